// rsf_cli.cpp -- `rsf3d`: evolves one volume from the command line.
//
// Drop-in for the reference's executable (CUDA_RSF/main.cpp): the same option
// names, defaults and meanings (main.cpp:86-99), long options only with
// unambiguous prefixes and `--name value` or `--name=value` (the Boost
// unix_style without short options, main.cpp:102-104), `--help` printing the
// option table and exiting with status 1 (main.cpp:107-110), phi0 built from
// the seed as sdf(seed - 13) (main.cpp:174-183), one "It takes X ms to
// calculate" line per iteration (main.cpp:296-307), phi saved as float32
// .npy (main.cpp:316).  The reference's --e weights both fitting terms and
// its epsilon is fixed at 0.2 (kernel.cu:214); --lambda1/--lambda2/--eps
// override them.  Where the reference would crash or read out of bounds
// (missing or mismatched input files, unknown options) this tool prints the
// problem and exits with status 2 (usage) or 3 (runtime).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "npy_io.h"
#include "rsf.h"

namespace {

struct Option {
    const char *name;
    bool takes_value;
    const char *def;
    const char *help;
};

const Option kOptions[] = {
    {"help", false, nullptr, "produce help message"},
    {"sigma", true, "5", "blur kernel for the fitting term (in pixels)"},
    {"t", true, "30", "total number of time steps"},
    {"dt", true, "0.1", "time step size"},
    {"meu", true, "1", "weight for the regularization term"},
    {"e", true, "0.1", "weight for the fitting term (lambda1 = lambda2 = e)"},
    {"v", true, "0.0001", "weight for the smoothing term"},
    {"sigma2", true, "0", "weight for sigma2 (box radius (int)sigma2 of the e-term, 0..8)"},
    {"binary", true, nullptr, "binary seed surface (.npy)"},
    {"image", true, nullptr, "input image filename (.npy)"},
    {"ouput", true, "out.npy", "output level set (.npy)"},
    {"output", true, nullptr, "same as --ouput"},
    {"debug", false, nullptr, "output all debugging details"},
    {"eps", true, "0.2", "width of the regularised Heaviside (fixed at 0.2 in the reference)"},
    {"lambda1", true, nullptr, "weight of the outside fitting term (default: e)"},
    {"lambda2", true, nullptr, "weight of the inside fitting term (default: e)"},
    {"threshold", true, "13", "seed level: voxels with seed > threshold are inside"},
    {"boundary", true, "reference", "derivative boundary rule: reference | clamp"},
    {"arith", true, "portable", "arithmetic: portable (bit-exact with the CPU oracle) | reference"},
    {"data-term", true, "reference", "data term: reference ((I - f)^2 as kernel.cu) | gaussian (expanded RSF form)"},
    {"device", true, "0", "CUDA device ordinal"},
    {"quiet", false, nullptr, "one timing line for the whole evolution instead of one per step"},
};
constexpr int kNumOptions = sizeof(kOptions) / sizeof(kOptions[0]);

int canonical_ouput() {
    for (int i = 0; i < kNumOptions; i++)
        if (std::strcmp(kOptions[i].name, "ouput") == 0) return i;
    return -1;
}

void usage(FILE *out) {
    std::fprintf(out, "Allowed options:\n");
    for (const Option &o : kOptions) {
        std::string lhs = std::string("  --") + o.name;
        if (o.takes_value) lhs += o.def ? std::string(" arg (=") + o.def + ")" : std::string(" arg");
        std::fprintf(out, "%-30s %s\n", lhs.c_str(), o.help);
    }
}

// --output is another spelling of --ouput: both land on --ouput.
int canonical(int i) { return std::strcmp(kOptions[i].name, "output") == 0 ? canonical_ouput() : i; }

// Exact name first, then a unique prefix; -1 when unknown, -2 when ambiguous.
int find_option(const std::string &name) {
    for (int i = 0; i < kNumOptions; i++)
        if (name == kOptions[i].name) return canonical(i);
    int hit = -1;
    for (int i = 0; i < kNumOptions; i++) {
        if (std::strncmp(kOptions[i].name, name.c_str(), name.size()) == 0) {
            if (hit >= 0 && hit != canonical(i)) return -2;
            hit = canonical(i);
        }
    }
    return hit;
}

bool parse_float(const std::string &s, float &out) {
    char *end = nullptr;
    const float v = std::strtof(s.c_str(), &end);  // decimal to float in one rounding
    if (s.empty() || *end != '\0') return false;
    out = v;
    return true;
}

bool parse_int(const std::string &s, int &out) {
    char *end = nullptr;
    const long v = std::strtol(s.c_str(), &end, 10);
    if (s.empty() || *end != '\0' || v < -2147483647L || v > 2147483647L) return false;
    out = (int)v;
    return true;
}

int fail_rsf(rsf_status s, const char *what) {
    std::fprintf(stderr, "rsf3d: %s: %s (%s)\n", what, rsf_status_string(s), rsf_last_error());
    return 3;
}

int fail_cuda(cudaError_t e, const char *what) {
    std::fprintf(stderr, "rsf3d: %s: %s\n", what, cudaGetErrorString(e));
    return 3;
}

}  // namespace

int main(int argc, char **argv) {
    std::vector<std::string> value(kNumOptions);
    std::vector<bool> given(kNumOptions, false);
    for (int i = 0; i < kNumOptions; i++)
        if (kOptions[i].def) value[i] = kOptions[i].def;
    for (int a = 1; a < argc; a++) {
        std::string tok = argv[a];
        if (tok.size() < 3 || tok.compare(0, 2, "--") != 0) {
            std::fprintf(stderr, "rsf3d: unexpected argument '%s' (options are --name value)\n", tok.c_str());
            return 2;
        }
        std::string name = tok.substr(2), val;
        bool has_val = false;
        const size_t eq = name.find('=');
        if (eq != std::string::npos) {
            val = name.substr(eq + 1);
            name = name.substr(0, eq);
            has_val = true;
        }
        const int id = find_option(name);
        if (id == -2) {
            std::fprintf(stderr, "rsf3d: option '--%s' is ambiguous\n", name.c_str());
            return 2;
        }
        if (id < 0) {
            std::fprintf(stderr, "rsf3d: unrecognised option '--%s'\n", name.c_str());
            return 2;
        }
        if (kOptions[id].takes_value && !has_val) {
            if (a + 1 >= argc) {
                std::fprintf(stderr, "rsf3d: option '--%s' needs a value\n", kOptions[id].name);
                return 2;
            }
            val = argv[++a];
        } else if (!kOptions[id].takes_value && has_val) {
            std::fprintf(stderr, "rsf3d: option '--%s' takes no value\n", kOptions[id].name);
            return 2;
        }
        value[id] = val;
        given[id] = true;
    }
    auto idx = [](const char *n) { return find_option(n); };
    if (given[idx("help")]) {
        usage(stdout);
        return 1;
    }
    const bool debug = given[idx("debug")];
    const bool quiet = given[idx("quiet")];

    rsf_params p;
    rsf_params_default(&p);
    int T = 0, device = 0;
    float e = 0.0f;
    bool ok = parse_float(value[idx("sigma")], p.sigma) && parse_int(value[idx("t")], T) &&
              parse_float(value[idx("dt")], p.dt) && parse_float(value[idx("meu")], p.mu) &&
              parse_float(value[idx("e")], e) && parse_float(value[idx("v")], p.nu) &&
              parse_float(value[idx("sigma2")], p.sigma2) && parse_float(value[idx("eps")], p.eps) &&
              parse_int(value[idx("device")], device);
    float threshold = 13.0f;
    ok = ok && parse_float(value[idx("threshold")], threshold);
    p.lambda1 = p.lambda2 = e;
    if (ok && given[idx("lambda1")]) ok = parse_float(value[idx("lambda1")], p.lambda1);
    if (ok && given[idx("lambda2")]) ok = parse_float(value[idx("lambda2")], p.lambda2);
    if (!ok) {
        std::fprintf(stderr, "rsf3d: a numeric option has a malformed value\n");
        return 2;
    }
    if (T < 0) {
        std::fprintf(stderr, "rsf3d: --t must be >= 0\n");
        return 2;
    }
    const std::string &bnd = value[idx("boundary")], &arith = value[idx("arith")];
    if (bnd == "reference") p.boundary = RSF_BOUNDARY_REFERENCE;
    else if (bnd == "clamp") p.boundary = RSF_BOUNDARY_CLAMP;
    else {
        std::fprintf(stderr, "rsf3d: --boundary must be reference or clamp\n");
        return 2;
    }
    const std::string &dterm = value[idx("data-term")];
    if (dterm == "reference") p.data_term = RSF_DATA_TERM_REFERENCE;
    else if (dterm == "gaussian") p.data_term = RSF_DATA_TERM_GAUSSIAN;
    else {
        std::fprintf(stderr, "rsf3d: --data-term must be reference or gaussian\n");
        return 2;
    }
    if (arith == "portable") p.arith = RSF_ARITH_PORTABLE;
    else if (arith == "reference") p.arith = RSF_ARITH_REFERENCE;
    else {
        std::fprintf(stderr, "rsf3d: --arith must be portable or reference\n");
        return 2;
    }
    if (!given[idx("image")] || !given[idx("binary")]) {
        std::fprintf(stderr, "rsf3d: --image and --binary are required (see --help)\n");
        return 2;
    }
    const std::string &out_path = value[idx("ouput")];

    rsf::NpyVolume img, seed;
    std::string err = rsf::npy_load(value[idx("image")], img);
    if (err.empty()) err = rsf::npy_load(value[idx("binary")], seed);
    if (!err.empty()) {
        std::fprintf(stderr, "rsf3d: %s\n", err.c_str());
        return 3;
    }
    if (img.W != seed.W || img.H != seed.H || img.L != seed.L) {
        std::fprintf(stderr, "rsf3d: image (%lld x %lld x %lld) and seed (%lld x %lld x %lld) differ in shape\n",
                     (long long)img.W, (long long)img.H, (long long)img.L, (long long)seed.W, (long long)seed.H,
                     (long long)seed.L);
        return 3;
    }
    const int64_t W = img.W, H = img.H, L = img.L, N = W * H * L;
    if (debug) {
        std::printf("volume %lld x %lld x %lld (%s image), %d steps\n", (long long)W, (long long)H, (long long)L,
                    img.is_u8 ? "uint8" : "float32", T);
        std::printf("sigma %g dt %g mu %g lambda1 %g lambda2 %g nu %g eps %g sigma2 %g threshold %g\n", p.sigma, p.dt,
                    p.mu, p.lambda1, p.lambda2, p.nu, p.eps, p.sigma2, threshold);
    }

    cudaError_t ce = cudaSetDevice(device);
    if (ce != cudaSuccess) return fail_cuda(ce, "cudaSetDevice");
    rsf_workspace *ws = nullptr;
    rsf_status s = rsf_workspace_create(N, 1, &ws);
    if (s != RSF_OK) return fail_rsf(s, "workspace");
    const rsf_dtype img_dt = img.is_u8 ? RSF_U8 : RSF_F32;
    const rsf_dtype seed_dt = seed.is_u8 ? RSF_U8 : RSF_F32;
    const size_t img_bytes = (size_t)N * (img.is_u8 ? 1 : 4), seed_bytes = (size_t)N * (seed.is_u8 ? 1 : 4);
    void *d_img = nullptr, *d_seed = nullptr;
    float *d_phi = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int rc = 0;
    std::vector<float> phi;
    ce = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (ce == cudaSuccess) ce = cudaEventCreate(&ev0);
    if (ce == cudaSuccess) ce = cudaEventCreate(&ev1);
    if (ce == cudaSuccess) ce = cudaMalloc(&d_img, img_bytes);
    if (ce == cudaSuccess) ce = cudaMalloc(&d_seed, seed_bytes);
    if (ce == cudaSuccess) ce = cudaMalloc((void **)&d_phi, (size_t)N * sizeof(float));
    if (ce == cudaSuccess)
        ce = cudaMemcpyAsync(d_img, img.is_u8 ? (const void *)img.u8.data() : (const void *)img.f32.data(), img_bytes,
                             cudaMemcpyHostToDevice, st);
    if (ce == cudaSuccess)
        ce = cudaMemcpyAsync(d_seed, seed.is_u8 ? (const void *)seed.u8.data() : (const void *)seed.f32.data(),
                             seed_bytes, cudaMemcpyHostToDevice, st);
    if (ce != cudaSuccess) {
        rc = fail_cuda(ce, "device buffers");
        goto done;
    }
    s = rsf_signed_distance(ws, d_seed, seed_dt, threshold, d_phi, W, H, L, st);
    if (s != RSF_OK) {
        rc = fail_rsf(s, "initial level set");
        goto done;
    }
    if (debug && (s = rsf_set_kernel_timing(ws, 1)) != RSF_OK) {
        rc = fail_rsf(s, "kernel timing");
        goto done;
    }
    {
        const int chunks = quiet ? (T > 0 ? 1 : 0) : T;
        for (int c = 0; c < chunks; c++) {
            const int iters = quiet ? T : 1;
            cudaEventRecord(ev0, st);
            s = rsf_evolve(ws, &p, d_img, img_dt, d_phi, W, H, L, iters, st);
            if (s != RSF_OK) {
                rc = fail_rsf(s, "evolution");
                goto done;
            }
            cudaEventRecord(ev1, st);
            ce = cudaEventSynchronize(ev1);
            if (ce != cudaSuccess) {
                rc = fail_cuda(ce, "evolution");
                goto done;
            }
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, ev0, ev1);
            std::printf("It takes %g ms to calculate \n", ms);
        }
    }
    s = rsf_workspace_check(ws, st);
    if (s != RSF_OK) {
        rc = fail_rsf(s, "evolution");
        goto done;
    }
    if (debug) {
        double ms[4] = {0, 0, 0, 0};
        int64_t n[4] = {0, 0, 0, 0};
        if (rsf_kernel_times(ws, ms, n, 0) == RSF_OK) {
            const char *names[4] = {"x-pass", "y-pass", "z-pass", "stencil/update"};
            for (int k = 0; k < 4; k++)
                std::printf("%-15s %10.3f ms over %lld launches\n", names[k], ms[k], (long long)n[k]);
        }
    }
    phi.resize((size_t)N);
    ce = cudaMemcpy(phi.data(), d_phi, (size_t)N * sizeof(float), cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) {
        rc = fail_cuda(ce, "read back");
        goto done;
    }
    err = rsf::npy_save_f32(out_path, phi.data(), W, H, L);
    if (!err.empty()) {
        std::fprintf(stderr, "rsf3d: %s\n", err.c_str());
        rc = 3;
    }
done:
    cudaFree(d_img);
    cudaFree(d_seed);
    cudaFree(d_phi);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (st) cudaStreamDestroy(st);
    rsf_workspace_destroy(ws);
    return rc;
}
