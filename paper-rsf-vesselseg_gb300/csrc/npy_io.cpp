// npy_io.cpp -- .npy format version 1.0 - 3.0: magic "\x93NUMPY", version,
// header length (2 bytes for 1.0, 4 bytes after), a Python dict literal with
// 'descr', 'fortran_order' and 'shape', then the raw data.
#include "npy_io.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

namespace rsf {
namespace {

std::string dict_value(const std::string &hdr, const std::string &key) {
    const size_t k = hdr.find("'" + key + "'");
    if (k == std::string::npos) return "";
    size_t c = hdr.find(':', k);
    if (c == std::string::npos) return "";
    ++c;
    while (c < hdr.size() && hdr[c] == ' ') ++c;
    if (c >= hdr.size()) return "";
    if (hdr[c] == '\'') {
        const size_t e = hdr.find('\'', c + 1);
        return e == std::string::npos ? "" : hdr.substr(c + 1, e - c - 1);
    }
    if (hdr[c] == '(') {
        const size_t e = hdr.find(')', c);
        return e == std::string::npos ? "" : hdr.substr(c, e - c + 1);
    }
    size_t e = c;
    while (e < hdr.size() && hdr[e] != ',' && hdr[e] != '}') ++e;
    return hdr.substr(c, e - c);
}

template <typename T>
void convert(const std::vector<char> &raw, size_t n, std::vector<float> &out) {
    out.resize(n);
    for (size_t i = 0; i < n; i++) {
        T v;
        std::memcpy(&v, raw.data() + i * sizeof(T), sizeof(T));
        out[i] = (float)v;
    }
}

}  // namespace

std::string npy_load(const std::string &path, NpyVolume &out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return "cannot open " + path;
    char magic[6];
    if (!f.read(magic, 6) || std::memcmp(magic, "\x93NUMPY", 6) != 0) return path + ": not a .npy file";
    unsigned char ver[2];
    if (!f.read(reinterpret_cast<char *>(ver), 2)) return path + ": truncated header";
    uint32_t hlen = 0;
    if (ver[0] == 1) {
        unsigned char b[2];
        if (!f.read(reinterpret_cast<char *>(b), 2)) return path + ": truncated header";
        hlen = b[0] | (b[1] << 8);
    } else if (ver[0] == 2 || ver[0] == 3) {
        unsigned char b[4];
        if (!f.read(reinterpret_cast<char *>(b), 4)) return path + ": truncated header";
        hlen = b[0] | (b[1] << 8) | (b[2] << 16) | ((uint32_t)b[3] << 24);
    } else {
        return path + ": unsupported .npy version";
    }
    if (hlen > (1u << 20)) return path + ": header too long";
    std::string hdr(hlen, '\0');
    if (!f.read(&hdr[0], hlen)) return path + ": truncated header";
    const std::string descr = dict_value(hdr, "descr");
    const std::string fortran = dict_value(hdr, "fortran_order");
    const std::string shape = dict_value(hdr, "shape");
    if (descr.empty() || shape.empty()) return path + ": malformed header";
    std::vector<int64_t> dims;
    {
        std::string s = shape.substr(1, shape.size() - 2);
        std::stringstream ss(s);
        std::string tok;
        while (std::getline(ss, tok, ',')) {
            size_t a = tok.find_first_not_of(' ');
            if (a == std::string::npos) continue;
            char *end = nullptr;
            const long long d = std::strtoll(tok.c_str() + a, &end, 10);
            while (end && *end == ' ') ++end;
            if (!end || end == tok.c_str() + a || (*end != '\0' && *end != 'L')) return path + ": malformed shape";
            dims.push_back((int64_t)d);
        }
    }
    while (dims.size() > 3 && dims.front() == 1) dims.erase(dims.begin());
    if (dims.size() != 3) return path + ": expected a 3-D array";
    for (int64_t d : dims)
        if (d < 1) return path + ": empty array";
        else if (d > (int64_t(1) << 31)) return path + ": extent too large";
    if (dims[0] * dims[1] > (int64_t(1) << 40) / dims[2]) return path + ": array too large";
    const size_t n = (size_t)(dims[0] * dims[1] * dims[2]);
    const bool fortran_order = fortran.find("True") != std::string::npos;
    const char endian = descr[0];
    const char kind = descr.size() > 1 ? descr[1] : '?';
    const int size = descr.size() > 2 ? std::atoi(descr.c_str() + 2) : 0;
    if (endian == '>' && size > 1) return path + ": big-endian data is not supported";
    if (size < 1 || size > 8) return path + ": unsupported dtype " + descr;
    std::vector<char> raw(n * (size_t)size);
    if (!f.read(raw.data(), (std::streamsize)raw.size())) return path + ": truncated data";
    out.L = dims[0];
    out.H = dims[1];
    out.W = dims[2];
    out.is_u8 = kind == 'u' && size == 1;
    if (out.is_u8) {
        out.u8.assign(raw.begin(), raw.end());
    } else if (kind == 'f' && size == 4) {
        convert<float>(raw, n, out.f32);
    } else if (kind == 'f' && size == 8) {
        convert<double>(raw, n, out.f32);
    } else if (kind == 'i' && size == 1) {
        convert<int8_t>(raw, n, out.f32);
    } else if (kind == 'i' && size == 2) {
        convert<int16_t>(raw, n, out.f32);
    } else if (kind == 'u' && size == 2) {
        convert<uint16_t>(raw, n, out.f32);
    } else if (kind == 'i' && size == 4) {
        convert<int32_t>(raw, n, out.f32);
    } else if (kind == 'u' && size == 4) {
        convert<uint32_t>(raw, n, out.f32);
    } else if (kind == 'i' && size == 8) {
        convert<int64_t>(raw, n, out.f32);
    } else if (kind == 'b' && size == 1) {
        convert<uint8_t>(raw, n, out.f32);
    } else {
        return path + ": unsupported dtype " + descr;
    }
    if (fortran_order) {  // element (z, y, x) is at x*L*H + y*L + z: transpose to C order
        const int64_t L = out.L, H = out.H, W = out.W;
        if (out.is_u8) {
            std::vector<uint8_t> t(n);
            for (int64_t z = 0; z < L; z++)
                for (int64_t y = 0; y < H; y++)
                    for (int64_t x = 0; x < W; x++) t[(z * H + y) * W + x] = out.u8[(x * H + y) * L + z];
            out.u8.swap(t);
        } else {
            std::vector<float> t(n);
            for (int64_t z = 0; z < L; z++)
                for (int64_t y = 0; y < H; y++)
                    for (int64_t x = 0; x < W; x++) t[(z * H + y) * W + x] = out.f32[(x * H + y) * L + z];
            out.f32.swap(t);
        }
    }
    return "";
}

std::string npy_save_f32(const std::string &path, const float *data, int64_t W, int64_t H, int64_t L) {
    std::string hdr = "{'descr': '<f4', 'fortran_order': False, 'shape': (" + std::to_string(L) + ", " +
                      std::to_string(H) + ", " + std::to_string(W) + "), }";
    // pad so that magic + version + length + header is a multiple of 64 bytes
    const size_t total = 10 + hdr.size() + 1;
    hdr.append((64 - total % 64) % 64, ' ');
    hdr.push_back('\n');
    std::ofstream f(path, std::ios::binary);
    if (!f) return "cannot write " + path;
    const unsigned char head[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
    f.write(reinterpret_cast<const char *>(head), 8);
    const unsigned char len[2] = {(unsigned char)(hdr.size() & 0xff), (unsigned char)(hdr.size() >> 8)};
    f.write(reinterpret_cast<const char *>(len), 2);
    f.write(hdr.data(), (std::streamsize)hdr.size());
    f.write(reinterpret_cast<const char *>(data), (std::streamsize)(sizeof(float) * (size_t)(W * H * L)));
    return f ? "" : "write failed: " + path;
}

}  // namespace rsf
