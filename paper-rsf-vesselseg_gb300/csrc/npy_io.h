// npy_io.h -- minimal reader/writer of NumPy .npy files for 3-D volumes.
//
// The reference loads and saves its volumes with tiralib's load_npy/save_npy
// (CUDA_RSF/main.cpp:145,149,316).  Arrays are C order; a shape (L, H, W) has
// x fastest, the layout of the evolution.  Leading axes of length 1 are
// squeezed (U-Net outputs carry a channel axis).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace rsf {

struct NpyVolume {
    int64_t W = 0, H = 0, L = 0;
    bool is_u8 = false;             // the file held uint8 (kept as bytes)
    std::vector<uint8_t> u8;        // data when is_u8
    std::vector<float> f32;         // data otherwise, converted to float32
};

// Reads a .npy volume; returns an empty string on success, else the error.
std::string npy_load(const std::string &path, NpyVolume &out);
// Writes a float32 C-order (L, H, W) array.
std::string npy_save_f32(const std::string &path, const float *data, int64_t W, int64_t H, int64_t L);

}  // namespace rsf
