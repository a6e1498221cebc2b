// Shared helpers of the three stage drivers: raw little-endian array files in
// place of the reference's HDF5 datasets (libhdf5 is not available here), the
// same path names with ".bin" for ".h5", and CUDA / library checks that exit
// the way the reference programs do.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "kevd.h"

#define DRV_CUDA(x)                                                                       \
    do {                                                                                  \
        cudaError_t e_ = (x);                                                             \
        if (e_ != cudaSuccess) {                                                          \
            fprintf(stderr, "CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, \
                    __LINE__);                                                            \
            exit(1);                                                                      \
        }                                                                                 \
    } while (0)

#define DRV_KEVD(ctx, x)                                                                   \
    do {                                                                                   \
        int s_ = (x);                                                                      \
        if (s_ != KEVD_OK) {                                                               \
            fprintf(stderr, "%s: %s\n", kevd_status_name(s_), kevd_last_error(ctx));       \
            exit(s_);                                                                      \
        }                                                                                  \
    } while (0)

template <typename T>
std::vector<T> read_array(const char* path, size_t count) {
    std::vector<T> v(count);
    FILE* f = fopen(path, "rb");
    if (!f) {
        fprintf(stderr, "cannot open %s\n", path);
        exit(1);
    }
    if (fread(v.data(), sizeof(T), count, f) != count) {
        fprintf(stderr, "%s: expected %zu values\n", path, count);
        exit(1);
    }
    fclose(f);
    return v;
}

// Number of T values in a file.
template <typename T>
size_t array_length(const char* path) {
    FILE* f = fopen(path, "rb");
    if (!f) {
        fprintf(stderr, "cannot open %s\n", path);
        exit(1);
    }
    fseek(f, 0, SEEK_END);
    const long n = ftell(f);
    fclose(f);
    return (size_t)n / sizeof(T);
}

template <typename T>
void write_array(const char* path, const T* v, size_t count) {
    FILE* f = fopen(path, "wb");
    if (!f || fwrite(v, sizeof(T), count, f) != count) {
        fprintf(stderr, "cannot write %s\n", path);
        exit(1);
    }
    fclose(f);
}
