// Shared helpers of the three stage drivers: the reference's HDF5 datasets read and
// written through libkevdh5 (include/kevd_h5.h; libhdf5 is not needed), and CUDA /
// library checks that exit the way the reference programs do.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "kevd.h"
#include "kevd_h5.h"

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

// An HDF5 failure ends the program, as the reference's assert on every H5 call does.
#define DRV_H5(x)                                                   \
    do {                                                            \
        if ((x) != KEVD_H5_OK) {                                    \
            fprintf(stderr, "HDF5: %s\n", kevd_h5_last_error());   \
            exit(1);                                                \
        }                                                           \
    } while (0)

// Device memory in use at a labelled point, in the reference's format
// (ks_kevd.cu:98-110 mem_probe; one device, so always rank 0).
inline void mem_probe(const char* label) {
    DRV_CUDA(cudaDeviceSynchronize());
    size_t freeb = 0, totalb = 0;
    DRV_CUDA(cudaMemGetInfo(&freeb, &totalb));
    const double gib = 1024.0 * 1024.0 * 1024.0;
    printf("MEM[%-10s] rank 0: used %.3f GiB  free %.3f GiB\n", label, (double)(totalb - freeb) / gib,
           (double)freeb / gib);
    fflush(stdout);
}

template <typename T>
constexpr int32_t h5_type();
template <>
constexpr int32_t h5_type<float>() { return KEVD_H5_F32; }
template <>
constexpr int32_t h5_type<double>() { return KEVD_H5_F64; }
template <>
constexpr int32_t h5_type<uint64_t>() { return KEVD_H5_U64; }
template <>
constexpr int32_t h5_type<int64_t>() { return KEVD_H5_I64; }

// `count` elements of dataset `dset`, converted to T (ks_bandwidth.cu:51-83 h5read,
// ks_kevd.cu:134-243 h5read_float / h5read_double / h5read_sizet).
template <typename T>
std::vector<T> h5_read(const char* path, const char* dset, size_t count) {
    std::vector<T> v(count);
    DRV_H5(kevd_h5_read(path, dset, h5_type<T>(), v.data(), (int64_t)count));
    return v;
}

// Number of elements of a dataset (ks_kevd.cu:113-132 h5_num_elements).
inline size_t h5_count(const char* path, const char* dset) {
    int64_t n = 0;
    DRV_H5(kevd_h5_dataset_info(path, dset, &n, nullptr, nullptr, nullptr));
    return (size_t)n;
}

// A new file holding one dataset (ks_arpclm.cu:121-172 h5write_sizet / h5write_double).
template <typename T>
void h5_write_one(const char* path, const char* dset, const T* v, size_t count) {
    DRV_H5(kevd_h5_create(path));
    DRV_H5(kevd_h5_append(path, dset, h5_type<T>(), v, (int64_t)count));
}

// One more dataset in an existing file (ks_kevd.cu:247-290 h5add_double / h5add_float).
template <typename T>
void h5_add(const char* path, const char* dset, const T* v, size_t count) {
    DRV_H5(kevd_h5_append(path, dset, h5_type<T>(), v, (int64_t)count));
}
