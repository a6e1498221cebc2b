// FP32 squared distances of a 128 x 128 pair tile, shared by the calibration
// kernels (single dataset, batched work queue) and the pair-distance median.
// Thread (ty, tx) of a 16 x 16 CTA computes rows ri0 + ty + 16a (a < 8)
// against rows rj0 + tx + 16b (b < 8), each distance summed over the features
// in increasing order.  Features are staged 64 at a time with a row pitch of
// 66 floats: a thread reads two features of a row in one 8-byte shared load
// (16 loads per 256 FP32 operations, twice the work per load of 4-byte
// loads; 16-byte loads would need 32 more registers than the 128 that two
// CTAs per SM allow), and the 16 row addresses of a half-warp's loads fall in
// distinct banks.  A ragged last chunk is padded with a zero in both tiles,
// which adds an exact zero.
#pragma once

#include <cstdint>

namespace kevd {

constexpr int kPtTile = 128;
constexpr int kPtChunk = 64;
constexpr int kPtPitch = kPtChunk + 2;

// Stage features [c0, c0 + w) of rows [r0, r0 + 128) (zeros past N and past w,
// up to w rounded up to 2) into dst[128][kPtPitch].
__device__ __forceinline__ void pt_stage(const float* __restrict__ X, int64_t N, int d, int64_t r0, int c0, int w,
                                         float* dst) {
    const int w2 = (w + 1) & ~1;
    const bool vec = (d & 1) == 0 && ((uintptr_t)X & 7) == 0;
    if (vec) {
        const int nq = w2 >> 1;
        for (int e = threadIdx.x; e < kPtTile * nq; e += blockDim.x) {
            const int rr = e / nq, k2 = (e - rr * nq) << 1;
            const int64_t r = r0 + rr;
            const float2 v = (r < N) ? __ldg(reinterpret_cast<const float2*>(X + r * d + c0 + k2))
                                     : make_float2(0.f, 0.f);
            *reinterpret_cast<float2*>(dst + rr * kPtPitch + k2) = v;
        }
    } else {
        for (int e = threadIdx.x; e < kPtTile * w2; e += blockDim.x) {
            const int rr = e / w2, kk = e - rr * w2;
            const int64_t r = r0 + rr;
            dst[rr * kPtPitch + kk] = (r < N && kk < w) ? X[r * d + c0 + kk] : 0.f;
        }
    }
}

// D[a][b] = ||x_{ri0+ty+16a} - x_{rj0+tx+16b}||^2 (FP32).  Called by all 256
// threads of the CTA; xi, xj: 128 x kPtPitch floats each, 8-byte aligned.
__device__ __forceinline__ void pt_dist(const float* __restrict__ X, int64_t N, int d, int64_t ri0, int64_t rj0,
                                        float* xi, float* xj, int ty, int tx, float (&D)[8][8]) {
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int b = 0; b < 8; ++b) D[a][b] = 0.f;
    for (int c0 = 0; c0 < d; c0 += kPtChunk) {
        const int w = min(kPtChunk, d - c0);
        const int w2 = (w + 1) & ~1;
        __syncthreads();
        pt_stage(X, N, d, ri0, c0, w, xi);
        pt_stage(X, N, d, rj0, c0, w, xj);
        __syncthreads();
        for (int k = 0; k < w2; k += 2) {
            float2 vi[8], vj[8];
#pragma unroll
            for (int a = 0; a < 8; ++a) vi[a] = *reinterpret_cast<const float2*>(xi + (ty + 16 * a) * kPtPitch + k);
#pragma unroll
            for (int b = 0; b < 8; ++b) vj[b] = *reinterpret_cast<const float2*>(xj + (tx + 16 * b) * kPtPitch + k);
#pragma unroll
            for (int a = 0; a < 8; ++a)
#pragma unroll
                for (int b = 0; b < 8; ++b) {
                    float u = vi[a].x - vj[b].x;
                    D[a][b] = fmaf(u, u, D[a][b]);
                    u = vi[a].y - vj[b].y;
                    D[a][b] = fmaf(u, u, D[a][b]);
                }
        }
    }
}

}  // namespace kevd
