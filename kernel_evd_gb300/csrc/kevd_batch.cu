// Many uneven calibrations in one persistent launch.
//
// A batch of datasets (each its own X, N, d and eps sweep) is flattened into a
// device work queue of (dataset, tile range) items covering every dataset's
// lower-triangle 128 x 128 pair tiles.  One persistent grid (two CTAs per SM)
// takes items with an atomic counter, so the large datasets' items and the
// small datasets' items share the GPU without one launch per dataset and
// without idle SMs at the tail of a small dataset.  Each item writes its own
// FP64 partial per eps; a second kernel sums each dataset's items in item
// order, so the result does not depend on which CTA took which item.  The
// per-tile arithmetic is the single-dataset pass's (FP32 direct distances,
// ex2.approx, FP32 warp partials, FP64 accumulation).
//
// The launch sequence (counter reset, persistent kernel, reduction) has no host
// synchronisation or allocation once the queue is uploaded, so it can be
// captured in a CUDA graph and replayed.
#include "kevd_internal.cuh"
#include "kevd_pairtile.cuh"

#include <algorithm>
#include <cstring>
#include <vector>

namespace kevd {

namespace {

constexpr int kTile = 128;
constexpr int kMaxScalesB = 64;
constexpr int kMaxDB = 1024;

struct JobDesc {
    const float* X;
    int64_t N;
    int64_t n_tiles;
    int32_t d;
    int32_t n_scales;
    int32_t scale_off;   // into the flattened FP32 scale array (already x log2 e)
    int32_t item0;       // first item of the job
    int32_t n_items;
    int32_t pad;
};

struct Item {
    int32_t job;
    int32_t pad;
    int64_t t0, t1;      // tile range [t0, t1)
};

__device__ __forceinline__ float ex2f(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ void tile_ij(int64_t t, int64_t& ti, int64_t& tj) {
    int64_t i = (int64_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while (i * (i + 1) / 2 > t) --i;
    while ((i + 1) * (i + 2) / 2 <= t) ++i;
    ti = i;
    tj = t - i * (i + 1) / 2;
}

__global__ void __launch_bounds__(256, 2)
calibrate_queue_kernel(const JobDesc* __restrict__ jobs, const Item* __restrict__ items, int item_base,
                       int n_items, const float* __restrict__ c2all, int* __restrict__ counter,
                       double* __restrict__ partial) {
    extern __shared__ __align__(16) float sm[];
    float* xi = sm;
    float* xj = sm + kPtTile * kPtPitch;
    float* cs = xj + kPtTile * kPtPitch;     // kMaxScalesB
    float* red = cs + kMaxScalesB;           // 8 warps x kMaxScalesB
    __shared__ int cur;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    while (true) {
        __syncthreads();
        if (threadIdx.x == 0) cur = atomicAdd(counter, 1);
        __syncthreads();
        if (cur >= n_items) break;
        const int it = item_base + cur;
        const Item item = items[it];
        const JobDesc jb = jobs[item.job];
        const int d = jb.d, ns = jb.n_scales;
        for (int j = threadIdx.x; j < ns; j += blockDim.x) cs[j] = c2all[jb.scale_off + j];
        double acc = 0.0;   // thread j < ns owns eps j
        for (int64_t t = item.t0; t < item.t1; ++t) {
            int64_t ti, tj;
            tile_ij(t, ti, tj);
            float D[8][8];
            pt_dist(jb.X, jb.N, d, ti * kTile, tj * kTile, xi, xj, ty, tx, D);
            const int64_t gi0 = ti * kTile + ty, gj0 = tj * kTile + tx;
#pragma unroll
            for (int a = 0; a < 8; ++a)
#pragma unroll
                for (int b = 0; b < 8; ++b) {
                    const int64_t gi = gi0 + 16 * a, gj = gj0 + 16 * b;
                    if (!(gi < jb.N && gi > gj)) D[a][b] = __int_as_float(0x7f800000);
                }
            for (int j = 0; j < ns; ++j) {
                const float c = -cs[j];
                float s = 0.f;
#pragma unroll
                for (int a = 0; a < 8; ++a)
#pragma unroll
                    for (int b = 0; b < 8; ++b) s += ex2f(D[a][b] * c);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                if (lane == 0) red[warp * kMaxScalesB + j] = s;
            }
            __syncthreads();
            if (threadIdx.x < ns) {
                double w = 0.0;
#pragma unroll
                for (int q = 0; q < 8; ++q) w += (double)red[q * kMaxScalesB + threadIdx.x];
                acc += w;
            }
        }
        if (threadIdx.x < ns) partial[(int64_t)it * kMaxScalesB + threadIdx.x] = acc;
    }
}

__global__ void calibrate_queue_reduce_kernel(const JobDesc* __restrict__ jobs, int n_jobs,
                                              const double* __restrict__ partial, double* __restrict__ out) {
    const int job = blockIdx.x;
    if (job >= n_jobs) return;
    const JobDesc jb = jobs[job];
    for (int j = threadIdx.x; j < jb.n_scales; j += blockDim.x) {
        double s = 0.0;
        for (int q = 0; q < jb.n_items; ++q) s += partial[(int64_t)(jb.item0 + q) * kMaxScalesB + j];
        out[job * kMaxScalesB + j] = s;
    }
}

size_t queue_smem() {
    return (2 * kPtTile * (size_t)kPtPitch + kMaxScalesB + 8 * kMaxScalesB) * sizeof(float);
}

}  // namespace

int run_calibrate_batched(kevd_ctx* ctx, const kevd_calib_job* jobs, int n_jobs, int tiles_per_item,
                          cudaStream_t s) {
    if (!jobs || n_jobs < 1 || n_jobs > 4096 || tiles_per_item < 0)
        return set_error(ctx, KEVD_ERR_ARG, "calibrate_batched: need 1..4096 jobs");
    std::vector<JobDesc> hj(n_jobs);
    std::vector<Item> hi;
    std::vector<float> hc;
    int64_t total_tiles = 0;
    for (int q = 0; q < n_jobs; ++q) {
        const kevd_calib_job& j = jobs[q];
        if (!j.X || !j.scales || !j.sums || j.N < 1 || j.d < 1 || j.d > kMaxDB || j.n_scales < 1 ||
            j.n_scales > kMaxScalesB)
            return set_error(ctx, KEVD_ERR_ARG, "calibrate_batched: job %d needs N >= 1, 1 <= d <= %d, "
                             "1 <= n_scales <= %d", q, kMaxDB, kMaxScalesB);
        const int64_t nt = (j.N + kTile - 1) / kTile;
        total_tiles += nt * (nt + 1) / 2;
    }
    // item size: about 16 items per SM over the whole batch unless given
    int64_t per = tiles_per_item > 0 ? tiles_per_item
                                     : std::max<int64_t>(1, total_tiles / ((int64_t)ctx->num_sms * 16));
    // features are staged kPtChunk at a time, so shared memory does not depend on d
    // and one persistent launch serves every dataset of the batch
    std::vector<int> order(n_jobs);
    for (int q = 0; q < n_jobs; ++q) order[q] = q;
    for (int oi = 0; oi < n_jobs; ++oi) {
        const int q = order[oi];
        const kevd_calib_job& j = jobs[q];
        const int64_t nt = (j.N + kTile - 1) / kTile;
        const int64_t tiles = nt * (nt + 1) / 2;
        JobDesc& d = hj[q];
        d.X = j.X;
        d.N = j.N;
        d.n_tiles = tiles;
        d.d = j.d;
        d.n_scales = j.n_scales;
        d.scale_off = (int32_t)hc.size();
        d.item0 = (int32_t)hi.size();
        for (int e = 0; e < j.n_scales; ++e) {
            if (!(j.scales[e] > 0.0)) return set_error(ctx, KEVD_ERR_ARG, "calibrate_batched: scales must be positive");
            hc.push_back((float)(j.scales[e] * 1.4426950408889634));
        }
        for (int64_t t0 = 0; t0 < tiles; t0 += per) hi.push_back(Item{q, 0, t0, std::min(tiles, t0 + per)});
        d.n_items = (int32_t)hi.size() - d.item0;
        d.pad = 0;
    }
    if (hi.size() > (size_t)INT32_MAX / 2) return set_error(ctx, KEVD_ERR_ARG, "calibrate_batched: too many items");
    const int n_items = (int)hi.size();
    int st = KEVD_OK;
    JobDesc* dj = arena_get<JobDesc>(ctx, "cb.jobs", n_jobs, &st);
    Item* di = arena_get<Item>(ctx, "cb.items", n_items, &st);
    float* dc = arena_get<float>(ctx, "cb.c2", hc.size(), &st);
    int* counter = arena_get<int>(ctx, "cb.counter", 1, &st);
    double* partial = arena_get<double>(ctx, "cb.partial", (size_t)n_items * kMaxScalesB, &st);
    double* out = arena_get<double>(ctx, "cb.out", (size_t)n_jobs * kMaxScalesB, &st);
    if (st != KEVD_OK) return set_error(ctx, st, "calibrate_batched: out of device memory");
    KEVD_CUDA(ctx, cudaMemcpyAsync(dj, hj.data(), hj.size() * sizeof(JobDesc), cudaMemcpyHostToDevice, s));
    KEVD_CUDA(ctx, cudaMemcpyAsync(di, hi.data(), hi.size() * sizeof(Item), cudaMemcpyHostToDevice, s));
    KEVD_CUDA(ctx, cudaMemcpyAsync(dc, hc.data(), hc.size() * sizeof(float), cudaMemcpyHostToDevice, s));
    KEVD_CUDA(ctx, cudaMemsetAsync(counter, 0, sizeof(int), s));
    const size_t smem = queue_smem();
    KEVD_CUDA(ctx, raise_smem_limit(reinterpret_cast<const void*>(&calibrate_queue_kernel), (int)smem));
    {
        ProfScope ps(ctx, "calibrate_queue", s);
        calibrate_queue_kernel<<<ctx->num_sms * 2, 256, smem, s>>>(dj, di, 0, n_items, dc, counter, partial);
        KEVD_LAUNCH(ctx);
    }
    calibrate_queue_reduce_kernel<<<n_jobs, 64, 0, s>>>(dj, n_jobs, partial, out);
    KEVD_LAUNCH(ctx);
    std::vector<double> hout((size_t)n_jobs * kMaxScalesB);
    KEVD_CUDA(ctx, cudaMemcpyAsync(hout.data(), out, hout.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
    KEVD_CUDA(ctx, cudaStreamSynchronize(s));
    for (int q = 0; q < n_jobs; ++q)
        std::memcpy(jobs[q].sums, hout.data() + (size_t)q * kMaxScalesB, jobs[q].n_scales * sizeof(double));
    return KEVD_OK;
}

}  // namespace kevd
