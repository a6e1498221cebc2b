// Stage 2 driver (the reference's ./cuarpclm, ks_arpclm.cu:566-1152): block
// RPCholesky of the delay-embedded samples; writes L^{-1} and the pivot set
// and prints the per-round table.  Compile-time configuration as in the
// reference (ks_arpclm.cu:38, :587-602: L = 30 pi, 128 gridpoints, 32,831
// snapshots, Nq = 64, BLK = 512, bw = 0.8) except the round count: the
// reference's 64 rounds (rank 32,768) would need a 550 GB stored factor, so 8
// rounds (rank 4,096, 69 GB in FP32) are the default; the mixed form (FP32
// factor) stands for the reference's FP32 update; override with -D, or at run
// time with the flags of driver_args.h (none given: the configuration above).
#include <ctime>

#include "driver_args.h"
#include "driver_io.h"

#ifndef LFACT
#define LFACT 30
#endif
#ifndef MGRID
#define MGRID 128
#endif
#ifndef NDATA
#define NDATA 32831
#endif
#ifndef NQ
#define NQ 64
#endif
#ifndef BLK
#define BLK 512
#endif
#ifndef NROUNDS
#define NROUNDS 8
#endif
#ifndef BW
#define BW 0.8
#endif
#ifndef PRECISION
#define PRECISION KEVD_MIXED
#endif

int main(int argc, char** argv) {
    const time_t t0 = time(nullptr);
    DriverConfig cfg("cuarpclm", {{"lfact", LFACT, DriverSetting::kInt, "domain length factor in the file names"},
                                  {"mgrid", MGRID, DriverSetting::kInt, "gridpoints per snapshot"},
                                  {"ndata", NDATA, DriverSetting::kInt, "snapshots"},
                                  {"nq", NQ, DriverSetting::kInt, "delay window"},
                                  {"blk", BLK, DriverSetting::kInt, "proposals per round (1..512)"},
                                  {"nrounds", NROUNDS, DriverSetting::kInt, "rounds (rank <= blk x nrounds)"},
                                  {"bw", BW, DriverSetting::kReal, "bandwidth (scale 1 / (nq bw))"},
                                  {"precision", PRECISION == KEVD_FP64 ? 0 : 1, DriverSetting::kPrecision,
                                   "fp64 or mixed (FP32 factor)"}});
    cfg.parse(argc, argv);
    const size_t Lfact = cfg.size("lfact"), M = cfg.size("mgrid"), Ndata = cfg.size("ndata"), Nq = cfg.size("nq"),
                 Nrounds = cfg.size("nrounds");
    const int blk = cfg.integer("blk");
    const double bw = cfg.get("bw");
    const int32_t precision = cfg.get("precision") == 0 ? KEVD_FP64 : KEVD_MIXED;
    if (Nq < 1 || Nq > Ndata || M < 1 || blk < 1 || Nrounds < 1 || !(bw > 0)) {
        fprintf(stderr, "cuarpclm: need 1 <= nq <= ndata, mgrid, blk, nrounds >= 1 and bw > 0\n");
        return 2;
    }
    const size_t N = Ndata - Nq + 1, NM = N * M, rmax = Nrounds * (size_t)blk;
    char fname[256], linv_file[256], spiv_file[256];
    snprintf(fname, sizeof(fname), "data/ks_true_%zu_%zu_%zu_u32.h5", Ndata, M, Lfact);
    snprintf(linv_file, sizeof(linv_file), "data/linv_%zu_%zu_b%d_r%zu_%zu.h5", N, M, blk, Nrounds, Lfact);
    snprintf(spiv_file, sizeof(spiv_file), "data/spiv_%zu_%zu_b%d_r%zu_%zu.h5", N, M, blk, Nrounds, Lfact);
    if (cfg.print_only) {
        cfg.print(stdout);
        printf("input = %s:/u\noutput = %s:/linv\noutput = %s:/spiv\n", fname, linv_file, spiv_file);
        return 0;
    }
    printf("Data file: %s\nData set: u\n", fname);
    printf("Block size: %d  Devices: 1  Rows/device: %zu  Cols/device: %zu\n\n", blk, NM, rmax);
    std::vector<float> u = h5_read<float>(fname, "/u", Ndata * M);

    kevd_ctx* ctx = nullptr;
    if (kevd_ctx_create(0, &ctx) != KEVD_OK) {
        fprintf(stderr, "no CUDA device\n");
        return 1;
    }
    float *u_dev = nullptr, *X_dev = nullptr;
    void* F = nullptr;
    const size_t fsz = (precision == KEVD_FP64) ? sizeof(double) : sizeof(float);
    DRV_CUDA(cudaMalloc(&u_dev, u.size() * sizeof(float)));
    DRV_CUDA(cudaMalloc(&X_dev, NM * Nq * sizeof(float)));
    DRV_CUDA(cudaMalloc(&F, NM * rmax * fsz));
    DRV_CUDA(cudaMemcpy(u_dev, u.data(), u.size() * sizeof(float), cudaMemcpyHostToDevice));
    DRV_KEVD(ctx, kevd_hankel_rows(ctx, u_dev, (int64_t)Ndata, (int64_t)M, (int64_t)Nq, X_dev, nullptr));

    kevd_rpchol_params p = {};
    p.k_max = (int64_t)rmax;
    p.block = blk;
    p.max_rounds = (int32_t)Nrounds;
    p.tol = 1e-10;
    p.seed = 1234;
    p.precision = precision;
    std::vector<int64_t> spiv(rmax);
    std::vector<double> err(Nrounds);
    std::vector<int32_t> hm(Nrounds);
    kevd_rpchol_result res = {};
    DRV_KEVD(ctx, kevd_rpchol(ctx, X_dev, (int64_t)NM, (int32_t)Nq, 1.0 / ((double)Nq * bw), &p, F, (int64_t)rmax,
                              spiv.data(), err.data(), hm.data(), &res, nullptr));
    const size_t Nr = (size_t)res.rank;
    std::vector<double> linv(Nr * Nr);
    DRV_KEVD(ctx, kevd_linv_from_factor(ctx, F, precision, (int64_t)rmax, spiv.data(), (int64_t)Nr, linv.data(),
                                        nullptr));
    h5_write_one(linv_file, "/linv", linv.data(), linv.size());
    std::vector<uint64_t> spiv_u(spiv.begin(), spiv.begin() + Nr);
    h5_write_one(spiv_file, "/spiv", spiv_u.data(), spiv_u.size());

    printf("\nAccepted rank: %zu in %zu rounds\n", Nr, Nrounds);
    printf("# round accepted cumrank relerr\n");
    size_t cum = 0;
    for (size_t i = 0; i < Nrounds; ++i) {
        const size_t a = i < (size_t)res.rounds ? (size_t)hm[i] : 0;
        cum += a;
        printf("%zu %zu %zu %.5e\n", i, a, cum, i < (size_t)res.rounds ? err[i] : err[res.rounds - 1]);
    }
    cudaFree(F);
    cudaFree(X_dev);
    cudaFree(u_dev);
    kevd_ctx_destroy(ctx);
    printf("Total time: %.2f s\n", difftime(time(nullptr), t0));
    return 0;
}
