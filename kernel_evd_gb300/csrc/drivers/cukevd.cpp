// Stage 3 driver (the reference's ./cukevd, ks_kevd.cu:419-2403): bistochastic
// normalisation and EVD from the stage-2 outputs (L^{-1}, pivots); writes the
// eigenvalues (ascending) and the top k_out eigenvector block.  A library status
// other than KEVD_OK ends the program with that code, as the reference's
// MPI_Abort codes do.  Compile-time configuration as in the reference
// (ks_kevd.cu:439-481: L = 30 pi, 128 gridpoints, 32,831 snapshots, Nq = 64,
// bw = 0.8, k_out = 256), reading the stage-2 files of the cuarpclm defaults
// (BLK = 512, 8 rounds); the factor is formed and decomposed in the mixed form
// (FP32 factor: at rank 4,096 it and its column-major copy take 138 GB);
// override with -D.
#include <ctime>

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
#ifndef KOUT
#define KOUT 256
#endif
#ifndef PRECISION
#define PRECISION KEVD_MIXED
#endif

int main() {
    const time_t t0 = time(nullptr);
    const size_t Lfact = LFACT, M = MGRID, Ndata = NDATA, Nq = NQ, Nrounds = NROUNDS, k_out = KOUT;
    const size_t N = Ndata - Nq + 1, NM = N * M;
    char fname[256], linv_file[256], spiv_file[256], out_file[256];
    snprintf(fname, sizeof(fname), "data/ks_true_%zu_%zu_%zu_u32.h5", Ndata, M, Lfact);
    snprintf(linv_file, sizeof(linv_file), "data/linv_%zu_%zu_b%d_r%zu_%zu.h5", N, M, BLK, Nrounds, Lfact);
    snprintf(spiv_file, sizeof(spiv_file), "data/spiv_%zu_%zu_b%d_r%zu_%zu.h5", N, M, BLK, Nrounds, Lfact);
    snprintf(out_file, sizeof(out_file), "data/evd_%zu_%zu_%zu_%zu_%zu.h5", N, M, Nq, k_out, Lfact);
    DRV_H5(kevd_h5_create(out_file));
    printf("Data file: %s\nData set: u\n", fname);
    std::vector<float> u = h5_read<float>(fname, "/u", Ndata * M);
    const size_t Nr = h5_count(spiv_file, "/spiv");
    if (h5_count(linv_file, "/linv") != Nr * Nr) {
        fprintf(stderr, "%s: /linv is not %zu x %zu\n", linv_file, Nr, Nr);
        return 1;
    }
    std::vector<uint64_t> spiv_u = h5_read<uint64_t>(spiv_file, "/spiv", Nr);
    std::vector<double> linv = h5_read<double>(linv_file, "/linv", Nr * Nr);
    std::vector<int64_t> spiv(spiv_u.begin(), spiv_u.end());
    printf("Rank: %zu  k_out: %zu\n", Nr, k_out);

    kevd_ctx* ctx = nullptr;
    if (kevd_ctx_create(0, &ctx) != KEVD_OK) {
        fprintf(stderr, "no CUDA device\n");
        return 1;
    }
    float *u_dev = nullptr, *X_dev = nullptr, *U_dev = nullptr;
    double* F = nullptr;
    DRV_CUDA(cudaMalloc(&u_dev, u.size() * sizeof(float)));
    DRV_CUDA(cudaMalloc(&X_dev, NM * Nq * sizeof(float)));
    DRV_CUDA(cudaMalloc(&F, NM * Nr * (PRECISION == KEVD_FP64 ? sizeof(double) : sizeof(float))));
    DRV_CUDA(cudaMalloc(&U_dev, NM * k_out * sizeof(float)));
    DRV_CUDA(cudaMemcpy(u_dev, u.data(), u.size() * sizeof(float), cudaMemcpyHostToDevice));
    DRV_KEVD(ctx, kevd_hankel_rows(ctx, u_dev, (int64_t)Ndata, (int64_t)M, (int64_t)Nq, X_dev, nullptr));
    DRV_KEVD(ctx, kevd_factor_from_linv(ctx, X_dev, (int64_t)NM, (int32_t)Nq, 1.0 / ((double)Nq * BW), spiv.data(),
                                        (int64_t)Nr, linv.data(), PRECISION, F, (int64_t)Nr, nullptr));
    std::vector<double> lam(Nr);
    kevd_evd_info info = {};
    DRV_KEVD(ctx, kevd_bistochastic_evd(ctx, F, PRECISION, (int64_t)NM, (int64_t)Nr, (int64_t)Nr, (int32_t)k_out,
                                        lam.data(), U_dev, &info, nullptr, nullptr));
    std::vector<float> U(NM * k_out);
    DRV_CUDA(cudaMemcpy(U.data(), U_dev, U.size() * sizeof(float), cudaMemcpyDeviceToHost));
    h5_add(out_file, "/lam", lam.data(), lam.size());
    h5_add(out_file, "/U", U.data(), U.size());
    printf("trace(A) = %.10e  shift = %.5e\n", info.trace_A, info.shift);
    printf("Leading eigenvalues:");
    for (size_t j = 0; j < (k_out < 8 ? k_out : 8); ++j) printf(" %.10f", lam[Nr - 1 - j]);
    printf("\n");
    cudaFree(U_dev);
    cudaFree(F);
    cudaFree(X_dev);
    cudaFree(u_dev);
    kevd_ctx_destroy(ctx);
    printf("Total time: %.2f s\n", difftime(time(nullptr), t0));
    return 0;
}
