// Stage 1 driver (the reference's ./cuband, ks_bandwidth.cu:339-667): delay
// embedding of u, pair sums over the 36-bandwidth sweep, selection, bw0.out.
// Compile-time configuration as in the reference (ks_bandwidth.cu:359-365:
// L = 30 pi, 128 gridpoints, 4,607 snapshots, Nq = 512); override with -D, or at
// run time with the flags of driver_args.h (none given: the reference's run).
#include <cmath>
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
#define NDATA 4607
#endif
#ifndef NQ
#define NQ 512
#endif

int main(int argc, char** argv) {
    const time_t t0 = time(nullptr);
    DriverConfig cfg("cuband", {{"lfact", LFACT, DriverSetting::kInt, "domain length factor in the file name"},
                                {"mgrid", MGRID, DriverSetting::kInt, "gridpoints per snapshot"},
                                {"ndata", NDATA, DriverSetting::kInt, "snapshots"},
                                {"nq", NQ, DriverSetting::kInt, "delay window"}});
    cfg.parse(argc, argv);
    const size_t Lfact = cfg.size("lfact"), M = cfg.size("mgrid"), Ndata = cfg.size("ndata"), Nq = cfg.size("nq");
    if (Nq < 1 || Nq > Ndata || M < 1) {
        fprintf(stderr, "cuband: need 1 <= nq <= ndata and mgrid >= 1\n");
        return 2;
    }
    const size_t N = Ndata - Nq + 1, NM = N * M;
    char fname[256];
    snprintf(fname, sizeof(fname), "data/ks_true_%zu_%zu_%zu_u32.h5", Ndata, M, Lfact);
    if (cfg.print_only) {
        cfg.print(stdout);
        printf("input = %s:/u\noutput = bw0.out\n", fname);
        return 0;
    }
    printf("Data file: %s\nData set: u\n", fname);
    std::vector<float> u = h5_read<float>(fname, "/u", Ndata * M);

    // the 36 candidate bandwidths: 1e-3 .. 9, nine per decade (float, as in the reference)
    std::vector<double> bw;
    for (float start : {1e-3f, 1e-2f, 1e-1f, 1.0f})
        for (int i = 0; i < 9; ++i) bw.push_back((double)(start + (float)i * start));
    const int nbw = (int)bw.size();
    std::vector<double> scales(nbw), sums(nbw), logS(nbw), slope(nbw);
    for (int j = 0; j < nbw; ++j) scales[j] = 1.0 / ((double)Nq * bw[j]);

    kevd_ctx* ctx = nullptr;
    if (kevd_ctx_create(0, &ctx) != KEVD_OK) {
        fprintf(stderr, "no CUDA device\n");
        return 1;
    }
    float *u_dev = nullptr, *X_dev = nullptr;
    DRV_CUDA(cudaMalloc(&u_dev, u.size() * sizeof(float)));
    DRV_CUDA(cudaMalloc(&X_dev, NM * Nq * sizeof(float)));
    DRV_CUDA(cudaMemcpy(u_dev, u.data(), u.size() * sizeof(float), cudaMemcpyHostToDevice));
    DRV_KEVD(ctx, kevd_hankel_rows(ctx, u_dev, (int64_t)Ndata, (int64_t)M, (int64_t)Nq, X_dev, nullptr));
    DRV_KEVD(ctx, kevd_calibrate(ctx, X_dev, (int64_t)NM, (int32_t)Nq, scales.data(), nbw, sums.data(), nullptr));
    int32_t idmax = 0;
    double eopt = 0.0, mdim = 0.0;
    DRV_KEVD(ctx, kevd_calibrate_select(bw.data(), sums.data(), nbw, (int64_t)NM, logS.data(), slope.data(),
                                        &idmax, &eopt, &mdim));
    FILE* f = fopen("bw0.out", "w");
    if (!f) {
        fprintf(stderr, "cannot write bw0.out\n");
        return 1;
    }
    for (int i = 1; i < nbw - 1; ++i) fprintf(f, "%.5e %.5e %.5e\n", bw[i], logS[i], slope[i - 1]);
    fprintf(f, "\n%.5e\n%.5e\n", eopt, mdim);
    fclose(f);
    cudaFree(u_dev);
    cudaFree(X_dev);
    kevd_ctx_destroy(ctx);
    printf("Optimal bandwidth: %.5e  dimension: %.5e\n", eopt, mdim);
    printf("Total time: %.2f s\n", difftime(time(nullptr), t0));
    return 0;
}
