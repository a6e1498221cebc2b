// Stage 3 driver (the reference's ./cukevd, ks_kevd.cu:419-2403): bistochastic
// normalisation and EVD from the stage-2 outputs (L^{-1}, pivots); writes the
// eigenvalues (ascending) and the top k_out eigenvector block.  A library status
// other than KEVD_OK ends the program with that code, as the reference's
// MPI_Abort codes do.  Compile-time configuration as in the reference
// (ks_kevd.cu:439-481: L = 30 pi, 128 gridpoints, 32,831 snapshots, Nq = 64,
// bw = 0.8, k_out = 256), reading the stage-2 files of the cuarpclm defaults
// (BLK = 512, 8 rounds); the factor is formed and decomposed in the mixed form
// (FP32 factor: at rank 4,096 it and its column-major copy take 138 GB);
// override with -D, or at run time with the flags of driver_args.h (none given:
// the configuration above).  -DDUMP_H5=1 (--dump 1) also writes the reference's
// optional dump file (ks_kevd.cu:483-484, :533-542) with its intermediates in its
// own basis.
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
#ifndef DUMP_H5
#define DUMP_H5 0
#endif
#ifndef MEM_CHECK
#define MEM_CHECK 0
#endif

// The reference's dump points (c1, p1, dtil, cq, pq, Atil, A, R, G, qtil, Btil, W,
// lam, Z, U in the order of ks_kevd.cu:809-2311) from the library's, which live in
// the basis of the stored factor F = K(:,S) L^{-T} (L^{-1} = linv, lower, r x r
// column-major): the reference's c1 = K(:,S)^T 1 = L c1_F, p1 = L^{-T} L^{-1} c1 =
// linv^T c1_F, likewise cq / pq; Atil = L A L^T and Btil = L B L^T; R = chol(A + sI)
// (upper); G = R L^{-1}; Z = L^{-T} Z_F.  The products with L are forward
// substitutions with linv; the host work is O(r^3), as the reference's own dump
// gathers r x r matrices to one rank.  V (the eigenvectors of W) is not kept by the
// library and is not dumped.
static void fwd_solve(const std::vector<double>& li, size_t r, double* x, size_t stride) {
    for (size_t i = 0; i < r; ++i) {
        double v = x[i * stride];
        for (size_t j = 0; j < i; ++j) v -= li[i + j * r] * x[j * stride];
        x[i * stride] = v / li[i + i * r];
    }
}

static std::vector<double> linv_t_times(const std::vector<double>& li, size_t r, const double* x) {
    std::vector<double> y(r, 0.0);
    for (size_t j = 0; j < r; ++j) {
        double v = 0.0;
        for (size_t i = j; i < r; ++i) v += li[i + j * r] * x[i];
        y[j] = v;
    }
    return y;
}

// L M L^T for a symmetric M (column-major): row-wise then column-wise substitution.
static std::vector<double> l_sym_lt(const std::vector<double>& li, size_t r, const std::vector<double>& m) {
    std::vector<double> x(m);
    for (size_t c = 0; c < r; ++c) fwd_solve(li, r, x.data() + c * r, 1);   // X = L M
    for (size_t i = 0; i < r; ++i) fwd_solve(li, r, x.data() + i, r);       // rows of X: X L^T
    return x;
}

static void write_dump(const char* path, size_t r, size_t nm, size_t k_out, const std::vector<double>& li,
                       const kevd_evd_dump& d, double shift, const std::vector<double>& lam,
                       const std::vector<float>& U) {
    DRV_H5(kevd_h5_create(path));
    std::vector<double> c1(d.c1, d.c1 + r), cq(d.cq, d.cq + r);
    const std::vector<double> p1 = linv_t_times(li, r, d.c1), pq = linv_t_times(li, r, d.cq);
    fwd_solve(li, r, c1.data(), 1);
    fwd_solve(li, r, cq.data(), 1);
    const std::vector<double> A(d.A, d.A + r * r), B(d.B, d.B + r * r);
    std::vector<double> R(r * r, 0.0), G(r * r, 0.0), Z(r * k_out, 0.0);
    for (size_t j = 0; j < r; ++j) {                        // A + sI = R^T R, R upper
        double v = A[j + j * r] + shift;
        for (size_t k = 0; k < j; ++k) v -= R[k + j * r] * R[k + j * r];
        if (!(v > 0.0)) {
            fprintf(stderr, "dump: A + sI is not positive definite at %zu\n", j);
            exit(1);
        }
        const double rjj = std::sqrt(v);
        R[j + j * r] = rjj;
        for (size_t i = j + 1; i < r; ++i) {
            double w = A[j + i * r];
            for (size_t k = 0; k < j; ++k) w -= R[k + j * r] * R[k + i * r];
            R[j + i * r] = w / rjj;
        }
    }
    for (size_t j = 0; j < r; ++j)                          // G = R L^{-1}
        for (size_t i = 0; i < r; ++i) {
            double v = 0.0;
            for (size_t k = (i > j ? i : j); k < r; ++k) v += R[i + k * r] * li[k + j * r];
            G[i + j * r] = v;
        }
    for (size_t c = 0; c < k_out; ++c) {                    // Z = L^{-T} Z_F
        const std::vector<double> z = linv_t_times(li, r, d.Z + c * r);
        for (size_t i = 0; i < r; ++i) Z[i + c * r] = z[i];
    }
    h5_add(path, "c1", c1.data(), r);
    h5_add(path, "p1", p1.data(), r);
    h5_add(path, "dtil", d.dtil, nm);
    h5_add(path, "cq", cq.data(), r);
    h5_add(path, "pq", pq.data(), r);
    h5_add(path, "Atil", l_sym_lt(li, r, A).data(), r * r);
    h5_add(path, "A", A.data(), r * r);
    h5_add(path, "R", R.data(), r * r);
    h5_add(path, "G", G.data(), r * r);
    h5_add(path, "qtil", d.qtil, nm);
    h5_add(path, "Btil", l_sym_lt(li, r, B).data(), r * r);
    h5_add(path, "W", d.W, r * r);
    h5_add(path, "lam", lam.data(), r);
    h5_add(path, "Z", Z.data(), r * k_out);
    h5_add(path, "U", U.data(), nm * k_out);
}

int main(int argc, char** argv) {
    const time_t t0 = time(nullptr);
    DriverConfig cfg("cukevd", {{"lfact", LFACT, DriverSetting::kInt, "domain length factor in the file names"},
                                {"mgrid", MGRID, DriverSetting::kInt, "gridpoints per snapshot"},
                                {"ndata", NDATA, DriverSetting::kInt, "snapshots"},
                                {"nq", NQ, DriverSetting::kInt, "delay window"},
                                {"blk", BLK, DriverSetting::kInt, "stage-2 block size (in the file names)"},
                                {"nrounds", NROUNDS, DriverSetting::kInt, "stage-2 rounds (in the file names)"},
                                {"bw", BW, DriverSetting::kReal, "bandwidth (scale 1 / (nq bw))"},
                                {"kout", KOUT, DriverSetting::kInt, "eigenvectors written to /U (1..256)"},
                                {"precision", PRECISION == KEVD_FP64 ? 0 : 1, DriverSetting::kPrecision,
                                 "fp64 or mixed (FP32 factor)"},
                                {"dump", DUMP_H5, DriverSetting::kFlag, "1: also write the dump file"},
                                {"memcheck", MEM_CHECK, DriverSetting::kFlag,
                                 "1: print device memory in use at labelled points"}});
    cfg.parse(argc, argv);
    const size_t Lfact = cfg.size("lfact"), M = cfg.size("mgrid"), Ndata = cfg.size("ndata"), Nq = cfg.size("nq"),
                 Nrounds = cfg.size("nrounds"), k_out = cfg.size("kout");
    const int blk = cfg.integer("blk");
    const double bw = cfg.get("bw");
    const int32_t precision = cfg.get("precision") == 0 ? KEVD_FP64 : KEVD_MIXED;
    const bool dump_h5 = cfg.get("dump") != 0, mem_check = cfg.get("memcheck") != 0;
    if (Nq < 1 || Nq > Ndata || M < 1 || k_out < 1 || !(bw > 0)) {
        fprintf(stderr, "cukevd: need 1 <= nq <= ndata, mgrid, kout >= 1 and bw > 0\n");
        return 2;
    }
    const size_t N = Ndata - Nq + 1, NM = N * M;
    char fname[256], linv_file[256], spiv_file[256], out_file[256], dump_file[256];
    snprintf(fname, sizeof(fname), "data/ks_true_%zu_%zu_%zu_u32.h5", Ndata, M, Lfact);
    snprintf(linv_file, sizeof(linv_file), "data/linv_%zu_%zu_b%d_r%zu_%zu.h5", N, M, blk, Nrounds, Lfact);
    snprintf(spiv_file, sizeof(spiv_file), "data/spiv_%zu_%zu_b%d_r%zu_%zu.h5", N, M, blk, Nrounds, Lfact);
    snprintf(out_file, sizeof(out_file), "data/evd_%zu_%zu_%zu_%zu_%zu.h5", N, M, Nq, k_out, Lfact);
    snprintf(dump_file, sizeof(dump_file), "data/kevd_dump_%zu_%zu_%zu.h5", N, M, Lfact);
    if (cfg.print_only) {
        cfg.print(stdout);
        printf("input = %s:/u\ninput = %s:/linv\ninput = %s:/spiv\noutput = %s:/lam,/U\n", fname, linv_file,
               spiv_file, out_file);
        if (dump_h5) printf("output = %s\n", dump_file);
        return 0;
    }
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
    DRV_CUDA(cudaMalloc(&F, NM * Nr * (precision == KEVD_FP64 ? sizeof(double) : sizeof(float))));
    DRV_CUDA(cudaMalloc(&U_dev, NM * k_out * sizeof(float)));
    DRV_CUDA(cudaMemcpy(u_dev, u.data(), u.size() * sizeof(float), cudaMemcpyHostToDevice));
    if (mem_check) mem_probe("post-init");
    DRV_KEVD(ctx, kevd_hankel_rows(ctx, u_dev, (int64_t)Ndata, (int64_t)M, (int64_t)Nq, X_dev, nullptr));
    DRV_KEVD(ctx, kevd_factor_from_linv(ctx, X_dev, (int64_t)NM, (int32_t)Nq, 1.0 / ((double)Nq * bw), spiv.data(),
                                        (int64_t)Nr, linv.data(), precision, F, (int64_t)Nr, nullptr));
    std::vector<double> lam(Nr);
    kevd_evd_info info = {};
    kevd_evd_dump dump = {};
    std::vector<double> d_c1, d_dtil, d_cq, d_qtil, d_A, d_B, d_W, d_Z;
    if (dump_h5) {
        d_c1.resize(Nr);
        d_dtil.resize(NM);
        d_cq.resize(Nr);
        d_qtil.resize(NM);
        d_A.resize(Nr * Nr);
        d_B.resize(Nr * Nr);
        d_W.resize(Nr * Nr);
        d_Z.resize(Nr * k_out);
        dump = {d_c1.data(), d_dtil.data(), d_cq.data(), d_qtil.data(), d_A.data(), d_B.data(), d_W.data(),
                d_Z.data()};
    }
    if (mem_check) mem_probe("pre-pass1");
    DRV_KEVD(ctx, kevd_bistochastic_evd(ctx, F, precision, (int64_t)NM, (int64_t)Nr, (int64_t)Nr, (int32_t)k_out,
                                        lam.data(), U_dev, &info, dump_h5 ? &dump : nullptr, nullptr));
    if (mem_check) mem_probe("post-pass4");
    std::vector<float> U(NM * k_out);
    DRV_CUDA(cudaMemcpy(U.data(), U_dev, U.size() * sizeof(float), cudaMemcpyDeviceToHost));
    h5_add(out_file, "/lam", lam.data(), lam.size());
    h5_add(out_file, "/U", U.data(), U.size());
    if (dump_h5) {
        write_dump(dump_file, Nr, NM, k_out, linv, dump, info.shift, lam, U);
        printf("Dump: %s\n", dump_file);
    }
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
