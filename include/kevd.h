/*
 * kevd.h -- C ABI of the GB300 kernel low-rank pipeline.
 *
 * The reference (cval26/kernel_evd) exposes its three stages as standalone
 * programs whose boundary is a process plus files:
 *
 *   ./cuband    ks_bandwidth.cu:339-667   bandwidth calibration  -> bw0.out
 *   ./cuarpclm  ks_arpclm.cu:566-1152     block RPCholesky       -> linv, spiv
 *   ./cukevd    ks_kevd.cu:419-2403       bistochastic EVD       -> lam, U
 *
 * Each entry point below replaces the compute of one stage (or one piece of
 * it) and is what a caller of that stage binds: the drivers in
 * kernel_evd_gb300/csrc/drivers reproduce the programs' invocation and file
 * layout on top of it, and the Python package binds it through ctypes.
 *
 * Conventions
 *   - Every function returns an int status (enum kevd_status); no exceptions
 *     or exits cross the boundary.  kevd_last_error() describes the failure.
 *   - Pointers documented "device" are caller-owned device buffers; "host"
 *     are caller-owned host buffers.  Sample matrices X are row-major
 *     N x d float32 (one sample per row, d contiguous).
 *   - stream is a cudaStream_t passed as void* (NULL = legacy default stream).
 *     Calls enqueue work on it and return after the host-visible outputs are
 *     written (they synchronise the stream when they return host data).
 *   - A context is bound to one device and is not internally locked: use one
 *     context per host thread.
 *   - Sample dimension d (features per state): 1..1024 everywhere; rows are
 *     staged in shared memory a fixed-width chunk of features at a time, so
 *     the reference's delay windows (Nq = 512) are accepted as they are.
 *   - Kernel: K(i,j) = exp(-scale * ||x_i - x_j||^2).  The Hankel view of the
 *     reference uses scale = 1/(Nq*bw) (ks_arpclm.cu:275); dense states use
 *     scale = 1/eps.
 */
#ifndef KEVD_H
#define KEVD_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct kevd_ctx kevd_ctx;

enum kevd_status {
    KEVD_OK = 0,
    KEVD_ERR_ARG = 1,           /* invalid argument or unsupported size       */
    KEVD_ERR_CUDA = 2,          /* CUDA runtime / cuBLAS / cuSOLVER failure   */
    KEVD_ERR_NONPOS_DTIL = 3,   /* dtil <= 0: ks_kevd.cu:1170-1181 (abort 2)  */
    KEVD_ERR_POTRF = 4,         /* chol(A+sI) failed: ks_kevd.cu:1510-1520 (3)*/
    KEVD_ERR_NONPOS_QTIL = 5,   /* qtil <= 0: ks_kevd.cu:1692-1703 (abort 4)  */
    KEVD_ERR_SYEVD = 6,         /* eigensolver failed: ks_kevd.cu:1904-1913 (5)*/
    KEVD_ERR_NOMEM = 7,         /* device allocation failed                   */
    KEVD_ERR_TIMEOUT = 8        /* a bounded device wait gave up              */
};

enum kevd_precision {
    KEVD_FP64 = 0,   /* plain form: factor and all arithmetic in FP64          */
    KEVD_MIXED = 1   /* factor F in FP32, FP64 in the pivot block, residual
                        diagonal, scaling vectors and the k x k eigensolve   */
};

/* ---- context ---------------------------------------------------------- */
int kevd_ctx_create(int device, kevd_ctx** out);
void kevd_ctx_destroy(kevd_ctx* ctx);
const char* kevd_last_error(const kevd_ctx* ctx);
const char* kevd_status_name(int status);
int kevd_abi_version(void);

/* Profiling.  While enabled, CUDA events are recorded on the launching stream
 * around each of this library's kernels; kevd_profile_read returns, for the
 * idx-th kernel name, its accumulated device time and launch count (it
 * synchronises the pending events).  Enabling resets the counters.
 * kevd_launch_count counts every kernel this library launched. */
int kevd_profile_enable(kevd_ctx* ctx, int on);
int kevd_profile_read(kevd_ctx* ctx, int idx, char* name, int name_len,
                      double* total_ms, int64_t* count);
int64_t kevd_launch_count(const kevd_ctx* ctx);

/* Issue-rate probe for roofline denominators (no reference counterpart; a
 * measurement aid).  kind 0: MUFU ex2 evaluations per second; 1: FP32 FMAs
 * per second; 2: FP64 FMAs per second; 3: FP32 FMAs per second issued as
 * packed pairs (fma.rn.f32x2, two per instruction); each from independent dependency
 * chains over every SM, at the clock the GPU runs during the call.  ms: the
 * best of three timed launches.  Synchronises the stream. */
int kevd_peak_rate(kevd_ctx* ctx, int32_t kind, double* ops_per_s, double* ms, void* stream);

/* ---- sample views ------------------------------------------------------ */

/* Materialise the delay-embedded samples of the reference programs as rows.
 * u: device, M*Ndata floats, time fastest.  X: device, (Ndata-Nq+1)*M x Nq.
 * Row i = gridpoint i/N, time i%N (ks_arpclm.cu:263-268,
 * ks_bandwidth.cu:168-169). */
int kevd_hankel_rows(kevd_ctx* ctx, const float* u, int64_t Ndata, int64_t M,
                     int64_t Nq, float* X, void* stream);

/* Kernel block out[r*ld + c] = K(row_r, cols[c]) in FP64 (precision
 * KEVD_FP64, out is double*) or FP32 (KEVD_MIXED, out is float*).
 * rows: device index array, or NULL for the contiguous rows row0..row0+nrows-1.
 * cols: device index array.  Replaces compute_kblock<T>
 * (ks_arpclm.cu:242-280, ks_kevd.cu:302-340). */
int kevd_kernel_block(kevd_ctx* ctx, const float* X, int64_t N, int32_t d,
                      double scale, const int64_t* rows, int64_t row0,
                      int64_t nrows, const int64_t* cols, int64_t ncols,
                      int32_t precision, void* out, int64_t ld, void* stream);

/* ---- stage 1: bandwidth calibration (ks_bandwidth.cu) ------------------ */

/* sums[j] = sum over i > l of exp(-scales[j] * ||x_i - x_l||^2), FP64, over
 * the strict lower triangle.  All n_scales values are accumulated in one pass
 * over the pair tiles.  Replaces dmat_comp + 36 x kernelsum_comp
 * (ks_bandwidth.cu:181-325, :537-577); the reference's per-summand 1/NM is
 * applied by kevd_calibrate_select.  scales, sums: host, n_scales <= 256. */
int kevd_calibrate(kevd_ctx* ctx, const float* X, int64_t N, int32_t d,
                   const double* scales, int32_t n_scales, double* sums,
                   void* stream);

/* The plain FP64 form of kevd_calibrate (FP64 distances from the FP32 states,
 * FP64 exp): the precision reference for the fused pass, as the reference's
 * FP64 programs are for its FP32 kernels.  Same arguments and limits. */
int kevd_calibrate_fp64(kevd_ctx* ctx, const float* X, int64_t N, int32_t d,
                        const double* scales, int32_t n_scales, double* sums,
                        void* stream);

/* kevd_calibrate for callers that cannot call cudaMalloc: a process whose
 * device memory is fully reserved by a pool it does not own (another
 * framework's caching allocator, or a host application that gives the plugin
 * a fixed budget), or a service that forbids allocation once it has started.
 * No reference counterpart.  Needs no context and allocates nothing: its
 * scratch is a fixed device array of about 160 KB that every GPU loading the
 * library keeps until exit.  Limits: n_scales <= 64 (KEVD_ERR_ARG beyond).
 * The first call on a device (and on each further context of that device)
 * resolves the array's device address with that device current; make that
 * first call before any stream capture.  Calls share the array: calls that
 * overlap on the GPU race.  The call synchronises the stream.  A CUDA error
 * already pending on the calling thread is reported as KEVD_ERR_CUDA, left in
 * place, and nothing is enqueued.  X: device; scales, sums: host. */
int kevd_calibrate_noalloc(const float* X, int64_t N, int32_t d,
                           const double* scales, int32_t n_scales,
                           double* sums, void* stream);

/* Many calibrations of uneven size in one persistent launch (no reference
 * counterpart: the reference calibrates one dataset per program run).  Every
 * job's lower-triangle pair tiles are cut into work items of tiles_per_item
 * tiles (0: chosen from the batch size) and placed in one device work queue; a
 * persistent grid takes items with an atomic counter and a second kernel sums
 * each job's item partials in item order (deterministic).  Per job: sums[j] as
 * kevd_calibrate, n_scales <= 64, d <= 1024.  X: device; scales, sums: host. */
typedef struct {
    const float* X;
    int64_t N;
    int32_t d;
    int32_t n_scales;
    const double* scales;
    double* sums;
} kevd_calib_job;
int kevd_calibrate_batched(kevd_ctx* ctx, const kevd_calib_job* jobs,
                           int32_t n_jobs, int32_t tiles_per_item,
                           void* stream);

/* Host post-processing of ks_bandwidth.cu:612-642 in FP64:
 * logS[i] = log(2 sums[i]/NM + 1); slope[i-1] = centred difference at bw[i]
 * (n-2 values); idmax = first arg-max; eopt = bw[idmax+1];
 * mdim = 2 slope[idmax].  All pointers host. */
int kevd_calibrate_select(const double* bw, const double* sums, int32_t n,
                          int64_t NM, double* logS, double* slope,
                          int32_t* idmax, double* eopt, double* mdim);

/* Squared-distance median over pairs i > l.  n_pairs == 0: exact, over all
 * N(N-1)/2 pairs (lower median).  n_pairs > 0: over the seeded sample of
 * pair indices (pi[s], pl[s]) given on the device. */
int kevd_pair_median(kevd_ctx* ctx, const float* X, int64_t N, int32_t d,
                     const int64_t* pi, const int64_t* pl, int64_t n_pairs,
                     double* median, void* stream);

/* ---- stage 2: block RPCholesky (ks_arpclm.cu) -------------------------- */

typedef struct {
    int64_t k_max;          /* factor capacity (target rank)                 */
    int32_t block;          /* proposals per round b, 1..512 (the reference's
                               BLK; rounds accepting more than 64 columns
                               update them in passes of 64)                   */
    int32_t max_rounds;     /* round limit                                    */
    double tol;             /* rejection tolerance (reference: 1e-10); the
                               mixed form also rejects H_ii <= 16 x 2^-24 K_ii
                               (FP32 rounding level of the factor) and stops
                               once the trace error is at or below that level */
    double err_target;      /* stop once trace error <= this (0: never)       */
    uint64_t seed;          /* Philox key when uniforms == NULL               */
    const double* uniforms; /* host, optional: max_rounds x 2 x block draws in
                               (0,1]; [r][0][:] proposals, [r][1][:] accepts  */
    int32_t precision;      /* enum kevd_precision                            */
} kevd_rpchol_params;

typedef struct {
    int64_t rank;           /* realised rank r                                */
    int32_t rounds;         /* rounds executed                                */
    double trace_error;     /* tr(K - F F^T)/tr(K) after the last round       */
} kevd_rpchol_result;

/* Factor K ~= F F^T with F = K(:,S) L^{-T}.  F: device, N x ldF, double
 * (KEVD_FP64) or float (KEVD_MIXED), ldF >= k_max; columns [0, rank) are
 * written.  piv: host, k_max int64 (pivots in acceptance order, the
 * reference's /spiv).  err, accepted: host, max_rounds entries (per-round
 * trace error and accepted count, the reference's round table
 * ks_arpclm.cu:1129-1136).  Replaces the round loop ks_arpclm.cu:793-1046.
 * KEVD_MIXED runs the residual update on the tensor cores when ldF % 4 == 0
 * and F is 16-byte aligned, unless the kernel is nearly diagonal (fewer than
 * half of 4,096 sampled kernel values reach 2^-24: the call then makes one
 * 4-byte device-to-host copy before the round loop and keeps the FP32 SIMT
 * update); otherwise the FP32 SIMT update. */
int kevd_rpchol(kevd_ctx* ctx, const float* X, int64_t N, int32_t d,
                double scale, const kevd_rpchol_params* params, void* F,
                int64_t ldF, int64_t* piv, double* err, int32_t* accepted,
                kevd_rpchol_result* result, void* stream);

/* Many mixed-precision factorisations at once (no reference counterpart).
 * Each job has its own X (device), FP32 factor F (device, N x ldF) and seed;
 * piv (host, k_max entries) receives the pivots and result the rank, rounds
 * and trace error.  use_graph != 0: the round loops of all jobs are captured
 * as parallel branches of one CUDA graph (forked from stream, joined back)
 * and launched once; every job runs max_rounds rounds on the device (kernels
 * return at once after the stop).  use_graph == 0: the same work is issued on
 * one stream per job. */
typedef struct {
    const float* X;
    int64_t N;
    int32_t d;
    int32_t block;
    double scale;
    void* F;
    int64_t ldF;
    int64_t k_max;
    int32_t max_rounds;
    int32_t pad;
    uint64_t seed;
    int64_t* piv;
    kevd_rpchol_result result;
} kevd_rpchol_job;
int kevd_rpchol_batched(kevd_ctx* ctx, kevd_rpchol_job* jobs, int32_t n_jobs,
                        int32_t use_graph, void* stream);

/* The reference's /linv output: L^{-1} (r x r, column-major, lower, zeros
 * stored) with L = F(S,:) (ks_arpclm.cu:1055-1095).  F: device; piv: host;
 * Linv: host. */
int kevd_linv_from_factor(kevd_ctx* ctx, const void* F, int32_t precision,
                          int64_t ldF, const int64_t* piv, int64_t r,
                          double* Linv, void* stream);

/* ---- stage 3: bistochastic normalisation + EVD (ks_kevd.cu) ------------ */

typedef struct {
    double trace_A;         /* tr(A), A = F^T Dtil^{-2} F                     */
    double shift;           /* s = DBL_EPSILON tr(A) (ks_kevd.cu:1481-1499)    */
} kevd_evd_info;

/* Optional host copies of the intermediates (the reference's dump points,
 * ks_kevd.cu:483-484); any pointer may be NULL. */
typedef struct {
    double* c1;    /* k      F^T 1                                           */
    double* dtil;  /* N      F c1                                            */
    double* cq;    /* k      F^T dtil^{-1}                                   */
    double* qtil;  /* N      F cq                                            */
    double* A;     /* k x k  F^T Dtil^{-2} F   (column-major, full)          */
    double* B;     /* k x k  F^T Qtil^{-1} F                                 */
    double* W;     /* k x k  R B R^T                                         */
    double* Z;     /* k x k_out  R^{-1} V[:, top k_out] (column-major)       */
} kevd_evd_dump;

/* Weighted Gram G = F^T diag(s)^2 F (k x k, column-major, both triangles) --
 * the Atil / Btil accumulation of ks_kevd.cu:1091-1159, :1627-1685 on a stored
 * factor.  F: device N x ldF (double for KEVD_FP64, float for KEVD_MIXED: the
 * FP32 factor is contracted on the tensor cores as a two-term f16 split,
 * scaled by powers of two to max |F| and max s^2, with FP64 accumulation
 * across row chunks).  s: device, N doubles.  G: device. */
int kevd_weighted_gram(kevd_ctx* ctx, const void* F, int32_t precision,
                       int64_t N, int64_t k, int64_t ldF, const double* s,
                       double* G, void* stream);

/* Kuramoto-Sivashinsky trajectories on the GPU: the synthetic data of the
 * workloads, by the scheme of the reference's generator (ks_datagen.py:21-101:
 * ETDRK4 in FP64 on real-FFT coefficients, quadratic term dealiased by the 3/2
 * rule).  n_traj trajectories of one grid size M (a power of two, 4 .. 128).
 * Trajectory t starts from the M/2+1 rfft
 * coefficients vhat0[t] (complex, interleaved re/im), steps with the ETDRK4
 * coefficients coef[t] (6 x (M/2+1): E, E2, Q, f1, f2, f3) and the dealiased
 * -1/2 d/dx factor g[t] (complex, interleaved), discards n_warm steps and writes
 * n_snap[t] states of M floats (time-major) to the device buffer out[t].  coef,
 * g, vhat0, n_snap and out are host arrays of n_traj entries each; the call
 * returns when the trajectories are written.  precision: KEVD_FP64 steps in
 * FP64 as the reference does (slow on the GB300's FP64 pipe); KEVD_MIXED steps in
 * FP32, about 20x faster, statistically the same attractor but a different
 * chaotic trajectory after a few Lyapunov times. */
int kevd_ks_generate(kevd_ctx* ctx, int32_t n_traj, int32_t M, int32_t precision, const double* coef,
                     const double* g, const double* vhat0, int64_t n_warm,
                     const int64_t* n_snap, float* const* out, void* stream);

/* Both Grams of the bistochastic EVD in one pass over F: G = F^T diag(s)^2 F
 * and G2 = F^T diag(s2)^2 F (the Atil and Btil accumulations of
 * ks_kevd.cu:1091-1159 and :1627-1685, which the reference runs as two
 * passes).  For KEVD_MIXED each F tile is loaded once and feeds both; the
 * results equal two kevd_weighted_gram calls bit for bit.  Arguments as for
 * kevd_weighted_gram. */
int kevd_weighted_gram2(kevd_ctx* ctx, const void* F, int32_t precision,
                        int64_t N, int64_t k, int64_t ldF, const double* s,
                        const double* s2, double* G, double* G2, void* stream);

/* Bistochastic EVD of Khat = F F^T.  F: device N x ldF (double or float by
 * precision), k <= 8192.  lam: host, k eigenvalues ascending.  U: device,
 * N x k_out float row-major, columns ascending (the last is the leading
 * eigenvector), k_out <= 256 (the reference's k_out, ks_kevd.cu:481); the
 * reference's /lam and /U (ks_kevd.cu:1932-1940, :2301-2308).  In the mixed
 * form the leading min(k_out, 32) eigenpairs (eigenvalues and U columns) are
 * refined against F in FP64 (Rayleigh-Ritz); the others come from the k x k
 * eigensolve. */
int kevd_bistochastic_evd(kevd_ctx* ctx, const void* F, int32_t precision,
                          int64_t N, int64_t k, int64_t ldF, int32_t k_out,
                          double* lam, float* U, kevd_evd_info* info,
                          kevd_evd_dump* dump, void* stream);

/* F = K(:,S) L^{-T} from the reference's stage-2 outputs (/linv, /spiv), so
 * that kevd_bistochastic_evd consumes them as ./cukevd does
 * (ks_kevd.cu:760-2308).  piv, Linv: host (Linv r x r column-major).
 * F: device N x ldF, double or float by precision. */
int kevd_factor_from_linv(kevd_ctx* ctx, const float* X, int64_t N, int32_t d,
                          double scale, const int64_t* piv, int64_t r,
                          const double* Linv, int32_t precision, void* F,
                          int64_t ldF, void* stream);

/* Nystrom factor of a given pivot set in FP64 arithmetic: F = K(:,S) L^{-T}
 * with L L^T = K(S,S) (ks_arpclm.cu's factor for the accepted pivots,
 * README_arpclm.md:21-47), written as double (KEVD_FP64) or rounded to float
 * (KEVD_MIXED).  Used to compare a mixed-precision run against the FP64 EVD of
 * the same pivots.  piv: host; F: device N x ldF. */
int kevd_factor_from_pivots(kevd_ctx* ctx, const float* X, int64_t N, int32_t d,
                            double scale, const int64_t* piv, int64_t r,
                            int32_t precision, void* F, int64_t ldF,
                            void* stream);

/* Out-of-sample (Nystrom) eigenfunctions of new states Y (device, n x d):
 * Uy[j,:] = (K(y_j,S) Z') / (K(y_j,S) p1'), the pass-4 formula
 * (ks_kevd.cu:2246-2269) applied to new rows; the model (landmarks S, Z', p1')
 * is prepared by kevd_nystrom_prepare from a factor and its EVD. */
typedef struct kevd_model kevd_model;
int kevd_nystrom_prepare(kevd_ctx* ctx, const float* X, int64_t N, int32_t d,
                         double scale, const void* F, int32_t precision,
                         int64_t ldF, const int64_t* piv, int64_t r,
                         int32_t k_out, kevd_model** model, void* stream);
int kevd_nystrom_eval(kevd_ctx* ctx, const kevd_model* model, const float* Y,
                      int64_t n, float* Uy, void* stream);
void kevd_model_destroy(kevd_model* model);

/* ---- serving loop (no reference counterpart) ----------------------------
 * The reference runs its three stages as batch programs.  The server keeps
 * factorized models resident on one GPU and answers eigenfunction queries
 * against them while new factorizations run:
 *  - a factorization request (host X, N x d) is admitted when a worker is
 *    free and its HBM footprint fits the budget left by running
 *    factorizations and resident models; it runs block RPCholesky, the
 *    bistochastic EVD and kevd_nystrom_prepare on its worker's own stream,
 *    then frees everything except the model;
 *  - query requests (host Y, n x d) for a model are batched: whatever is
 *    queued for the model with the oldest pending query, up to
 *    max_query_batch states, is evaluated in one kevd_nystrom_eval launch
 *    (rows are evaluated independently, so a query's result does not depend
 *    on the batch it joined).
 * Y and out stay owned by the caller and must remain valid until
 * kevd_server_wait has returned for that request. */
typedef struct kevd_server kevd_server;

typedef struct {
    int32_t device;            /* CUDA device ordinal                         */
    int32_t factor_workers;    /* concurrent factorizations, 1..16            */
    int64_t max_query_batch;   /* states per query launch, >= 1              */
    uint64_t hbm_budget_bytes; /* admission budget (bytes of device memory)   */
    double batch_window_us;    /* batcher waits this long before taking a
                                  batch, letting it fill (0: no wait)         */
} kevd_server_config;

typedef struct {
    int32_t status;            /* kevd_status of the request                  */
    int64_t model_id;          /* factorization: id of the resident model     */
    double latency_s;          /* submit -> done                              */
    double queue_s;            /* submit -> started                           */
    int64_t batch_rows;        /* query: states in the launch(es) it joined   */
    double trace_error;        /* factorization: tr(K - FF^T)/tr(K)           */
    int64_t rank;              /* factorization: realised rank                */
    char message[192];         /* failure description (empty on success)      */
} kevd_request_info;

int kevd_server_create(const kevd_server_config* cfg, kevd_server** server);
/* Device bytes the server charges against its budget for a factorization of
 * N x d states to rank k (X, F and its column-major copy, workspaces); -1 for
 * invalid sizes.  A resident model is charged r (4 d + 8 (k_out + 1)) bytes. */
int64_t kevd_factorization_footprint(int64_t N, int32_t d, int64_t k,
                                     int32_t k_out, int32_t precision);
/* Stops the workers after the requests already running; queued requests are
 * dropped.  Frees every resident model. */
void kevd_server_destroy(kevd_server* server);
/* X is copied at submission.  KEVD_ERR_NOMEM when the footprint can never fit
 * the budget. */
int kevd_server_submit_factorization(kevd_server* server, const float* X,
                                     int64_t N, int32_t d, double scale,
                                     int64_t k, int32_t block, int32_t k_out,
                                     uint64_t seed, int32_t precision,
                                     int64_t* request_id);
/* out: host, n x k_out float (row-major). */
int kevd_server_submit_query(kevd_server* server, int64_t model_id,
                             const float* Y, int64_t n, float* out,
                             int64_t* request_id);
/* Blocks until the request is done (KEVD_ERR_TIMEOUT after timeout_s, the
 * request stays pending).  Once it returns KEVD_OK the id is retired. */
int kevd_server_wait(kevd_server* server, int64_t request_id, double timeout_s,
                     kevd_request_info* info);
/* Frees a resident model; KEVD_ERR_ARG while queries for it are pending. */
int kevd_server_release_model(kevd_server* server, int64_t model_id);
/* Latency percentiles over finished requests of one type (0 factorization,
 * 1 query), in seconds. */
int kevd_server_stats(kevd_server* server, int32_t type, double* p50,
                      double* p99, int64_t* count);
/* Bytes charged against the budget, running factorizations, resident models,
 * and the largest number of factorizations that ever ran at once. */
int kevd_server_memory(kevd_server* server, int64_t* used_bytes,
                       int32_t* active_factorizations, int32_t* models,
                       int32_t* peak_active);

#ifdef __cplusplus
}
#endif

#endif /* KEVD_H */
