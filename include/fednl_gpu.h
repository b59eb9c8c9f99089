/*
 * fednl_gpu.h -- C ABI of the GB300 (sm_103a) FedNL round engine.
 *
 * Drop-in for the hot path of u-FedNL (dopt): the per-client L2-logistic oracle, the FedNL
 * compressors on the upper triangle of H_i - shift_i, the shift update, the master aggregation
 * and the Option-B Cholesky Newton step.  Plain C types only (no CUDA or torch types); every
 * entry point returns an int status (FEDNL_OK or a negative fednl_status code) and
 * fednl_gpu_last_error() describes the last failure of the calling thread.
 *
 * Threading: a handle is not thread-safe; calls on one handle are serialised on the handle's
 * own CUDA stream.  Different handles may be used from different threads.
 *
 * Index convention (identical to the reference): a selected Hessian entry (i, j), i <= j, is
 * reported as the flat column-major index j * lda + i, where lda is the reference build's
 * leading dimension (d rounded up to 4 in its default AVX2 build).
 */
#ifndef FEDNL_GPU_H
#define FEDNL_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum fednl_status {
    FEDNL_OK = 0,
    FEDNL_EINVAL = -1,     /* bad argument or call order */
    FEDNL_ENOMEM = -2,     /* device or host allocation failed */
    FEDNL_ECUDA = -3,      /* a CUDA runtime call failed */
    FEDNL_ENOTPD = -4,     /* Option-B matrix H + l I not positive definite */
    FEDNL_ETIMEOUT = -5,   /* a bounded device-side wait ran out */
    FEDNL_ENODEV = -6      /* no usable CUDA device */
} fednl_status;

/* Same numbering as the reference's enum Compressor
 * (dopt/bin_fednl_local/include/UsedTypes.h:18-26). */
typedef enum fednl_compressor {
    FEDNL_IDENTITY = 0,
    FEDNL_RANDK = 1,
    FEDNL_TOPK = 2,
    FEDNL_RANDSEQK = 3,
    FEDNL_TOPLEK = 4,
    FEDNL_NATURAL = 5,
    FEDNL_RANDK_PHILOX = 6      /* project-defined RandK stream: k positions from a Philox4x32-10-keyed
                                   Feistel permutation of the upper positions (no reference counterpart) */
} fednl_compressor;

typedef enum fednl_feature_format {
    FEDNL_FEATURES_AUTO = 0,    /* binary if every feature is 0 or 1, dense otherwise */
    FEDNL_FEATURES_BINARY = 1,  /* {0,1} features: bit-packed per client and feature */
    FEDNL_FEATURES_DENSE = 2    /* arbitrary FP64 features */
} fednl_feature_format;

/* Problem description.  Mirrors the reference's train() configuration
 * (dopt/bin_fednl_local/include/TrainLoop.h:103-735 and Args.h). */
typedef struct fednl_problem_desc {
    int32_t d;                  /* dimension including the intercept attribute */
    int32_t lda;                /* leading dimension for flat indices; 0 = reference default (d up to x4) */
    int32_t n_clients;
    const int32_t* n_samples;   /* host [n_clients]; uneven sizes allowed */
    double lambda;              /* L2 regulariser */
    int32_t compressor;         /* fednl_compressor */
    int32_t k;                  /* compressor k (ignored for Identity / Natural, which send all of U) */
    double alpha;               /* shift learning rate */
    int32_t workers;            /* reference --workers W: client c runs on worker c mod W (TopLEK streams) */
    uint32_t seed_base;         /* RandK / RandSeqK client seed = seed_base + c (reference: 123) */
    uint32_t toplek_seed;       /* initial state of each worker's TopLEK generator (reference: 1234) */
    int32_t feature_format;     /* fednl_feature_format */
    /* FedNL-PP (dopt/bin_fednl_local_pp, TrainLoop.h:279-287): clients_per_round > 0 selects the
     * partial-participation algorithm with that many sampled clients per round (--clients-per-round);
     * 0 = plain FedNL (bin_fednl_local) */
    int32_t clients_per_round;
    uint32_t client_seed;       /* FedNL-PP sampler seed (--client-selection-seed, reference: 1234) */
    /* FedNL options of bin_fednl_local (TrainLoop.h:300-360, 1383-1640) */
    int32_t option_a;           /* 1: Option A, Cholesky of H + lambda I (--fednl-option-a); 0: Option B */
    int32_t line_search;        /* 1: FedNL-LS backtracking on the iterate (--line_search); not with PP */
    double ls_c, ls_gamma;      /* --c_line_search, --gamma_line_search */
    int32_t ls_max_steps;       /* --max_line_search_steps (reference default 5) */
    int32_t track_f;            /* 1: form f(x) at every round's starting iterate (--tracking) */
    /* Arithmetic order (plain FedNL only): FEDNL_ORDER_FIXED (0) is the engine's own fixed order,
     * reproducible on every GPU and equal to the test oracle bit for bit; FEDNL_ORDER_REFERENCE (1)
     * performs the IEEE operations of the reference's AVX2 build without FMA in its order
     * (two-Vec4d dot products and norms, vectorclass exp/log in SIMD lanes, up-looking Cholesky,
     * TopLEK window numerators one by one), which reproduces the reference's rounds bit for bit;
     * the reference's scalar libm exp tail is replaced by the correctly rounded exp. */
    int32_t arith_order;
    int32_t reserved;           /* must be zero */
} fednl_problem_desc;

enum { FEDNL_ORDER_FIXED = 0, FEDNL_ORDER_REFERENCE = 1 };

typedef struct fednl_round_stats {
    int32_t round;              /* index of the round just completed */
    int32_t status;             /* FEDNL_OK or FEDNL_ENOTPD for this round */
    double grad_norm;           /* ||g|| of the aggregated gradient at the round's starting iterate
                                   (FedNL-PP: of the true gradient over all clients, TrainLoop.h:1166) */
    double l;                   /* Option-B regulariser l = mean_i Lk_i (FedNL-PP: running mean) */
} fednl_round_stats;

typedef struct fednl_handle_s* fednl_handle;

/* ---- lifecycle ---------------------------------------------------------------------------- */

/* Replaces the setup of train() (TrainLoop.h:103-735): sizes, device buffers, stream. */
int fednl_gpu_create(const fednl_problem_desc* desc, fednl_handle* out);
int fednl_gpu_destroy(fednl_handle h);

/* Client data, host row-major features [sum n_i][d] (clients concatenated in order) and labels
 * [sum n_i] in {-1,+1}.  Replaces the per-client L2RegulirizeLogisticRegression construction
 * (TrainLoop.h:601-605; logistic_regression.h:26-76). */
int fednl_gpu_upload_client_data(fednl_handle h, const double* features, const double* labels);
/* Client data as binary features in CSR form (the LIBSVM rows of dataset_loader_fs.h:607-870): for
 * every sample, clients concatenated in order, the ascending column indices (0-based, < d) of its
 * attributes equal to 1 (rowptr [sum n_i + 1], colidx [rowptr[sum n_i]]) and its label.  The bit
 * layout of A_i is packed on the device; the results equal those of fednl_gpu_upload_client_data
 * with the same features as dense 0/1 rows. */
int fednl_gpu_upload_client_csr(fednl_handle h, const int32_t* rowptr, const int32_t* colidx, const double* labels);

/* The common-sample lists that both uploads build for the binary Hessian's list kernel, built on the
 * host from 0/1 features given as CSR rows (as for fednl_gpu_upload_client_csr; clients' samples in
 * order, n_samples[c] of client c); no device is used.  Per client c and upper position
 * p = b (b + 1) / 2 + a (a <= b), code[c * ustr + p] (ustr = U rounded up to a multiple of 32) is
 * 0x7fff when no sample holds both attributes, the client-local index of the one sample that does,
 * 0x8000 | the number of its record within the 512-position segment when several do, 0xc000 | a on
 * the diagonal, and 0xa000 | a in the last column when every sample of the client has the last
 * attribute set (an intercept, whose entries come from attribute sums); padding is 0x7fff.
 * seg[c * (nseg + 1) + g] is the first record of segment g (nseg = ceil(U / 512)), rec[r] the first
 * of record r's samples in hits (client-local indices in sample order; rec[records] = their total).
 * sizes[0..3] receive the entry counts of code, seg, rec and hits and *maxrec the most records in
 * one segment (at least 1); call with NULL outputs to get the sizes.  Returns FEDNL_EINVAL when the
 * rows are bad or the lists are not built for this problem (a client over 0x7ffe samples, d over
 * 0x1fff, over 16 sample pairs per upper position in a client, over 64 M pairs in all). */
int fednl_gpu_hit_lists(int32_t d, int32_t nclients, const int32_t* n_samples, const int32_t* rowptr,
                        const int32_t* colidx, int64_t* sizes, int32_t* maxrec, uint16_t* code, uint32_t* seg,
                        uint32_t* rec, uint16_t* hits);

/* shift_i = H_i(x0), H = mean_i shift_i, x = x0 (x0 NULL = zeros, the reference default).
 * Replaces TrainLoop.h:639-643 and :732-735. */
int fednl_gpu_init_shifts(fednl_handle h, const double* x0);

/* One FedNL round (Option B): clients' oracle, compression, shift update; master aggregation,
 * Cholesky of H + l I and x -= dx.  Replaces one iteration of TrainLoop.h:991-1698. */
int fednl_gpu_round(fednl_handle h, fednl_round_stats* stats);

/* `rounds` rounds back to back (CUDA-graph replays); grad_norms (host, may be NULL) receives
 * ||g|| per round.  Returns the status of the first failing round, if any. */
int fednl_gpu_run(fednl_handle h, int32_t rounds, double* grad_norms);

/* ---- state readback (host buffers) -------------------------------------------------------- */
int fednl_gpu_get_x(fednl_handle h, double* x);                 /* [d] */
int fednl_gpu_set_x(fednl_handle h, const double* x);           /* [d] */
int fednl_gpu_get_grad(fednl_handle h, double* g);              /* [d] aggregated gradient */
int fednl_gpu_get_H(fednl_handle h, double* H);                 /* [d * lda] column-major, upper current */
int fednl_gpu_get_shift(fednl_handle h, int32_t client, double* shift);   /* [d * lda] symmetric */
double fednl_gpu_get_l(fednl_handle h);
double fednl_gpu_get_lk(fednl_handle h, int32_t client);
/* Last round's message of a client, exactly as the reference master adds it to H:
 * flat indices (ascending, except RandSeqK's window order) and values. */
int fednl_gpu_get_message(fednl_handle h, int32_t client, uint32_t* idx, double* val, int32_t* count);

/* FedNL-PP readback (bin_fednl_local_pp): the last round's sampled clients in ascending order
 * (clientHasBeenSelected, UsedTypes.h:169-182; *count = tau), the true gradient at the round's
 * starting iterate (computeFullGradient, TrainLoop.h:117-129) and a client's running direction
 * x Lk + shift x - grad with its last sent difference (LocalWorkerForFedNL_*.h "gradient like
 * direction").  EINVAL on a handle without FedNL-PP. */
int fednl_gpu_get_selected(fednl_handle h, int32_t* clients, int32_t* count);

/* f(x) at the last round's starting iterate (function_aggregation, TrainLoop.h:1511-1541; needs
 * line_search or track_f, else NAN) and the number of objective evaluations of the last round's
 * line search (0 without FedNL-LS). */
double fednl_gpu_get_f(fednl_handle h);
int32_t fednl_gpu_get_ls_steps(fednl_handle h);
int fednl_gpu_get_true_grad(fednl_handle h, double* g);                    /* [d] */
int fednl_gpu_get_dir(fednl_handle h, int32_t client, double* dir, double* ddir);   /* [d] each */

/* ---- operator-level entry points (host buffers in, host buffers out) ----------------------- */

/* getTopKFromUpperDiagonalPart<ignoreSign=true>
 * (dopt/dopt/math_routines/include/SpecialMathRoutinesForMatrix.h:229-366) on n_mat matrices,
 * each column-major d x lda.  idx receives n_mat * k flat indices, ascending per matrix. */
int fednl_gpu_topk(const double* mats, int32_t n_mat, int32_t d, int32_t lda, int32_t k, uint32_t* idx);

/* getTopLEKFromUpperDiagonalPart<ignoreSign=true> (SpecialMathRoutinesForMatrix.h:377-511) with
 * delta = k / U.  Matrix t draws from worker stream worker_of[t] (NULL = all on stream 0); the
 * n_workers generator states (RandomGenRealLinear, :383) are read and advanced in place; matrices
 * of one stream consume it in increasing t.  idx: n_mat * k slots, counts[t] entries used. */
int fednl_gpu_toplek(const double* mats, int32_t n_mat, int32_t d, int32_t lda, int32_t k,
                     int32_t n_workers, const int32_t* worker_of, uint32_t* worker_states,
                     uint32_t* idx, int32_t* counts);

/* generateRandKItemsInUpperTriangularPart (SpecialMathRoutinesForMatrix.h:95-107): one draw of
 * k sorted flat indices per generator; states[n_gen] (RandomGenIntegerLinear) advanced in place. */
int fednl_gpu_randk(uint32_t* states, int32_t n_gen, int32_t d, int32_t lda, int32_t k, uint32_t* idx);

/* generateRandSeqKItemsInUpperTriangularPart (SpecialMathRoutinesForMatrix.h:137-169). */
int fednl_gpu_randseqk(uint32_t* states, int32_t n_gen, int32_t d, int32_t lda, int32_t k, uint32_t* idx);

/* applyNaturalCompressor (dopt/dopt/linalg_matrices/include/MatrixNMD.h:2009-2031) on n values;
 * packed (may be NULL) receives the reference wire format of consecutive pairs,
 * 3 bytes per pair (pack2FP64NoMantissa, dopt/dopt/system/include/FloatUtils.h:193-221). */
int fednl_gpu_natural(const double* in, int64_t n, double* out, uint8_t* packed);

/* Shift update of the sparse compressors, batched over n_mat clients (LocalWorkerForFedNL_TopK.h:
 * 103-129, RandK.h:136-162): for every selected flat index f = j * lda + i (i <= j) of client m,
 * item = diffs[m][f] * value_mult, shifts[m][f] += alpha * item and, for i != j, the mirror
 * shifts[m][i * lda + j] += alpha * item.  value_mult is 1 for TopK / TopLEK and U / k for RandK /
 * RandSeqK (RandK.h:90).  shifts and diffs: n_mat column-major d x lda matrices; shifts is updated
 * in place.  idx[m * k_stride + t], t < counts[m]: the client's selected flat indices (distinct
 * upper entries; anything else returns FEDNL_EINVAL). */
int fednl_gpu_shift_update(double* shifts, const double* diffs, int32_t n_mat, int32_t d, int32_t lda,
                           const uint32_t* idx, const int32_t* counts, int32_t k_stride, double alpha,
                           double value_mult);

/* Master aggregation of one round (TrainLoop.h:1100-1333 with --debug forcesequpdate): the clients'
 * gradients grads[n_clients][d] summed in client order then times 1/n into g[d]; their Lk summed in
 * client order then times 1/n into *l; every client's message values added to H (column-major
 * d x lda, upper entries updated in place) in client order: H[idx[c * k_stride + t]] +=
 * vals[c * k_stride + t] for t < counts[c] (values as the master adds them: the worker's alpha / n
 * pre-scaling included).  k_stride = 0: no Hessian messages (idx, vals, counts unused). */
int fednl_gpu_aggregate(int32_t n_clients, int32_t d, int32_t lda, const double* grads, const double* lks,
                        const uint32_t* idx, const double* vals, const int32_t* counts, int32_t k_stride,
                        double* H, double* g, double* l);

/* Identity compressor, batched over n_mat clients (LocalWorkerForFedNL_Identical.h:80-94): the
 * message of client m is every upper entry of diffs[m] in the upper-index order (column j, rows
 * 0..j): idx_out[m * U + p] its flat index, val_out[m * U + p] = diff * prescale (prescale = alpha / n,
 * TrainLoop.h:531); shifts[m] += alpha * diffs[m] on both triangles (in place).  shifts, idx_out and
 * val_out may each be NULL. */
int fednl_gpu_compress_identity(const double* diffs, int32_t n_mat, int32_t d, int32_t lda, double alpha,
                                double prescale, double* shifts, uint32_t* idx_out, double* val_out);

/* Logistic oracle of one client: evaluateGradient and evaluateHessian<true, 4>
 * (dopt/dopt/optimization_problems/include/ml/logistic_regression.h:148-547).
 * features row-major [n][d], labels [n]; grad [d]; hess [d * lda] column-major symmetric. */
int fednl_gpu_logreg_oracle(const double* features, const double* labels, int32_t n, int32_t d,
                            int32_t lda, double lambda, const double* x, double* grad, double* hess);

/* Option-B solve: choleskyFactorization<.., true, true>(Ltr, H, l) then forward / backward
 * substitution (CholeskyFactorization.h:153-272, ElementarySolvers.h:71-224).  H column-major
 * d x lda, only the upper triangle is read.  Returns FEDNL_ENOTPD if H + l I is not positive
 * definite. */
int fednl_gpu_optionb_solve(const double* H, int32_t d, int32_t lda, double l, const double* g, double* dx);

/* The mixed-precision form's solve of (H + l I) dx = g: FP32 Cholesky factor in one CTA's shared
 * memory (d up to about 300), one step of iterative refinement on a float-float residual of H held
 * as an FP32 pair, dx in FP64.  Host buffers, H column-major upper (lda >= d). */
int fednl_gpu_optionb_solve_mixed(const double* H, int32_t d, int32_t lda, double l, const double* g, double* dx);

/* The same system by the FP32 Cholesky on a cooperative grid (fednl_mx_set_solver 2): at most
 * `refine` FP64-residual refinement steps (0..8; they stop once a correction is at most 2^-30 of the
 * solution), `grid` CTAs of a cooperative launch, or -n for one thread-block cluster of n <= 16 CTAs
 * synchronised by the cluster barrier (0: a cluster of 16 up to d = 512, else one CTA per tile of the
 * first trailing update), d up to 1312.  A pivot that loses more than 18 bits in FP32 hands the
 * system to the FP64 solve, which returns FEDNL_ENOTPD for a matrix that is not positive definite.
 * Host buffers. */
int fednl_gpu_optionb_solve32(const double* H, int32_t d, int32_t lda, double l, const double* g, double* dx,
                              int32_t refine, int32_t grid);

/* Self-test of the FP64 Cholesky's square root and reciprocal (integer arithmetic, correctly
 * rounded): n inputs from a seeded generator (random bit patterns of every exponent and sign,
 * significands near 0 and 1, squares and their neighbours); counts of results that differ bit for bit
 * from the hardware sqrt and 1.0 / x. */
int fednl_gpu_selftest_rn(int64_t n, uint64_t seed, int64_t* sqrt_mismatches, int64_t* rcp_mismatches);

/* Measurement of this GPU's FP64 pipe (no counterpart in the reference; the denominator of the FP64
 * kernels' roofline): lane operations per second of dependent FP64 fma and add chains with all SMs
 * full of warps (8 chains a thread), in G op/s, and the clock cycles of one dependent FP64 add in a
 * single warp.  `iters` operations per chain. */
int fednl_gpu_fp64_rate(int64_t iters, double* fma_gops, double* add_gops, double* add_latency_cycles);

/* Allocation-free Option-B solve.  It has no counterpart in the reference; it is for callers that
 * cannot allocate device memory: a host framework that owns all device memory through its own
 * allocator (a cudaMalloc beside it would fail or fragment its pool), a process running under a
 * fixed device-memory budget, or a latency-critical loop in which cudaMalloc / cudaFree would
 * synchronise the device.  It computes what fednl_gpu_optionb_solve computes (the same kernel and
 * operation order, so the same bits) and allocates nothing:
 *   - H (column-major d x lda, upper triangle read), g and dx are DEVICE pointers the caller owns;
 *   - the call runs on `stream` (a cudaStream_t, NULL = the default stream) and waits for that
 *     stream to finish the solve before it returns the status (FEDNL_OK, FEDNL_ENOTPD,
 *     FEDNL_ETIMEOUT);
 *   - its scratch is one fixed device array of the library, about 1 MB, which every device that
 *     loads the library holds until the process exits; so d is at most 512, and a larger d returns
 *     FEDNL_EINVAL with a message naming the limit;
 *   - the first call on a device does a one-time set-up with that device current: it looks up the
 *     array's device address, which can load the library's device code on that device (and so
 *     reserve the array at that moment); make that first call before any stream capture, and before
 *     measuring free device memory;
 *   - every call uses the same array and finds the previous call's contents there; the call clears
 *     what must start at zero.  Calls that overlap on the GPU (other streams or host threads at the
 *     same time) race on the array: serialise them. */
int fednl_gpu_optionb_solve_noalloc(const double* H, int32_t d, int32_t lda, double l, const double* g,
                                    double* dx, void* stream);

/* ---- instrumentation ---------------------------------------------------------------------- */

/* Device time of `rounds` rounds replayed as in fednl_gpu_run, each bracketed by CUDA events on
 * the handle's stream.  Before each round a buffer of flush_bytes is rewritten outside the
 * bracket so that every round starts with a cold L2 (0 = no flush).  Replaces the reference's
 * wall-clock round timer (dopt/bin_fednl_local/include/TrainLoop.h:1669-1670, :1715).
 * per_round_ms (may be NULL) receives each round's time. */
int fednl_gpu_time_rounds(fednl_handle h, int32_t rounds, int64_t flush_bytes, double* total_ms,
                          double* per_round_ms);

/* Per-kernel breakdown of the same rounds: launched kernel by kernel with CUDA events between the
 * launches on the handle's stream.  kernel_ms[t] (capacity 64) receives the mean time of the t-th
 * launch of a round; names receives the kernel names separated by ';'. */
int fednl_gpu_profile_kernels(fednl_handle h, int32_t rounds, int64_t flush_bytes, int32_t* n_kernels,
                              double* kernel_ms, char* names, int32_t names_len);

const char* fednl_gpu_last_error(void);

/* ---- tensor-core (tcgen05) operators of the mixed-precision form ---------------------------- */
/* Weighted Gram matrices H_c = X_c^T diag(w) X_c + lambda I of dense FP32 client blocks on the
 * tensor cores (TF32 inputs, FP32 accumulation in tensor memory): the Hessian sum of
 * evaluateHessian (logistic_regression.h:365-547) with w = D_s.  features: host [sum n][d]
 * row-major FP32 (clients in order), weights: host [sum n] FP32, out: host [n_clients][d][d]
 * row-major FP32 of which the upper 128 x 128 tiles (row tile <= column tile) are written.
 * d must be a multiple of 128. */
int fednl_gpu_weighted_gram_tf32(const float* features, const float* weights, const int32_t* n_samples,
                                 int32_t n_clients, int32_t d, float lambda, float* out);

/* ---- the mixed-precision round (FP32 features) --------------------------------------------- */
/* The FedNL round with client Hessians on the tensor cores: per client H_c = X_c^T diag(D) X_c +
 * lambda I in TF32 with FP32 accumulation (tcgen05; d padded to a multiple of 128 with zero
 * features), fused with the FP32 shift difference and its Frobenius norm; margins and gradients in
 * FP32 pairs (about 2^-44 relative); master H, aggregation and the Option-B Cholesky solve in FP64.
 * Compressors: FEDNL_RANDK_PHILOX (selection fused into the Gram epilogue), FEDNL_TOPK and
 * FEDNL_TOPLEK on the FP32 differences (radix select of the k largest magnitudes, ties to the lower
 * packed position; TopLEK's window rule on that set with a Philox draw for the boundary entry).
 * desc: Option B, no PP / LS.  features: host [sum n][d] FP32.  The entry points mirror
 * fednl_gpu_create / upload / init_shifts / run / get_*. */
typedef struct fednl_mx_handle_s* fednl_mx_handle;
int fednl_mx_create(const fednl_problem_desc* desc, fednl_mx_handle* out);
int fednl_mx_destroy(fednl_mx_handle h);
int fednl_mx_upload_client_data(fednl_mx_handle h, const float* features, const double* labels);
int fednl_mx_init_shifts(fednl_mx_handle h, const double* x0);
int fednl_mx_run(fednl_mx_handle h, int32_t rounds, double* grad_norms);
/* device-timed rounds (CUDA events around each graph replay; flush_bytes > 0 writes a buffer of that
 * size before every round so that each starts with a cold L2) */
int fednl_mx_time_rounds(fednl_mx_handle h, int32_t rounds, int64_t flush_bytes, double* total_ms,
                         double* per_round_ms);
/* mean per-launch time of the round's 9 kernels (names ';'-separated), CUDA events between launches */
int fednl_mx_profile_kernels(fednl_mx_handle h, int32_t rounds, double* kernel_ms, char* names, int32_t names_len);
int fednl_mx_get_x(fednl_mx_handle h, double* x);
int fednl_mx_get_grad(fednl_mx_handle h, double* g);
double fednl_mx_get_l(fednl_mx_handle h);
/* Newton solve of the round: 0 = FP64 cooperative Cholesky (default), 1 = FP32 Cholesky in one CTA's
 * shared memory with one refinement step on a float-float residual (d up to about 300), 2 = FP32
 * Cholesky on a cooperative grid with FP64-residual refinement until the correction is at most 2^-30
 * of the solution, six steps at most (d up to 1312; a pivot that loses more than 18 bits in FP32
 * hands the system to the FP64 solve in the same launch) */
int fednl_mx_set_solver(fednl_mx_handle h, int32_t solver);
/* the last round's FP32 differences H_c - shift_c (packed upper, [U]; RandK-Philox: only the
 * selected positions are current), selected packed positions, and the FP32 shift of a client */
int fednl_mx_get_diff(fednl_mx_handle h, int32_t client, float* diff);
int fednl_mx_get_selection(fednl_mx_handle h, int32_t client, uint32_t* pos, int32_t* count);
int fednl_mx_get_shift(fednl_mx_handle h, int32_t client, float* shift);

/* ---- wire format of the distributed binaries -------------------------------------------------- */
/* The bytes a u-FedNL distributed client (bin_fednl_distr_client) sends its master for one client's
 * last round: the gradient packet, Lk (FEDNL_WIRE_LK, Option B), the Hessian message in chunks of
 * 359 entries in the compressor's layout (TopK / TopLEK / RandK / RandSeqK: indices and scaled items;
 * Natural: 3 bytes per pair of upper entries plus a trailing pair; Identity: all scaled items),
 * f_i (FEDNL_WIRE_FI, tracking or line search) and the round-finished packet (FEDNL_WIRE_FINISH).
 * Packet = signal byte, LEB128 length, payload (UsedTypes.h:1022-1125).  With out == NULL only
 * *len is set (the size needed).  Plain FedNL handles only. */
enum {
    FEDNL_WIRE_LK = 1,
    FEDNL_WIRE_FI = 2,
    FEDNL_WIRE_FINISH = 4,
    FEDNL_WIRE_RANDK_INDICES = 8   /* --transfer_indicies_for_randk */
};
int fednl_gpu_encode_client_round(fednl_handle h, int32_t client, int32_t flags, uint8_t* out, int64_t cap,
                                  int64_t* len);
int fednl_gpu_get_client_grad(fednl_handle h, int32_t client, double* g);     /* [d] the client's gradient */
int fednl_gpu_get_diff(fednl_handle h, int32_t client, double* diff);         /* [U] H_c - shift_c, packed upper */

/* ---- serving: a round split into its client phase and a batched solve ------------------------ */
/* Everything of one round up to the master's aggregation, on the handle's stream (plain FedNL). */
int fednl_gpu_client_phase(fednl_handle h);
int fednl_mx_client_phase(fednl_mx_handle h);
/* The Option-B solves that end the rounds of every listed handle in one cooperative launch (each
 * problem gets a group of CTAs and its own barrier words; more problems than resident CTAs take
 * successive launches).  Results equal those of fednl_gpu_round bit for bit. */
int fednl_gpu_solve_batch(fednl_handle* handles, int32_t n, fednl_mx_handle* mixed, int32_t n_mixed);
/* waits for the handle's last round and reports it as fednl_gpu_round does */
int fednl_gpu_round_result(fednl_handle h, fednl_round_stats* stats);
int fednl_mx_round_result(fednl_mx_handle h, fednl_round_stats* stats);
/* ---- autotuning ------------------------------------------------------------------------------ */
/* Measures the launch shapes of the round's Newton solve on the handle's current system (scratch
 * outputs: the run's state does not change) and keeps the fastest; results are cached per d for the
 * process.  FP64 handles: the cooperative Cholesky's CTA count (results are identical for every
 * count).  Mixed handles: the solver (FP64 cooperative, FP32 cooperative with refinement, or, d up
 * to about 300, the FP32 shared-memory factor with refinement) and the chosen one's CTA count. */
int fednl_gpu_autotune(fednl_handle h, int32_t* chol_grid, double* solve_ms);
/* the launch shape fednl_gpu_autotune chose for the binary-feature Hessian kernel, measured per
 * (d, bucket of the clients' largest n_i: n_i in (2^(b-1), 2^b] is bucket b) and cached for the
 * process: threads per block (128, 256, 512), whether the attribute masks are staged in shared
 * memory, the bucket, and the chosen shape's launch time in ms (0 before tuning or for dense
 * features); results do not depend on the shape */
int fednl_gpu_autotune_shapes(fednl_handle h, int32_t* hess_threads, int32_t* hess_masks_in_smem, int32_t* ni_bucket,
                              double* hess_ms);
int fednl_mx_autotune(fednl_mx_handle h, int32_t* solver, int32_t* chol_grid, double* solve_ms);
/* the binary-feature Hessian's kernel: kind 0 intersects the attribute masks staged in shared
 * memory, 1 the masks read from global memory, 2 reads the lists of common samples built at upload
 * (built when no client has more than 16 U attribute pairs, n_i < 32767 and d < 8192;
 * lists_built says whether they were); threads per block 128, 256 or 512.  The upload
 * picks kind 2 when the lists exist, fednl_gpu_autotune measures every available pair; the set
 * call overrides it.  Results are identical for every kind and shape. */
int fednl_gpu_hess_schedule(fednl_handle h, int32_t* kind, int32_t* threads, int32_t* lists_built);
int fednl_gpu_set_hess_schedule(fednl_handle h, int32_t kind, int32_t threads);

/* free and total device memory (admission by free memory) */
int fednl_gpu_mem_info(int64_t* free_bytes, int64_t* total_bytes);
/* device bytes a handle of this desc holds: its state plus (FP64) a dense bound on the client data
 * or (mixed) the padded feature-major copy and the upload's staging buffer */
int fednl_gpu_footprint(const fednl_problem_desc* desc, int64_t* bytes);
int fednl_mx_footprint(const fednl_problem_desc* desc, int64_t* bytes);

/* ---- the serving loop ------------------------------------------------------------------------
 * Independent problems are submitted at any time (the client data is copied), admitted in arrival
 * order as device memory (footprint + reserve <= free, held footprints <= budget) and live slots
 * allow, and advance one round per fednl_server_tick: every live problem's client phase on its own
 * stream, then one batched Option-B solve launch for all of them.  A problem retires when its ||g||
 * is at most its tolerance or it has run max_rounds rounds; its iterate stays readable. */
typedef enum fednl_precision {
    FEDNL_PRECISION_FP64 = 0,   /* the FP64 engine (features: double, S x d row-major) */
    FEDNL_PRECISION_MIXED = 1   /* the mixed-precision engine (features: float, S x d row-major) */
} fednl_precision;

typedef enum fednl_problem_state {
    FEDNL_PROBLEM_QUEUED = 0,
    FEDNL_PROBLEM_LIVE = 1,
    FEDNL_PROBLEM_DONE = 2,
    FEDNL_PROBLEM_FAILED = 3
} fednl_problem_state;

typedef struct fednl_problem_status {
    int32_t state;              /* fednl_problem_state */
    int32_t rounds;             /* rounds run */
    int32_t error;              /* status code of a failed problem */
    int32_t d;
    double grad_norm;           /* ||g|| of the last round (-1 before the first) */
    double t_submit_ms, t_admit_ms, t_done_ms;   /* since fednl_server_create; -1 until reached */
    int64_t bytes;              /* admission footprint */
} fednl_problem_status;

typedef struct fednl_tick_stats {
    int32_t live;               /* problems that ran a round in this tick */
    int32_t admitted, retired;  /* joined the live set at this tick; retired in it */
    int32_t pending;            /* queued or being admitted after the tick */
    double tick_ms;             /* host wall time of the round phase */
    double device_ms;           /* device time of the tick: first client phase to the batched solve's end */
    int64_t held_bytes;         /* footprints of the problems live after the tick */
    int64_t device_free, device_total;
} fednl_tick_stats;

/* The serving loop.  A server admits submitted problems on its own host thread (handle creation,
 * client-data upload and initial shifts, in arrival order, while the queue head fits in free
 * device memory less the reserve, the byte budget and the live-slot limit) and releases retired
 * problems there too; each fednl_server_tick adds the problems admitted since the last tick and runs
 * one round of every live problem (client phases on their own streams, one batched Newton solve). */
typedef struct fednl_server_s* fednl_server;
/* budget_bytes: cap on the live problems' footprints (0: none); reserve_bytes: device memory left
 * free; max_live: live-slot limit (0: none) */
int fednl_server_create(int64_t budget_bytes, int64_t reserve_bytes, int32_t max_live, fednl_server* out);
int fednl_server_destroy(fednl_server s);
int fednl_server_submit(fednl_server s, const fednl_problem_desc* desc, int32_t precision, const void* features,
                        const double* labels, double tol, int32_t max_rounds, int64_t* id);
/* The same without a copy: the server reads `features` and `labels` when it admits the problem, so
 * the caller keeps them valid and unchanged until the problem's state leaves FEDNL_PROBLEM_QUEUED
 * (for callers whose payloads are large or shared between problems). */
int fednl_server_submit_ref(fednl_server s, const fednl_problem_desc* desc, int32_t precision, const void* features,
                            const double* labels, double tol, int32_t max_rounds, int64_t* id);
int fednl_server_tick(fednl_server s, fednl_tick_stats* stats);
int fednl_server_status(fednl_server s, int64_t id, fednl_problem_status* status, double* x /* [d] or NULL */);
/* per (problem, round) latencies in ms, in completion order; count = how many were recorded */
int fednl_server_latencies(fednl_server s, double* out, int64_t cap, int64_t* count);
/* per tick with live problems, the tick's device time in ms (no admission work is in it: problems
 * are admitted on the server's own host thread); count = how many were recorded */
int fednl_server_device_times(fednl_server s, double* out, int64_t cap, int64_t* count);
/* the CUDA stream (a cudaStream_t) a handle's work runs on, for callers that order their own work
 * around it; NULL for a NULL handle */
void* fednl_gpu_stream(fednl_handle h);
void* fednl_mx_stream(fednl_mx_handle h);

/* ---- the reference's local driver ---------------------------------------------------------- */
/* Callback of doptExecuteLocal (bin_fednl_local/include/TrainCallbaksShared.h:11-14): dimension,
 * ||g|| of the last round, ||g||^2 / (2 mu) and 2 ||g||^2 / mu with mu = lambda
 * (TrainLoop.h:1854-1860, ConvexOptimizationRoutines.h:13-27). */
typedef void (*fednl_result_callback)(int x_dimension, double grad_norm, double f_gap_bound, double x_gap_bound);

/* doptExecuteLocal (bin_fednl_local/src/mainShared.cpp:15-38) on the GB300 engine: the command is
 * bin_fednl_local's command line (--train_dataset, --clients, --reshuffle_train, --add_intercept,
 * --lambda, --rounds, --workers, --algorithm fednl1, --compressor identical|natural|randk|topk|
 * toplek|seqk, --k_compressor_as_d_mult, --alpha_step_size or --theoretical_alpha with
 * --use_theoretical_alpha_option_1|2, --fednl-option-a|b, --line_search with --c_line_search,
 * --gamma_line_search, --max_line_search_steps, --tracking, --out, --debug).  Returns the
 * reference's TrainReturnCodes (0 ok, -1 missing argument, -2 wrong argument, -3 dataset missing,
 * -4 parse error, -5 split error, -6 saving failed, -7 internal error, -8 unknown debug mode).
 * Engine option: --gpu-arith-order reference|fixed (default reference: the rounds reproduce the
 * reference's values bit for bit; fixed: the engine's faster fixed order). */
int fednl_gpu_execute_local(const char* command, fednl_result_callback callback);

/* The reference's own exported symbols, so that a program linked against the reference's
 * shared_bin_fednl_local / shared_bin_fednl_local_pp can load this library instead.
 * doptExecuteLocal replaces bin_fednl_local/exported/FedNLLocalShared.h:8-17 (the same as
 * fednl_gpu_execute_local).  doptExecuteLocalPP replaces
 * bin_fednl_local_pp/exported/FedNLPPLocalShared.h:8-16: bin_fednl_local_pp's command line, i.e. the
 * flags above without the line search plus --clients-per-round (required, 1..clients; the client
 * sampler's seed is the reference's fixed 1234, Args.h:243-264); the rounds run in the engine's
 * fixed order; the callback receives the dimension (TrainLoop.h:1870-1871); the tracking records
 * carry NaN in place of f(x).  Same return codes. */
typedef void (*ResultCallbackLocal)(int xDimension, double discrWithOptSolution, double discrWithOptValue,
                                    double L2NormInLastIterate);
typedef void (*ResultCallbackLocalPP)(int xDimension);
int doptExecuteLocal(const char* command, ResultCallbackLocal resultCallback);
int doptExecuteLocalPP(const char* command, ResultCallbackLocalPP resultCallback);

/* The reference's LIBSVM text loader (dataset_loader_fs.h:380-885 as TrainLoop.h:124-180 drives
 * it): labels remapped to +-1 around the mean of the smallest and largest label, attribute
 * indices shifted by the smallest index found, optional intercept attribute (= 1) last.  Host only,
 * no device needed.  Call with features = labels = NULL to get n_samples and d, then again with
 * buffers of n_samples * d (row-major) and n_samples doubles.  Returns 0, -3 (file missing) or -4
 * (parse error, or not exactly two label values). */
int fednl_gpu_load_libsvm(const char* path, int32_t add_intercept, int32_t* n_samples, int32_t* d,
                          double* features, double* labels);

#ifdef __cplusplus
}
#endif
#endif
