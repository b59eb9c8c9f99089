/*
 * fednl_oracle.h -- CPU restatement of the u-FedNL (dopt) FedNL round, used as TEST
 * INFRASTRUCTURE ONLY.
 *
 * This library is the parity oracle for the GB300 kernels in ufednl_gb300/csrc.  Only the
 * test-suite, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it; the product
 * path (libfednl_gpu.so) never links, loads or calls it.
 *
 * Every function restates the reference algorithm in plain C and cites the reference file:line
 * it follows (paths relative to the ufednl repository root).  The restatement is pinned by the
 * golden vectors in tests/golden/, which were produced by compiling the reference's own headers
 * (oracle/ref_harness.cpp, built by oracle/Makefile into oracle/_ref/).
 */
#ifndef FEDNL_ORACLE_H
#define FEDNL_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Compressor ids: same numbering as enum Compressor, dopt/bin_fednl_local/include/UsedTypes.h:18-26 */
#define ORC_IDENTITY 0
#define ORC_RANDK    1
#define ORC_TOPK     2
#define ORC_RANDSEQK 3
#define ORC_TOPLEK   4
#define ORC_NATURAL  5
#define ORC_RANDK_PHILOX 6   /* project-defined RandK stream (Philox-keyed permutation), no reference counterpart */

typedef struct orc_problem {
    int32_t d;                 /* dimension including the intercept column */
    int32_t lda;               /* leading dimension of d x d matrices (AVX2 build: d rounded up to 4) */
    int32_t n_clients;
    const int32_t* n_samples;  /* [n_clients] */
    const double* features;    /* [sum n_i][d] row-major, clients concatenated in order */
    const double* labels;      /* [sum n_i], values in {-1,+1} */
    double lambda;
    int32_t compressor;        /* ORC_* */
    int32_t k;                 /* compressor k (Identity/Natural: ignored, U is used) */
    double alpha;              /* shift learning rate */
    int32_t workers;           /* reference --workers W (client c runs on worker c mod W) */
    int32_t threads;           /* OS threads this oracle uses for the client phase (<= workers) */
    uint32_t seed_base;        /* RandK/RandSeqK client seed = seed_base + c (reference: 123) */
    uint32_t toplek_seed;      /* initial seed of each worker's TopLEK generator (reference: 1234) */
    int32_t pp;                /* 1: FedNL-PP (dopt/bin_fednl_local_pp), 0: FedNL */
    int32_t clients_per_round; /* FedNL-PP tau (--clients-per-round) */
    uint32_t client_seed;      /* FedNL-PP client sampler seed (--client-selection-seed, reference: 1234) */
    int32_t option_a;          /* 1: FedNL Option A, Cholesky of H + lambda I (--fednl-option-a) */
    int32_t line_search;       /* 1: FedNL-LS backtracking on the iterate (--line_search) */
    double ls_c, ls_gamma;     /* --c_line_search, --gamma_line_search */
    int32_t ls_max_steps;      /* --max_line_search_steps (reference default 5) */
    int32_t track_f;           /* 1: form f(x) every round (--tracking) */
    int32_t ref_order;         /* 1: the reference's own operation order (lane-ordered dot products,
                                  vectorclass exp/log, up-looking Cholesky, sequential TopLEK window) */
} orc_problem;

typedef struct orc_state orc_state;

/* ---- LCG generators (dopt/dopt/random) ------------------------------------------------- */
uint32_t orc_lcg_int_next(uint32_t* state);          /* RandomGenIntegerLinear::generateInteger */
double   orc_lcg_int_unit(uint32_t* state);          /* RandomGenIntegerLinear::generateRealInUnitInterval */
double   orc_lcg_real_unit(uint32_t* state);         /* RandomGenRealLinear::generateRealInUnitInterval */
size_t   orc_round_to_nearest(double v);             /* roundToNearestInt<size_t> */

/* ---- index helpers and compressors ---------------------------------------------------- */
size_t orc_upper_count(int32_t d);
void   orc_upper_indices(int32_t d, int32_t lda, uint32_t* out);
void   orc_shuffle_partial(uint32_t* arr, size_t n, size_t k, uint32_t* state);
void   orc_randk(uint32_t* state, int32_t k, size_t U, const uint32_t* upper, uint32_t* out);
void   orc_randseqk(uint32_t* state, int32_t k, size_t U, const uint32_t* upper, uint32_t* out);
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) */
void   orc_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* k distinct upper positions of draw number `draw` of client `client`: images of 0..k-1 under a
 * Philox-keyed Feistel permutation of [0, 2^b) walked into [0, U); out = sorted flat indices */
void   orc_randk_philox(uint32_t seed, uint32_t client, uint32_t draw, int32_t k, size_t U, const uint32_t* upper,
                        uint32_t* out);
/* TopK over |m[upper[..]]| of a full d x lda column-major matrix; writes k sorted flat indices */
int32_t orc_topk(const double* m, int32_t k, size_t U, const uint32_t* upper, uint32_t* out);
/* TopLEK; frob_sq = squared L2 norm of the whole d x lda buffer; returns the count written */
int32_t orc_toplek(const double* m, int32_t lda, int32_t k, size_t U, const uint32_t* upper,
                   double delta, double frob_sq, uint32_t* rng_state, uint32_t* out);
double  orc_natural(double v);                       /* mantissa truncation, MatrixNMD.h:2013-2031 */
uint32_t orc_pack2_natural(double a, double b);      /* pack2FP64NoMantissa, FloatUtils.h:193-221 */
double  orc_l2sq(const double* v, size_t n);          /* fixed chunked order, see the .c file */
double  orc_frob_sym(const double* m, int32_t d, int32_t lda);
double  orc_exp(double x);
double  orc_log(double x);
/* reference-order arithmetic (ref_order = 1) */
double  orc_ref_dot(const double* a, const double* b, size_t n);
double  orc_ref_norm2(const double* a, size_t n);
double  orc_exp_vcl(double x);
double  orc_exp_cr(double x);
double  orc_log_vcl(double x);
double  orc_frob_ref(const double* m, int32_t d, int32_t lda);
void    orc_margin_ref(const double* atr, int32_t d, int32_t lda, int32_t n, const double* x, double* m);
void    orc_sigmoid_ref(const double* m, int32_t n, double* sig);
double  orc_client_function_ref(const double* sig, int32_t n, const double* x, int32_t d, double lambda);
int     orc_cholesky_ref(const double* h, int32_t d, int32_t lda, double l, double* ltr);
void    orc_solve_chol_ref(const double* ltr, int32_t d, int32_t lda, const double* b, double* x);
int32_t orc_toplek_ref(const double* m, int32_t lda, int32_t k, size_t U, const uint32_t* upper,
                       double delta, double frob_sq, uint32_t* rng_state, uint32_t* out);
/* L2-logistic objective of one client from its sigmoid values (evaluateFunction(x, margin, sigmoid),
 * logistic_regression.h:119-123): -mean log sigma_s + lambda/2 ||x||^2 */
double  orc_client_function(const double* sig, int32_t n, const double* x, int32_t d, double lambda);

/* ---- logistic-regression oracle (one client) ------------------------------------------ */
/* atr: d x n col-major with leading dimension lda, column s = b_s * a_s */
void orc_margin(const double* atr, int32_t d, int32_t lda, int32_t n, const double* x, double* m);
void orc_sigmoid(const double* m, int32_t n, double* sig);
void orc_gradient(const double* atr, int32_t d, int32_t lda, int32_t n, const double* x,
                  const double* sig, double lambda, double* g);
/* full symmetric d x lda Hessian (+lambda on the diagonal) */
void orc_hessian(const double* atr, int32_t d, int32_t lda, int32_t n, const double* sig,
                 double lambda, double* h);

/* ---- Option-B solve -------------------------------------------------------------------- */
/* LDL^T of (upper(h) + l I) into ltr (d x lda: upper = multipliers of L^T with D on the diagonal,
 * mirrored into the lower part); 1 on success, 0 for a negative pivot */
int  orc_ldlt(const double* h, int32_t d, int32_t lda, double l, double* ltr);
void orc_solve_ldlt(const double* ltr, int32_t d, int32_t lda, const double* b, double* x);

/* ---- whole FedNL run (forcesequpdate semantics: master merges clients in order) -------- */
orc_state* orc_create(const orc_problem* p, const double* x0);
void   orc_destroy(orc_state* s);
/* one round; *grad_norm = ||aggregated gradient at the round's starting iterate|| */
int    orc_round(orc_state* s, double* grad_norm);
void   orc_get_x(const orc_state* s, double* x);
void   orc_get_H(const orc_state* s, double* h);            /* master H, d x lda */
void   orc_get_shift(const orc_state* s, int32_t c, double* sh);
double orc_get_l(const orc_state* s);
void   orc_get_grad(const orc_state* s, double* g);
/* last round's message of client c: indices (flat) and values; returns count */
int32_t orc_get_message(const orc_state* s, int32_t c, uint32_t* idx, double* val);
/* last round's Lk of client c */
double orc_get_lk(const orc_state* s, int32_t c);

/* ---- FedNL-PP extras ------------------------------------------------------------------- */
/* true gradient (mean of every client's gradient at the round's starting iterate; its norm is what
 * orc_round returns in PP mode) */
void   orc_get_true_grad(const orc_state* s, double* g);
/* the round's sampled clients in ascending order; returns tau */
int32_t orc_get_selected(const orc_state* s, int32_t* out);
/* f(x) at the last round's starting iterate (tracking / line search) and the number of line-search
 * evaluations the last round made */
double  orc_get_f(const orc_state* s);
int32_t orc_get_ls_steps(const orc_state* s);
/* client c's running direction (x Lk + shift x - grad) and its last sent difference */
void   orc_get_dir(const orc_state* s, int32_t c, double* dir, double* ddir);

#ifdef __cplusplus
}
#endif
#endif
