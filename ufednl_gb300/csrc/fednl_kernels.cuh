// fednl_kernels.cuh -- sm_103a kernels of one FedNL round.
//
// Storage (one problem, resident in HBM):
//   * symmetric d x d matrices (client shifts, differences, the master H, the Cholesky factor)
//     are stored as their packed upper triangle: position p = j (j + 1) / 2 + i for i <= j.
//     This is exactly the order of the reference's upper-index list (column j, rows 0..j,
//     dopt/dopt/math_routines/include/SpecialMathRoutinesForMatrix.h:35-64), so "scan order",
//     "ascending flat index j * lda + i" and "ascending p" coincide.  Half the bytes of the
//     reference's full d x lda buffers; the lower triangle is its mirror.
//   * binary {0,1} features: per client and attribute one bit per sample (feature-major
//     bitmasks) plus a per-sample CSR list of nonzero attributes;
//   * dense features: row-major [sample][d] FP64.
//
// Floating-point discipline: wherever the reference fixes an operation order, the kernels
// perform the same IEEE operations in the same order with explicit __d*_rn intrinsics (no
// fused multiply-add), so that values match the CPU oracle bit for bit given identical inputs.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "fednl_philox.cuh"

namespace fednl {

constexpr int kMaxK = 9600;             // largest TopK/TopLEK k: heap, chain and staging fit in 227 KB of shared memory

struct Dev {
    // sizes and scalars
    int d, lda, U, nc, k, comp, W, SW, nfpart, nseg;
    int ustr;               // row stride of the per-client [U] arrays (U rounded up to 32)
    double lambda, alpha, prescale, inv_n, mult;
    // clients
    const int* ns;          // [nc]
    const int* soff;        // [nc + 1]
    const int* client_of;   // [S]
    const long long* fboff; // [nc] u64 offset of the client's d x words bitmask block
    // features
    const int* rowptr;      // [S + 1]  binary: nonzero attributes of each sample
    const int* colidx;      // [nnz]
    const unsigned long long* fbits;
    const double* A;        // dense [S][d]
    const double* lab;      // [S]
    // state
    double* x;              // [d]
    double* H;              // [U] master
    double* g;              // [d]
    double* shift;          // [nc][ustr]
    double* diff;           // [nc][ustr]
    double* Dv;             // [S] Hessian weights D_s
    double* qb;             // [S] gradient weights b_s * q_s
    double* gc;             // [nc][d]
    double* dsum;           // [nc][d] sum of D_s over the samples with attribute j set (Hessian diagonal - lambda)
    const int* icpt;        // [nc] 1 if the client's last attribute is 1 for every sample (intercept)
    double* Fpart;          // [nc][nseg] segment sums of ||diff||_F^2 (512 upper positions each)
    double* F;              // [nc] ||diff||_F^2
    double* lk;             // [nc]
    unsigned* sel;          // [nc][SW] selection bitmaps over p
    int* cnt;               // [nc]
    int* needs;             // [nc] TopLEK: rounding draw needed
    double* pdraw;          // [nc]
    int* minidx;            // [nc]
    unsigned* wstate;       // [W] TopLEK generators
    unsigned* rstate;       // [nc] RandK / RandSeqK generators
    int* rseq;              // [nc] RandSeqK window start
    unsigned long long* hmap; // [nc][hcap] RandK virtual-shuffle map
    int hcap;
    double* work;           // [U] Cholesky factor
    double* dx;             // [d]
    double* ybuf;           // [d]
    double* rinv;           // [d] 1 / r_kk of the last factorization
    double* hist;           // [max_rounds] ||g|| history
    int* round_ctr;         // [1]
    int* status;            // [1]
    double* stats;          // [2] ||g||, l
    int hist_cap;
    unsigned* bar;          // [4] grid barrier: arrival count, generation, error flag
    // FedNL-PP (bin_fednl_local_pp); act == nullptr: every client takes part (plain FedNL)
    int pp, n_act;          // n_act: clients processed this round (tau, or nc without PP)
    const int* act;         // [n_act] processed clients in ascending order
    int* is_sel;            // [nc]
    int* perm;              // [nc] the sampler's permutation (when it does not fit in shared memory)
    unsigned* sampler;      // [1] client sampler (RandomGenIntegerLinear)
    double* hbuf;           // [nc][ustr] the round's client Hessians (Lk after the update)
    double* dir;            // [nc][d] localGradient = x Lk + shift x - grad
    double* ddir;           // [nc][d] its last sent difference
    double* dlk;            // [nc] last sent Lk difference
    double* gprev;          // [d] running mean of the directions
    double* lprev;          // [1] running mean of Lk
    double* tg;             // [d] true gradient at the round's starting iterate
    // objective values (tracking) and FedNL-LS
    int fmode;              // 1: form -log sigma_s per sample and f_i per client every round
    double* fterm;          // [S] -log sigma_s at the last evaluated point
    double* fi;             // [nc] f_i at the last evaluated point
    double* xprev;          // [d] x_k during the line search
    double* ls;             // [5] line search: t, -(dx . g), done, evaluations, solve succeeded
    unsigned* hdone;        // [nc] Hessian blocks of a client finished this round (the last one forms F)
    // binary Hessian from the clients' static common-sample lists (k_hess_hits)
    const unsigned short* hcode; // [nc][ustr] per upper position (see k_hess_hits)
    const unsigned* hseg;        // [nc][nseg + 1] first multi-sample record of each segment
    const unsigned* hrec;        // [records + 1] first common sample of each record in hhits
    const unsigned short* hhits; // common samples of the multi-sample records, in sample order
    // the reference's arithmetic order (fednl_refmode.cuh)
    int ref;                // 1: FEDNL_ORDER_REFERENCE
    double* rref;           // [(d+1)(d+2)/2] Cholesky factor with y as column d
    double* racc;           // [9][(d+1)(d+2)/2] lane and tail accumulators of its dot products
};

// ---- helpers -------------------------------------------------------------------------------

// p -> (i, j) with p = j (j + 1) / 2 + i, i <= j; FP32 square root plus exact integer correction
__device__ __forceinline__ void upper_ij(int p, int& i, int& j)
{
    int jj = (int)((sqrtf(8.0f * (float)p + 1.0f) - 1.0f) * 0.5f);
    while (jj > 0 && (long long)jj * (jj + 1) / 2 > p) --jj;
    while ((long long)(jj + 1) * (jj + 2) / 2 <= p) ++jj;
    j = jj;
    i = p - (int)((long long)jj * (jj + 1) / 2);
}

__device__ __forceinline__ bool upper_is_diag(int p)
{
    int i, j;
    upper_ij(p, i, j);
    return i == j;
}

// RandomGenIntegerLinear step (dopt/dopt/random/include/RandomGenIntegerLinear.h:107-123)
__device__ __forceinline__ unsigned lcg_int_next(unsigned& s)
{
    s = 214013u * s + 2531011u;
    return s;
}

// RandomGenIntegerLinear::generateRealInUnitInterval (RandomGenIntegerLinear.h:49-58)
__device__ __forceinline__ double lcg_int_unit(unsigned& s)
{
    s = 214013u * s + 2531011u;
    return __dmul_rn((double)s, 1.0 / 4294967295.0);
}

// RandomGenRealLinear::generateRealInUnitInterval (RandomGenRealLinear.h:54-59)
__device__ __forceinline__ double lcg_real_unit(unsigned& s)
{
    unsigned t = 214013u * s + 2531011u;
    s = t % 4294967295u;
    return __dmul_rn((double)s, 1.0 / 4294967295.0);
}

// roundToNearestInt<size_t> (dopt/dopt/math_routines/include/SimpleMathRoutines.h:408-414)
__device__ __forceinline__ unsigned long long round_to_nearest(double v)
{
    unsigned long long t = (unsigned long long)v;
    if (__dsub_rn(v, (double)t) > 0.5) return t + 1;
    return t;
}

__device__ __forceinline__ double natural_trunc(double v)
{
    return __longlong_as_double(__double_as_longlong(v) & ~((1ll << 52) - 1));
}

// exp(x), own implementation with the same IEEE operation sequence as the CPU oracle: Cody-Waite
// reduction x = k ln2 + r (ln2 = 32-bit head + tail: the two-part ln2 published with fdlibm's
// e_exp.c / e_log.c, 6.93147180369123816490e-01 + 1.90821492927058770002e-10), r as a double-double, exp(r) = 1 + r + r^2/2
// + r^3/6 + r^4 P(r) with the leading terms summed through exact two-sum / two-product errors and
// the Taylor tail in double, one final rounding, scaling by 2^k.  Error before the last rounding
// about 1e-3 ulp.
__device__ __forceinline__ double pow2i(int k) { return __longlong_as_double((long long)(k + 1023) << 52); }

__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e)
{
    double t = __dadd_rn(a, b);
    double bb = __dsub_rn(t, a);
    e = __dadd_rn(__dsub_rn(a, __dsub_rn(t, bb)), __dsub_rn(b, bb));
    s = t;
}

__device__ __forceinline__ double fednl_exp(double x)
{
    if (x != x) return x;
    if (x > 709.782712893384) return __longlong_as_double(0x7ff0000000000000ll);
    if (x < -745.1332191019412) return 0.0;
    const double ln2_hi = 6.93147180369123816490e-01, ln2_lo = 1.90821492927058770002e-10;
    double kd = rint(__dmul_rn(x, 1.4426950408889634));
    double t = fma(-kd, ln2_hi, x);
    double pl_hi = __dmul_rn(kd, ln2_lo);
    double pl_lo = fma(kd, ln2_lo, -pl_hi);
    double r_hi, e0;
    two_sum(t, -pl_hi, r_hi, e0);
    double r_lo = __dsub_rn(e0, pl_lo);
    double r2 = __dmul_rn(r_hi, r_hi);
    double r2e = fma(r_hi, r_hi, -r2);
    double r3 = __dmul_rn(r2, r_hi);
    double r3e = __dadd_rn(fma(r2, r_hi, -r3), __dmul_rn(r2e, r_hi));
    double q = 1.6059043836821613e-10;
    q = fma(q, r_hi, 2.0876756987868100e-09);
    q = fma(q, r_hi, 2.5052108385441720e-08);
    q = fma(q, r_hi, 2.7557319223985893e-07);
    q = fma(q, r_hi, 2.7557319223985888e-06);
    q = fma(q, r_hi, 2.4801587301587302e-05);
    q = fma(q, r_hi, 1.9841269841269841e-04);
    q = fma(q, r_hi, 1.3888888888888889e-03);
    q = fma(q, r_hi, 8.3333333333333332e-03);
    q = fma(q, r_hi, 4.1666666666666664e-02);
    double tail = __dmul_rn(__dmul_rn(r2, r2), q);
    const double c6 = 1.6666666666666666e-01, c6e = 9.2518585385429707e-18;
    double s3 = __dmul_rn(r3, c6);
    double s3e = __dadd_rn(fma(r3, c6, -s3), __dadd_rn(__dmul_rn(r3e, c6), __dmul_rn(r3, c6e)));
    double s, e1, e2, e3;
    two_sum(1.0, r_hi, s, e1);
    two_sum(s, __dmul_rn(r2, 0.5), s, e2);
    two_sum(s, s3, s, e3);
    double lo = __dadd_rn(__dadd_rn(__dadd_rn(e1, e2), e3), __dadd_rn(__dadd_rn(__dmul_rn(r2e, 0.5), s3e), tail));
    lo = fma(r_lo, __dadd_rn(1.0, r_hi), lo);
    double p = __dadd_rn(s, lo);
    int k = (int)kd;
    if (k > 1000) return __dmul_rn(__dmul_rn(p, pow2i(k - 1000)), pow2i(1000));
    if (k < -1000) return __dmul_rn(__dmul_rn(p, pow2i(k + 1000)), pow2i(-1000));
    return __dmul_rn(p, pow2i(k));
}

// Natural logarithm (the CPU oracle's orc_log, operation for operation): x = 2^e m, m in
// [sqrt(1/2), sqrt(2)), log m = 2 atanh((m - 1)/(m + 1)) with the quotient as a double-double, the
// odd series to s^23/23 for the tail, e ln 2 in two parts.  Below one ulp of error.
__device__ __forceinline__ double fednl_log(double x)
{
    if (x != x) return x;
    if (x < 0.0) return __longlong_as_double(0x7ff8000000000000ll);
    if (x == 0.0) return __longlong_as_double((long long)0xfff0000000000000ull);
    if (x == __longlong_as_double(0x7ff0000000000000ll)) return x;
    long long b = __double_as_longlong(x);
    int e = 0;
    if ((b >> 52) == 0) {
        x = __dmul_rn(x, 18014398509481984.0);
        b = __double_as_longlong(x);
        e = -54;
    }
    e += (int)(b >> 52) - 1023;
    double m = __longlong_as_double((b & 0x000fffffffffffffll) | 0x3ff0000000000000ll);
    if (m > 1.4142135623730951) {
        m = __dmul_rn(m, 0.5);
        e += 1;
    }
    const double ln2_hi = 6.93147180369123816490e-01, ln2_lo = 1.90821492927058770002e-10;
    const double f = __dsub_rn(m, 1.0);
    double g_hi, g_lo;
    two_sum(m, 1.0, g_hi, g_lo);
    const double s_hi = __ddiv_rn(f, g_hi);
    const double r = __dsub_rn(fma(-s_hi, g_hi, f), __dmul_rn(s_hi, g_lo));
    const double s_lo = __ddiv_rn(r, g_hi);
    const double z = __dmul_rn(s_hi, s_hi);
    double q = 1.0 / 23.0;
    q = fma(q, z, 1.0 / 21.0);
    q = fma(q, z, 1.0 / 19.0);
    q = fma(q, z, 1.0 / 17.0);
    q = fma(q, z, 1.0 / 15.0);
    q = fma(q, z, 1.0 / 13.0);
    q = fma(q, z, 1.0 / 11.0);
    q = fma(q, z, 1.0 / 9.0);
    q = fma(q, z, 1.0 / 7.0);
    q = fma(q, z, 1.0 / 5.0);
    q = fma(q, z, 1.0 / 3.0);
    const double tail = __dmul_rn(__dmul_rn(__dmul_rn(s_hi, z), q), 2.0);
    const double ed = (double)e;
    double h, l;
    two_sum(__dmul_rn(ed, ln2_hi), __dmul_rn(s_hi, 2.0), h, l);
    l = __dadd_rn(l, __dadd_rn(__dadd_rn(__dmul_rn(s_lo, 2.0), tail), __dmul_rn(ed, ln2_lo)));
    return __dadd_rn(h, l);
}

__device__ __forceinline__ double rcp_rn_int(double r);

// 1 / (1 + exp(-m)); the correctly rounded reciprocal from integer arithmetic equals the IEEE
// division 1.0 / (1 + e) bit for bit and keeps the FP64 pipe free
__device__ __forceinline__ double fednl_sigmoid(double m)
{
    return rcp_rn_int(__dadd_rn(1.0, fednl_exp(-m)));
}

// Sum of one aligned 32-term chunk held one term per lane: the halving tree
// v[l] += v[l + h], h = 16, 8, 4, 2, 1 (valid in lane 0).  Chunk sums are then added in order by
// one thread.  The CPU oracle sums in exactly this order.
__device__ __forceinline__ double chunk_tree(double v)
{
    for (int h = 16; h > 0; h >>= 1) v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, h));
    return v;
}

template <int NT>
__device__ __forceinline__ double block_sum(double v, double* red)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < NT / 32; ++w) r += red[w];
    return r;  // valid in thread 0
}

// ---- 1. margins, sigmoid and the per-sample weights ----------------------------------------
// logistic_regression.h:88-101 (margin, sigmoid), :148-161 (q_s = (1 - sigma_s)(-1/n)),
// :387-393 (D_s = (1/n)((1 - sigma_s) sigma_s)).  Binary features: the margin is the sequential
// sum of x over the sample's nonzero attributes in ascending order, times the label -- the same
// IEEE additions as the reference's dot product with the +-1 / 0 column.
__global__ void k_margin_binary(Dev P, int S)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    int c = P.client_of[s];
    double acc = 0.0;
    for (int t = P.rowptr[s]; t < P.rowptr[s + 1]; ++t) acc = __dadd_rn(acc, P.x[P.colidx[t]]);
    double b = P.lab[s];
    double m = (b == 1.0) ? acc : -acc;
    double sig = fednl_sigmoid(m);
    double inv_m = 1.0 / (double)P.ns[c];
    double z1 = __dsub_rn(1.0, sig);
    P.Dv[s] = __dmul_rn(inv_m, __dmul_rn(z1, sig));
    double q = __dmul_rn(z1, -inv_m);
    P.qb[s] = (b == 1.0) ? q : __dmul_rn(-1.0, q);
    if (P.fmode) P.fterm[s] = -fednl_log(sig);
}

// dense features: column s of Atr is b_s * a_s (logistic_regression.h:45-75)
__global__ void k_margin_dense(Dev P, int S)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    int c = P.client_of[s];
    double b = P.lab[s];
    const double* a = P.A + (size_t)s * P.d;
    double acc = 0.0;
    for (int i = 0; i < P.d; ++i) {
        double u = (b == 1.0) ? a[i] : __dmul_rn(a[i], -1.0);
        acc = __dadd_rn(acc, __dmul_rn(u, P.x[i]));
    }
    double sig = fednl_sigmoid(acc);
    double inv_m = 1.0 / (double)P.ns[c];
    double z1 = __dsub_rn(1.0, sig);
    P.Dv[s] = __dmul_rn(inv_m, __dmul_rn(z1, sig));
    P.qb[s] = __dmul_rn(z1, -inv_m);   // dense: the label enters through u
    if (P.fmode) P.fterm[s] = -fednl_log(sig);
}

// acc + the weights of the samples whose bits are set in the attribute's W mask words, added in
// sample order.  A full word (every sample of 64, as the intercept column's) takes the 64 adds with
// their loads issued ahead: the chain is then the FP64 add latency alone, not a bit walk per term.
__device__ __forceinline__ double attr_sum(const unsigned long long* fb, int W, const double* wv, double acc)
{
    for (int w = 0; w < W; ++w) {
        unsigned long long m = fb[w];
        if (m == ~0ull) {
            const double* v = wv + w * 64;
#pragma unroll 16
            for (int t = 0; t < 64; ++t) acc = __dadd_rn(acc, v[t]);
            continue;
        }
        while (m) {
            const int b = w * 64 + __ffsll((long long)m) - 1;
            m &= m - 1;
            acc = __dadd_rn(acc, wv[b]);
        }
    }
    return acc;
}

// The engine's fixed order for the attribute sums of {0,1} features (gradient and dsum): the
// samples holding the attribute are taken in 64-sample words; a word's terms are summed in sample
// order (its first term exactly), and the word sums are added to acc in word order (the CPU
// oracle's blocked_attr_sum).  One FP64 add per set bit, in a single loop over the bits whose
// adds are branch-free: a bit that opens a new word adds the finished word sum into acc, any other
// bit adds its term into the open word sum.  The lanes of a warp then issue one FP64 instruction
// per step of the longest bit list, not per word of it.
__device__ __forceinline__ double attr_sum_blocked(const unsigned long long* fb, int W, const double* wv, double acc)
{
    int w = 0;
    unsigned long long m = fb[0];
    while (!m && ++w < W) m = fb[w];
    if (!m) return acc;
    int pw = w;
    double part = wv[w * 64 + __ffsll((long long)m) - 1];
    m &= m - 1;
    for (;;) {
        while (!m && ++w < W) m = fb[w];
        if (!m) break;
        const double v = wv[w * 64 + __ffsll((long long)m) - 1];
        m &= m - 1;
        const bool nw = w != pw;
        const double sum = __dadd_rn(nw ? acc : part, nw ? part : v);
        acc = nw ? sum : acc;
        part = nw ? v : sum;
        pw = w;
    }
    return __dadd_rn(acc, part);
}

// ---- 2. client gradients g_c = lambda x + sum_s Atr[:, s] q_s (samples in order) ----------
// One block per (client, range of attributes); the client's weights are staged in shared memory.
// The same bit loop also forms dsum_j = sum of D_s over the samples with attribute j set, which is
// bit for bit the Hessian diagonal before lambda (and the intercept column) of evaluateHessian.
__global__ void k_grad_binary(Dev P)
{
    extern __shared__ double s_w[];    // [n] b_s q_s, then [n] D_s
    const int c = blockIdx.y;
    const int n = P.ns[c], W = (n + 63) >> 6, off = P.soff[c];
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        s_w[t] = P.qb[off + t];
        s_w[n + t] = P.Dv[off + t];
    }
    __syncthreads();
    // lane pair (2j, 2j+1): the gradient sum and the diagonal sum of attribute j walk the same bits,
    // one FP64 add each per bit (a warp issues one FP64 instruction per bit, not two)
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = t >> 1, which = t & 1;
    if (j >= P.d) return;
    const unsigned long long* fb = P.fbits + P.fboff[c] + (size_t)j * W;
    const double* wv = s_w + (which ? n : 0);
    const double a0 = which ? 0.0 : __dmul_rn(P.x[j], P.lambda);
    const double acc = P.ref ? attr_sum(fb, W, wv, a0) : attr_sum_blocked(fb, W, wv, a0);
    if (which) P.dsum[(size_t)c * P.d + j] = acc;
    else P.gc[(size_t)c * P.d + j] = acc;
}

// The clients' bit layout (k_hess_binary's masks: per client, per attribute, one bit per sample,
// 64 samples a word) from the samples' CSR columns, one thread per sample: the CSR upload packs A_i
// on the device (dataset_loader_fs.h:607-870 reads the same rows into the reference's matrices).
__global__ void k_pack_bits(const int* __restrict__ rowptr, const int* __restrict__ colidx, const int* client_of,
                            const int* soff, const int* ns, const long long* fboff, int S, unsigned long long* fbits)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const int c = client_of[s], ls = s - soff[c], W = (ns[c] + 63) >> 6;
    unsigned long long* fb = fbits + fboff[c];
    for (int u = rowptr[s]; u < rowptr[s + 1]; ++u)
        atomicOr(fb + (size_t)colidx[u] * W + (ls >> 6), 1ull << (ls & 63));
}

// ---- 1 + 2 fused for binary features: one CTA per client -----------------------------------
// The client's margins, sigmoid values and weights (k_margin_binary's operations, one sample per
// thread), then its gradient and attribute sums (k_grad_binary's, blocked order, a lane pair per
// attribute) with the weights already in shared memory: one launch for the client oracle.  When the
// client's last attribute is an intercept (set in every sample), the block's last warp forms its two
// sums alone: the word sums in parallel, one lane per word, then added in word order, so that the
// longest chain of dependent adds is 63 + W instead of n.  blockDim.x is a multiple of 32.
__global__ void k_client_binary(Dev P)
{
    extern __shared__ double s_w[];    // [n] b_s q_s, [n] D_s, [2][W] intercept word sums
    __shared__ double s_inv;
    const int c = blockIdx.x;
    const int n = P.ns[c], W = (n + 63) >> 6, off = P.soff[c];
    // the round's solve finds its grid-barrier words and error flag at zero (no solve runs now)
    if (c == 0 && threadIdx.x < 4) P.bar[threadIdx.x] = 0u;
    if (threadIdx.x == 0) s_inv = 1.0 / (double)n;      // one FP64 division per client
    __syncthreads();
    const double inv_m = s_inv;
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const int s = off + t;
        double acc = 0.0;
        for (int u = P.rowptr[s]; u < P.rowptr[s + 1]; ++u) acc = __dadd_rn(acc, P.x[P.colidx[u]]);
        const double b = P.lab[s];
        const double m = (b == 1.0) ? acc : -acc;
        const double sig = fednl_sigmoid(m);
        const double z1 = __dsub_rn(1.0, sig);
        const double dv = __dmul_rn(inv_m, __dmul_rn(z1, sig));
        const double q = __dmul_rn(z1, -inv_m);
        const double qb = (b == 1.0) ? q : __dmul_rn(-1.0, q);
        P.Dv[s] = dv;
        P.qb[s] = qb;
        if (P.fmode) P.fterm[s] = -fednl_log(sig);
        s_w[t] = qb;
        s_w[n + t] = dv;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const bool icw = P.icpt[c] != 0;
    if (icw && warp == nw - 1) {
        double* part = s_w + 2 * n;
        for (int t = lane; t < 2 * W; t += 32) {
            const int which = t >= W ? 1 : 0, w = t - which * W;
            const double* v = s_w + which * n + w * 64;
            double a = v[0];
            if (w * 64 + 64 <= n) {
#pragma unroll 21
                for (int k = 1; k < 64; ++k) a = __dadd_rn(a, v[k]);
            } else {
                for (int k = 1; k < n - w * 64; ++k) a = __dadd_rn(a, v[k]);
            }
            part[t] = a;
        }
        __syncwarp();
        if (lane < 2) {
            const int j = P.d - 1;
            double acc = lane ? 0.0 : __dmul_rn(P.x[j], P.lambda);
            for (int w = 0; w < W; ++w) acc = __dadd_rn(acc, part[lane * W + w]);
            if (lane) P.dsum[(size_t)c * P.d + j] = acc;
            else P.gc[(size_t)c * P.d + j] = acc;
        }
        return;
    }
    const int nt = icw ? blockDim.x - 32 : blockDim.x;
    const int na = icw ? P.d - 1 : P.d;
    for (int t = threadIdx.x; t < 2 * na; t += nt) {
        const int j = t >> 1, which = t & 1;
        const unsigned long long* fb = P.fbits + P.fboff[c] + (size_t)j * W;
        const double* wv = s_w + (which ? n : 0);
        const double acc = attr_sum_blocked(fb, W, wv, which ? 0.0 : __dmul_rn(P.x[j], P.lambda));
        if (which) P.dsum[(size_t)c * P.d + j] = acc;
        else P.gc[(size_t)c * P.d + j] = acc;
    }
}

__global__ void k_grad_dense(Dev P)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int c = blockIdx.y;
    if (j >= P.d) return;
    int n = P.ns[c], off = P.soff[c];
    double g = __dmul_rn(P.x[j], P.lambda);
    for (int s = 0; s < n; ++s) {
        double a = P.A[(size_t)(off + s) * P.d + j];
        double u = (P.lab[off + s] == 1.0) ? a : __dmul_rn(a, -1.0);
        g = __dadd_rn(g, __dmul_rn(u, P.qb[off + s]));
    }
    P.gc[(size_t)c * P.d + j] = g;
}

// ---- 3. client Hessians fused with the difference and its Frobenius norm ------------------
// evaluateHessian<true,4> (logistic_regression.h:365-547): entry (i, j) is the sum over samples
// in order of u_i (D_s u_j); for {0,1} features every nonzero term equals D_s exactly, so the
// entry is the in-order sum of D_s over the samples where both attributes are set (bitmask
// AND).  Then + lambda on the diagonal.  mode 0: diff = H_i - shift_i (TopK.h:70-71) and the
// partial sums of ||diff||_F^2 over the full symmetric matrix; mode 1: shift_i = H_i(x0); mode 2
// (FedNL-PP): mode 0 and H_i kept for the Lk taken after the shift update; mode 3: the difference
// only (the selection kernel forms the norms).  Grid y runs over the processed clients (P.act).
constexpr int kHessThreads = 256;
constexpr int kHessPerBlock = 4096;     // upper entries per block

// Fixed-order ||diff||_F^2 (the CPU oracle's orc_frob_sym): each warp owns one segment of 512
// upper positions; lane l accumulates its 16 squares with fused multiply-adds, diagonal (a) and
// off-diagonal (b) apart, then contributes a + 2 b to the segment's halving tree.
__device__ __forceinline__ double segment_value(double a, double b) { return __dadd_rn(a, __dmul_rn(b, 2.0)); }

// F_c = ||diff_c||_F^2 as the in-order sum of the client's segment sums, and Lk = sqrt(F_c)
// (TopK.h:74-78); one warp, 32 segment sums loaded at a time and added one by one
__device__ __forceinline__ void client_fsum_warp(const Dev& P, int c, int lane)
{
    const double* fp = P.Fpart + (size_t)c * P.nseg;
    double f = 0.0;
    for (int q0 = 0; q0 < P.nseg; q0 += 32) {
        const double v = (q0 + lane < P.nseg) ? __ldcg(fp + q0 + lane) : 0.0;
        const int cnt = min(32, P.nseg - q0);
        for (int t = 0; t < cnt; ++t) f = __dadd_rn(f, __shfl_sync(0xffffffffu, v, t));
    }
    if (lane == 0) {
        P.F[c] = f;
        if (!P.pp) P.lk[c] = sqrt(f);    // FedNL-PP takes Lk after the update (k_pp_dir)
    }
}

// Called by every block of a Hessian launch after its Fpart stores: the last of a client's blocks
// (gridDim.x of them) forms F_c and Lk, then re-arms the client's counter for the next round.
__device__ __forceinline__ void client_fsum_last_block(const Dev& P, int c)
{
    __shared__ int s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(P.hdone + c, 1u) == gridDim.x - 1;
    __syncthreads();
    if (s_last && threadIdx.x < 32) {
        __threadfence();
        client_fsum_warp(P, c, threadIdx.x);
        if (threadIdx.x == 0) P.hdone[c] = 0u;
    }
}

template <bool SMEM_BITS, int NT>
__global__ void __launch_bounds__(NT) k_hess_binary(Dev P, int mode)
{
    extern __shared__ unsigned long long s_fb[];
    const int c = P.act ? P.act[blockIdx.y] : blockIdx.y;
    const int n = P.ns[c], W = (n + 63) >> 6, off = P.soff[c];
    const unsigned long long* gfb = P.fbits + P.fboff[c];
    double* s_D;
    const unsigned long long* fb;
    if (SMEM_BITS) {
        for (int t = threadIdx.x; t < P.d * W; t += blockDim.x) s_fb[t] = gfb[t];
        s_D = (double*)(s_fb + (size_t)P.d * W);
        fb = s_fb;
    } else {
        s_D = (double*)s_fb;
        fb = gfb;
    }
    for (int t = threadIdx.x; t < n; t += blockDim.x) s_D[t] = P.Dv[off + t];
    // the diagonal entries sum_s D_s a_si + lambda, formed once per block: in the entry loop a
    // diagonal lane would cost its warp a whole FP64 instruction
    double* s_dl = s_D + n;
    const double* dsum = P.dsum + (size_t)c * P.d;
    for (int t = threadIdx.x; t < P.d; t += blockDim.x) s_dl[t] = __dadd_rn(dsum[t], P.lambda);
    __syncthreads();

    const size_t base = (size_t)c * P.ustr;
    const bool icpt = P.icpt[c] != 0;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int seg = blockIdx.x * (NT / 32) + warp;     // 512 positions per warp, NT / 32 warps per block
    const int p_seg = seg * 512;
    double fa = 0.0, fb2 = 0.0;
    int i, j;
    upper_ij(p_seg + lane, i, j);
    for (int q = 0; q < 16; ++q) {
        const int p = p_seg + 32 * q + lane;
        if (p >= P.U) break;
        if (q > 0) {                   // advance (i, j) by 32 packed positions
            i += 32;
            while (i > j) {
                i -= j + 1;
                ++j;
            }
        }
        double h;
        if (i == j) {
            h = s_dl[i];
        } else if (icpt && j == P.d - 1) {
            h = dsum[i];               // samples with attribute i set, all of which have the intercept
        } else {
            const unsigned long long* mi = fb + (size_t)i * W;
            const unsigned long long* mj = fb + (size_t)j * W;
            // Per 32 mask words: pass 1, without branches, finds the words holding samples with
            // both attributes set; pass 2 sums over those words only, in sample order.  The sum's
            // first term is 0 + D_s = D_s exactly (D_s >= 0), so it costs no FP64 add: on this part
            // a warp's FP64 instruction takes the pipe for ~64 cycles however few lanes are active,
            // and most entries have at most one sample with both attributes set
            h = 0.0;
            bool first = true;
            for (int w0 = 0; w0 < W; w0 += 32) {
                const int w1 = min(W, w0 + 32);
                unsigned nz = 0u;
                for (int w = w0; w < w1; ++w) nz |= (unsigned)((mi[w] & mj[w]) != 0ull) << (w - w0);
                while (nz) {
                    const int w = w0 + __ffs(nz) - 1;
                    nz &= nz - 1u;
                    unsigned long long m = mi[w] & mj[w];
                    if (first) {
                        const int b = __ffsll((long long)m) - 1;
                        m &= m - 1;
                        h = s_D[w * 64 + b];
                        first = false;
                    }
                    while (m) {
                        const int b = __ffsll((long long)m) - 1;
                        m &= m - 1;
                        h = __dadd_rn(h, s_D[w * 64 + b]);
                    }
                }
            }
        }
        if (mode == 1) {
            P.shift[base + p] = h;
        } else {
            if (mode == 2) P.hbuf[base + p] = h;
            const double df = __dsub_rn(h, P.shift[base + p]);
            P.diff[base + p] = df;
            if (mode != 3) {
                const double r = fma(df, df, i == j ? fa : fb2);     // one FP64 instruction per warp
                if (i == j) fa = r;
                else fb2 = r;
            }
        }
    }
    if ((mode == 0 || mode == 2) && p_seg < P.U) {
        const double cs = chunk_tree(segment_value(fa, fb2));
        if (lane == 0) P.Fpart[(size_t)c * P.nseg + seg] = cs;
    }
    if ((mode == 0 || mode == 2) && !P.ref) client_fsum_last_block(P, c);
}

// dense FP64: the reference's per-entry order u_i (D_s u_j), samples in order
__global__ void __launch_bounds__(kHessThreads) k_hess_dense(Dev P, int mode)
{
    const int c = P.act ? P.act[blockIdx.y] : blockIdx.y;
    const int n = P.ns[c], off = P.soff[c];
    const size_t base = (size_t)c * P.ustr;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int seg = blockIdx.x * (kHessThreads / 32) + warp;
    const int p_seg = seg * 512;
    double fa = 0.0, fb2 = 0.0;
    for (int q = 0; q < 16; ++q) {
        const int p = p_seg + 32 * q + lane;
        if (p >= P.U) break;
        int i, j;
        upper_ij(p, i, j);
        double h = 0.0;
        for (int s = 0; s < n; ++s) {
            const double* a = P.A + (size_t)(off + s) * P.d;
            const bool pos = P.lab[off + s] == 1.0;
            const double ui = pos ? a[i] : __dmul_rn(a[i], -1.0);
            const double uj = pos ? a[j] : __dmul_rn(a[j], -1.0);
            h = __dadd_rn(h, __dmul_rn(ui, __dmul_rn(P.Dv[off + s], uj)));
        }
        if (i == j) h = __dadd_rn(h, P.lambda);
        if (mode == 1) {
            P.shift[base + p] = h;
        } else {
            if (mode == 2) P.hbuf[base + p] = h;
            const double df = __dsub_rn(h, P.shift[base + p]);
            P.diff[base + p] = df;
            if (mode != 3) {
                const double r = fma(df, df, i == j ? fa : fb2);     // one FP64 instruction per warp
                if (i == j) fa = r;
                else fb2 = r;
            }
        }
    }
    if ((mode == 0 || mode == 2) && p_seg < P.U) {
        const double cs = chunk_tree(segment_value(fa, fb2));
        if (lane == 0) P.Fpart[(size_t)c * P.nseg + seg] = cs;
    }
    if ((mode == 0 || mode == 2) && !P.ref) client_fsum_last_block(P, c);
}

// master H = mean_i shift_i after the initial shifts (TrainLoop.h:639-643, :732-735)
__global__ void k_h_init(Dev P)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.U) return;
    double h = 0.0;
    for (int c = 0; c < P.nc; ++c) h = __dadd_rn(h, P.shift[(size_t)c * P.ustr + p]);
    P.H[p] = __dmul_rn(h, P.inv_n);
}

// ---- 4. TopK / TopLEK: exact emulation of the reference's 4-ary heap ------------------------
// dopt/dopt/math_routines/include/MinHeap.h (D = 4) as used by getTopKFromUpperDiagonalPart and
// getTopLEKFromUpperDiagonalPart (SpecialMathRoutinesForMatrix.h:229-511).  The reference's
// minHeapify keeps comparing a node's children with the value that moved up on the previous
// level (MinHeap.h:259-286), so its "heap" is not a true heap and the selected set is not the
// plain top-k by magnitude; every comparison, swap and tie is reproduced here step by step.
//
// * Keys are the IEEE bit patterns of |v| compared as unsigned 64-bit integers: for non-negative
//   doubles this order is exactly the floating-point order (GB300's FP64 compares are slow).
// * buildMinHeap runs level by level in parallel: sifts of nodes on one level touch disjoint
//   subtrees, so the result equals the reference's descending-index order.
// * The scanned entries stream into shared memory by bulk asynchronous copies (cp.async.bulk with
//   an mbarrier per buffer, double-buffered); one warp tests them 256 at a time, each lane its
//   first entry above the root, one warp-wide minimum per replacement.  The heap's top two levels
//   live in registers during the scan, the same in every lane, and the warp replaces the root in
//   step: most root replacements stop within the top three levels (the carried comparison value
//   ends the walk early), so a replacement is a few compares and at most one shared-memory load.
// * TopLEK extracts in chunks of 32 recording the order in place (extracFromMinHeap leaves the
//   extracted element at the array's end, MinHeap.h:133-140) and stops after the chunk that opens
//   the rounding window; the top two heap levels live in registers during the extraction.  The
//   window numerator uses the fixed parallel order of the CPU oracle (chunked tree for the heap's
//   terms, chunked doubling scan plus in-order carries for the extracted terms).
struct HeapS {
    unsigned long long* key;   // bits of |value|
    unsigned* hid;             // packed upper position p
};

__device__ __forceinline__ unsigned long long abs_bits(double v)
{
    return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}

__device__ __forceinline__ void heap_swap(HeapS& h, int a, int b)
{
    unsigned long long tk = h.key[a];
    h.key[a] = h.key[b];
    h.key[b] = tk;
    unsigned ti = h.hid[a];
    h.hid[a] = h.hid[b];
    h.hid[b] = ti;
}

// minHeapify, MinHeap.h:255-290.  The entry (ck, ci) enters at node i with the carried comparison
// value lv.  The reference walks the children in order and moves to a child whose value is
// strictly below the running value, so it lands on the leftmost child holding the children's
// minimum whenever that minimum is strictly below lv; the carried value then becomes that
// minimum (the value that moved up, not the entry being sifted).  A two-level tree with strict
// '<' finds the same child.  The key array is placed so that the four children 4i+1..4i+4 of a
// node start on a 32-byte boundary (two 16-byte loads), the id array so that they start on a
// 16-byte boundary.  The path moves up one node and (ck, ci) is written where the walk stops,
// which equals the reference's chain of swaps.
__device__ __forceinline__ void heap_descend(HeapS& h, int i, int n, unsigned long long lv,
                                             unsigned long long ck, unsigned ci)
{
    for (;;) {
        const int f = 4 * i + 1;
        int lo;
        unsigned long long m;
        if (f + 3 < n) {
            const ulonglong2 a = *reinterpret_cast<const ulonglong2*>(h.key + f);
            const ulonglong2 b = *reinterpret_cast<const ulonglong2*>(h.key + f + 2);
            const bool r12 = a.y < a.x, r34 = b.y < b.x;
            const unsigned long long m12 = r12 ? a.y : a.x, m34 = r34 ? b.y : b.x;
            const bool r = m34 < m12;
            m = r ? m34 : m12;
            lo = f + (r ? (r34 ? 3 : 2) : (r12 ? 1 : 0));
        } else {
            if (f >= n) break;
            lo = f;
            m = h.key[f];
            for (int c = f + 1; c < n; ++c) {
                const unsigned long long cv = h.key[c];
                if (cv < m) {
                    m = cv;
                    lo = c;
                }
            }
        }
        if (!(lv > m)) break;
        h.key[i] = m;
        h.hid[i] = h.hid[lo];
        i = lo;
        lv = m;
    }
    h.key[i] = ck;
    h.hid[i] = ci;
}

__device__ __forceinline__ void heap_sift(HeapS& h, int i, int heap_size)
{
    const unsigned long long kv = h.key[i];
    heap_descend(h, i, heap_size, kv, kv, h.hid[i]);
}

constexpr int kSelThreads = 128;
constexpr int kSelStage = 2048;                    // doubles per staging buffer (16 KB)
constexpr long long kSelWaitCycles = 2000000000ll; // bounded mbarrier wait (~1 s)

// c v^2 with c = 1 on the diagonal and 2 off it
__device__ __forceinline__ double term_of(unsigned long long key, unsigned p)
{
    double v = __longlong_as_double((long long)key);
    double t = __dmul_rn(v, v);
    return upper_is_diag((int)p) ? t : __dmul_rn(t, 2.0);
}

// increaseMinimumInMinHeap (MinHeap.h:78-85): the root takes (cand, p) and sifts down; returns the
// new root value, which the scanning warp compares against next
__device__ __forceinline__ unsigned long long heap_replace_root(HeapS& h, int k, unsigned long long cand, unsigned p)
{
    if (k < 5) {
        heap_descend(h, 0, k, cand, cand, p);
        return h.key[0];
    }
    const ulonglong2 a = *reinterpret_cast<const ulonglong2*>(h.key + 1);
    const ulonglong2 b = *reinterpret_cast<const ulonglong2*>(h.key + 3);
    const bool r12 = a.y < a.x, r34 = b.y < b.x;
    const unsigned long long m12 = r12 ? a.y : a.x, m34 = r34 ? b.y : b.x;
    const bool r = m34 < m12;
    const unsigned long long m = r ? m34 : m12;
    if (!(cand > m)) {
        h.key[0] = cand;
        h.hid[0] = p;
        return cand;
    }
    const int lo = 1 + (r ? (r34 ? 3 : 2) : (r12 ? 1 : 0));
    h.key[0] = m;
    h.hid[0] = h.hid[lo];
    heap_descend(h, lo, k, m, cand, p);
    return m;
}

// heap_replace_root with the heap's levels 0 and 1 in registers (K0..K4, I0..I4; k >= 21, so levels
// 0-2 are complete): the same comparisons and moves, level 2 and below in shared memory
__device__ __forceinline__ unsigned long long heap_replace_root_r(HeapS& h, int k, unsigned long long cand, unsigned p,
                                                                  unsigned long long& K0, unsigned long long& K1,
                                                                  unsigned long long& K2, unsigned long long& K3,
                                                                  unsigned long long& K4, unsigned& I0, unsigned& I1,
                                                                  unsigned& I2, unsigned& I3, unsigned& I4)
{
    const bool r12 = K2 < K1, r34 = K4 < K3;
    const unsigned long long m12 = r12 ? K2 : K1, m34 = r34 ? K4 : K3;
    const bool r = m34 < m12;
    const unsigned long long m = r ? m34 : m12;
    if (!(cand > m)) {
        K0 = cand;
        I0 = p;
        return cand;
    }
    const int lo = r ? (r34 ? 4 : 3) : (r12 ? 2 : 1);
    K0 = m;
    I0 = lo == 1 ? I1 : lo == 2 ? I2 : lo == 3 ? I3 : I4;
    // the children of lo (level 2) against the value that moved up
    const int f = 4 * lo + 1;
    const ulonglong2 a = *reinterpret_cast<const ulonglong2*>(h.key + f);
    const ulonglong2 b = *reinterpret_cast<const ulonglong2*>(h.key + f + 2);
    const bool s01 = a.y < a.x, s23 = b.y < b.x;
    const unsigned long long n01 = s01 ? a.y : a.x, n23 = s23 ? b.y : b.x;
    const bool sr = n23 < n01;
    const unsigned long long m2 = sr ? n23 : n01;
    unsigned long long nk = cand;
    unsigned ni = p;
    if (m > m2) {
        const int gp = f + (sr ? (s23 ? 3 : 2) : (s01 ? 1 : 0));
        nk = m2;
        ni = h.hid[gp];
        heap_descend(h, gp, k, m2, cand, p);
    }
    if (lo == 1) { K1 = nk; I1 = ni; }
    else if (lo == 2) { K2 = nk; I2 = ni; }
    else if (lo == 3) { K3 = nk; I3 = ni; }
    else { K4 = nk; I4 = ni; }
    return m;
}

// dynamic shared memory of k_select: two staging buffers, key[k] (three slots ahead and 32 bytes
// of alignment slack), terms[k], hid[k] (three slots ahead, 16 bytes of slack), chunk sums
__host__ __device__ inline size_t select_smem_bytes(int k)
{
    return 2 * (size_t)kSelStage * 8 + 32 + ((size_t)k + 3) * 8 /*key*/ + (size_t)k * 8 /*terms*/ + 16 +
           ((size_t)k + 3) * 4 /*hid*/ + 8 + ((size_t)(k + 31) / 32) * 8 /*chunk sums*/;
}

template <typename T>
__device__ __forceinline__ T* align_up_ptr(void* p, size_t a)
{
    return reinterpret_cast<T*>(((size_t)p + a - 1) & ~(a - 1));
}

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)));
}

__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, unsigned bytes, unsigned long long* bar)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// bounded wait for the given phase parity; false if it did not complete in time
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity)
{
    const long long t0 = clock64();
    for (;;) {
        unsigned done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(smem_addr(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > kSelWaitCycles) return false;
    }
}

// The binary Hessian (k_hess_binary's sums: in-order over the samples holding both attributes,
// the first term exact) from lists of common samples built once from the static features, so no
// masks are intersected in the rounds.  hcode[p] describes upper position p:
//   < 0x7fff           the one sample holding both attributes: the entry is D_s
//   0x7fff             no such sample: 0
//   0x8000 | m         the segment's m-th entry with several common samples (a record)
//   0xa000 | i         intercept column (i, d-1): dsum_i
//   0xc000 | i         diagonal (i, i): dsum_i + lambda
// Each warp owns a segment of 512 positions.  Its lane 0 first starts a bulk copy of the segment's
// shift values into shared memory (one mbarrier per warp) and every lane loads its 16 codes into
// registers; while they fly the block stages D_s and dsum and the warp sums its segment's records, a
// lane per record (the warp's FP64 instructions then serve up to 32 multi-sample entries at once, not
// the few lanes of a 32-position row that hold one).  Then the positions are formed as
// k_hess_binary forms them.  64 registers and 4 KB of staging a warp let an SM hold 32 warps.
constexpr unsigned kHitNone = 0x7fffu;

__host__ __device__ inline size_t hits_stage_bytes(int nt) { return (size_t)(nt / 32) * 512 * 8; }

__device__ __forceinline__ void bulk_copy_1d(void* dst, const void* src, unsigned bytes, unsigned long long* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

template <int NT>
__global__ void __launch_bounds__(NT, 1024 / NT) k_hess_hits(Dev P, int mode, int maxrec)
{
    // [NT / 32][512] shift values, [n] D_s, [d] dsum, [d] diagonal values, [NT / 32][maxrec] record sums
    extern __shared__ __align__(16) double s_hx[];
    __shared__ __align__(8) unsigned long long s_bar[NT / 32];
    const int c = P.act ? P.act[blockIdx.y] : blockIdx.y;
    const int n = P.ns[c], off = P.soff[c];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int seg = blockIdx.x * (NT / 32) + warp;
    const int p_seg = seg * 512;
    const bool live = p_seg < P.U;
    const int cnt = live ? min(512, P.U - p_seg) : 0;
    const size_t base = (size_t)c * P.ustr;
    double* s_sh = s_hx + (size_t)warp * 512;
    const bool staged = live && mode != 1;
    if (staged && lane == 0) {
        // rows start 16-byte aligned (ustr is a multiple of 32, segments of 512); the size rounded up
        // to 16 bytes stays inside the client's row of ustr entries
        const unsigned bs = (unsigned)((cnt * 8 + 15) & ~15);
        mbar_init(&s_bar[warp]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(&s_bar[warp])),
                     "r"(bs)
                     : "memory");
        bulk_copy_1d(s_sh, P.shift + base + p_seg, bs, &s_bar[warp]);
    }
    unsigned cds[8];      // the warp's codes of rows 2 u and 2 u + 1, two to a register
#pragma unroll
    for (int u = 0; u < 8; ++u) {
        const int t0 = 64 * u + lane, t1 = t0 + 32;
        const unsigned c0 = t0 < cnt ? (unsigned)P.hcode[base + p_seg + t0] : kHitNone;
        const unsigned c1 = t1 < cnt ? (unsigned)P.hcode[base + p_seg + t1] : kHitNone;
        cds[u] = c0 | (c1 << 16);
    }
    double* s_D = s_hx + (size_t)(NT / 32) * 512;
    double* s_ds = s_D + n;
    double* s_dl = s_ds + P.d;
    const double* dsum = P.dsum + (size_t)c * P.d;
    for (int t = threadIdx.x; t < n; t += blockDim.x) s_D[t] = P.Dv[off + t];
    for (int t = threadIdx.x; t < P.d; t += blockDim.x) {
        const double v = dsum[t];
        s_ds[t] = v;
        s_dl[t] = __dadd_rn(v, P.lambda);
    }
    __syncthreads();

    double* s_r = s_dl + P.d + (size_t)warp * maxrec;
    double fa = 0.0, fb2 = 0.0;
    if (live) {
        const unsigned* sg = P.hseg + (size_t)c * (P.nseg + 1) + seg;
        const unsigned r0 = sg[0], r1 = sg[1];
        for (unsigned b = r0; b < r1; b += 32) {
            const unsigned r = b + lane;
            if (r < r1) {
                const unsigned e0 = P.hrec[r], e1 = P.hrec[r + 1];
                double h = s_D[P.hhits[e0]];
                unsigned e = e0 + 1;
                for (; e + 4 <= e1; e += 4) {     // four indices and values loaded ahead of the adds
                    const double v0 = s_D[P.hhits[e]], v1 = s_D[P.hhits[e + 1]];
                    const double v2 = s_D[P.hhits[e + 2]], v3 = s_D[P.hhits[e + 3]];
                    h = __dadd_rn(h, v0);
                    h = __dadd_rn(h, v1);
                    h = __dadd_rn(h, v2);
                    h = __dadd_rn(h, v3);
                }
                for (; e < e1; ++e) h = __dadd_rn(h, s_D[P.hhits[e]]);
                s_r[r - r0] = h;
            }
        }
        __syncwarp();
        if (staged && !mbar_wait(&s_bar[warp], 0u)) {     // the copy never completed: report it, form nothing
            if (lane == 0) {
                mbar_wait(&s_bar[warp], 0u);
                atomicExch(P.status, -5);     // FEDNL_ETIMEOUT
            }
        } else {
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                const int t = 32 * q + lane;
                if (t >= cnt) break;
                const int p = p_seg + t;
                const unsigned cd = (cds[q >> 1] >> (16 * (q & 1))) & 0xffffu;
                double h;
                bool diag = false;
                if (cd < kHitNone) h = s_D[cd];
                else if (cd == kHitNone) h = 0.0;
                else if (cd >= 0xc000u) {
                    h = s_dl[cd & 0x3fffu];
                    diag = true;
                } else if (cd >= 0xa000u) h = s_ds[cd & 0x1fffu];
                else h = s_r[cd & 0x1fffu];
                if (mode == 1) {
                    P.shift[base + p] = h;
                } else {
                    if (mode == 2) P.hbuf[base + p] = h;
                    const double df = __dsub_rn(h, s_sh[t]);
                    P.diff[base + p] = df;
                    if (mode != 3) {
                        const double r = fma(df, df, diag ? fa : fb2);     // one FP64 instruction per warp
                        if (diag) fa = r;
                        else fb2 = r;
                    }
                }
            }
        }
    }
    if ((mode == 0 || mode == 2) && live) {
        const double cs = chunk_tree(segment_value(fa, fb2));
        if (lane == 0) P.Fpart[(size_t)c * P.nseg + seg] = cs;
    }
    if ((mode == 0 || mode == 2) && !P.ref) client_fsum_last_block(P, c);
}

// Worker w's draws.  FRESH: the flags were written by other CTAs of the same launch (read through
// L2, selection words and counts updated atomically).
template <bool FRESH>
__device__ __forceinline__ void toplek_draws(int w, int n_mat, int W, const int* worker_of, unsigned* wstate,
                                             const int* needs, const double* pdraw, const int* minidx, unsigned* sel,
                                             int SW, int* cnt)
{
    unsigned st = wstate[w];
    auto keep = [&](int c, unsigned p) {     // w.p. 1 - p keep the element (insertInMinHeap)
        if (FRESH) {
            atomicOr(&sel[(size_t)c * SW + (p >> 5)], 1u << (p & 31));
            atomicAdd(&cnt[c], 1);
        } else {
            sel[(size_t)c * SW + (p >> 5)] |= 1u << (p & 31);
            cnt[c] += 1;
        }
    };
    if (worker_of) {
        for (int c = 0; c < n_mat; ++c) {
            int owner = worker_of[c];
            if (owner != w || !(FRESH ? __ldcg(needs + c) : needs[c])) continue;
            double u = lcg_real_unit(st);
            if (u > (FRESH ? __ldcg(pdraw + c) : pdraw[c])) keep(c, (unsigned)(FRESH ? __ldcg(minidx + c) : minidx[c]));
        }
    } else {
        // clients w, w + W, ... in order; their flags loaded eight at a time ahead of the draws
        for (int c0 = w; c0 < n_mat; c0 += 8 * W) {
            int nd[8], mi[8];
            double pd[8];
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                const int c = c0 + t * W;
                nd[t] = c < n_mat ? (FRESH ? __ldcg(needs + c) : needs[c]) : 0;
                pd[t] = c < n_mat ? (FRESH ? __ldcg(pdraw + c) : pdraw[c]) : 0.0;
                mi[t] = c < n_mat ? (FRESH ? __ldcg(minidx + c) : minidx[c]) : 0;
            }
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                const int c = c0 + t * W;
                if (c >= n_mat || !nd[t]) continue;
                double u = lcg_real_unit(st);
                if (u > pd[t]) keep(c, (unsigned)mi[t]);
            }
        }
    }
    wstate[w] = st;
}

// The master's aggregation: g = (1/n) sum_c g_c per coordinate, l = (1/n) sum_c Lk_c, clients in
// order (TrainLoop.h:1100-1333).
struct MasterAgg {
    const double* gc;      // [nc][d]
    const double* lk;      // [nc]
    double* g;             // [d]
    double* stats;         // stats[1] = l
    int d, nc;
    double inv_n;
};

// coordinate j: 32 clients' values loaded ahead of their in-order additions
__device__ __forceinline__ void master_g(const MasterAgg& A, int j)
{
    double g = 0.0;
    for (int c0 = 0; c0 < A.nc; c0 += 32) {
        double v[32];
#pragma unroll
        for (int t = 0; t < 32; ++t) v[t] = (c0 + t < A.nc) ? A.gc[(size_t)(c0 + t) * A.d + j] : 0.0;
#pragma unroll
        for (int t = 0; t < 32; ++t)
            if (c0 + t < A.nc) g = __dadd_rn(g, v[t]);
    }
    A.g[j] = __dmul_rn(g, A.inv_n);
}

// l = (1/n) sum_c Lk_c by one warp: 32 values loaded at a time, added in client order
__device__ __forceinline__ double lk_mean(const double* lk, int nc, double inv_n, int lane)
{
    double l = 0.0;
    for (int c0 = 0; c0 < nc; c0 += 32) {
        const double v = (c0 + lane < nc) ? lk[c0 + lane] : 0.0;
        const int cnt = min(32, nc - c0);
        for (int t = 0; t < cnt; ++t) l = __dadd_rn(l, __shfl_sync(0xffffffffu, v, t));
    }
    return __dmul_rn(l, inv_n);
}

__device__ __forceinline__ void master_l(const MasterAgg& A, int lane)
{
    const double l = lk_mean(A.lk, A.nc, A.inv_n, lane);
    if (lane == 0) A.stats[1] = l;
}

// Work fused into k_select.  TopLEK's rounding draws: the launch's last CTA to finish (counted on
// ctr, which it returns to zero) makes every worker's draws (k_toplek_rng's work) once all clients'
// window flags are written; ctr == nullptr: no draws in this launch.  The master's aggregation
// (agg.gc != nullptr): CTA 0's three other warps form l and g while its first warp walks the heap.
struct SelectDraws {
    unsigned* ctr;
    int n_mat, W;
    unsigned* wstate;
    MasterAgg agg;
    // norms != 0: warps 1-3 form the client's ||diff||_F^2 (F, its segment sums in fpart) and Lk
    int norms, nseg;
    double* fpart;     // [n_mat][nseg]
    double* lk;        // [n_mat]
};

// The difference's squared Frobenius norm in the fixed segment order (k_hess_binary's, the CPU
// oracle's orc_frob_sym) and Lk = sqrt of it (TopK.h:74-78), formed by warps 1-3 of the selection
// kernel while warp 0 walks the heap: segment seg holds 512 upper positions, lane l squares
// positions 32 q + l into fused multiply-adds (diagonal and off-diagonal apart, loaded ahead) and
// gives a + 2 b to the segment's halving tree; warp 1 then adds the segment sums in order.
__device__ __forceinline__ void select_norms(const SelectDraws& dr, const double* __restrict__ v, int U, int c,
                                          double* F, int warp, int lane)
{
    double* fp = dr.fpart + (size_t)c * dr.nseg;
    for (int seg = warp - 1; seg < dr.nseg; seg += 3) {
        const int p_seg = seg * 512;
        double x[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int p = p_seg + 32 * q + lane;
            x[q] = p < U ? v[p] : 0.0;
        }
        double fa = 0.0, fb2 = 0.0;
        int i, j;
        upper_ij(p_seg + lane, i, j);
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            if (p_seg + 32 * q + lane >= U) break;
            if (q > 0) {
                i += 32;
                while (i > j) {
                    i -= j + 1;
                    ++j;
                }
            }
            const double r = fma(x[q], x[q], i == j ? fa : fb2);
            if (i == j) fa = r;
            else fb2 = r;
        }
        const double cs = chunk_tree(segment_value(fa, fb2));
        if (lane == 0) fp[seg] = cs;
    }
    asm volatile("bar.sync 1, 96;" ::: "memory");
    if (warp == 1) {
        double f = 0.0;
        for (int q0 = 0; q0 < dr.nseg; q0 += 32) {
            const double t = (q0 + lane < dr.nseg) ? fp[q0 + lane] : 0.0;
            const int cnt = min(32, dr.nseg - q0);
            for (int u = 0; u < cnt; ++u) f = __dadd_rn(f, __shfl_sync(0xffffffffu, t, u));
        }
        if (lane == 0) {
            F[c] = f;
            dr.lk[c] = sqrt(f);
        }
    }
}

__device__ __forceinline__ void select_finish(const SelectDraws& dr, const int* needs, const double* pdraw,
                                              const int* minidx, unsigned* sel, int SW, int* cnt)
{
    if (!dr.ctr) return;
    __shared__ int s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(dr.ctr, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    for (int w = threadIdx.x; w < dr.W; w += blockDim.x)
        toplek_draws<true>(w, dr.n_mat, dr.W, nullptr, dr.wstate, needs, pdraw, minidx, sel, SW, cnt);
    if (threadIdx.x == 0) *dr.ctr = 0u;
}

// vals: [n_mat][ustr] packed upper values (signed), rows 16-byte aligned (ustr even); F: [n_mat]
// squared Frobenius norms.  Output: sel bitmap per matrix, cnt (entries kept before the rounding
// draw), TopLEK draw request.  err: set to 1 if a bounded wait ran out.
__global__ void __maxnreg__(192) k_select(const double* __restrict__ vals, int ustr, int U, int k,
                                                        int lek, double delta, double* F,
                                                        unsigned* sel, int SW, int* cnt, int* needs,
                                                        double* pdraw, int* minidx, int* err, const int* act,
                                                        int ref, SelectDraws dr)
{
    extern __shared__ __align__(16) unsigned long long s_dyn[];
    __shared__ __align__(8) unsigned long long s_bar[2];
    __shared__ int s_keep, s_fail;
    const int c = act ? act[blockIdx.x] : blockIdx.x;
    const double* v = vals + (size_t)c * ustr;
    unsigned* sc = sel + (size_t)c * SW;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nwarps = blockDim.x >> 5;
    for (int w = tid; w < SW; w += blockDim.x) sc[w] = 0u;
    if (k >= U) {       // SpecialMathRoutinesForMatrix.h:279-280 / :395-396: every upper index
        __syncthreads();
        for (int w = tid; w < SW; w += blockDim.x) {
            int lo = w * 32, n = min(32, U - lo);
            sc[w] = (n == 32) ? 0xffffffffu : ((1u << n) - 1u);
        }
        if (tid == 0) {
            cnt[c] = U;
            if (needs) needs[c] = 0;
        }
        if (dr.norms && warp != 0) select_norms(dr, v, U, c, F, warp, lane);
        if (dr.agg.gc && blockIdx.x == 0 && warp != 0) {
            if (warp == 1) {
                if (dr.agg.lk) master_l(dr.agg, lane);
            } else {
                for (int j = tid - 64; j < dr.agg.d; j += blockDim.x - 64) master_g(dr.agg, j);
            }
        }
        select_finish(dr, needs, pdraw, minidx, sel, SW, cnt);
        return;
    }
    double* stage = (double*)s_dyn;                                          // [2][kSelStage]
    HeapS h;
    h.key = align_up_ptr<unsigned long long>(s_dyn + 2 * kSelStage, 32) + 3;  // [k], key+1 32-byte aligned
    double* terms = (double*)(h.key + k);                                    // [k]
    h.hid = align_up_ptr<unsigned>(terms + k, 16) + 3;                       // [k], hid+1 16-byte aligned
    double* csum = align_up_ptr<double>(h.hid + k, 8);                       // [ceil(k/32)]

    // scanned region [k, U) streamed in chunks starting at an even element (16-byte aligned)
    const int s0 = k & ~1;
    const int n_chunks = (U - s0 + kSelStage - 1) / kSelStage;
    if (tid == 0) {
        s_fail = 0;
        mbar_init(&s_bar[0]);
        mbar_init(&s_bar[1]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        for (int q = 0; q < 2 && q < n_chunks; ++q) {
            const int st = s0 + q * kSelStage;
            const int len = min(kSelStage, ustr - st);
            tma_load_1d(stage + q * kSelStage, v + st, (unsigned)len * 8u, &s_bar[q]);
        }
    }
    for (int t = tid; t < k; t += blockDim.x) {
        h.key[t] = abs_bits(v[t]);
        h.hid[t] = (unsigned)t;
    }
    __syncthreads();
    // buildMinHeap (MinHeap.h:147-191) level by level, deepest first
    {
        const int start = (k + 4 - 2) / 4;
        int lvl = 0, lo = 0;
        while (lo + (1 << (2 * lvl)) <= start) {   // level of `start`
            lo += 1 << (2 * lvl);
            ++lvl;
        }
        for (; lvl >= 0; --lvl) {
            const int first = ((1 << (2 * lvl)) - 1) / 3;
            const int last = min(first + (1 << (2 * lvl)) - 1, start);
            for (int i = first + tid; i <= last; i += blockDim.x) heap_sift(h, i, k);
            __syncthreads();
        }
    }
    // scan, SpecialMathRoutinesForMatrix.h:300-318
    if (warp != 0) {
        if (dr.norms) select_norms(dr, v, U, c, F, warp, lane);
        if (dr.agg.gc && blockIdx.x == 0) {      // the master's aggregation beside the heap walk
            if (warp == 1) {
                if (dr.agg.lk) master_l(dr.agg, lane);
            } else {
                for (int j = tid - 64; j < dr.agg.d; j += blockDim.x - 64) master_g(dr.agg, j);
            }
        }
    } else {
        unsigned long long root = h.key[0];
        // levels 0 and 1 of the heap live in registers during the scan (k >= 21), the same in every
        // lane: the warp replaces the root in step, without a divergent branch or a broadcast
        const bool regs = k >= 21;
        unsigned long long K0 = 0, K1 = 0, K2 = 0, K3 = 0, K4 = 0;
        unsigned I0 = 0, I1 = 0, I2 = 0, I3 = 0, I4 = 0;
        if (regs) {
            K0 = h.key[0]; K1 = h.key[1]; K2 = h.key[2]; K3 = h.key[3]; K4 = h.key[4];
            I0 = h.hid[0]; I1 = h.hid[1]; I2 = h.hid[2]; I3 = h.hid[3]; I4 = h.hid[4];
        }
        for (int q = 0; q < n_chunks; ++q) {
            const int b = q & 1;
            if (!mbar_wait(&s_bar[b], (unsigned)(q >> 1) & 1u)) {
                if (lane == 0) s_fail = 1;
                break;
            }
            const int st = s0 + q * kSelStage;
            const int len = min(kSelStage, U - st);
            const double* buf = stage + b * kSelStage;
            // 256 entries per step, 8 per lane in lane-contiguous groups of 32 (entry e = 32 j + lane
            // of the step).  Each pass finds the first entry above the root that comes after the last
            // one taken (each lane its own first, then the warp minimum) and replaces the root with
            // it.  The root of this heap can also decrease (a deeper element may move up), so every
            // remaining entry is tested again after each replacement.  Entries outside [k, U) read as
            // 0, which never exceeds the root.
            for (int o = 0; o < len; o += 256) {
                unsigned long long v[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int idx = o + j * 32 + lane;
                    v[j] = (idx < len && st + idx >= k) ? abs_bits(buf[idx]) : 0ull;
                }
                int done = -1;                           // last entry taken in this step
                for (;;) {
                    unsigned e = 0xffffffffu;
                    unsigned long long mine = 0ull;
#pragma unroll
                    for (int j = 7; j >= 0; --j)
                        if (v[j] > root && j * 32 + lane > done) {
                            e = (unsigned)(j * 32 + lane);
                            mine = v[j];
                        }
                    e = __reduce_min_sync(0xffffffffu, e);
                    if (e == 0xffffffffu) break;
                    const unsigned long long cand = __shfl_sync(0xffffffffu, mine, (int)(e & 31u));
                    done = (int)e;
                    if (regs) {
                        root = heap_replace_root_r(h, k, cand, (unsigned)(st + o + done), K0, K1, K2, K3, K4, I0, I1,
                                                   I2, I3, I4);
                        __syncwarp();
                    } else {
                        unsigned long long nr = 0ull;
                        if (lane == 0) nr = heap_replace_root(h, k, cand, (unsigned)(st + o + done));
                        root = __shfl_sync(0xffffffffu, nr, 0);
                    }
                }
            }
            __syncwarp();
            if (lane == 0 && q + 2 < n_chunks) {       // refill this buffer with chunk q + 2
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                const int nst = s0 + (q + 2) * kSelStage;
                const int nlen = min(kSelStage, ustr - nst);
                tma_load_1d(stage + b * kSelStage, v + nst, (unsigned)nlen * 8u, &s_bar[b]);
            }
        }
        if (regs && lane == 0) {
            h.key[0] = K0; h.key[1] = K1; h.key[2] = K2; h.key[3] = K3; h.key[4] = K4;
            h.hid[0] = I0; h.hid[1] = I1; h.hid[2] = I2; h.hid[3] = I3; h.hid[4] = I4;
        }
    }
    __syncthreads();
    if (s_fail) {   // a copy never completed: give the copies in flight a bounded chance, report
        if (tid == 0) {
            for (int q = 0; q < 2; ++q) mbar_wait(&s_bar[q], 0u);
            *err = 1;
            cnt[c] = 0;
            if (needs) needs[c] = 0;
        }
        select_finish(dr, needs, pdraw, minidx, sel, SW, cnt);
        return;
    }
    int keep = k;
    if (lek) {
        const int nch = (k + 31) / 32;
        // heap terms in heap-array order, chunk trees, then the chunk sums in order
        for (int t = tid; t < k; t += blockDim.x) terms[t] = term_of(h.key[t], h.hid[t]);
        __syncthreads();
        if (!ref) {
            for (int q = warp; q < nch; q += nwarps) {
                const int t = q * 32 + lane;
                const double cs = chunk_tree(t < k ? terms[t] : 0.0);
                if (lane == 0) csum[q] = cs;
            }
        }
        __syncthreads();
        if (warp == 0) {
            const double fr = __ldcg(F + c);     // formed by warp 1 when the norms are formed here
            double num0;
            if (ref) {   // the reference's order: ||M||^2 minus each heap term in heap-array order
                double nm = fr;
                if (lane == 0)
                    for (int t = 0; t < k; ++t) nm = __dsub_rn(nm, terms[t]);
                num0 = __shfl_sync(0xffffffffu, nm, 0);
            } else {
                double sh = 0.0;
                if (lane == 0)
                    for (int q = 0; q < nch; ++q) sh = __dadd_rn(sh, csum[q]);
                num0 = __dsub_rn(fr, __shfl_sync(0xffffffffu, sh, 0));
            }
            // window test of SpecialMathRoutinesForMatrix.h:475-476 on the numerators before (prev) and
            // after (next) extraction m: hi > prev and omd < next + eps
            const double omd = __dmul_rn(__dsub_rn(1.0, delta), fr);
            const double eps = __dmul_rn(1e-1, fr);
            const double hi = __dadd_rn(omd, eps);
            int first = k;
            double prev_hit = 0.0, next_hit = 0.0;
            // Each numerator is num0 plus non-negative terms, added with monotone rounding, so none is
            // below num0: if hi > num0 fails no extraction opens the window, and none is made.
            if (hi > num0) {
                // Extraction (extracFromMinHeap, MinHeap.h:125-141) in chunks of 32: element m lands at
                // position k-1-m.  After each chunk the warp forms the chunk's numerators (doubling
                // scan of its terms, plus the carry of the chunks before it) and stops at the first
                // chunk holding a window hit.  Extractions after the hit only reorder positions
                // [0, k-1-first), whose set is what is kept.  While the heap has more than 21
                // entries, positions 0..4 live in lane 0's registers.
                unsigned long long K0 = 0, K1 = 0, K2 = 0, K3 = 0, K4 = 0;
                unsigned I0 = 0, I1 = 0, I2 = 0, I3 = 0, I4 = 0;
                int size = k;
                bool live = false;
                if (lane == 0 && k > 21) {
                    K0 = h.key[0]; K1 = h.key[1]; K2 = h.key[2]; K3 = h.key[3]; K4 = h.key[4];
                    I0 = h.hid[0]; I1 = h.hid[1]; I2 = h.hid[2]; I3 = h.hid[3]; I4 = h.hid[4];
                    live = true;
                }
                double carry = num0, prev_last = num0;
                for (int q = 0; q < nch; ++q) {
                    if (lane == 0) {
                        const int target = max(k - 32 * (q + 1), 1);     // heap size after this chunk
                        for (; live && size > max(target, 21); --size) {
                            const int n = size - 1;                      // heap size after the swap
                            const unsigned long long LK = h.key[n];
                            const unsigned LI = h.hid[n];
                            // level-2 keys (positions 5..20), loaded ahead of the level-1 decision
                            unsigned long long G[16];
#pragma unroll
                            for (int t = 0; t < 8; ++t) {
                                const ulonglong2 g2 = *reinterpret_cast<const ulonglong2*>(h.key + 5 + 2 * t);
                                G[2 * t] = g2.x;
                                G[2 * t + 1] = g2.y;
                            }
                            h.key[n] = K0;
                            h.hid[n] = I0;
                            // level 1, leftmost minimum of the children, moved up if strictly below L
                            const bool r12 = K2 < K1, r34 = K4 < K3;
                            const unsigned long long m12 = r12 ? K2 : K1, m34 = r34 ? K4 : K3;
                            const bool r = m34 < m12;
                            const unsigned long long lv = r ? m34 : m12;
                            const int lo = r ? (r34 ? 4 : 3) : (r12 ? 2 : 1);
                            if (!(LK > lv)) {
                                K0 = LK;
                                I0 = LI;
                                continue;
                            }
                            // root takes the child, the child's slot takes L (still in registers)
                            if (lo == 1) { K0 = K1; I0 = I1; K1 = LK; I1 = LI; }
                            else if (lo == 2) { K0 = K2; I0 = I2; K2 = LK; I2 = LI; }
                            else if (lo == 3) { K0 = K3; I0 = I3; K3 = LK; I3 = LI; }
                            else { K0 = K4; I0 = I4; K4 = LK; I4 = LI; }
                            // level 2: children of `lo` against the value that moved up (lv)
                            const int gb = 4 * (lo - 1);
                            const unsigned long long g0 = lo == 1 ? G[0] : lo == 2 ? G[4] : lo == 3 ? G[8] : G[12];
                            const unsigned long long g1 = lo == 1 ? G[1] : lo == 2 ? G[5] : lo == 3 ? G[9] : G[13];
                            const unsigned long long g2 = lo == 1 ? G[2] : lo == 2 ? G[6] : lo == 3 ? G[10] : G[14];
                            const unsigned long long g3 = lo == 1 ? G[3] : lo == 2 ? G[7] : lo == 3 ? G[11] : G[15];
                            const bool s01 = g1 < g0, s23 = g3 < g2;
                            const unsigned long long n01 = s01 ? g1 : g0, n23 = s23 ? g3 : g2;
                            const bool sr = n23 < n01;
                            const unsigned long long lv2 = sr ? n23 : n01;
                            if (!(lv > lv2)) continue;
                            const int gp = 5 + gb + (sr ? (s23 ? 3 : 2) : (s01 ? 1 : 0));
                            const unsigned GI = h.hid[gp];
                            if (lo == 1) { K1 = lv2; I1 = GI; }
                            else if (lo == 2) { K2 = lv2; I2 = GI; }
                            else if (lo == 3) { K3 = lv2; I3 = GI; }
                            else { K4 = lv2; I4 = GI; }
                            // L enters at gp; deeper levels carry the value that moved up, as the reference
                            heap_descend(h, gp, n, lv2, LK, LI);
                        }
                        if (live && size <= 21) {
                            h.key[0] = K0; h.key[1] = K1; h.key[2] = K2; h.key[3] = K3; h.key[4] = K4;
                            h.hid[0] = I0; h.hid[1] = I1; h.hid[2] = I2; h.hid[3] = I3; h.hid[4] = I4;
                            live = false;
                        }
                        for (; size > target; --size) {
                            const int n = size - 1;
                            const unsigned long long LK = h.key[n];
                            const unsigned LI = h.hid[n];
                            h.key[n] = h.key[0];
                            h.hid[n] = h.hid[0];
                            heap_descend(h, 0, n, LK, LK, LI);
                        }
                    }
                    __syncwarp();
                    const int m = q * 32 + lane;
                    double x = (m < k) ? term_of(h.key[k - 1 - m], h.hid[k - 1 - m]) : 0.0;
                    if (ref) {   // numerators one extraction at a time (every lane walks the same chain)
                        int hit = -1;
                        double run = carry, ph = 0.0, nh = 0.0;
                        const int nq = min(32, k - q * 32);
                        for (int t = 0; t < nq; ++t) {
                            const double tt = __shfl_sync(0xffffffffu, x, t);
                            const double nx = __dadd_rn(run, tt);
                            if (hi > run && omd < __dadd_rn(nx, eps)) {
                                hit = t;
                                ph = run;
                                nh = nx;
                                break;
                            }
                            run = nx;
                        }
                        if (hit >= 0) {
                            first = q * 32 + hit;
                            prev_hit = ph;
                            next_hit = nh;
                            break;
                        }
                        carry = run;
                        continue;
                    }
                    for (int hh = 1; hh < 32; hh <<= 1) {
                        const double y = __shfl_up_sync(0xffffffffu, x, hh);
                        if (lane >= hh) x = __dadd_rn(x, y);
                    }
                    const double tot = __shfl_sync(0xffffffffu, x, min(31, k - 1 - q * 32));
                    const double nxt = __dadd_rn(carry, x);
                    double prv = __shfl_up_sync(0xffffffffu, nxt, 1);
                    if (lane == 0) prv = prev_last;
                    const unsigned hits = __ballot_sync(0xffffffffu, m < k && hi > prv && omd < __dadd_rn(nxt, eps));
                    if (hits) {
                        const int l = __ffs(hits) - 1;
                        first = q * 32 + l;
                        prev_hit = __shfl_sync(0xffffffffu, prv, l);
                        next_hit = __shfl_sync(0xffffffffu, nxt, l);
                        break;
                    }
                    prev_last = __shfl_sync(0xffffffffu, nxt, 31);
                    carry = __dadd_rn(carry, tot);
                }
                if (lane == 0 && live) {
                    h.key[0] = K0; h.key[1] = K1; h.key[2] = K2; h.key[3] = K3; h.key[4] = K4;
                    h.hid[0] = I0; h.hid[1] = I1; h.hid[2] = I2; h.hid[3] = I3; h.hid[4] = I4;
                }
                __syncwarp();
            }
            if (lane == 0) {
                if (first < k) {
                    pdraw[c] = __dadd_rn(__dsub_rn(omd, prev_hit), eps) / __dadd_rn(__dsub_rn(next_hit, prev_hit), eps);
                    needs[c] = 1;
                    minidx[c] = (int)h.hid[k - 1 - first];
                    s_keep = k - 1 - first;      // positions [0, k-1-first) stay in the heap
                } else {
                    needs[c] = 0;
                    pdraw[c] = 0.0;
                    minidx[c] = 0;
                    s_keep = 0;
                }
            }
        }
        __syncthreads();
        keep = s_keep;
    }
    for (int t = tid; t < keep; t += blockDim.x) {
        const unsigned p = h.hid[t];
        atomicOr(&sc[p >> 5], 1u << (p & 31));
    }
    if (tid == 0) cnt[c] = keep;
    select_finish(dr, needs, pdraw, minidx, sel, SW, cnt);
}

// TopLEK rounding draws: each reference worker w owns one thread_local RandomGenRealLinear
// (SpecialMathRoutinesForMatrix.h:383) and visits its clients c = w, w + W, ... in order
// (TrainLoop.h:664-686); a draw happens only when the rounding window was reached (:475-501).
__global__ void k_toplek_rng(int n_mat, int W, const int* worker_of, unsigned* wstate, const int* needs,
                             const double* pdraw, const int* minidx, unsigned* sel, int SW, int* cnt)
{
    int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= W) return;
    toplek_draws<false>(w, n_mat, W, worker_of, wstate, needs, pdraw, minidx, sel, SW, cnt);
}

// ---- 5. RandK / RandSeqK ---------------------------------------------------------------------
// generateRandKItemsInUpperTriangularPart (SpecialMathRoutinesForMatrix.h:95-107): partial
// Fisher-Yates over a copy of the upper-index list (dopt/dopt/random/include/Shuffle.h:76-93)
// with the client's RandomGenIntegerLinear; the shuffled array is virtual: only displaced
// positions are kept, in an open-addressing map in global scratch.  The first k entries, sorted,
// are the selection -- set as bits of the selection bitmap, whose ascending order is the sort.
__device__ __forceinline__ unsigned hmap_get(unsigned long long* m, int cap, unsigned key)
{
    unsigned hsh = (key * 2654435761u) & (unsigned)(cap - 1);
    for (;;) {
        unsigned long long e = m[hsh];
        if (e == ~0ull) return key;                    // untouched: identity
        if ((unsigned)(e >> 32) == key) return (unsigned)e;
        hsh = (hsh + 1) & (unsigned)(cap - 1);
    }
}

__device__ __forceinline__ void hmap_put(unsigned long long* m, int cap, unsigned key, unsigned val)
{
    unsigned hsh = (key * 2654435761u) & (unsigned)(cap - 1);
    for (;;) {
        unsigned long long e = m[hsh];
        if (e == ~0ull || (unsigned)(e >> 32) == key) {
            m[hsh] = ((unsigned long long)key << 32) | val;
            return;
        }
        hsh = (hsh + 1) & (unsigned)(cap - 1);
    }
}

__global__ void k_randk(unsigned* states, int n_gen, int U, int k, unsigned long long* hmap, int hcap,
                        unsigned* sel, int SW, int* cnt, const int* act)
{
    int c = act ? act[blockIdx.x] : blockIdx.x;
    unsigned long long* m = hmap + (size_t)c * hcap;
    unsigned* sc = sel + (size_t)c * SW;
    for (int t = threadIdx.x; t < hcap; t += blockDim.x) m[t] = ~0ull;
    for (int w = threadIdx.x; w < SW; w += blockDim.x) sc[w] = 0u;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned st = states[c];
        unsigned long long n_minus_i_minus_one = (unsigned long long)U - 1;
        for (int i = 0; i < k; ++i, --n_minus_i_minus_one) {
            double u = lcg_int_unit(st);
            unsigned long long r_off = round_to_nearest(__dmul_rn(u, (double)n_minus_i_minus_one));
            if (r_off != 0) {
                unsigned r = (unsigned)(i + r_off);
                unsigned vi = hmap_get(m, hcap, (unsigned)i);
                unsigned vr = hmap_get(m, hcap, r);
                hmap_put(m, hcap, (unsigned)i, vr);
                hmap_put(m, hcap, r, vi);
            }
        }
        states[c] = st;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < k; i += blockDim.x) {
        unsigned p = hmap_get(m, hcap, (unsigned)i);
        atomicOr(&sc[p >> 5], 1u << (p & 31));
    }
    if (threadIdx.x == 0) cnt[c] = k;
}

// Project-defined RandK stream (FEDNL_RANDK_PHILOX): the k positions of draw `draw` of client c are
// the images of 0..k-1 under a six-round Feistel permutation of [0, 2^(2h)) whose round function is
// Philox4x32-10 (Salmon et al., SC'11) keyed by (seed, c), walked back into [0, U).  Every position
// is formed independently, one thread each; the CPU oracle computes the same stream.
__global__ void k_randk_philox(unsigned* draws, int U, int k, int h, unsigned seed, unsigned* sel, int SW, int* cnt,
                               const int* act)
{
    const int c = act ? act[blockIdx.x] : blockIdx.x;
    unsigned* sc = sel + (size_t)c * SW;
    for (int w = threadIdx.x; w < SW; w += blockDim.x) sc[w] = 0u;
    const unsigned draw = draws[c];
    __syncthreads();
    for (int i = threadIdx.x; i < k; i += blockDim.x) {
        uint32_t y = philox_feistel((uint32_t)i, h, seed, (uint32_t)c, draw);
        while (y >= (uint32_t)U) y = philox_feistel(y, h, seed, (uint32_t)c, draw);   // ends: a cycle holds i < U
        atomicOr(&sc[y >> 5], 1u << (y & 31));
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        draws[c] = draw + 1;
        cnt[c] = k;
    }
}

// generateRandSeqKItemsInUpperTriangularPart (SpecialMathRoutinesForMatrix.h:137-169)
__global__ void k_randseqk(unsigned* states, int n_gen, int U, int k, int* rseq, unsigned* sel, int SW, int* cnt,
                           const int* act)
{
    int c = act ? act[blockIdx.x] : blockIdx.x;
    unsigned* sc = sel + (size_t)c * SW;
    for (int w = threadIdx.x; w < SW; w += blockDim.x) sc[w] = 0u;
    __shared__ unsigned s_r;
    if (threadIdx.x == 0) {
        unsigned st = states[c];
        s_r = (unsigned)((unsigned long long)lcg_int_next(st) % (unsigned long long)U);
        states[c] = st;
        rseq[c] = (int)s_r;
        cnt[c] = k;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < k; t += blockDim.x) {
        unsigned p = s_r + t;
        if (p >= (unsigned)U) p -= U;
        atomicOr(&sc[p >> 5], 1u << (p & 31));
    }
}

// ---- 6. shift update + master merge, clients in order ----------------------------------------
// Worker: shift[idx] += alpha * item (TopK.h:103-129, RandK.h:136-162; Identical/Natural: the
// whole symmetric difference).  Master: H[idx] += item * preScale in client order
// (TrainLoop.h:1126-1276 with forcesequpdate).  One thread per upper position, looping over the
// clients in order, so H receives exactly the reference's sequence of additions.
// Position p = 32 word + lane of one selection word, called by the 32 lanes of a converged warp
// (lanes past U take part in the shuffles only).  Per batch of 32 clients, lane t loads client t's
// word; 32 shuffles turn the words into each position's mask of selecting clients, and every lane
// walks its own mask in client order, four clients at a time with their loads issued together (the
// same operations as one position at a time).  Updates the selecting clients' shifts; returns the
// new H[p].
__device__ __forceinline__ double apply_word(const Dev& P, int p, int lane)
{
    const bool in = p < P.U;
    const int word = p >> 5;                      // the same for the whole warp
    const bool all = (P.comp == 0 || P.comp == 5);
    double h = in ? P.H[p] : 0.0;
    // each batch's client ids and selection words are loaded one batch ahead
    auto client_of_lane = [&](int c0) { return (c0 + lane < P.n_act) ? (P.act ? P.act[c0 + lane] : c0 + lane) : -1; };
    auto word_of = [&](int cl) { return cl < 0 ? 0u : (all ? 0xffffffffu : P.sel[(size_t)cl * P.SW + word]); };
    int cl_next = client_of_lane(0);
    unsigned wv_next = word_of(cl_next);
    for (int c0 = 0; c0 < P.n_act; c0 += 32) {
        const int cl = cl_next < 0 ? 0 : cl_next;
        const unsigned wv = wv_next;
        if (c0 + 32 < P.n_act) {
            cl_next = client_of_lane(c0 + 32);
            wv_next = word_of(cl_next);
        }
        unsigned mine = 0u;                       // bit t: client c0 + t selected my position
#pragma unroll
        for (int t = 0; t < 32; ++t) {
            const unsigned w = __shfl_sync(0xffffffffu, wv, t);
            mine |= ((w >> lane) & 1u) << t;
        }
        if (!in) mine = 0u;
        // each lane walks its own selecting clients, four at a time with their loads issued ahead:
        // the warp's FP64 instructions then serve the lanes' events side by side, not one client of
        // the batch at a time (most clients select one or two of a word's 32 positions)
        while (__any_sync(0xffffffffu, mine != 0u)) {
            int tt[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                tt[e] = mine ? __ffs(mine) - 1 : -1;
                mine &= mine - 1u;
            }
            double dv[4], sv[4];
            size_t qq[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int c = __shfl_sync(0xffffffffu, cl, tt[e] < 0 ? 0 : tt[e]);
                qq[e] = (size_t)c * P.ustr + p;
                if (tt[e] >= 0) {
                    dv[e] = P.diff[qq[e]];
                    sv[e] = P.shift[qq[e]];
                }
            }
#pragma unroll
            for (int e = 0; e < 4; ++e)
                if (tt[e] >= 0) {
                    double item, sent;
                    if (P.comp == 5) {                 // Natural: master adds preScale * trunc(diff)
                        item = natural_trunc(dv[e]);
                        sent = __dmul_rn(P.prescale, item);
                    } else {
                        item = (P.comp == 1 || P.comp == 3 || P.comp == 6) ? __dmul_rn(dv[e], P.mult) : dv[e];
                        sent = __dmul_rn(item, P.prescale);
                    }
                    P.shift[qq[e]] = __dadd_rn(sv[e], __dmul_rn(P.alpha, item));
                    h = __dadd_rn(h, sent);
                }
        }
    }
    return h;
}

// A warp covers the 32 positions of one selection word.  In the FP64 round the same work runs in
// the Option-B solve's first phase (chol_body, apply_first).
__global__ void __launch_bounds__(128) k_apply(Dev P)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x, lane = threadIdx.x & 31;
    const double h = apply_word(P, p, lane);      // blockDim % 32 == 0: the warp covers one word
    if (p < P.U) P.H[p] = h;
}

// ---- 7. master: g = (1/n) sum_c g_c, l = (1/n) sum_c Lk_c (TrainLoop.h:1100-1333) ------------
// One thread per coordinate (32-thread blocks spread over SMs); clients added in order, loads
// issued in batches of 32 ahead of the dependent additions.  The last block forms l.  In the FP64
// TopK / TopLEK round the same work runs in k_select's idle warps (MasterAgg).
constexpr int kAggThreads = 32;
__global__ void __launch_bounds__(kAggThreads) k_aggregate(Dev P)
{
    const MasterAgg A{P.gc, P.lk, P.g, P.stats, P.d, P.nc, P.inv_n};
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < P.d) master_g(A, j);
    if (blockIdx.x == gridDim.x - 1) master_l(A, threadIdx.x & 31);     // l on a block of its own, the last
}

// ---- 8. Option-B solve: Cholesky of H + l I, two triangular solves, x -= dx ------------------
// choleskyFactorization<.., true, true> (CholeskyFactorization.h:153-272) computes R = L^T with
// H + l I = R^T R reading only the upper triangle; forwardSubstitutionWithATranspose and
// backwardSubstitutionWithATranspose (ElementarySolvers.h:186-224, :71-128) solve R^T y = g and
// R dx = y.
__device__ __forceinline__ size_t up_pos(int i, int j) { return (size_t)j * (j + 1) / 2 + i; }

// ---- 8b. Option-B solve across the whole GPU -------------------------------------------------
// Blocked right-looking LDL^T (H + l I = L D L^T, L unit lower; the oracle's orc_ldlt order) in
// one cooperative launch.  Square-root free: the pivot chain of a column is the reciprocal of the
// pivot, one multiply and one fused multiply-add.  For each panel of kCholNB rows:
//   1. every CTA factors the kCholNB x kCholNB diagonal block redundantly in shared memory (no
//      barrier needed; CTA 0 writes it back) and, in the same column loop, the panel rows of its
//      own share of the columns right of the block (l_kj = a_kj (1 / d_k), then
//      a_ij = fma(-l_ki, a_kj, a_ij) with a_kj unscaled); on GB300 a warp's FP64 instructions
//      issue about once per 64 cycles and the correctly rounded reciprocal takes ~300 cycles, so
//      the loop keeps the pivot chain short (two CTA barriers per column) and spreads the updates
//      over all warps;
//   2. the panel's multipliers go to the packed factor and its unscaled rows right of the block to
//      the work array's panel buffer; grid barrier, then all threads apply the panel to the
//      trailing triangle entry by entry (a_ij = fma(-l_ki, a_kj, a_ij), k over the panel in
//      order); grid barrier.
// Every entry undergoes exactly the operation sequence of the unblocked right-looking algorithm,
// so the factor equals the CPU oracle's factor bit for bit.  g is appended as column d of the
// packed matrix: the strips and trailing updates then carry out the forward substitution L y = g
// (y_i = fma(-l_ti, y_t, y_i)), and the scaling of row t leaves z_t = y_t (1 / d_t) in column d.
// The backward substitution L^T x = z (unit diagonal) runs in CTA 0, blocked by 32 rows, same
// order as the oracle's.
constexpr int kCholNB = 32;
constexpr int kCholSlab = 8;                          // panel columns per CTA kept in shared memory
constexpr int kCoopThreads = 256;
constexpr long long kBarrierCycles = 4000000000ll;   // ~2 s at 2 GHz, then ETIMEOUT

// ---- correctly rounded square root and reciprocal without the FP64 pipe ----------------------
// On this part a warp's FP64 instructions (and 64-bit integer <-> float conversions) issue about once
// per 64 cycles, and the hardware sequences for sqrt and 1/x cost about 720 and 355 cycles on the
// Cholesky's pivot chain.  These give the same correctly rounded results from integer arithmetic:
// an FP32 estimate, Newton steps whose residuals are computed exactly in 64-bit integers (converted
// to FP32 through 32-bit integers only), and a final exact remainder test that decides the rounding.
// Outside their domain (sqrt: a not a positive normal; 1/x: the result not normal) they defer to
// the hardware operation.

// sqrt(a) = S 2^(e/2 - 52), S = the integer nearest sqrt(N), N = M 2^52, a = M 2^(e - 52) with e even
// and M in [2^52, 2^54).  The FP32 square root of M gives S within 2^29; the Newton step from
// s0 = r 2^26 uses the exact residual N - s0^2 = (M - r^2) 2^52 (|M - r^2| < 2^34) and lands within
// 53; the next one's residual N - T^2 fits in 64 bits (|.| < 2^61) and lands within 1/2; then
// (T + 1/2)^2 = T^2 + T + 1/4 decides: S = T + 1 when N - T^2 > T, T - 1 when N - T^2 <= -T.
__device__ __forceinline__ double sqrt_rn_int(double a)
{
    const unsigned long long ia = (unsigned long long)__double_as_longlong(a);
    const unsigned E = (unsigned)(ia >> 52);                       // sign bit included: 0 for a > 0
    if (E - 1u >= 2046u) return sqrt(a);                          // zero, negative, subnormal, inf, nan
    const int odd = (E & 1u) == 0u;                               // e = E - 1023 odd
    const unsigned long long M = ((ia & 0xFFFFFFFFFFFFFull) | (1ull << 52)) << odd;
    const int eh = ((int)E - 1023 - odd) / 2;
    const float fm = __fmul_rn(__uint2float_rn((unsigned)(M >> 22)), 4194304.0f);          // M (24 bits)
    const unsigned ri = __float2uint_rn(__fsqrt_rn(fm));
    const long long D0 = (long long)(M - (unsigned long long)ri * ri);
    const float d1 = __fdiv_rn(__fmul_rn(__int2float_rn((int)(D0 >> 3)), 268435456.0f),   // D0 2^25 / r
                               __uint2float_rn(ri));
    unsigned long long T = ((unsigned long long)ri << 26) + (unsigned long long)(long long)__float2int_rn(d1);
    const unsigned long long Nlo = M << 52;                      // N mod 2^64
    long long Rm = (long long)(Nlo - T * T);
    const float rf = __fmul_rn(__int2float_rn((int)(Rm >> 32)), 4294967296.0f);
    const float tf = __fmul_rn(__uint2float_rn((unsigned)(T >> 29)), 536870912.0f);
    T += (unsigned long long)(long long)__float2int_rn(__fdiv_rn(rf, __fmul_rn(tf, 2.0f)));
    Rm = (long long)(Nlo - T * T);
    if (Rm > (long long)T) ++T;
    else if (Rm <= -(long long)T) --T;
    return __longlong_as_double((long long)(((unsigned long long)(eh + 1023) << 52) + (T - (1ull << 52))));
}

// 1/r = Q 2^(970 - E), Q = the integer nearest 2^105 / M, r = M 2^(E - 1075), M in [2^52, 2^53).
// A float-float Newton step from the FP32 reciprocal of M (held as its top 24 bits plus the rest)
// gives Q within 361; the residual 2^105 - M Q is then exact in 64 bits (2^105 = 0 mod 2^64), one
// more step lands within 1/2 and 2|2^105 - M Q| < M decides the rounding (no ties: 2^106 / M is an
// odd integer for no M in range).
__device__ __forceinline__ double rcp_rn_int(double r)
{
    const unsigned long long ir = (unsigned long long)__double_as_longlong(r);
    const unsigned E = (unsigned)(ir >> 52);
    if (E - 1u >= 2044u) return 1.0 / r;                          // the result would not be normal
    const unsigned long long M = (ir & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const float mh = __fmul_rn(__uint2float_rn((unsigned)(M >> 29)), 536870912.0f);       // exact
    const float ml = __uint2float_rn((unsigned)(M & 0x1FFFFFFFull));
    const float y0 = __frcp_rn(mh);
    const float e = __fsub_rn(fmaf(-mh, y0, 1.0f), __fmul_rn(ml, y0));                   // 1 - M y0
    unsigned long long Q = ((unsigned long long)__float2uint_rn(__fmul_rn(y0, 0x1p76f)) << 29) +
                           (unsigned long long)(long long)__float2int_rn(__fmul_rn(__fmul_rn(y0, e), 0x1p105f));
    long long Rm = (long long)(0ull - M * Q);
    Q += (unsigned long long)(long long)__float2int_rn(
        __fmul_rn(__fmul_rn(__int2float_rn((int)(Rm >> 32)), 4294967296.0f), y0));
    Rm = (long long)(0ull - M * Q);
    if (2 * Rm > (long long)M) ++Q;
    else if (2 * Rm < -(long long)M) --Q;
    return __longlong_as_double((long long)(((unsigned long long)(2045u - E) << 52) + (Q - (1ull << 52))));
}

// r = RN(sqrt(a)) and inv = RN(1 / r) together, as the Cholesky's pivot needs them.  The square root
// runs as in sqrt_rn_int.  The reciprocal's float-float estimate Q0 ~ 2^105 / T1 is formed from the
// square root's first Newton value T1 (within 53 of the root S), independently of the square root's
// second step, so only its exact integer correction waits for S: Q0 is within 361 of 2^105 / T1 and
// 2^105 / T1 within 2 |T1 - S| + 1 of 2^105 / S, so the residual 2^105 - S Q0 stays below 2^62 and
// one correction step lands within 1/2 (the FP32 reciprocal of T1 differs from that of S by
// 2^-46 relative); the remainder test then rounds as in rcp_rn_int.  S = 2^53 (the root rounds up
// to the next power of two) gives r and 1 / r as exact powers of two.
__device__ __forceinline__ double sqrt_rcp_rn_int(double a, double& inv)
{
    const unsigned long long ia = (unsigned long long)__double_as_longlong(a);
    const unsigned E = (unsigned)(ia >> 52);
    if (E - 1u >= 2046u) {                                         // zero, negative, subnormal, inf, nan
        const double r = sqrt(a);
        inv = rcp_rn_int(r);
        return r;
    }
    const int odd = (E & 1u) == 0u;
    const unsigned long long M = ((ia & 0xFFFFFFFFFFFFFull) | (1ull << 52)) << odd;
    const int eh = ((int)E - 1023 - odd) / 2;
    const float fm = __fmul_rn(__uint2float_rn((unsigned)(M >> 22)), 4194304.0f);
    const unsigned ri = __float2uint_rn(__fsqrt_rn(fm));
    const long long D0 = (long long)(M - (unsigned long long)ri * ri);
    const float d1 = __fdiv_rn(__fmul_rn(__int2float_rn((int)(D0 >> 3)), 268435456.0f), __uint2float_rn(ri));
    unsigned long long T = ((unsigned long long)ri << 26) + (unsigned long long)(long long)__float2int_rn(d1);
    // reciprocal estimate from T1 (= T here), clamped to [2^52, 2^53) so that mh is exact and
    // y0 2^76 an integer; the clamp moves it no further from S < 2^53
    const unsigned long long T1 = min(max(T, 1ull << 52), (1ull << 53) - 1ull);
    const float mh = __fmul_rn(__uint2float_rn((unsigned)(T1 >> 29)), 536870912.0f);
    const float ml = __uint2float_rn((unsigned)(T1 & 0x1FFFFFFFull));
    const float y0 = __frcp_rn(mh);
    const float e = __fsub_rn(fmaf(-mh, y0, 1.0f), __fmul_rn(ml, y0));
    unsigned long long Q = ((unsigned long long)__float2uint_rn(__fmul_rn(y0, 0x1p76f)) << 29) +
                           (unsigned long long)(long long)__float2int_rn(__fmul_rn(__fmul_rn(y0, e), 0x1p105f));
    // square root, second step and rounding
    const unsigned long long Nlo = M << 52;
    long long Rm = (long long)(Nlo - T * T);
    const float rf = __fmul_rn(__int2float_rn((int)(Rm >> 32)), 4294967296.0f);
    const float tf = __fmul_rn(__uint2float_rn((unsigned)(T >> 29)), 536870912.0f);
    T += (unsigned long long)(long long)__float2int_rn(__fdiv_rn(rf, __fmul_rn(tf, 2.0f)));
    Rm = (long long)(Nlo - T * T);
    if (Rm > (long long)T) ++T;
    else if (Rm <= -(long long)T) --T;
    const double r = __longlong_as_double((long long)(((unsigned long long)(eh + 1023) << 52) + (T - (1ull << 52))));
    if (T == (1ull << 53)) {                                       // r = 2^(eh + 1)
        inv = __longlong_as_double((long long)((unsigned long long)(1022 - eh) << 52));
        return r;
    }
    // reciprocal of r = T 2^(eh - 52): Q = RN(2^105 / T), 1 / r = Q 2^(-53 - eh)
    long long Rq = (long long)(0ull - T * Q);
    Q += (unsigned long long)(long long)__float2int_rn(
        __fmul_rn(__fmul_rn(__int2float_rn((int)(Rq >> 32)), 4294967296.0f), y0));
    Rq = (long long)(0ull - T * Q);
    if (2 * Rq > (long long)T) ++Q;
    else if (2 * Rq < -(long long)T) --Q;
    inv = __longlong_as_double((long long)(((unsigned long long)(1022 - eh) << 52) + (Q - (1ull << 52))));
    return r;
}

// Bounded grid barrier of n cooperating CTAs on three words: bar[0] counts arrivals since the
// launch began (the e-th barrier completes when it reaches e n), bar[1] counts CTAs that have
// finished, bar[2] is the error flag.  One fence and one reduction per CTA, then a poll with acquire
// loads: no counter is reset between barriers.  Every CTA calls finish() once after its last
// barrier; the last one to do so returns both counters to zero for the next launch.  sync() returns
// false (error flag set) when the other CTAs did not arrive in time.
// A launch that is one thread-block cluster uses the cluster's hardware barrier instead (every
// thread of every CTA arrives with release and waits with acquire semantics; the callers' control
// flow is the same in every CTA, so every barrier is reached by all of them).
struct GridSync {
    unsigned* bar;
    unsigned n;
    bool cluster;
    unsigned epoch = 0;        // barriers this CTA has passed (kept by thread 0)

    __device__ GridSync(unsigned* b, unsigned nblk, bool in_cluster = false) : bar(b), n(nblk), cluster(in_cluster) {}

    __device__ bool sync()
    {
        if (cluster) {
            asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
            return true;
        }
        __shared__ int s_ok;
        __syncthreads();
        if (threadIdx.x == 0) {
            epoch += 1;
            const unsigned target = epoch * n;
            // arrival with release semantics: after the CTA barrier it publishes every thread's writes
            // of this CTA (the acquire load below makes the other CTAs' writes visible to this one)
            asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(bar) : "memory");
            volatile unsigned* verr = bar + 2;
            int ok = 1;
            const long long t0 = clock64();
            for (;;) {
                unsigned v;
                asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(bar) : "memory");
                if ((int)(v - target) >= 0) break;
                if (*verr) {
                    ok = 0;
                    break;
                }
                if (clock64() - t0 > kBarrierCycles) {
                    atomicExch(bar + 2, 1u);
                    ok = 0;
                    break;
                }
            }
            asm volatile("fence.acq_rel.gpu;" ::: "memory");      // the other CTAs' writes, for this CTA
            if (*verr) ok = 0;
            s_ok = ok;
        }
        __syncthreads();
        return s_ok != 0;
    }

    __device__ void finish()
    {
        if (cluster) return;
        __syncthreads();
        if (threadIdx.x == 0 && atomicAdd(bar + 1, 1u) == n - 1) {
            atomicExch(bar, 0u);
            atomicExch(bar + 1, 0u);
        }
    }
};

// Hin is the packed upper triangle, or (hin_lda > 0) a column-major matrix with that leading
// dimension of which the upper triangle is read.
// The solve of one problem by a group of G cooperating CTAs (this CTA is number bid of the group);
// the grid barrier counts the group's CTAs on P.bar.
// apply_first: the round's master merge (k_apply's work) runs first, each warp a selection word at
// a time, and the system is formed from the merged H (Hin must be P.H, packed).  apply_first 2:
// also l = (1/n) sum_c Lk_c (master_l's order) is formed here, by warp 0 of every CTA while the
// other warps merge, and added to the diagonal once known (lptr is not read).
__device__ __forceinline__ void chol_body(const Dev& P, const double* __restrict__ Hin, int hin_lda, const double* lptr,
                                          double lval, const double* __restrict__ gin, double* dxout, double* xupd,
                                          int record, unsigned G, unsigned bid, GridSync& gs, int apply_first = 0)
{
    __shared__ double Db[kCholNB][kCholNB + 1];
    __shared__ double Rb[kCholNB][kCholNB + 1];
    __shared__ double Sb[kCholNB][kCholSlab + 1];
    __shared__ double SR[kCholNB][kCholSlab + 1];
    __shared__ double s_inv[kCholNB];     // 1 / pivot (single column), p and r (pair)
    __shared__ double s_q[kCholNB];       // q of the pair starting at k
    __shared__ unsigned short s_ent[kCholNB * (kCholNB + 1) / 2];
    __shared__ int s_fail;
    __shared__ double s_yb[2][32];
    __shared__ double s_l;
    int ent_nb = -1;
    double l = (lptr && apply_first != 2) ? *lptr : lval;
    const int d = P.d;
    const int D = d + 1;                       // augmented by the right-hand side
    const int UA = D * (D + 1) / 2;
    double* A = P.work;                        // [UA]
    double* W = P.work + UA;                   // [kCholNB][D]: the panel's unscaled rows
    if (P.ls && bid == 0 && threadIdx.x == 0) P.ls[4] = 0.0;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int gtid = bid * blockDim.x + tid, gthreads = G * blockDim.x;
    if (apply_first) {
        const int U = d * (d + 1) / 2;
        const bool own_l = apply_first == 2;
        const int nmw = own_l ? kCoopThreads / 32 - 1 : kCoopThreads / 32;    // merging warps per CTA
        const int NMW = (int)G * nmw;
        if (own_l && warp == 0) {
            const double lm = lk_mean(P.lk, P.nc, P.inv_n, lane);
            if (lane == 0) {
                s_l = lm;
                if (bid == 0) P.stats[1] = lm;
            }
        } else {
            for (int wd = (int)bid * nmw + (own_l ? warp - 1 : warp); wd < (U + 31) >> 5; wd += NMW) {
                const int p = wd * 32 + lane;
                const double hv = apply_word(P, p, lane);
                if (p < U) {
                    P.H[p] = hv;
                    int i, j;
                    upper_ij(p, i, j);
                    A[p] = (i == j && !own_l) ? __dadd_rn(hv, l) : hv;
                }
            }
        }
        for (int p = U + gtid; p < UA; p += gthreads) A[p] = (p - U < d) ? gin[p - U] : 0.0;    // column d
        if (own_l) {     // + l on the diagonal entries this CTA's warps merged
            __syncthreads();
            l = s_l;
            for (int jj = tid; jj < d; jj += blockDim.x) {
                const int p = jj * (jj + 1) / 2 + jj;
                if (((p >> 5) % NMW) / nmw == (int)bid) A[p] = __dadd_rn(P.H[p], l);
            }
        }
    } else {
        for (int p = gtid; p < UA; p += gthreads) {
            int i, j;
            upper_ij(p, i, j);
            if (j < d) {
                const double hv = hin_lda > 0 ? Hin[(size_t)j * hin_lda + i] : Hin[p];
                A[p] = (i == j) ? __dadd_rn(hv, l) : hv;
            } else {
                A[p] = (i < d) ? gin[i] : 0.0;
            }
        }
    }
    if (!gs.sync()) goto timeout;
    for (int c0 = 0; c0 < d; c0 += kCholNB) {
        const int nb = min(kCholNB, d - c0), c1 = c0 + nb;
        // this CTA's panel columns right of the block: j = c1 + bid + s G, s < ns (kept in
        // shared memory, at most kCholSlab; any further ones are finished after the column loop)
        const int ntot = D > c1 ? (D - c1 - (int)bid + (int)G - 1) / (int)G : 0;
        const int ns = max(0, min(ntot, kCholSlab));
        for (int t = tid; t < nb * nb; t += blockDim.x) {
            int i = t % nb, j = t / nb;
            if (i <= j) Db[i][j] = A[up_pos(c0 + i, c0 + j)];
        }
        for (int t = tid; t < nb * ns; t += blockDim.x) {
            const int i = t % nb, sl = t / nb;
            Sb[i][sl] = A[up_pos(c0 + i, c1 + (int)bid + sl * (int)G)];
        }
        // block entries (i, j), i <= j, listed by descending i: those with i > k are a prefix
        if (nb != ent_nb) {
            for (int e = tid; e < nb * (nb + 1) / 2; e += blockDim.x) {
                int i = nb - 1, rem = e;
                while (rem >= nb - i) {
                    rem -= nb - i;
                    --i;
                }
                s_ent[e] = (unsigned short)((i << 8) | (i + rem));
            }
            ent_nb = nb;
        }
        if (tid == 0) s_fail = 0;
        __syncthreads();
        // Column loop over the panel's pivot blocks: the pairs (k, k+1), k even (2x2 blocks of D),
        // and a single column last when nb is odd.  Warp 0 runs only the pivot chain, one block
        // ahead: while the others apply block k it applies block k to the next block's own three
        // entries (a lane per multiplier, then a lane per entry) and forms that block's det, its
        // correctly rounded reciprocal and D^{-1} = [[p, q], [q, r]] (a lane per entry).  Six other
        // warps form the multipliers of rows k and k+1 (l1 = fma(p, w1, q w2), l2 = fma(q, w1, r w2)
        // into Rb / SR, a thread per row and column) and apply block k (two fused multiply-adds) to
        // every other entry below row k+1.  Each of their threads owns fixed entries for the whole panel and keeps them in
        // registers: block entries e = ut + 192 q of the descending-row list (rows 1..nb-1) and slab
        // entries (row nb-1 - e / ns, slab column e mod ns) likewise, so the entries still active at
        // block k (row > k+1) fill the lowest slots of consecutive threads.  An entry is written to
        // Db / Sb when its row becomes one of the next pivot rows (the entries of the block after
        // the next one block earlier, for the chain).  Warp 4 stays idle: it shares warp 0's SM
        // sub-partition, whose FP64 pipe the chain needs.
        constexpr int kSlotsB = (kCholNB * (kCholNB - 1) / 2 + kCoopThreads - 65) / (kCoopThreads - 64);
        constexpr int kSlotsS = ((kCholNB - 1) * kCholSlab + kCoopThreads - 65) / (kCoopThreads - 64);
        const int ut = (warp < 4 ? warp - 1 : warp - 2) * 32 + lane;    // 0..191 for the update warps
        double vb[kSlotsB], vs[kSlotsS];
        int ib[kSlotsB], jb[kSlotsB], is_[kSlotsS], ss[kSlotsS];
        if (warp != 0 && warp != 4) {
            const int nbe = nb * (nb - 1) / 2;     // block entries below row 0
#pragma unroll
            for (int q = 0; q < kSlotsB; ++q) {
                const int e = ut + q * (kCoopThreads - 64);
                ib[q] = -1;
                jb[q] = 0;
                vb[q] = 0.0;
                if (e < nbe) {
                    const unsigned v = s_ent[e];
                    ib[q] = (int)(v >> 8);
                    jb[q] = (int)(v & 0xffu);
                    vb[q] = Db[ib[q]][jb[q]];
                }
            }
#pragma unroll
            for (int q = 0; q < kSlotsS; ++q) {     // the first slab entries on warps 5-7, one per sub-partition
                const int e = (ut + 96) % (kCoopThreads - 64) + q * (kCoopThreads - 64);
                is_[q] = -1;
                ss[q] = 0;
                vs[q] = 0.0;
                if (ns > 0 && e < (nb - 1) * ns) {
                    is_[q] = nb - 1 - e / ns;
                    ss[q] = e - (e / ns) * ns;
                    vs[q] = Sb[is_[q]][ss[q]];
                }
            }
        }
        // Warp 0: the parameters of the block at k2 from its (updated) entries a, b, c (b, c unused
        // for a single column): the pivot block goes to Rb (0 between the rows of a pair), D^{-1} to
        // s_inv / s_q, and a negative a or det (not NaN, not -0) fails the factorisation.
        auto block_params = [&](int k2, bool pair2, double a, double b, double c) {
            const auto neg = [](double v) {
                const long long vb_ = __double_as_longlong(v), mag = vb_ & 0x7fffffffffffffffll;
                return vb_ < 0 && mag != 0 && mag <= 0x7ff0000000000000ll;
            };
            if (pair2) {
                const double det = fma(a, c, -__dmul_rn(b, b));
                const double rdet = rcp_rn_int(det);
                if (lane < 3) {     // p = c rdet, q = -(b rdet), r = a rdet, a lane each
                    const double v = __dmul_rn(lane == 0 ? c : lane == 1 ? b : a, rdet);
                    if (lane == 0) s_inv[k2] = v;
                    else if (lane == 1) s_q[k2] = -v;
                    else s_inv[k2 + 1] = v;
                }
                if (lane == 0) {
                    Rb[k2][k2] = a;
                    Rb[k2][k2 + 1] = 0.0;
                    Rb[k2 + 1][k2 + 1] = c;
                    if (neg(a) || neg(det)) s_fail = 1;
                }
            } else {
                const double inv = rcp_rn_int(a);
                if (lane == 0) {
                    Rb[k2][k2] = a;
                    s_inv[k2] = inv;
                    if (neg(a)) s_fail = 1;
                }
            }
        };
        if (warp == 0) block_params(0, nb > 1, Db[0][0], nb > 1 ? Db[0][1] : 0.0, nb > 1 ? Db[1][1] : 0.0);
        __syncthreads();
        for (int k = 0; k < nb; k += 2) {
            if (s_fail) break;
            const bool pair = k + 1 < nb;
            if (warp == 0) {
                const int k2 = k + 2;
                if (pair && k2 < nb) {
                    // block k applied to the next block's entries: lane t < 4 forms the multiplier of
                    // row k2 + (t >> 1) (t even: l1 = fma(p, w1, q w2), t odd: l2 = fma(q, w1, r w2)),
                    // lane e < 3 then updates entry e of (k2,k2), (k2,k2+1), (k2+1,k2+1)
                    const bool pair2 = k2 + 1 < nb;
                    const double p = s_inv[k], r = s_inv[k + 1], q = s_q[k];
                    const int mc = k2 + ((lane >> 1) & 1);
                    const int mcol = (lane < 4 && (pair2 || mc == k2)) ? mc : k2;
                    const double x1 = Db[k][mcol], x2 = Db[k + 1][mcol];
                    const bool odd = lane & 1;
                    const double ml = fma(odd ? q : p, x1, __dmul_rn(odd ? r : q, x2));
                    const int er = k2 + (lane == 2 ? 1 : 0), ec = k2 + (lane >= 1 ? 1 : 0);
                    const int src = 2 * (er - k2);
                    const double m1 = __shfl_sync(0xffffffffu, ml, src), m2 = __shfl_sync(0xffffffffu, ml, src + 1);
                    const bool live = lane < 3 && (pair2 || lane == 0);
                    const int erc = live ? er : k2, ecc = live ? ec : k2;
                    double e = fma(-m1, Db[k][ecc], Db[erc][ecc]);
                    e = fma(-m2, Db[k + 1][ecc], e);
                    const double na = __shfl_sync(0xffffffffu, e, 0), nbv = __shfl_sync(0xffffffffu, e, 1),
                                 nc = __shfl_sync(0xffffffffu, e, 2);
                    block_params(k2, pair2, na, nbv, nc);
                }
            } else if (warp != 4) {
                if (pair) {
                    const double p = s_inv[k], r = s_inv[k + 1], q = s_q[k];
                    // a thread per (row, column) of the multipliers: warps 1-3, one per sub-partition
                    const int nd = nb - 2 - k;                 // block columns k+2 .. nb-1
                    const int o = ut & 1, cix = ut >> 1;
                    const double ca = o ? q : p, cb = o ? r : q;
                    if (cix < nd) {
                        const int j = k + 2 + cix;
                        Rb[k + o][j] = fma(ca, Db[k][j], __dmul_rn(cb, Db[k + 1][j]));
                    } else if (cix < nd + ns) {
                        const int sl = cix - nd;
                        SR[k + o][sl] = fma(ca, Sb[k][sl], __dmul_rn(cb, Sb[k + 1][sl]));
                    }
                    asm volatile("bar.sync 1, 192;" ::: "memory");
#pragma unroll
                    for (int q2 = 0; q2 < kSlotsB; ++q2) {
                        const int i = ib[q2], j = jb[q2];
                        if (i > k + 1 && !(j <= k + 3)) {      // the next block's own entries are the chain's
                            double v = fma(-Rb[k][i], Db[k][j], vb[q2]);
                            vb[q2] = fma(-Rb[k + 1][i], Db[k + 1][j], v);
                            if (i <= k + 3 || j <= k + 5) Db[i][j] = vb[q2];
                        }
                    }
#pragma unroll
                    for (int q2 = 0; q2 < kSlotsS; ++q2) {
                        const int i = is_[q2];
                        if (i > k + 1) {
                            double v = fma(-Rb[k][i], Sb[k][ss[q2]], vs[q2]);
                            vs[q2] = fma(-Rb[k + 1][i], Sb[k + 1][ss[q2]], v);
                            if (i <= k + 3) Sb[i][ss[q2]] = vs[q2];
                        }
                    }
                } else if (ut < ns) {      // the single last column: only the slab's row k is scaled
                    SR[k][ut] = __dmul_rn(Sb[k][ut], s_inv[k]);
                }
            }
            __syncthreads();
        }
        if (s_fail) {   // identical decision in every CTA: all leave together
            if (bid == 0 && tid == 0) {
                *P.status = -4;
                if (record) *P.round_ctr += 1;
            }
            return;
        }
        if (bid == 0) {
            for (int t = tid; t < nb * nb; t += blockDim.x) {
                int i = t % nb, j = t / nb;
                if (i <= j) A[up_pos(c0 + i, c0 + j)] = Rb[i][j];
            }
            for (int t = tid; t < nb; t += blockDim.x) P.rinv[c0 + t] = s_inv[t];
        }
        for (int t = tid; t < nb * ns; t += blockDim.x) {
            const int i = t % nb, sl = t / nb;
            const int j = c1 + (int)bid + sl * (int)G;
            A[up_pos(c0 + i, j)] = SR[i][sl];
            W[(size_t)i * D + j] = Sb[i][sl];
        }
        // panel columns beyond the slab (very large d only): one column per warp, same blocks
        {
            const int wp = tid >> 5;
            for (int sl = kCholSlab + wp; sl < ntot; sl += kCoopThreads / 32) {
                const int j = c1 + (int)bid + sl * (int)G;
                double a = (lane < nb) ? A[up_pos(c0 + lane, j)] : 0.0;
                for (int k = 0; k < nb; k += 2) {
                    const double w1 = __shfl_sync(0xffffffffu, a, k);     // a_kj, a_k+1,j final and unscaled
                    if (k + 1 < nb) {
                        const double w2 = __shfl_sync(0xffffffffu, a, k + 1);
                        const double p = s_inv[k], r = s_inv[k + 1], q = s_q[k];
                        if (lane == k) {
                            W[(size_t)k * D + j] = w1;
                            a = fma(p, w1, __dmul_rn(q, w2));
                        } else if (lane == k + 1) {
                            W[(size_t)(k + 1) * D + j] = w2;
                            a = fma(q, w1, __dmul_rn(r, w2));
                        } else if (lane > k + 1 && lane < nb) {
                            a = fma(-Rb[k][lane], w1, a);
                            a = fma(-Rb[k + 1][lane], w2, a);
                        }
                    } else if (lane == k) {
                        W[(size_t)k * D + j] = w1;
                        a = __dmul_rn(a, s_inv[k]);
                    }
                }
                if (lane < nb) A[up_pos(c0 + lane, j)] = a;
            }
        }
        if (c1 >= d) break;
        if (!gs.sync()) goto timeout;
        // trailing update, entries (i, j) with c1 <= i <= j < D (column d carries y)
        {
            const int m = D - c1;
            const int T = m * (m + 1) / 2;
            for (int e = gtid; e < T; e += gthreads) {
                int ii, jj;
                upper_ij(e, ii, jj);
                const int i = c1 + ii, j = c1 + jj;
                const double* ci = A + up_pos(0, i);
                const double* wj = W + j;
                double u[kCholNB], w[kCholNB];     // multipliers l_ki, unscaled a_kj, loaded ahead
#pragma unroll
                for (int k = 0; k < kCholNB; ++k) {
                    u[k] = k < nb ? ci[c0 + k] : 0.0;
                    w[k] = k < nb ? wj[(size_t)k * D] : 0.0;
                }
                double a = A[up_pos(i, j)];
#pragma unroll
                for (int k = 0; k < kCholNB; ++k)
                    if (k < nb) a = fma(-u[k], w[k], a);
                A[up_pos(i, j)] = a;
            }
        }
        if (!gs.sync()) goto timeout;
    }
    if (!gs.sync()) goto timeout;
    if (bid != 0) return;
    {
        // L^T dx = z (z in column d), blocked by 32 rows (CTA 0)
        double* y = P.ybuf;
        double gs = 0.0;
        for (int i = tid; i < d; i += blockDim.x) {
            y[i] = A[up_pos(i, d)];
            gs += gin[i] * gin[i];
        }
        if (record) {   // ||g|| for the round statistics
            for (int o = 16; o > 0; o >>= 1) gs += __shfl_down_sync(0xffffffffu, gs, o);
            __shared__ double s_gs[kCoopThreads / 32];
            if (lane == 0) s_gs[tid >> 5] = gs;
            __syncthreads();
            if (tid == 0) {
                double t = 0.0;
                for (int w = 0; w < kCoopThreads / 32; ++w) t += s_gs[w];
                P.stats[0] = sqrt(t);
            }
        }
        // Blocks of 32 rows from the bottom.  Warp 0 solves a block (lane = row, the block's
        // triangle in registers), then applies the block's solution to the next block's rows, which
        // it keeps in registers; meanwhile warps 1-3 and 5-7 apply it to all rows above.  Warp 4
        // shares warp 0's sub-partition and runs no FP64 instruction: it stages the triangle (Db)
        // and the rectangle of the update (Rb) of the block after the current one into shared
        // memory, each as soon as warp 0 has taken the current one into registers (named barriers
        // 3 and 2), so warp 0 reads no global memory.  A row receives its updates in descending t
        // order whichever warp applies them.
        const int nblocks = (d + 31) / 32;
        auto stage_t = [&](int blk) {
            const int b1 = d - 32 * blk, b0 = max(0, b1 - 32), nbk = b1 - b0;
#pragma unroll 8
            for (int s = 0; s < 32; ++s) Db[lane][s] = (lane < s && s < nbk) ? A[up_pos(b0 + lane, b0 + s)] : 0.0;
        };
        auto stage_r = [&](int blk) {
            const int b1 = d - 32 * blk, b0 = max(0, b1 - 32), nbk = b1 - b0, n0 = max(0, b0 - 32);
#pragma unroll 8
            for (int s = 0; s < 32; ++s)
                Rb[lane][s] = (s < nbk && n0 + lane < b0) ? A[up_pos(n0 + lane, b0 + s)] : 0.0;
        };
        if (warp == 4) {
            stage_t(0);
            stage_r(0);
        }
        __syncthreads();
        double v = 0.0;
        if (tid < 32) {
            const int b1 = d, b0 = max(0, d - 32);
            v = (lane < b1 - b0) ? y[b0 + lane] : 0.0;
        }
        for (int blk = 0; blk < nblocks; ++blk) {
            const int b1 = d - 32 * blk, b0 = max(0, b1 - 32), nbk = b1 - b0;
            if (tid < 32) {
                double ar[32];
#pragma unroll
                for (int s = 0; s < 32; ++s) ar[s] = Db[lane][s];
                asm volatile("bar.arrive 3, 64;" ::: "memory");   // warp 4 may refill Db
#pragma unroll
                for (int s = 31; s >= 0; --s) {
                    if (s < nbk) {
                        const double yt = __shfl_sync(0xffffffffu, v, s);
                        if (lane < s) v = fma(-ar[s], yt, v);
                    }
                }
                if (lane < nbk) {
                    y[b0 + lane] = v;
                    s_yb[blk & 1][lane] = v;
                }
            } else if (warp == 4) {
                asm volatile("bar.sync 3, 64;" ::: "memory");
                if (blk + 1 < nblocks) stage_t(blk + 1);
            }
            __syncthreads();
            const int n0 = max(0, b0 - 32);                 // next block: rows [n0, b0)
            if (tid < 32) {
                double av[32];
#pragma unroll
                for (int s = 0; s < 32; ++s) av[s] = Rb[lane][s];
                asm volatile("bar.arrive 2, 64;" ::: "memory");   // warp 4 may refill Rb
                if (b0 > 0) {
                    const int i = n0 + lane;
                    double w = (i < b0) ? y[i] : 0.0;
#pragma unroll
                    for (int s = 31; s >= 0; --s)
                        if (s < nbk) w = fma(-av[s], s_yb[blk & 1][s], w);
                    v = w;
                }
            } else if (warp == 4) {
                asm volatile("bar.sync 2, 64;" ::: "memory");
                if (blk + 1 < nblocks) stage_r(blk + 1);
            } else {
                const int ut = (warp < 4 ? warp - 1 : warp - 2) * 32 + lane;
                for (int i = ut; i < n0; i += blockDim.x - 64) {
                    double av[32];
#pragma unroll
                    for (int s = 0; s < 32; ++s) av[s] = (s < nbk) ? A[up_pos(i, b0 + s)] : 0.0;
                    double w = y[i];
#pragma unroll
                    for (int s = 31; s >= 0; --s)
                        if (s < nbk) w = fma(-av[s], s_yb[blk & 1][s], w);
                    y[i] = w;
                }
            }
        }
        __syncthreads();
        for (int i = tid; i < d; i += blockDim.x) {
            const double dxi = y[i];
            if (dxout) dxout[i] = dxi;
            if (xupd) xupd[i] = __dsub_rn(xupd[i], dxi);
        }
        if (record && tid == 0) {
            int r = *P.round_ctr;
            if (r < P.hist_cap) P.hist[r] = P.stats[0];
            *P.round_ctr = r + 1;
        }
        if (P.ls && tid == 0) P.ls[4] = 1.0;
    }
    return;
timeout:
    if (bid == 0 && threadIdx.x == 0) {
        *P.status = -5;
        if (record) *P.round_ctr += 1;
    }
}

__global__ void __launch_bounds__(kCoopThreads) k_chol_coop(Dev P, const double* __restrict__ Hin, int hin_lda,
                                                            const double* lptr, double lval,
                                                            const double* __restrict__ gin, double* dxout,
                                                            double* xupd, int record, int apply_first)
{
    GridSync gs(P.bar, gridDim.x);
    chol_body(P, Hin, hin_lda, lptr, lval, gin, dxout, xupd, record, gridDim.x, blockIdx.x, gs, apply_first);
    gs.finish();
}

// Several independent Option-B solves in one cooperative launch (the serving loop's tick): job j
// owns CTAs [cta0, cta0 + ncta) and its own barrier words, so problems of different d proceed
// side by side.
struct CholJob {
    Dev P;
    const double* Hin;
    int hin_lda;
    const double* lptr;
    double lval;
    const double* gin;
    double* dxout;
    double* xupd;
    int record, cta0, ncta;
};

__global__ void __launch_bounds__(kCoopThreads) k_chol_batched(const CholJob* __restrict__ jobs, int njobs)
{
    int j = 0;
    while (j + 1 < njobs && (int)blockIdx.x >= jobs[j + 1].cta0) ++j;
    const CholJob& J = jobs[j];
    if ((int)blockIdx.x >= J.cta0 + J.ncta) return;
    GridSync gs(J.P.bar, (unsigned)J.ncta);
    chol_body(J.P, J.Hin, J.hin_lda, J.lptr, J.lval, J.gin, J.dxout, J.xupd, J.record, (unsigned)J.ncta,
              blockIdx.x - (unsigned)J.cta0, gs);
    gs.finish();
}

// ---- operator-level helpers -----------------------------------------------------------------
// Shift update of the sparse compressors (LocalWorkerForFedNL_TopK.h:103-129; RandK.h:136-162):
// for every selected flat index j*lda + i of matrix m, item = diff[idx] (times U/k for RandK and
// RandSeqK, already part of the message), shift[idx] += alpha item and, off the diagonal, the mirror
// shift[i*lda + j] += alpha item.  One thread per (matrix, selected entry); the entries of one matrix
// are distinct upper positions, so no two threads touch the same element.
__global__ void k_op_shift_update(double* shifts, const double* diffs, int n_mat, int lda, size_t full,
                                  const unsigned* idx, const int* counts, int kstride, double alpha, double mult)
{
    const int m = blockIdx.y;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n_mat || t >= counts[m]) return;
    const unsigned f = idx[(size_t)m * kstride + t];
    const unsigned jc = f / (unsigned)lda, ir = f - jc * (unsigned)lda;
    const double item = (mult == 1.0) ? diffs[(size_t)m * full + f] : __dmul_rn(diffs[(size_t)m * full + f], mult);
    const double upd = __dmul_rn(alpha, item);
    double* sh = shifts + (size_t)m * full;
    sh[f] = __dadd_rn(sh[f], upd);
    if (ir != jc) {
        const size_t g = (size_t)ir * lda + jc;
        sh[g] = __dadd_rn(sh[g], upd);
    }
}

// Master aggregation (TrainLoop.h:1100-1333 with forcesequpdate): g = (sum of the clients'
// gradients in client order) * (1/n), l = (sum of Lk in client order) * (1/n); H[idx] += value for
// every client message in client order.  One thread per H position of the upper triangle walks the
// clients in order (each client's message holds a position at most once), one per coordinate of g.
__global__ void k_op_aggregate_g(const double* grads, const double* lks, int nc, int d, double inv_n, double* g,
                                 double* l)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < d) {
        double s = 0.0;
        for (int c = 0; c < nc; ++c) s = __dadd_rn(s, grads[(size_t)c * d + j]);
        g[j] = __dmul_rn(s, inv_n);
    }
    if (j == 0) {
        double s = 0.0;
        for (int c = 0; c < nc; ++c) s = __dadd_rn(s, lks[c]);
        *l = __dmul_rn(s, inv_n);
    }
}

// per client: the message's upper positions scattered into a [nc][U] map of message slots (-1: none)
__global__ void k_op_message_slots(const unsigned* idx, const int* counts, int kstride, int nc, int lda, int* slot,
                                   int U)
{
    const int c = blockIdx.y;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc || t >= counts[c]) return;
    const unsigned f = idx[(size_t)c * kstride + t];
    const unsigned jc = f / (unsigned)lda, ir = f - jc * (unsigned)lda;
    const size_t p = (size_t)jc * (jc + 1) / 2 + ir;
    slot[(size_t)c * U + p] = t;
}

__global__ void k_op_aggregate_h(double* H, int d, int lda, int U, const double* vals, const int* slot, int kstride,
                                 int nc)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= U) return;
    int i, j;
    upper_ij(p, i, j);
    const size_t f = (size_t)j * lda + i;
    double h = H[f];
    for (int c = 0; c < nc; ++c) {
        const int t = slot[(size_t)c * U + p];
        if (t >= 0) h = __dadd_rn(h, vals[(size_t)c * kstride + t]);
    }
    H[f] = h;
}

// Identity compressor (LocalWorkerForFedNL_Identical.h:80-94): the message is every upper entry
// times alpha / n in the upper-index order (column j, rows 0..j); the shift receives alpha diff on
// both triangles.  One thread per (matrix, upper position).
__global__ void k_op_identity(const double* diffs, double* shifts, int n_mat, int lda, size_t full, int U,
                              double alpha, double prescale, unsigned* idx_out, double* val_out)
{
    const int m = blockIdx.y;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n_mat || p >= U) return;
    int i, j;
    upper_ij(p, i, j);
    const size_t f = (size_t)j * lda + i;
    const double item = diffs[(size_t)m * full + f];
    if (idx_out) idx_out[(size_t)m * U + p] = (unsigned)f;
    if (val_out) val_out[(size_t)m * U + p] = __dmul_rn(item, prescale);
    if (shifts) {
        const double upd = __dmul_rn(alpha, item);
        double* sh = shifts + (size_t)m * full;
        sh[f] = __dadd_rn(sh[f], upd);
        if (i != j) {
            const size_t g = (size_t)i * lda + j;
            sh[g] = __dadd_rn(sh[g], upd);
        }
    }
}
// pack the upper triangle of n column-major d x lda matrices and their full squared norms
__global__ void k_pack_upper(const double* full, int d, int lda, int U, int ustr, double* packed)
{
    int t = blockIdx.y;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < ustr; p += gridDim.x * blockDim.x) {
        double v = 0.0;
        if (p < U) {
            int i, j;
            upper_ij(p, i, j);
            v = full[(size_t)t * d * lda + (size_t)j * lda + i];
        }
        packed[(size_t)t * ustr + p] = v;
    }
}

// squared L2 norm of whole d x lda buffers in the chunked order (chunk sums by the warp tree,
// then in order by one thread); csum: [n_mat][ceil(len / 32)] scratch
__global__ void __launch_bounds__(256) k_l2sq_full(const double* full, long long len, double* csum, double* out)
{
    int t = blockIdx.x;
    const double* m = full + (size_t)t * len;
    long long nch = (len + 31) / 32;
    double* cs = csum + (size_t)t * nch;
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (long long q = warp; q < nch; q += blockDim.x / 32) {
        long long e = q * 32 + lane;
        double v = (e < len) ? __dmul_rn(m[e], m[e]) : 0.0;
        double s = chunk_tree(v);
        if (lane == 0) cs[q] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double f = 0.0;
        for (long long q = 0; q < nch; ++q) f = __dadd_rn(f, cs[q]);
        out[t] = f;
    }
}

__global__ void k_natural(const double* in, long long n, double* out)
{
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n) out[e] = natural_trunc(in[e]);
}

// Reference wire format of the Natural message (LocalWorkerForFedNL_Natural.h:92-126): entries
// are packed pairwise, 3 bytes per pair [signA(1) expA(11) signB(1) expB(11)]
// (pack2FP64NoMantissa, FloatUtils.h:193-221), followed by one trailing block made of the
// packer's two slots as they stand: (last, second-to-last) for odd n, the final pair again for
// even n.  Block q < n/2 packs (2q, 2q+1); block n/2 is the trailing one.
__global__ void k_natural_pack(const double* in, long long n, unsigned char* packed)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long nb = n / 2 + 1;
    if (q >= nb || n < 1) return;
    long long ia, ib;
    if (q < n / 2) {
        ia = 2 * q;
        ib = 2 * q + 1;
    } else if (n & 1) {
        ia = n - 1;
        ib = (n >= 2) ? n - 2 : n - 1;
    } else {
        ia = n - 2;
        ib = n - 1;
    }
    unsigned long long a = (unsigned long long)__double_as_longlong(in[ia]);
    unsigned long long b = (unsigned long long)__double_as_longlong(in[ib]);
    unsigned v = ((unsigned)(a >> 63) << 23) | ((unsigned)((a >> 52) & 0x7FF) << 12) |
                 ((unsigned)(b >> 63) << 11) | (unsigned)((b >> 52) & 0x7FF);
    packed[3 * q + 0] = (unsigned char)(v & 0xFF);
    packed[3 * q + 1] = (unsigned char)((v >> 8) & 0xFF);
    packed[3 * q + 2] = (unsigned char)((v >> 16) & 0xFF);
}


// ---- 8c. objective values and FedNL-LS --------------------------------------------------------
// f_i = -mean_s log sigma_s + (lambda / 2) ||x||^2 (evaluateFunction(x, margin, sigmoid),
// logistic_regression.h:119-123); the per-sample terms come from the margin kernels.  Sums in the
// CPU oracle's chunked order (halving tree over 32 terms, chunks in order).
__device__ __forceinline__ double warp_chunked_sum(const double* v, int n)
{
    const int lane = threadIdx.x & 31;
    double total = 0.0;
    for (int base = 0; base < n; base += 32) {
        const double cs = chunk_tree(base + lane < n ? v[base + lane] : 0.0);
        total = __dadd_rn(total, __shfl_sync(0xffffffffu, cs, 0));
    }
    return total;
}

__device__ __forceinline__ double warp_chunked_sumsq(const double* v, int n)
{
    const int lane = threadIdx.x & 31;
    double total = 0.0;
    for (int base = 0; base < n; base += 32) {
        const double t = base + lane < n ? v[base + lane] : 0.0;
        const double cs = chunk_tree(__dmul_rn(t, t));
        total = __dadd_rn(total, __shfl_sync(0xffffffffu, cs, 0));
    }
    return total;
}

// one warp per client; skipped once the line search has finished (gate = P.ls)
__global__ void k_fclient(Dev P, const double* x, const double* gate)
{
    if (gate && gate[2] != 0.0) return;
    const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (c >= P.nc) return;
    const int n = P.ns[c];
    const double loss = __ddiv_rn(warp_chunked_sum(P.fterm + P.soff[c], n), (double)n);
    const double xs = warp_chunked_sumsq(x, P.d);
    if ((threadIdx.x & 31) == 0) P.fi[c] = __dadd_rn(loss, __dmul_rn(__dmul_rn(P.lambda, 0.5), xs));
}

// master: f = (chunked sum of f_i) / n into out (function_aggregation, TrainLoop.h:1511-1541)
__global__ void k_fmaster(Dev P, double* out)
{
    const double f = __dmul_rn(warp_chunked_sum(P.fi, P.nc), P.inv_n);
    if (threadIdx.x == 0) *out = f;
}

// FedNL-LS (TrainLoop.h:1543-1640): t = 1, -(dx . g) in the chunked order, x_k kept; nothing to
// search when the solve failed
__global__ void k_ls_init(Dev P)
{
    __shared__ double s_dg[1024];
    for (int i = threadIdx.x; i < P.d && i < 1024; i += blockDim.x) s_dg[i] = __dmul_rn(P.dx[i], P.g[i]);
    for (int i = threadIdx.x; i < P.d; i += blockDim.x) P.xprev[i] = P.x[i];
    __syncthreads();
    if (threadIdx.x < 32) {
        double dg = 0.0;
        if (P.d <= 1024) {
            dg = warp_chunked_sum(s_dg, P.d);
        } else {       // larger d: the same chunked order, terms formed on the fly
            const int lane = threadIdx.x;
            for (int base = 0; base < P.d; base += 32) {
                const int i = base + lane;
                const double cs = chunk_tree(i < P.d ? __dmul_rn(P.dx[i], P.g[i]) : 0.0);
                dg = __dadd_rn(dg, __shfl_sync(0xffffffffu, cs, 0));
            }
        }
        if (threadIdx.x == 0) {
            P.ls[0] = 1.0;
            P.ls[1] = -dg;
            P.ls[2] = P.ls[4] != 0.0 ? 0.0 : 1.0;
            P.ls[3] = 0.0;
        }
    }
}

// trial point x = x_k - t dx
__global__ void k_ls_trial(Dev P)
{
    if (P.ls[2] != 0.0) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P.d) P.x[i] = __dsub_rn(P.xprev[i], __dmul_rn(P.ls[0], P.dx[i]));
}

// -log sigma_s at the trial point
__global__ void k_ls_margin(Dev P, int S)
{
    if (P.ls[2] != 0.0) return;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    double m;
    const double b = P.lab[s];
    if (P.A == nullptr) {
        double acc = 0.0;
        for (int t = P.rowptr[s]; t < P.rowptr[s + 1]; ++t) acc = __dadd_rn(acc, P.x[P.colidx[t]]);
        m = (b == 1.0) ? acc : -acc;
    } else {
        const double* a = P.A + (size_t)s * P.d;
        double acc = 0.0;
        for (int i = 0; i < P.d; ++i) {
            const double u = (b == 1.0) ? a[i] : __dmul_rn(a[i], -1.0);
            acc = __dadd_rn(acc, __dmul_rn(u, P.x[i]));
        }
        m = acc;
    }
    P.fterm[s] = -fednl_log(fednl_sigmoid(m));
}

// Armijo test f(x) <= f(x_k) + (c t)(-(dx . g)); t *= gamma after a failure
__global__ void k_ls_check(Dev P, double c, double gamma)
{
    if (P.ls[2] != 0.0) return;
    const double fr = __dmul_rn(warp_chunked_sum(P.fi, P.nc), P.inv_n);
    if (threadIdx.x == 0) {
        P.ls[3] = __dadd_rn(P.ls[3], 1.0);
        const double t = P.ls[0];
        if (fr <= __dadd_rn(P.stats[2], __dmul_rn(__dmul_rn(c, t), P.ls[1]))) P.ls[2] = 1.0;
        else P.ls[0] = __dmul_rn(t, gamma);
    }
}

// ---- 9. FedNL-PP (dopt/bin_fednl_local_pp) ----------------------------------------------------
// Client sampler (TrainLoop.h:1150-1157): a fresh 0..n-1 is shuffled for tau steps by the partial
// Fisher-Yates of Shuffle.h:76-93 with the sampler's RandomGenIntegerLinear; its first tau entries
// are this round's clients, processed and merged in ascending client order (forcesequpdate).  One
// CTA; the permutation lives in shared memory when it fits (smem_perm), else in global scratch.
// needs[] is cleared so that the TopLEK draw kernel skips clients that were not sampled.
constexpr int kPPThreads = 256;

__global__ void __launch_bounds__(kPPThreads) k_pp_sample(int n, int tau, unsigned* sampler, int* gperm, int* act,
                                                          int* is_sel, int* needs, int smem_perm)
{
    extern __shared__ int s_perm[];
    __shared__ int s_wsum[kPPThreads / 32];
    int* perm = smem_perm ? s_perm : gperm;
    const int tid = threadIdx.x;
    for (int i = tid; i < n; i += blockDim.x) {
        perm[i] = i;
        is_sel[i] = 0;
        if (needs) needs[i] = 0;
    }
    __syncthreads();
    if (tid == 0) {
        unsigned st = *sampler;
        unsigned long long n_minus_i_minus_one = (unsigned long long)n - 1;
        for (int i = 0; i < tau; ++i, --n_minus_i_minus_one) {
            const double u = lcg_int_unit(st);
            const unsigned long long r_off = round_to_nearest(__dmul_rn(u, (double)n_minus_i_minus_one));
            if (r_off != 0) {
                const int r = i + (int)r_off;
                const int a = perm[i], b = perm[r];
                perm[i] = b;
                perm[r] = a;
            }
        }
        *sampler = st;
    }
    __syncthreads();
    for (int t = tid; t < tau; t += blockDim.x) is_sel[perm[t]] = 1;
    __syncthreads();
    // ascending compaction: thread t owns clients [t * per, (t + 1) * per)
    const int per = (n + blockDim.x - 1) / blockDim.x;
    const int lo = min(n, tid * per), hi = min(n, lo + per);
    int cnt = 0;
    for (int c = lo; c < hi; ++c) cnt += is_sel[c];
    int incl = cnt;
    const int lane = tid & 31, warp = tid >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) s_wsum[warp] = incl;
    __syncthreads();
    int base = 0;
    for (int w = 0; w < warp; ++w) base += s_wsum[w];
    int pos = base + incl - cnt;
    for (int c = lo; c < hi; ++c)
        if (is_sel[c]) act[pos++] = c;
}

// True gradient at the round's starting iterate (computeFullGradient, TrainLoop.h:117-129), in
// the fixed blocked order of the CPU oracle: in-order sums over blocks of 32 consecutive clients,
// block sums in order, then / n.  One warp per coordinate; lane l owns blocks l, l + 32, ...
// The last CTA also records ||true gradient|| (sequential sum of squares) as the round's norm.
__global__ void k_pp_truegrad(Dev P)
{
    const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (i < P.d) {
        const int nb = (P.nc + 31) / 32;
        double acc = 0.0;
        for (int b0 = 0; b0 < nb; b0 += 32) {
            const int b = b0 + lane;
            double bs = 0.0;
            if (b < nb) {
                const int c0 = b * 32, c1 = min(P.nc, c0 + 32);
                bs = P.gc[(size_t)c0 * P.d + i];
                for (int c = c0 + 1; c < c1; ++c) bs = __dadd_rn(bs, P.gc[(size_t)c * P.d + i]);
            }
            const int cntb = min(32, nb - b0);
            for (int t = 0; t < cntb; ++t) {
                const double v = __shfl_sync(0xffffffffu, bs, t);
                acc = (b0 + t == 0) ? v : __dadd_rn(acc, v);
            }
        }
        if (lane == 0) P.tg[i] = __ddiv_rn(acc, (double)P.nc);
    }
}

__global__ void k_pp_norm(Dev P)
{
    if (threadIdx.x != 0) return;
    double gs = 0.0;
    for (int i = 0; i < P.d; ++i) gs = __dadd_rn(gs, __dmul_rn(P.tg[i], P.tg[i]));
    const double gn = sqrt(gs);
    P.stats[0] = gn;
    const int r = *P.round_ctr;
    if (r < P.hist_cap) P.hist[r] = gn;
    *P.round_ctr = r + 1;
}

// ||shift - H_i||_F^2 after the shift update (the PP workers' "Put Lk", e.g. RandSeqK.h:166-173) in
// the segment order of k_hess_binary: warp per 512 upper positions, diagonal and off-diagonal
// accumulators apart, halving tree.
__global__ void __launch_bounds__(kHessThreads) k_pp_lkpart(Dev P)
{
    const int c = P.act[blockIdx.y];
    const size_t base = (size_t)c * P.ustr;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int seg = blockIdx.x * (kHessThreads / 32) + warp;
    const int p_seg = seg * 512;
    double fa = 0.0, fb2 = 0.0;
    for (int q = 0; q < 16; ++q) {
        const int p = p_seg + 32 * q + lane;
        if (p >= P.U) break;
        const double df = __dsub_rn(P.shift[base + p], P.hbuf[base + p]);
        const bool dg = upper_is_diag(p);
        const double r = fma(df, df, dg ? fa : fb2);
        if (dg) fa = r;
        else fb2 = r;
    }
    if (p_seg < P.U) {
        const double cs = chunk_tree(segment_value(fa, fb2));
        if (lane == 0) P.Fpart[(size_t)c * P.nseg + seg] = cs;
    }
}

// Per processed client: Lk = ||shift - H_i||_F (segment sums in order), its difference, and the
// direction dir = x Lk + shift x - grad with shift x swept column by column
// (MatrixNMD::matrixVectorMultiply, MatrixNMD.h:1299-1325); the difference to the previous
// direction is what the client sends.
__global__ void k_pp_dir(Dev P)
{
    __shared__ double s_lk;
    const int c = P.act[blockIdx.x];
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        const double* fp = P.Fpart + (size_t)c * P.nseg;
        double f = 0.0;
        for (int q0 = 0; q0 < P.nseg; q0 += 32) {
            const double v = (q0 + lane < P.nseg) ? fp[q0 + lane] : 0.0;
            const int cnt = min(32, P.nseg - q0);
            for (int t = 0; t < cnt; ++t) f = __dadd_rn(f, __shfl_sync(0xffffffffu, v, t));
        }
        if (lane == 0) {
            const double lk = sqrt(f);
            P.dlk[c] = __dsub_rn(lk, P.lk[c]);
            P.lk[c] = lk;
            s_lk = lk;
        }
    }
    __syncthreads();
    const double lk = s_lk;
    const double* sh = P.shift + (size_t)c * P.ustr;
    for (int i = threadIdx.x; i < P.d; i += blockDim.x) {
        double y = 0.0;
        for (int j = 0; j < P.d; ++j) {
            const int a = min(i, j), b = max(i, j);
            y = __dadd_rn(y, __dmul_rn(sh[(size_t)b * (b + 1) / 2 + a], P.x[j]));
        }
        const size_t q = (size_t)c * P.d + i;
        const double dv = __dsub_rn(__dadd_rn(__dmul_rn(P.x[i], lk), y), P.gc[q]);
        P.ddir[q] = __dsub_rn(dv, P.dir[q]);
        P.dir[q] = dv;
    }
}

// Master (TrainLoop.h:1168-1450): g = (sum of the sent direction differences) / n + g_prev and
// l = (sum of the Lk differences) / n + l_prev, processed clients in ascending order.
__global__ void k_pp_aggregate(Dev P)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P.d) {
        double g = 0.0;
        for (int s = 0; s < P.n_act; ++s) g = __dadd_rn(g, P.ddir[(size_t)P.act[s] * P.d + i]);
        g = __dadd_rn(__dmul_rn(g, P.inv_n), P.gprev[i]);
        P.gprev[i] = g;
        P.g[i] = g;
    }
    if (i == 0) {
        double l = 0.0;
        for (int s = 0; s < P.n_act; ++s) l = __dadd_rn(l, P.dlk[P.act[s]]);
        l = __dadd_rn(__dmul_rn(l, P.inv_n), *P.lprev);
        *P.lprev = l;
        P.stats[1] = l;
    }
}

// FedNL-PP initial state (LocalWorkerForFedNL_RandSeqK.h:22-31 and TrainLoop.h:1064-1080):
// Lk = 0, dir = shift x0 - grad(x0) per client; g_prev = mean dir (clients in order), l_prev = 0.
__global__ void k_pp_init_dir(Dev P)
{
    const int c = blockIdx.x;
    const double* sh = P.shift + (size_t)c * P.ustr;
    for (int i = threadIdx.x; i < P.d; i += blockDim.x) {
        double y = 0.0;
        for (int j = 0; j < P.d; ++j) {
            const int a = min(i, j), b = max(i, j);
            y = __dadd_rn(y, __dmul_rn(sh[(size_t)b * (b + 1) / 2 + a], P.x[j]));
        }
        const size_t q = (size_t)c * P.d + i;
        P.dir[q] = __dsub_rn(y, P.gc[q]);
        P.ddir[q] = 0.0;
    }
    if (threadIdx.x == 0) {
        P.lk[c] = 0.0;
        P.dlk[c] = 0.0;
    }
}

__global__ void k_pp_init_mean(Dev P)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P.d) {
        double g = 0.0;
        for (int c = 0; c < P.nc; ++c) g = __dadd_rn(g, P.dir[(size_t)c * P.d + i]);
        P.gprev[i] = __dmul_rn(g, P.inv_n);
    }
    if (i == 0) {
        double l = 0.0;
        for (int c = 0; c < P.nc; ++c) l = __dadd_rn(l, P.lk[c]);
        *P.lprev = __dmul_rn(l, P.inv_n);
    }
}

}  // namespace fednl
