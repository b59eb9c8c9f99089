// fednl_refmode.cuh -- the round in the reference's own operation order (desc.arith_order = 1).
//
// The reference's AVX2 build (dopt SUPPORT_CPU_AVX_256_bits=1, SUPPORT_CPU_FMA_EXT=0, no FMA
// contraction) fixes the order of every floating-point operation of a round.  The kernels here
// perform the same IEEE operations in the same order, so a round reproduces the reference's values
// bit for bit given the same inputs:
//   * margins: one Vec4d accumulator, attribute j < 4 floor(d/4) into lane j mod 4, reduced as
//     (c0 + c2) + (c1 + c3), the remaining attributes added in order
//     (MatrixNMD_SIMD_double.h:1256-1430);
//   * sigmoid: the vectorclass exp in SIMD lanes (exp_d<Vec4d>, vectormath_exp.h:141-230) for
//     samples s < 8 floor(n/8); libm's exp on the scalar tail, here the correctly rounded exp
//     (glibc returns the other neighbour for a few inputs in ten thousand);
//   * ||diff||_F from the upper part (MatrixNMD_SIMD_double.h:1068-1253): eight lane accumulators
//     shared by all columns, a scalar for each column's tail rows and one for the diagonal;
//   * TopLEK's window numerators one by one in heap-array and then extraction order
//     (SpecialMathRoutinesForMatrix.h:435-503), in k_select;
//   * Cholesky (CholeskyFactorization.h:153-272) and the two triangular solves
//     (ElementarySolvers.h:71-224) with two-Vec4d dot products: element k < 8 floor(n/8) into lane
//     k mod 8, lanes reduced as (0 + h(c0..c3)) + h(c4..c7), h(c) = (c0 + c2) + (c1 + c3), the tail
//     summed in order from 0 and added last (LightVector_SIMD_double.h:233-380);
//   * the objective's loss with the vectorclass log in lanes (log_d<Vec4d>, vectormath_exp.h:947-1003).
#pragma once

#include "fednl_kernels.cuh"

namespace fednl {
namespace refo {

// ---- scalar restatements of the reference's lane arithmetic -------------------------------------

// exp_d<Vec4d, 0, 0> of one lane, without FMA (mul_add(a, b, c) = a b + c, nmul_add(a, b, c) = c - a b)
__device__ __forceinline__ double exp_vcl(double x0)
{
    if (x0 != x0) return x0;
    if (!(fabs(x0) < 708.39)) return x0 < 0.0 ? 0.0 : __longlong_as_double(0x7ff0000000000000ll);
    const double p2 = 0x1p-1, p3 = 0x1.5555555555555p-3, p4 = 0x1.5555555555555p-5, p5 = 0x1.1111111111111p-7;
    const double p6 = 0x1.6c16c16c16c17p-10, p7 = 0x1.a01a01a01a01ap-13, p8 = 0x1.a01a01a01a01ap-16;
    const double p9 = 0x1.71de3a556c734p-19, p10 = 0x1.27e4fb7789f5cp-22, p11 = 0x1.ae64567f544e4p-26;
    const double p12 = 0x1.1eed8eff8d898p-29, p13 = 0x1.6124613a86d09p-33;
    const double ln2d_hi = 0.693145751953125, ln2d_lo = 1.42860682030941723212E-6;
    const double r = rint(__dmul_rn(x0, 1.44269504088896340736));
    double x = __dsub_rn(x0, __dmul_rn(r, ln2d_hi));
    x = __dsub_rn(x, __dmul_rn(r, ln2d_lo));
    const double x2 = __dmul_rn(x, x), x4 = __dmul_rn(x2, x2), x8 = __dmul_rn(x4, x4);
    const double hi = __dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(p13, x), p12), x4),
                                __dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(p11, x), p10), x2), __dadd_rn(__dmul_rn(p9, x), p8)));
    const double lo = __dadd_rn(
        __dmul_rn(__dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(p7, x), p6), x2), __dadd_rn(__dmul_rn(p5, x), p4)), x4),
        __dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(p3, x), p2), x2), x));
    const double z = __dadd_rn(__dmul_rn(hi, x8), lo);
    return __dmul_rn(__dadd_rn(z, 1.0), pow2i((int)r));
}

struct dd {
    double hi, lo;
};

__device__ __forceinline__ dd dd_norm(double s, double e)
{
    const double t = __dadd_rn(s, e);
    return dd{t, __dsub_rn(e, __dsub_rn(t, s))};
}

__device__ __forceinline__ dd dd_add(dd a, dd b)
{
    double s, e;
    two_sum(a.hi, b.hi, s, e);
    e = __dadd_rn(e, __dadd_rn(a.lo, b.lo));
    return dd_norm(s, e);
}

__device__ __forceinline__ dd dd_mul(dd a, dd b)
{
    const double p = __dmul_rn(a.hi, b.hi);
    double e = __fma_rn(a.hi, b.hi, -p);
    e = __dadd_rn(e, __dadd_rn(__dmul_rn(a.hi, b.lo), __dmul_rn(a.lo, b.hi)));
    return dd_norm(p, e);
}

// Correctly rounded exp (own method): x = k ln2 + r with ln2 in three parts (30-bit head: k L1 and
// x - k L1 exact), r as a double-double; exp(r 2^-10) by its Taylor series to degree 9 in
// double-double arithmetic, squared ten times; one rounding of hi + lo; exact scaling by 2^k.
// Below 2^-90 relative error before the rounding: the correctly rounded result for normal results.
__device__ __forceinline__ double exp_cr(double x)
{
    if (x != x) return x;
    if (x > 709.782712893384) return __longlong_as_double(0x7ff0000000000000ll);
    if (x < -745.1332191019412) return 0.0;
    const double L1 = 0x1.62e42fe8p-1, L2 = 0x1.e8e7bcd5e4f1ep-31, L3 = -0x1.8cff81a12a17ep-85;
    const double fh[10] = {1.0, 1.0, 0x1p-1, 0x1.5555555555555p-3, 0x1.5555555555555p-5, 0x1.1111111111111p-7,
                           0x1.6c16c16c16c17p-10, 0x1.a01a01a01a01ap-13, 0x1.a01a01a01a01ap-16, 0x1.71de3a556c734p-19};
    const double fl[10] = {0.0, 0.0, 0.0, 0x1.5555555555555p-57, 0x1.5555555555555p-59, 0x1.1111111111111p-63,
                           -0x1.f49f49f49f49fp-65, 0x1.a01a01a01a01ap-73, 0x1.a01a01a01a01ap-76, -0x1.c154f8ddc6c00p-73};
    const double kd = rint(__dmul_rn(x, 0x1.71547652b82fep+0));
    const double r1 = __dsub_rn(x, __dmul_rn(kd, L1));
    const double p2 = __dmul_rn(kd, L2);
    const double p2e = __fma_rn(kd, L2, -p2);
    double s, e;
    two_sum(r1, -p2, s, e);
    e = __dsub_rn(__dsub_rn(e, p2e), __dmul_rn(kd, L3));
    dd y = dd_norm(s, e);
    y.hi = __dmul_rn(y.hi, 0x1p-10);
    y.lo = __dmul_rn(y.lo, 0x1p-10);
    dd t{fh[9], fl[9]};
#pragma unroll
    for (int n = 8; n >= 0; --n) t = dd_add(dd_mul(t, y), dd{fh[n], fl[n]});
#pragma unroll
    for (int q = 0; q < 10; ++q) t = dd_mul(t, t);
    const double p = __dadd_rn(t.hi, t.lo);
    const int k = (int)kd;
    if (k > 1000) return __dmul_rn(__dmul_rn(p, pow2i(k - 1000)), pow2i(1000));
    if (k < -1000) return __dmul_rn(__dmul_rn(p, pow2i(k + 1000)), pow2i(-1000));
    return __dmul_rn(p, pow2i(k));
}

// log_d<Vec4d, 0> of one lane, without FMA, for positive normal inputs (zero -> -inf, +inf -> +inf)
__device__ __forceinline__ double log_vcl(double x1)
{
    if (x1 != x1 || x1 < 0.0) return __longlong_as_double(0x7ff8000000000000ll);
    if (x1 == 0.0) return __longlong_as_double((long long)0xfff0000000000000ull);
    if (x1 == __longlong_as_double(0x7ff0000000000000ll)) return x1;
    const double ln2_hi = 0.693359375, ln2_lo = -2.121944400546905827679E-4;
    const double P0 = 7.70838733755885391666E0, P1 = 1.79368678507819816313E1, P2 = 1.44989225341610930846E1;
    const double P3 = 4.70579119878881725854E0, P4 = 4.97494994976747001425E-1, P5 = 1.01875663804580931796E-4;
    const double Q0 = 2.31251620126765340583E1, Q1 = 7.11544750618563894466E1, Q2 = 8.29875266912776603211E1;
    const double Q3 = 4.52279145837532221105E1, Q4 = 1.12873587189167450590E1;
    const unsigned long long b = (unsigned long long)__double_as_longlong(x1);
    double x = __longlong_as_double((long long)((b & 0x000FFFFFFFFFFFFFull) | 0x3FE0000000000000ull));
    double fe = __dsub_rn((double)(long long)(b >> 52), 1023.0);
    if (x > __dmul_rn(1.41421356237309504880, 0.5)) fe = __dadd_rn(fe, 1.0);
    else x = __dadd_rn(x, x);
    x = __dsub_rn(x, 1.0);
    const double xx2 = __dmul_rn(x, x), xx4 = __dmul_rn(xx2, xx2);
    double px = __dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(P3, x), P2), xx2),
                          __dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(P5, x), P4), xx4), __dadd_rn(__dmul_rn(P1, x), P0)));
    const double x2 = __dmul_rn(x, x);
    px = __dmul_rn(px, __dmul_rn(x, x2));
    const double qx = __dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(Q3, x), Q2), xx2),
                                __dadd_rn(__dmul_rn(__dadd_rn(Q4, x), xx4), __dadd_rn(__dmul_rn(Q1, x), Q0)));
    double res = __ddiv_rn(px, qx);
    res = __dadd_rn(__dmul_rn(fe, ln2_lo), res);
    res = __dadd_rn(res, __dsub_rn(x, __dmul_rn(x2, 0.5)));
    res = __dadd_rn(__dmul_rn(fe, ln2_hi), res);
    return res;
}

// the reference's sigmoid of sample sl of a client with n samples (elementwiseSigmoid,
// VectorND_Raw_SIMD_double.h:1596-1650)
__device__ __forceinline__ double sigmoid_at(double m, int sl, int n)
{
    const double e = (sl < (n & ~7)) ? exp_vcl(-m) : exp_cr(-m);
    return __ddiv_rn(1.0, __dadd_rn(1.0, e));
}

// -log sigma of the loss (logisticUnweightedLossFromMarginSigmoid, :1464-1532): vectorclass log in
// the lanes, the own log on the tail (the reference takes libm's there)
__device__ __forceinline__ double negloss_at(double sig, int sl, int n)
{
    return (sl < (n & ~7)) ? -log_vcl(sig) : -fednl_log(sig);
}

// (0 + h(c0..c3)) + h(c4..c7) with h(c) = (c0 + c2) + (c1 + c3): the two-Vec4d reduction
__device__ __forceinline__ double lanes8(const double* c)
{
    double fin = __dadd_rn(0.0, __dadd_rn(__dadd_rn(c[0], c[2]), __dadd_rn(c[1], c[3])));
    return __dadd_rn(fin, __dadd_rn(__dadd_rn(c[4], c[6]), __dadd_rn(c[5], c[7])));
}

// two-Vec4d dot product of a[i] b[i], i < n, by one thread
__device__ __forceinline__ double dot8_seq(const double* a, const double* b, int n)
{
    double c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const int items = n & ~7;
    int i = 0;
    for (; i < items; i += 8)
#pragma unroll
        for (int l = 0; l < 8; ++l) c[l] = __dadd_rn(c[l], __dmul_rn(a[i + l], b[i + l]));
    double rest = 0.0;
    for (; i < n; ++i) rest = __dadd_rn(rest, __dmul_rn(a[i], b[i]));
    return __dadd_rn(lanes8(c), rest);
}

// the same by the 32 lanes of a warp: lanes 0-7 take the Vec4d lanes, lane 8 the tail; the result
// is valid in lane 0
__device__ __forceinline__ double dot8_warp(const double* a, const double* b, int n)
{
    const int lane = threadIdx.x & 31;
    const int items = n & ~7;
    double acc = 0.0;
    if (lane < 8) {
        for (int i = lane; i < items; i += 8) acc = __dadd_rn(acc, __dmul_rn(a[i], b[i]));
    } else if (lane == 8) {
        for (int i = items; i < n; ++i) acc = __dadd_rn(acc, __dmul_rn(a[i], b[i]));
    }
    double c[8];
#pragma unroll
    for (int l = 0; l < 8; ++l) c[l] = __shfl_sync(0xffffffffu, acc, l);
    const double rest = __shfl_sync(0xffffffffu, acc, 8);
    return __dadd_rn(lanes8(c), rest);
}

}  // namespace refo

// ---- 1r. margins, sigmoid and per-sample weights in the reference's order ---------------------
// Binary features: the nonzero products are +-x_j (labels +-1), zero products leave a lane
// unchanged, so a lane sums x over the sample's set attributes of its residue class; the label
// multiplies the finished sum (negation commutes with round-to-nearest).
__device__ __forceinline__ void margin_weights_ref(const Dev& P, int s, double m)
{
    const int c = P.client_of[s];
    const int n = P.ns[c], sl = s - P.soff[c];
    const double sig = refo::sigmoid_at(m, sl, n);
    const double inv_m = 1.0 / (double)n;
    const double z1 = __dsub_rn(1.0, sig);
    const double b = P.lab[s];
    P.Dv[s] = __dmul_rn(inv_m, __dmul_rn(z1, sig));
    const double q = __dmul_rn(z1, -inv_m);
    P.qb[s] = (P.A != nullptr || b == 1.0) ? q : __dmul_rn(-1.0, q);   // dense: the label enters through u
    if (P.fmode) P.fterm[s] = refo::negloss_at(sig, sl, n);
}

__device__ __forceinline__ double margin_binary_ref(const Dev& P, const double* x, int s)
{
    const int cb = P.d & ~3;
    double c0 = 0.0, c1 = 0.0, c2 = 0.0, c3 = 0.0;
    int t = P.rowptr[s];
    const int t1 = P.rowptr[s + 1];
    for (; t < t1; ++t) {
        const int j = P.colidx[t];
        if (j >= cb) break;
        const double v = x[j];
        switch (j & 3) {
        case 0: c0 = __dadd_rn(c0, v); break;
        case 1: c1 = __dadd_rn(c1, v); break;
        case 2: c2 = __dadd_rn(c2, v); break;
        default: c3 = __dadd_rn(c3, v); break;
        }
    }
    double acc = __dadd_rn(__dadd_rn(c0, c2), __dadd_rn(c1, c3));
    for (; t < t1; ++t) acc = __dadd_rn(acc, x[P.colidx[t]]);
    return (P.lab[s] == 1.0) ? acc : -acc;
}

__device__ __forceinline__ double margin_dense_ref(const Dev& P, const double* x, int s)
{
    const int d = P.d, cb = d & ~3;
    const double b = P.lab[s];
    const double* a = P.A + (size_t)s * d;
    double c[4] = {0.0, 0.0, 0.0, 0.0};
    int j = 0;
    for (; j < cb; j += 4)
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            const double u = (b == 1.0) ? a[j + l] : __dmul_rn(a[j + l], -1.0);
            c[l] = __dadd_rn(c[l], __dmul_rn(u, x[j + l]));
        }
    double acc = __dadd_rn(__dadd_rn(c[0], c[2]), __dadd_rn(c[1], c[3]));
    for (; j < d; ++j) {
        const double u = (b == 1.0) ? a[j] : __dmul_rn(a[j], -1.0);
        acc = __dadd_rn(acc, __dmul_rn(u, x[j]));
    }
    return acc;
}

__global__ void k_margin_ref(Dev P, int S)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const double m = (P.A == nullptr) ? margin_binary_ref(P, P.x, s) : margin_dense_ref(P, P.x, s);
    margin_weights_ref(P, s, m);
}

// FedNL-LS trial point: -log sigma_s only
__global__ void k_ls_margin_ref(Dev P, int S)
{
    if (P.ls[2] != 0.0) return;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const double m = (P.A == nullptr) ? margin_binary_ref(P, P.x, s) : margin_dense_ref(P, P.x, s);
    const int c = P.client_of[s];
    const int n = P.ns[c], sl = s - P.soff[c];
    P.fterm[s] = refo::negloss_at(refo::sigmoid_at(m, sl, n), sl, n);
}

// ---- 3r. ||diff||_F^2 from the packed upper part, per processed client ----------------------
// One CTA per client.  The ten running sums of the reference's loop are chains of dependent FP64
// adds (eight lane accumulators shared by all columns: column j, rows i < 8 floor(j/8) with
// i mod 8 = lane; one scalar for rows 8 floor(j/8) .. j-1; one for the diagonal), and a dependent
// FP64 add costs about 64 cycles on this part, so everything else is taken off those chains: warps
// 1..7 stage the squares of the coming columns into a ring of shared-memory buffers while warp 0's
// lanes 0..9 add one column's squares to their sums.
constexpr int kFrobRefThreads = 256;
constexpr int kFrobRing = 4;                       // ring buffers: a column is added 3 steps after staging

__global__ void __launch_bounds__(kFrobRefThreads) k_frob_ref(Dev P)
{
    extern __shared__ double s_sq[];               // [kFrobRing][d]
    const int c = P.act ? P.act[blockIdx.x] : blockIdx.x;
    const double* v = P.diff + (size_t)c * P.ustr;
    const int d = P.d, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    double acc = 0.0;
    // step j0: warps 1..7 stage column j0 into buffer j0 % kFrobRing; warp 0 adds column
    // j0 - (kFrobRing - 1), staged kFrobRing - 1 barriers earlier, from its buffer (a different one)
    for (int j0 = 0; j0 < d + kFrobRing - 1; ++j0) {
        if (warp > 0 && j0 < d) {
            double* buf = s_sq + (size_t)(j0 % kFrobRing) * d;
            const double* col = v + (size_t)j0 * (j0 + 1) / 2;
            for (int i = tid - 32; i <= j0; i += kFrobRefThreads - 32) buf[i] = __dmul_rn(col[i], col[i]);
        }
        const int j = j0 - (kFrobRing - 1);
        if (warp == 0 && j >= 0) {
            const double* buf = s_sq + (size_t)(j % kFrobRing) * d;
            const int items = j & ~7;
            if (lane < 8) {
                for (int i = lane; i < items; i += 8) acc = __dadd_rn(acc, buf[i]);
            } else if (lane == 8) {
                for (int i = items; i < j; ++i) acc = __dadd_rn(acc, buf[i]);
            } else if (lane == 9) {
                acc = __dadd_rn(acc, buf[j]);
            }
        }
        __syncthreads();
    }
    if (warp == 0) {
        double c8[8];
#pragma unroll
        for (int l = 0; l < 8; ++l) c8[l] = __shfl_sync(0xffffffffu, acc, l);
        const double rest = __shfl_sync(0xffffffffu, acc, 8);
        const double diag = __shfl_sync(0xffffffffu, acc, 9);
        if (lane == 0) {
            double out = refo::lanes8(c8);
            out = __dadd_rn(out, rest);
            const double f = __dadd_rn(__dadd_rn(out, out), diag);
            P.F[c] = f;
            if (!P.pp) P.lk[c] = sqrt(f);
        }
    }
}

// ---- 8cr. objective values ------------------------------------------------------------------
// f_i = loss + (lambda / 2) ||x||^2 (evaluateFunction(x, margin, sigmoid), logistic_regression.h:
// 119-123): the loss's lanes over the client's samples, its tail, (fin + rest) / n; one warp per
// client; skipped once the line search has finished (gate = P.ls)
__global__ void k_fclient_ref(Dev P, const double* x, const double* gate)
{
    if (gate && gate[2] != 0.0) return;
    const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (c >= P.nc) return;
    const int lane = threadIdx.x & 31;
    const int n = P.ns[c];
    const double* ft = P.fterm + P.soff[c];
    const int items = n & ~7;
    double acc = 0.0;
    if (lane < 8) {
        for (int i = lane; i < items; i += 8) acc = __dadd_rn(acc, ft[i]);
    } else if (lane == 8) {
        for (int i = items; i < n; ++i) acc = __dadd_rn(acc, ft[i]);
    }
    double c8[8];
#pragma unroll
    for (int l = 0; l < 8; ++l) c8[l] = __shfl_sync(0xffffffffu, acc, l);
    const double rest = __shfl_sync(0xffffffffu, acc, 8);
    const double loss = __ddiv_rn(__dadd_rn(refo::lanes8(c8), rest), (double)n);
    const double xs = refo::dot8_warp(x, x, P.d);
    if (lane == 0) P.fi[c] = __dadd_rn(loss, __dmul_rn(__ddiv_rn(P.lambda, 2.0), xs));
}

// master: f = (f_0 + f_1 + ... in client order) / n (function_aggregation, TrainLoop.h:1511-1541)
__device__ __forceinline__ double client_mean_ref(const Dev& P)
{
    double s = 0.0;
    for (int c = 0; c < P.nc; ++c) s = __dadd_rn(s, P.fi[c]);
    return __dmul_rn(s, P.inv_n);
}

__global__ void k_fmaster_ref(Dev P, double* out)
{
    if (threadIdx.x == 0) *out = client_mean_ref(P);
}

// FedNL-LS: t = 1, -(dx . g) as the reference's dot product, x_k kept
__global__ void k_ls_init_ref(Dev P)
{
    for (int i = threadIdx.x; i < P.d; i += blockDim.x) P.xprev[i] = P.x[i];
    if (threadIdx.x < 32) {
        const double dg = refo::dot8_warp(P.dx, P.g, P.d);
        if (threadIdx.x == 0) {
            P.ls[0] = 1.0;
            P.ls[1] = -dg;
            P.ls[2] = P.ls[4] != 0.0 ? 0.0 : 1.0;
            P.ls[3] = 0.0;
        }
    }
}

__global__ void k_ls_check_ref(Dev P, double c, double gamma)
{
    if (P.ls[2] != 0.0) return;
    if (threadIdx.x == 0) {
        const double fr = client_mean_ref(P);
        P.ls[3] = __dadd_rn(P.ls[3], 1.0);
        const double t = P.ls[0];
        if (fr <= __dadd_rn(P.stats[2], __dmul_rn(__dmul_rn(c, t), P.ls[1]))) P.ls[2] = 1.0;
        else P.ls[0] = __dmul_rn(t, gamma);
    }
}

// ---- 8r. Option-B solve in the reference's order -------------------------------------------
// choleskyFactorization<.., true, true> computes column i of R (= L^T) row by row:
// R_ji = (1 / R_jj)(H_ji - R[0:j, i] . R[0:j, j]) for j < i, then R_ii = sqrt((H_ii + l) -
// ||R[0:i, i]||^2); forwardSubstitutionWithATranspose gives y_j = (g_j - R[0:j, j] . y[0:j]) / R_jj,
// backwardSubstitutionWithATranspose x_i = (y_i - R[i, i+1:d] . x[i+1:d]) / R_ii, all dot products
// in the two-Vec4d order.  In the dot of entry (j, i) over k < j, row k goes to lane k mod 8 when
// k < 8 floor(j/8) and to the in-order tail otherwise; the terms of each lane and of the tail are
// added in increasing k, which is the order in which the rows of R are finished.  So the kernel runs
// right-looking over blocks of 8 rows with nine accumulators per entry of the augmented matrix
// [H | g] (g as column d, whose entries become y):
//   1. CTA 0 finishes the block's rows one by one (pivot, then the row's entries from their
//      accumulators with the reference's expression; the block's later rows collect the row in
//      their tails);
//   2. grid barrier; every CTA adds the block's 8 rows to lane l of the entries below the block
//      (row 8b + l into lane l: one product and one add per lane and entry); grid barrier.
// The backward substitution runs in one warp of CTA 0: for each row from the bottom, lanes 0-7 form
// the Vec4d lanes of its dot product and lane 8 the tail.  Every value equals the reference's.
constexpr int kRefCholThreads = 256;

__device__ __forceinline__ size_t apos(int j, int i) { return (size_t)i * (i + 1) / 2 + j; }

__global__ void __launch_bounds__(kRefCholThreads) k_chol_ref(Dev P, const double* __restrict__ Hin,
                                                              const double* lptr, double lval,
                                                              const double* __restrict__ gin, double* dxout,
                                                              double* xupd, int record)
{
    GridSync gs(P.bar, gridDim.x);
    __shared__ double s_r, s_inv;
    __shared__ int s_bad;
    const int d = P.d, tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31;
    const size_t Ua = (size_t)(d + 1) * (d + 2) / 2;
    double* R = P.rref;                       // [Ua] R, column d = y
    double* acc = P.racc;                     // [9][Ua]: lanes 0..7, then the tail
    volatile unsigned* badflag = P.bar + 3;   // not positive definite, set by CTA 0 before a barrier
    const double l = lptr ? *lptr : lval;
    if (P.ls && blockIdx.x == 0 && tid == 0) P.ls[4] = 0.0;
    if (blockIdx.x == 0 && tid == 0) *badflag = 0u;
    {
        const size_t gtid = (size_t)blockIdx.x * nthr + tid, gthr = (size_t)gridDim.x * nthr;
        for (size_t p = gtid; p < 9 * Ua; p += gthr) acc[p] = 0.0;
    }
    if (!gs.sync()) goto timeout;
    for (int k0 = 0; k0 < d; k0 += 8) {
        const int k1 = min(k0 + 8, d);
        if (blockIdx.x == 0) {
            for (int k = k0; k < k1; ++k) {
                if (tid == 0) {
                    double c8[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) c8[q] = acc[q * Ua + apos(k, k)];
                    const double sq = __dadd_rn(refo::lanes8(c8), acc[8 * Ua + apos(k, k)]);
                    const double a = __dsub_rn(__dadd_rn(Hin[up_pos(k, k)], l), sq);
                    s_bad = (a < 0.0) ? 1 : 0;
                    double inv;
                    const double r = sqrt_rcp_rn_int(a, inv);
                    s_r = r;
                    s_inv = inv;
                    R[apos(k, k)] = r;
                }
                __syncthreads();
                if (s_bad) break;
                const double r = s_r, inv = s_inv;
                for (int i = k + 1 + tid; i <= d; i += nthr) {
                    double c8[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) c8[q] = acc[q * Ua + apos(k, i)];
                    const double dot = __dadd_rn(refo::lanes8(c8), acc[8 * Ua + apos(k, i)]);
                    R[apos(k, i)] = (i < d) ? __dmul_rn(inv, __dsub_rn(Hin[up_pos(k, i)], dot))
                                            : __ddiv_rn(__dsub_rn(gin[k], dot), r);
                }
                __syncthreads();
                // the block's later rows j collect row k in their tails: entries (j, i), j <= i <= d
                for (int j = k + 1; j < k1; ++j) {
                    const double rkj = R[apos(k, j)];
                    for (int i = j + tid; i <= d; i += nthr)
                        acc[8 * Ua + apos(j, i)] = __dadd_rn(acc[8 * Ua + apos(j, i)], __dmul_rn(rkj, R[apos(k, i)]));
                }
                __syncthreads();
            }
            if (tid == 0 && s_bad) *badflag = 1u;
        }
        if (!gs.sync()) goto timeout;
        if (*badflag) {
            if (blockIdx.x == 0 && tid == 0) {
                *P.status = -4;
                if (record) *P.round_ctr += 1;
            }
            gs.finish();
            return;
        }
        if (k1 - k0 == 8 && k1 < d) {
            // lane l of every entry (j, i), k1 <= j <= min(i, d - 1), k1 <= i <= d, adds row k0 + l
            for (int i = k1 + (int)blockIdx.x; i <= d; i += (int)gridDim.x) {
                double ri[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) ri[q] = R[apos(k0 + q, i)];
                const int jmax = min(i, d - 1);
                for (int j = k1 + tid; j <= jmax; j += nthr) {
                    const size_t pe = apos(j, i);
#pragma unroll
                    for (int q = 0; q < 8; ++q)
                        acc[q * Ua + pe] = __dadd_rn(acc[q * Ua + pe], __dmul_rn(R[apos(k0 + q, j)], ri[q]));
                }
            }
            if (!gs.sync()) goto timeout;
        }
    }
    if (blockIdx.x != 0) {
        gs.finish();
        return;
    }
    {
        double* x = P.ybuf;                  // [d]
        if (tid < 32) {
            for (int i = d - 1; i >= 0; --i) {
                const int len = d - 1 - i, items = len & ~7;
                double a = 0.0;
                if (lane < 8) {
                    for (int q = lane; q < items; q += 8) a = __dadd_rn(a, __dmul_rn(R[apos(i, i + 1 + q)], x[i + 1 + q]));
                } else if (lane == 8) {
                    for (int q = items; q < len; ++q) a = __dadd_rn(a, __dmul_rn(R[apos(i, i + 1 + q)], x[i + 1 + q]));
                }
                double c8[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) c8[q] = __shfl_sync(0xffffffffu, a, q);
                const double rest = __shfl_sync(0xffffffffu, a, 8);
                if (lane == 0) x[i] = __ddiv_rn(__dsub_rn(R[apos(i, d)], __dadd_rn(refo::lanes8(c8), rest)), R[apos(i, i)]);
                __syncwarp();
            }
            if (record) {
                const double gsq = refo::dot8_warp(gin, gin, d);
                if (lane == 0) P.stats[0] = sqrt(gsq);
            }
        }
        __syncthreads();
        for (int i = tid; i < d; i += nthr) {
            const double dxi = x[i];
            if (dxout) dxout[i] = dxi;
            if (xupd) xupd[i] = __dsub_rn(xupd[i], dxi);
        }
        if (record && tid == 0) {
            const int r = *P.round_ctr;
            if (r < P.hist_cap) P.hist[r] = P.stats[0];
            *P.round_ctr = r + 1;
        }
        if (P.ls && tid == 0) P.ls[4] = 1.0;
    }
    gs.finish();
    return;
timeout:
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *P.status = -5;
        if (record) *P.round_ctr += 1;
    }
}

}  // namespace fednl
