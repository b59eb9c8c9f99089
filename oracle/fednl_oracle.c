/*
 * fednl_oracle.c -- CPU restatement of the u-FedNL (dopt) FedNL round.  TEST INFRASTRUCTURE:
 * the parity oracle for the GB300 kernels and the timed CPU port in bench.py.  Nothing in
 * the product library (libfednl_gpu.so) links or calls this file.
 *
 * Each function cites the reference file:line it restates (paths relative to the ufednl
 * repository root).  Floating-point formulas keep the reference's operation order where the
 * reference fixes it (per-entry sample order of the Hessian and gradient sums, products as
 * written); SIMD horizontal-sum orders of dot products and norms are restated as sequential
 * sums, which changes results by a few ulps only.  In the fixed order (not ref_order), {0,1}
 * features take their attribute sums (gradient, Hessian diagonal, intercept column) in 64-sample
 * words (blocked_attr_sum), the GPU engine's order for them.  The file is compiled with
 * -ffp-contract=off so that no multiply-add is fused.
 */
#include "fednl_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ================================================================================== */
/* LCG generators                                                                     */
/* ================================================================================== */

/* RandomGenIntegerLinear: x <- 214013 x + 2531011 (mod 2^32)
 * dopt/dopt/random/include/RandomGenIntegerLinear.h:107-123, src/RandomGenIntegerLinear.cpp:12-19 */
uint32_t orc_lcg_int_next(uint32_t* state)
{
    *state = 214013u * (*state) + 2531011u;
    return *state;
}

/* RandomGenIntegerLinear::generateRealInUnitInterval, RandomGenIntegerLinear.h:49-58 */
double orc_lcg_int_unit(uint32_t* state)
{
    *state = 214013u * (*state) + 2531011u;
    return (double)(*state) * (1.0 / 4294967295.0);
}

/* RandomGenRealLinear::generateRealInUnitInterval: (a x + c) mod 2^32, then mod (2^32 - 1)
 * dopt/dopt/random/include/RandomGenRealLinear.h:54-59, src/RandomGenRealLinear.cpp:5-8 */
double orc_lcg_real_unit(uint32_t* state)
{
    uint32_t t = 214013u * (*state) + 2531011u;
    *state = t % 4294967295u;
    return (double)(*state) * (1.0 / 4294967295.0);
}

/* roundToNearestInt<size_t>, dopt/dopt/math_routines/include/SimpleMathRoutines.h:408-414 */
size_t orc_round_to_nearest(double v)
{
    size_t t = (size_t)v;
    if (v - (double)t > 0.5)
        return t + 1;
    return t;
}

/* ================================================================================== */
/* Upper-triangle indices and compressors                                             */
/* ================================================================================== */

size_t orc_upper_count(int32_t d) { return ((size_t)d * (size_t)(d + 1)) / 2; }

/* indiciesForUpperTriangularPart: column j, rows 0..j, flat index j*LDA + i
 * dopt/dopt/math_routines/include/SpecialMathRoutinesForMatrix.h:35-64 */
void orc_upper_indices(int32_t d, int32_t lda, uint32_t* out)
{
    size_t w = 0;
    for (int32_t j = 0; j < d; ++j)
        for (int32_t i = 0; i <= j; ++i)
            out[w++] = (uint32_t)j * (uint32_t)lda + (uint32_t)i;
}

/* Philox4x32-10: ten rounds of (hi0, lo0) = 0xD2511F53 c0, (hi1, lo1) = 0xCD9E8D57 c2,
 * c = (hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0), the key bumped by the Weyl constants
 * (0x9E3779B9, 0xBB67AE85) between rounds (Salmon et al., SC'11). */
void orc_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3], k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0, hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

/* Feistel permutation of [0, 2^(2h)) with six rounds whose round function is Philox keyed by
 * (seed, client) on the counter (right half, round, draw, 'RAND') */
static uint32_t feistel(uint32_t x, int h, uint32_t seed, uint32_t client, uint32_t draw)
{
    uint32_t mask = (1u << h) - 1u, L = x >> h, R = x & mask;
    for (uint32_t r = 0; r < 6; ++r) {
        uint32_t ctr[4] = {R, r, draw, 0x52414E44u}, key[2] = {seed, client}, o[4];
        orc_philox4x32(ctr, key, o);
        uint32_t nl = R, nr = L ^ (o[0] & mask);
        L = nl;
        R = nr;
    }
    return (L << h) | R;
}

static int philox_half_bits(size_t U)
{
    int b = 0;
    while (((size_t)1 << b) < U)
        ++b;
    if (b < 2)
        b = 2;
    return (b + 1) / 2;
}

static uint32_t philox_position(uint32_t i, size_t U, int h, uint32_t seed, uint32_t client, uint32_t draw)
{
    uint32_t y = feistel(i, h, seed, client, draw);
    while ((size_t)y >= U)                    /* cycle walking: a permutation of [0, U) */
        y = feistel(y, h, seed, client, draw);
    return y;
}

void orc_randk_philox(uint32_t seed, uint32_t client, uint32_t draw, int32_t k, size_t U, const uint32_t* upper,
                      uint32_t* out)
{
    int h = philox_half_bits(U);
    uint8_t* mark = (uint8_t*)calloc(U, 1);
    for (int32_t i = 0; i < k; ++i)
        mark[philox_position((uint32_t)i, U, h, seed, client, draw)] = 1;
    int32_t w = 0;
    for (size_t p = 0; p < U; ++p)
        if (mark[p])
            out[w++] = upper[p];
    free(mark);
}

/* Partial Fisher-Yates with early stop, dopt/dopt/random/include/Shuffle.h:31-95 (active loop :76-93) */
void orc_shuffle_partial(uint32_t* arr, size_t n, size_t k, uint32_t* state)
{
    size_t n_minus_i_minus_one = n - 1;
    for (size_t i = 0; i < k; ++i, --n_minus_i_minus_one) {
        double u = orc_lcg_int_unit(state);
        size_t r_off = orc_round_to_nearest(u * (double)n_minus_i_minus_one);
        if (r_off != 0) {
            uint32_t t = arr[i];
            arr[i] = arr[i + r_off];
            arr[i + r_off] = t;
        }
    }
}

static int cmp_u32(const void* a, const void* b)
{
    uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
    return (x > y) - (x < y);
}

/* generateRandKItemsInUpperTriangularPart, SpecialMathRoutinesForMatrix.h:95-107 */
void orc_randk(uint32_t* state, int32_t k, size_t U, const uint32_t* upper, uint32_t* out)
{
    uint32_t* tmp = (uint32_t*)malloc(U * sizeof(uint32_t));
    memcpy(tmp, upper, U * sizeof(uint32_t));
    orc_shuffle_partial(tmp, U, (size_t)k, state);
    memcpy(out, tmp, (size_t)k * sizeof(uint32_t));
    qsort(out, (size_t)k, sizeof(uint32_t), cmp_u32);
    free(tmp);
}

/* generateRandSeqKItemsInUpperTriangularPart, SpecialMathRoutinesForMatrix.h:137-169 */
void orc_randseqk(uint32_t* state, int32_t k, size_t U, const uint32_t* upper, uint32_t* out)
{
    uint32_t r = (uint32_t)((size_t)orc_lcg_int_next(state) % U);
    for (int32_t t = 0; t < k; ++t) {
        size_t p = (size_t)r + (size_t)t;
        if (p >= U)
            p -= U;
        out[t] = upper[p];
    }
}

/* ---- 4-ary min-heap of flat indices keyed by |m[index]| --------------------------- */
/* dopt/dopt/math_routines/include/MinHeap.h (D = 4) */
typedef struct {
    uint32_t* data;
    size_t size;
    const double* m;
} orc_heap;

static inline double hkey(const orc_heap* h, uint32_t idx) { return fabs(h->m[idx]); }

/* minHeapify, MinHeap.h:255-290: leftmost strictly-smaller child wins */
static void heap_sift(orc_heap* h, size_t i, size_t heap_size)
{
    double lowest_value = hkey(h, h->data[i]);
    for (;;) {
        size_t lowest = i;
        size_t first = 4 * i + 1;
        size_t last = first + 4 < heap_size ? first + 4 : heap_size;
        for (size_t c = first; c < last; ++c) {
            double cv = hkey(h, h->data[c]);
            if (lowest_value > cv) {
                lowest = c;
                lowest_value = cv;
            }
        }
        if (lowest != i) {
            uint32_t t = h->data[i];
            h->data[i] = h->data[lowest];
            h->data[lowest] = t;
            i = lowest;
        } else {
            break;
        }
    }
}

/* buildMinHeap, MinHeap.h:147-191: Floyd build starting at (sz + D - 2) / D */
static void heap_build(orc_heap* h)
{
    size_t i = (h->size + 4 - 2) / 4;
    for (;;) {
        heap_sift(h, i, h->size);
        if (i == 0)
            break;
        --i;
    }
}

/* extracFromMinHeap, MinHeap.h:125-141 */
static uint32_t heap_extract(orc_heap* h)
{
    uint32_t res = h->data[0];
    size_t n = h->size;
    uint32_t t = h->data[0];
    h->data[0] = h->data[n - 1];
    h->data[n - 1] = t;
    heap_sift(h, 0, n - 1);
    h->size = n - 1;
    return res;
}

/* insertInMinHeap, MinHeap.h:92-103 */
static void heap_insert(orc_heap* h, uint32_t v)
{
    size_t i = h->size++;
    h->data[i] = v;
    while (i != 0 && hkey(h, h->data[(i - 1) / 4]) > hkey(h, h->data[i])) {
        size_t p = (i - 1) / 4;
        uint32_t t = h->data[p];
        h->data[p] = h->data[i];
        h->data[i] = t;
        i = p;
    }
}

static double chunked_sum(const double* t, size_t n);

/* Heap phase shared by TopK and TopLEK: SpecialMathRoutinesForMatrix.h:291-318 (TopK) and
 * :406-433 (TopLEK).  Seeds the heap with the first k upper indices, then replaces the root
 * by every later entry whose magnitude is strictly larger. */
static void topk_heap_scan(orc_heap* h, int32_t k, size_t U, const uint32_t* upper)
{
    memcpy(h->data, upper, (size_t)k * sizeof(uint32_t));
    h->size = (size_t)k;
    heap_build(h);
    double min_value = hkey(h, h->data[0]);
    for (size_t i = (size_t)k; i < U; ++i) {
        uint32_t cand = upper[i];
        if (hkey(h, cand) > min_value) {
            h->data[0] = cand;                 /* increaseMinimumInMinHeap, MinHeap.h:78-85 */
            heap_sift(h, 0, h->size);
            min_value = hkey(h, h->data[0]);
        }
    }
}

/* getTopKFromUpperDiagonalPart<ignoreSign=true>, SpecialMathRoutinesForMatrix.h:229-366 */
int32_t orc_topk(const double* m, int32_t k, size_t U, const uint32_t* upper, uint32_t* out)
{
    if ((size_t)k >= U) {
        memcpy(out, upper, U * sizeof(uint32_t));
        return (int32_t)U;
    }
    orc_heap h;
    h.data = out;
    h.m = m;
    topk_heap_scan(&h, k, U, upper);
    qsort(out, (size_t)k, sizeof(uint32_t), cmp_u32);
    return k;
}

/* getTopLEKFromUpperDiagonalPart<ignoreSign=true>, SpecialMathRoutinesForMatrix.h:377-511.
 * rng_state is the calling worker thread's RandomGenRealLinear state (thread_local, :383). */
static int32_t toplek_ref_window(orc_heap* h, const double* m, int32_t lda, size_t K, double frob_sq,
                                 double one_minus_delta_xf, double eps, uint32_t* rng_state);

static int32_t toplek_impl(const double* m, int32_t lda, int32_t k, size_t U, const uint32_t* upper,
                           double delta, double frob_sq, uint32_t* rng_state, uint32_t* out, int ref_order)
{
    double one_minus_delta = 1.0 - delta;
    double one_minus_delta_xf = one_minus_delta * frob_sq;
    double eps = 1e-1 * frob_sq;

    if ((size_t)k >= U) {
        memcpy(out, upper, U * sizeof(uint32_t));
        return (int32_t)U;
    }

    orc_heap h;
    h.data = out;
    h.m = m;
    topk_heap_scan(&h, k, U, upper);
    if (ref_order) {
        int32_t keep = toplek_ref_window(&h, m, lda, (size_t)k, frob_sq, one_minus_delta_xf, eps, rng_state);
        qsort(out, (size_t)keep, sizeof(uint32_t), cmp_u32);
        return keep;
    }

    /* Numerator of the rounding window (:435-503).  The reference subtracts the heap's terms from
     * ||M||^2 one by one in heap-array order and then adds back the extracted terms one by one in
     * extraction order.  Restated with a fixed order the GB300 kernel also uses: the heap's terms
     * (c v^2, c = 1 on the diagonal, 2 off it) are summed by chunked_sum in heap-array order and
     * subtracted once; the prefix sums of the extracted terms are formed per chunk of 32 by the
     * inclusive doubling scan s_l += s_{l-h} (h = 1, 2, 4, 8, 16) and carried from chunk to chunk
     * in order.  The values differ from the reference's by a few ulps, which matters only if the
     * window boundary falls within those ulps.  Every numerator is num0 plus non-negative terms
     * (monotone rounding), so when the window's upper bound does not exceed num0 no extraction
     * opens it and none is made.  Otherwise the heap is extracted in chunks of 32; the extracted
     * element lands at the array's end (MinHeap.h:133-140), so the elements not extracted by step
     * m are the array prefix of length k - 1 - m whatever later extractions do, and extraction
     * stops after the chunk that holds the first window hit. */
    size_t K = (size_t)k;
    double* terms = (double*)malloc(K * sizeof(double));
    for (size_t i = 0; i < K; ++i) {
        uint32_t index = h.data[i];
        double item = m[index];
        uint32_t jc = index / (uint32_t)lda, ir = index - jc * (uint32_t)lda;
        terms[i] = (ir == jc) ? item * item : (item * item) * 2.0;
    }
    double num0 = frob_sq - chunked_sum(terms, K);
    double hi = one_minus_delta_xf + eps;
    size_t keep = 0;
    if (hi > num0) {
        double carry = num0, prev_last = num0;
        size_t size = K;
        for (size_t q = 0; q < K; q += 32) {
            size_t target = (K - q > 32) ? K - q - 32 : 1;     /* heap size after this chunk */
            for (; size > target; --size) {                   /* extracFromMinHeap */
                uint32_t t = h.data[0];
                h.data[0] = h.data[size - 1];
                h.data[size - 1] = t;
                heap_sift(&h, 0, size - 1);
            }
            double v[32], w[32];
            int n = (int)((K - q) < 32 ? (K - q) : 32);
            for (int l = 0; l < 32; ++l) {                     /* extracted term m is at K - 1 - m */
                if (l < n) {
                    uint32_t index = h.data[K - 1 - (q + (size_t)l)];
                    double item = m[index];
                    uint32_t jc = index / (uint32_t)lda, ir = index - jc * (uint32_t)lda;
                    v[l] = (ir == jc) ? item * item : (item * item) * 2.0;
                } else {
                    v[l] = 0.0;
                }
            }
            for (int hh = 1; hh < 32; hh <<= 1) {
                for (int l = 0; l < 32; ++l)
                    w[l] = (l >= hh) ? v[l] + v[l - hh] : v[l];
                memcpy(v, w, sizeof(v));
            }
            int hit = -1;
            double prev = prev_last, nx = 0.0;
            for (int l = 0; l < n; ++l) {
                prev = (l == 0) ? prev_last : carry + v[l - 1];
                nx = carry + v[l];
                if (hi > prev && one_minus_delta_xf < nx + eps) {
                    hit = l;
                    break;
                }
            }
            if (hit >= 0) {
                size_t mm = q + (size_t)hit;
                double p = (one_minus_delta_xf - prev + eps) / (nx - prev + eps);
                keep = K - 1 - mm;
                if (orc_lcg_real_unit(rng_state) > p)
                    keep += 1;        /* insertInMinHeap of the extracted element: it is at position K-1-mm */
                break;
            }
            prev_last = carry + v[n - 1];
            carry = carry + v[n - 1];
        }
    }
    free(terms);
    qsort(out, keep, sizeof(uint32_t), cmp_u32);
    return (int32_t)keep;
}

int32_t orc_toplek(const double* m, int32_t lda, int32_t k, size_t U, const uint32_t* upper,
                   double delta, double frob_sq, uint32_t* rng_state, uint32_t* out)
{
    return toplek_impl(m, lda, k, U, upper, delta, frob_sq, rng_state, out, 0);
}

int32_t orc_toplek_ref(const double* m, int32_t lda, int32_t k, size_t U, const uint32_t* upper,
                       double delta, double frob_sq, uint32_t* rng_state, uint32_t* out)
{
    return toplek_impl(m, lda, k, U, upper, delta, frob_sq, rng_state, out, 1);
}

/* The rounding window in the reference's own order (SpecialMathRoutinesForMatrix.h:435-503): the
 * numerator starts at ||M||^2 and loses c v^2 (c = 1 on the diagonal, 2.0 * v * v off it) for every
 * heap entry in heap-array order; then the heap is extracted one minimum at a time (MinHeap.h:133-140
 * extraction, the extracted element lands at the array's end) and the numerator gains the extracted
 * entry's term; the first step with (1-delta)||M||^2 + eps > prev and (1-delta)||M||^2 < next + eps
 * draws u from the worker's generator and re-inserts the extracted entry when u > p.  Returns the
 * number of kept entries, which are the array prefix (plus the re-inserted one at its end). */
static int32_t toplek_ref_window(orc_heap* h, const double* m, int32_t lda, size_t K, double frob_sq,
                                 double one_minus_delta_xf, double eps, uint32_t* rng_state)
{
    double numerator = frob_sq;
    for (size_t i = 0; i < K; ++i) {
        uint32_t index = h->data[i];
        double item = m[index];
        uint32_t jc = index / (uint32_t)lda, ir = index - jc * (uint32_t)lda;
        numerator = (ir == jc) ? numerator - item * item : numerator - (2.0 * item) * item;
    }
    size_t size = K;
    while (size > 0) {
        double prev = numerator;
        uint32_t t = h->data[0];
        h->data[0] = h->data[size - 1];
        h->data[size - 1] = t;
        heap_sift(h, 0, size - 1);
        size -= 1;
        double item = m[t];
        uint32_t jc = t / (uint32_t)lda, ir = t - jc * (uint32_t)lda;
        numerator = (ir == jc) ? numerator + item * item : numerator + (2.0 * item) * item;
        double next = numerator;
        if (one_minus_delta_xf + eps > prev && one_minus_delta_xf < next + eps) {
            double p = (one_minus_delta_xf - prev + eps) / (next - prev + eps);
            if (orc_lcg_real_unit(rng_state) > p)
                size += 1;     /* insertInMinHeap: the extracted entry still sits at position size */
            break;
        }
    }
    return (int32_t)size;
}

/* applyNaturalCompressorNaive: sign and exponent kept, mantissa zeroed, MatrixNMD.h:2013-2031 */
double orc_natural(double v)
{
    uint64_t b;
    memcpy(&b, &v, 8);
    b &= ~((((uint64_t)1) << 52) - 1);
    memcpy(&v, &b, 8);
    return v;
}

/* pack2FP64NoMantissa: [signA(1) expA(11) signB(1) expB(11)], dopt/dopt/system/include/FloatUtils.h:193-221 */
uint32_t orc_pack2_natural(double a, double b)
{
    uint64_t ba, bb;
    memcpy(&ba, &a, 8);
    memcpy(&bb, &b, 8);
    uint32_t sa = (uint32_t)(ba >> 63), ea = (uint32_t)((ba >> 52) & 0x7FF);
    uint32_t sb = (uint32_t)(bb >> 63), eb = (uint32_t)((bb >> 52) & 0x7FF);
    return (sa << 23) | (ea << 12) | (sb << 11) | eb;
}

/* Sum of t[0..n) in a fixed order: chunks of 32 consecutive terms (the last one zero-padded)
 * are each reduced by the halving tree v[l] += v[l + h], h = 16, 8, 4, 2, 1, and the chunk sums
 * are added in order.  The reference's norm (VectorND_Raw_SIMD_double.h:749-800) sums in its
 * SIMD lane order; any fixed order agrees with it to a few ulps, and this one is also the order
 * of the GB300 kernels (a warp-shuffle tree per 32 entries). */
static double chunked_sum(const double* t, size_t n)
{
    double total = 0.0;
    for (size_t base = 0; base < n; base += 32) {
        double v[32];
        for (int l = 0; l < 32; ++l)
            v[l] = (base + (size_t)l < n) ? t[base + (size_t)l] : 0.0;
        for (int h = 16; h > 0; h >>= 1)
            for (int l = 0; l < h; ++l)
                v[l] = v[l] + v[l + h];
        total = total + v[0];
    }
    return total;
}

/* squared L2 norm of a buffer (frobeniusNormSquareForSymmetricMatrixFromUpPart on the full
 * d x lda buffer, MatrixNMD.h:486-488) */
double orc_l2sq(const double* v, size_t n)
{
    double* t = (double*)malloc((n ? n : 1) * sizeof(double));
    for (size_t i = 0; i < n; ++i)
        t[i] = v[i] * v[i];
    double s = chunked_sum(t, n);
    free(t);
    return s;
}

/* ||M||_F^2 of a symmetric d x lda matrix from its upper part (the reference's
 * frobeniusNormForSymmetricMatrixFromUpPart over the full buffer, MatrixNMD.h:478-488), in a fixed
 * order that the GB300 kernel follows exactly: upper positions p (column j, rows 0..j) are cut into
 * segments of 512; inside a segment, lane l = p mod 32 accumulates m_p^2 over its 16 positions in
 * order with fused multiply-adds (a_l = fma(m_p, m_p, a_l)), diagonal entries into a_l and
 * off-diagonal ones into b_l; lane l contributes
 * v_l = a_l + 2 b_l, the 32 lane values are reduced by the halving tree, and the segment sums are
 * added in order. */
double orc_frob_sym(const double* m, int32_t d, int32_t lda)
{
    size_t U = orc_upper_count(d);
    uint32_t* col = (uint32_t*)malloc(U * sizeof(uint32_t));
    uint32_t* row = (uint32_t*)malloc(U * sizeof(uint32_t));
    size_t p = 0;
    for (int32_t j = 0; j < d; ++j)
        for (int32_t i = 0; i <= j; ++i, ++p) {
            col[p] = (uint32_t)j;
            row[p] = (uint32_t)i;
        }
    double total = 0.0;
    for (size_t seg = 0; seg < U; seg += 512) {
        double v[32];
        for (int l = 0; l < 32; ++l) {
            double a = 0.0, b = 0.0;
            for (int q = 0; q < 16; ++q) {
                size_t pp = seg + 32 * (size_t)q + (size_t)l;
                if (pp >= U)
                    continue;
                double x = m[(size_t)col[pp] * lda + row[pp]];
                if (row[pp] == col[pp])
                    a = fma(x, x, a);
                else
                    b = fma(x, x, b);
            }
            v[l] = a + b * 2.0;
        }
        for (int h = 16; h > 0; h >>= 1)
            for (int l = 0; l < h; ++l)
                v[l] = v[l] + v[l + h];
        total = total + v[0];
    }
    free(col);
    free(row);
    return total;
}

/* ================================================================================== */
/* Logistic-regression oracle                                                         */
/* dopt/dopt/optimization_problems/include/ml/logistic_regression.h                   */
/* ================================================================================== */

/* evaluateClassificationMargin, :88-92 (m = Atr^T x) */
void orc_margin(const double* atr, int32_t d, int32_t lda, int32_t n, const double* x, double* m)
{
    for (int32_t s = 0; s < n; ++s) {
        const double* col = atr + (size_t)s * lda;
        double acc = 0.0;
        for (int32_t i = 0; i < d; ++i)
            acc += col[i] * x[i];
        m[s] = acc;
    }
}

/* exp(x), own implementation (the GB300 kernels run the identical operation sequence, so both
 * give the same bits on every platform).  Method: Cody-Waite reduction x = k ln2 + r with ln2 split
 * into a 32-bit head and a tail, r kept as a double-double (r_hi, r_lo); exp(r) = 1 + r + r^2/2 +
 * r^3/6 + r^4 P(r), the first four terms summed with exact two-sum / two-product error terms and
 * the Taylor tail P (1/24 ... 1/13!) in double; one final rounding; then scaling by 2^k.  The error
 * before the final rounding is about 1e-3 ulp (the two-part ln2 is the split published with fdlibm's
 * e_exp.c / e_log.c), so results are correctly rounded except in rare
 * near-halfway cases.  The reference's sigmoid uses the vectorclass exp in SIMD lanes and libm exp
 * for the tail (VectorND_Raw_SIMD_double.h:1596-1650), both within an ulp of this. */
static double pow2i(int k)
{
    uint64_t b = (uint64_t)(k + 1023) << 52;
    double v;
    memcpy(&v, &b, 8);
    return v;
}

static void two_sum(double a, double b, double* s, double* e)
{
    double t = a + b;
    double bb = t - a;
    *e = (a - (t - bb)) + (b - bb);
    *s = t;
}

double orc_exp(double x)
{
    if (x != x)
        return x;
    if (x > 709.782712893384)
        return 1.0 / 0.0;
    if (x < -745.1332191019412)
        return 0.0;
    const double ln2_hi = 6.93147180369123816490e-01, ln2_lo = 1.90821492927058770002e-10;
    double kd = rint(x * 1.4426950408889634);
    double t = fma(-kd, ln2_hi, x);                 /* exact */
    double pl_hi = kd * ln2_lo;
    double pl_lo = fma(kd, ln2_lo, -pl_hi);
    double r_hi, e0;
    two_sum(t, -pl_hi, &r_hi, &e0);
    double r_lo = e0 - pl_lo;
    /* r^2 and r^3 with their rounding errors */
    double r2 = r_hi * r_hi;
    double r2e = fma(r_hi, r_hi, -r2);
    double r3 = r2 * r_hi;
    double r3e = fma(r2, r_hi, -r3) + r2e * r_hi;
    /* tail r^4 (1/24 + r/120 + ... + r^9/13!) */
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
    double tail = (r2 * r2) * q;
    /* r^3 / 6 as head + error (1/6 = c6 + c6e) */
    const double c6 = 1.6666666666666666e-01, c6e = 9.2518585385429707e-18;
    double s3 = r3 * c6;
    double s3e = fma(r3, c6, -s3) + (r3e * c6 + r3 * c6e);
    /* 1 + r_hi + r2/2 + s3, exactly as double-doubles, then all small terms */
    double s, e1, e2, e3;
    two_sum(1.0, r_hi, &s, &e1);
    two_sum(s, r2 * 0.5, &s, &e2);
    two_sum(s, s3, &s, &e3);
    double lo = ((e1 + e2) + e3) + ((r2e * 0.5 + s3e) + tail);
    lo = fma(r_lo, 1.0 + r_hi, lo);                  /* exp(r_hi + r_lo) ~ exp(r_hi)(1 + r_lo) */
    double p = s + lo;
    int k = (int)kd;
    if (k > 1000)
        return (p * pow2i(k - 1000)) * pow2i(1000);
    if (k < -1000)
        return (p * pow2i(k + 1000)) * pow2i(-1000);
    return p * pow2i(k);
}

/* Natural logarithm, own implementation shared bit for bit with the GB300 kernels: x = 2^e m with
 * m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(s) with s = (m - 1)/(m + 1) (m - 1 exact by Sterbenz,
 * m + 1 and s carried as double-doubles), the odd series 2 s^3 (1/3 + s^2/5 + ... + s^20/23) for
 * the tail (|s| < 0.172, so 11 terms reach 2^-58 relative), and e ln 2 from the same two-part ln 2
 * as orc_exp.  Errors stay below one ulp; results need not equal libm's. */
double orc_log(double x)
{
    if (x != x)
        return x;
    if (x < 0.0)
        return 0.0 / 0.0;
    if (x == 0.0)
        return -1.0 / 0.0;
    if (x == 1.0 / 0.0)
        return x;
    uint64_t b;
    memcpy(&b, &x, 8);
    int e = 0;
    if ((b >> 52) == 0) {                     /* subnormal: scale into the normal range */
        x = x * 18014398509481984.0;          /* 2^54 */
        memcpy(&b, &x, 8);
        e = -54;
    }
    e += (int)(b >> 52) - 1023;
    uint64_t mb = (b & 0x000fffffffffffffull) | 0x3ff0000000000000ull;
    double m;
    memcpy(&m, &mb, 8);
    if (m > 1.4142135623730951) {
        m = m * 0.5;
        e += 1;
    }
    const double ln2_hi = 6.93147180369123816490e-01, ln2_lo = 1.90821492927058770002e-10;
    double f = m - 1.0;
    double g_hi, g_lo;
    two_sum(m, 1.0, &g_hi, &g_lo);
    double s_hi = f / g_hi;
    double r = fma(-s_hi, g_hi, f) - s_hi * g_lo;
    double s_lo = r / g_hi;
    double z = s_hi * s_hi;
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
    double tail = ((s_hi * z) * q) * 2.0;
    double ed = (double)e;
    double h, l;
    two_sum(ed * ln2_hi, s_hi * 2.0, &h, &l);
    l = l + ((s_lo * 2.0 + tail) + ed * ln2_lo);
    return h + l;
}

/* ================================================================================== */
/* Reference arithmetic order (orc_problem.ref_order = 1)                             */
/* The operation sequence of the reference's AVX2 build without FMA (the reference's   */
/* SUPPORT_CPU_AVX_256_bits=1, SUPPORT_CPU_FMA_EXT=0 with -mno-fma -ffp-contract=off). */
/* ================================================================================== */

/* Dot product in the reference's lane order (LightVectorND::operator& and
 * dotProductForAlignedMemory, dopt/dopt/linalg_vectors/include_internal/LightVector_SIMD_double.h:233-313,
 * :316-380; VectorNDRaw::operator&, VectorND_Raw_SIMD_double.h:253): two Vec4d accumulators, element
 * e < 8 floor(n/8) goes to lane e mod 8 (products rounded, then added); each Vec4d is reduced as
 * (c0 + c2) + (c1 + c3) (horizontal_add, vectorclass/vectorf256.h:1967); the two results are added
 * to 0 in order; the tail e >= 8 floor(n/8) is summed in order from 0 and added last. */
double orc_ref_dot(const double* a, const double* b, size_t n)
{
    double c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    size_t items = n & ~(size_t)7;
    size_t i = 0;
    for (; i < items; i += 8)
        for (int l = 0; l < 8; ++l)
            c[l] = c[l] + a[i + (size_t)l] * b[i + (size_t)l];
    double r0 = (c[0] + c[2]) + (c[1] + c[3]);
    double r1 = (c[4] + c[6]) + (c[5] + c[7]);
    double fin = 0.0;
    fin = fin + r0;
    fin = fin + r1;
    double rest = 0.0;
    for (; i < n; ++i)
        rest = rest + a[i] * b[i];
    return fin + rest;
}

/* Squared L2 norm in the same lane order (vectorL2NormSquare, VectorND_Raw_SIMD_double.h:749-800;
 * LightVectorND::vectorL2NormSquareForAlignedMemory, LightVector_SIMD_double.h:772-830) */
double orc_ref_norm2(const double* a, size_t n)
{
    return orc_ref_dot(a, a, n);
}

/* The vectorclass exp of one SIMD lane (exp_d<Vec4d, 0, 0>, dopt/dopt/3rdparty/vectorclass/
 * vectormath_exp.h:141-230, without FMA: mul_add(a, b, c) = a*b + c, nmul_add(a, b, c) = c - a*b,
 * vectorf256.h:2148-2179): r = round(x log2e) (nearest even), x - r ln2_hi - r ln2_lo, the Taylor
 * polynomial 1/2! .. 1/13! in the grouping of polynomial_13m (vectormath_common.h:311-321), then
 * (z + 1) 2^r.  Lanes outside |x| < 708.39 give 0 / +inf, NaN passes through. */
double orc_exp_vcl(double x0)
{
    if (x0 != x0)
        return x0;
    if (!(fabs(x0) < 708.39))
        return (x0 < 0) ? 0.0 : 1.0 / 0.0;
    const double p2 = 1. / 2., p3 = 1. / 6., p4 = 1. / 24., p5 = 1. / 120., p6 = 1. / 720., p7 = 1. / 5040.;
    const double p8 = 1. / 40320., p9 = 1. / 362880., p10 = 1. / 3628800., p11 = 1. / 39916800.;
    const double p12 = 1. / 479001600., p13 = 1. / 6227020800.;
    const double ln2d_hi = 0.693145751953125, ln2d_lo = 1.42860682030941723212E-6;
    const double log2e = 1.44269504088896340736;
    double r = rint(x0 * log2e);
    double x = x0 - r * ln2d_hi;
    x = x - r * ln2d_lo;
    double x2 = x * x, x4 = x2 * x2, x8 = x4 * x4;
    double hi = (p13 * x + p12) * x4 + ((p11 * x + p10) * x2 + (p9 * x + p8));
    double lo = ((p7 * x + p6) * x2 + (p5 * x + p4)) * x4 + ((p3 * x + p2) * x2 + x);
    double z = hi * x8 + lo;
    return (z + 1.0) * pow2i((int)r);
}

/* Correctly rounded exp (own method, used for the reference's scalar tail, which calls libm exp):
 * x = k ln2 + r with ln2 in three parts (30-bit head, so k*L1 and x - k*L1 are exact), r kept as a
 * double-double; exp(r 2^-10) by its Taylor series to degree 9 in double-double arithmetic, squared
 * ten times; one rounding of hi + lo, then the exact scaling by 2^k.  The double-double error is
 * below 2^-90 relative, so the result is the correctly rounded one for every result in the normal
 * range except inputs within 2^-90 of a rounding boundary.  libm's exp is within 0.51 ulp and equals
 * the correctly rounded value for all but a few inputs in ten thousand (measured on glibc 2.39). */
typedef struct { double hi, lo; } orc_dd;

static inline orc_dd dd_norm(double s, double e)
{
    double t = s + e;
    orc_dd r = {t, e - (t - s)};
    return r;
}

static inline orc_dd dd_add(orc_dd a, orc_dd b)
{
    double s, e;
    two_sum(a.hi, b.hi, &s, &e);
    e = e + (a.lo + b.lo);
    return dd_norm(s, e);
}

static inline orc_dd dd_mul(orc_dd a, orc_dd b)
{
    double p = a.hi * b.hi;
    double e = fma(a.hi, b.hi, -p);
    e = e + (a.hi * b.lo + a.lo * b.hi);
    return dd_norm(p, e);
}

double orc_exp_cr(double x)
{
    if (x != x)
        return x;
    if (x > 709.782712893384)
        return 1.0 / 0.0;
    if (x < -745.1332191019412)
        return 0.0;
    static const double L1 = 0x1.62e42fe8p-1, L2 = 0x1.e8e7bcd5e4f1ep-31, L3 = -0x1.8cff81a12a17ep-85;
    static const double inv_fact[10][2] = {
        {1.0, 0.0}, {1.0, 0.0}, {0x1p-1, 0.0}, {0x1.5555555555555p-3, 0x1.5555555555555p-57},
        {0x1.5555555555555p-5, 0x1.5555555555555p-59}, {0x1.1111111111111p-7, 0x1.1111111111111p-63},
        {0x1.6c16c16c16c17p-10, -0x1.f49f49f49f49fp-65}, {0x1.a01a01a01a01ap-13, 0x1.a01a01a01a01ap-73},
        {0x1.a01a01a01a01ap-16, 0x1.a01a01a01a01ap-76}, {0x1.71de3a556c734p-19, -0x1.c154f8ddc6c00p-73}};
    double kd = rint(x * 0x1.71547652b82fep+0);
    double r1 = x - kd * L1;                      /* exact */
    double p2 = kd * L2;
    double p2e = fma(kd, L2, -p2);
    double s, e;
    two_sum(r1, -p2, &s, &e);
    e = (e - p2e) - kd * L3;
    orc_dd y = dd_norm(s, e);
    y.hi = y.hi * 0x1p-10;
    y.lo = y.lo * 0x1p-10;
    orc_dd t = {inv_fact[9][0], inv_fact[9][1]};
    for (int n = 8; n >= 0; --n) {
        orc_dd c = {inv_fact[n][0], inv_fact[n][1]};
        t = dd_add(dd_mul(t, y), c);
    }
    for (int q = 0; q < 10; ++q)
        t = dd_mul(t, t);
    double p = t.hi + t.lo;
    int k = (int)kd;
    if (k > 1000)
        return (p * pow2i(k - 1000)) * pow2i(1000);
    if (k < -1000)
        return (p * pow2i(k + 1000)) * pow2i(-1000);
    return p * pow2i(k);
}

/* The vectorclass log of one SIMD lane (log_d<Vec4d, 0>, vectormath_exp.h:947-1003, without FMA):
 * x = fraction_2(x1) in [0.5, 1), fe = exponent_f(x1); x <= sqrt(2)/2 is doubled, otherwise fe + 1;
 * x - 1; res = P5(x) x^3 / Q5n(x) (polynomial_5 / polynomial_5n groupings, vectormath_common.h:206-223);
 * res += fe ln2_lo; res += x - 0.5 x^2; res += fe ln2_hi.  Zero gives -inf, +inf itself, negative
 * and NaN inputs NaN; subnormal inputs are outside the reference's use (sigmoid values). */
double orc_log_vcl(double x1)
{
    if (x1 != x1 || x1 < 0.0)
        return 0.0 / 0.0;
    if (x1 == 0.0)
        return -1.0 / 0.0;
    if (x1 == 1.0 / 0.0)
        return x1;
    const double ln2_hi = 0.693359375, ln2_lo = -2.121944400546905827679E-4;
    const double P0 = 7.70838733755885391666E0, P1 = 1.79368678507819816313E1, P2 = 1.44989225341610930846E1;
    const double P3 = 4.70579119878881725854E0, P4 = 4.97494994976747001425E-1, P5 = 1.01875663804580931796E-4;
    const double Q0 = 2.31251620126765340583E1, Q1 = 7.11544750618563894466E1, Q2 = 8.29875266912776603211E1;
    const double Q3 = 4.52279145837532221105E1, Q4 = 1.12873587189167450590E1;
    const double sqrt2_half = 1.41421356237309504880 * 0.5;
    uint64_t b;
    memcpy(&b, &x1, 8);
    uint64_t fb = (b & 0x000FFFFFFFFFFFFFull) | 0x3FE0000000000000ull;
    double x;
    memcpy(&x, &fb, 8);
    double fe = (double)(int64_t)(b >> 52) - 1023.0;
    if (x > sqrt2_half)
        fe = fe + 1.0;
    else
        x = x + x;
    x = x - 1.0;
    double xx2 = x * x, xx4 = xx2 * xx2;
    double px = (P3 * x + P2) * xx2 + ((P5 * x + P4) * xx4 + (P1 * x + P0));
    double x2 = x * x;
    px = px * (x * x2);
    double qx = (Q3 * x + Q2) * xx2 + ((Q4 + x) * xx4 + (Q1 * x + Q0));
    double res = px / qx;
    res = fe * ln2_lo + res;
    res = res + (x - x2 * 0.5);
    res = fe * ln2_hi + res;
    return res;
}

/* margins in the reference's order (the AVX2 specialisation of matrixVectorMultiplyWithPreTranspose,
 * dopt/dopt/linalg_matrices/include/include_internal/MatrixNMD_SIMD_double.h:1256-1430): one Vec4d
 * accumulator, attribute j < 4 floor(d/4) to lane j mod 4 (a_j x_j rounded, then added), reduced as
 * (c0 + c2) + (c1 + c3), then the remaining attributes added one by one in order. */
void orc_margin_ref(const double* atr, int32_t d, int32_t lda, int32_t n, const double* x, double* m)
{
    int32_t cb = d & ~3;
    for (int32_t s = 0; s < n; ++s) {
        const double* a = atr + (size_t)s * lda;
        double c[4] = {0, 0, 0, 0};
        int32_t j = 0;
        for (; j < cb; j += 4)
            for (int l = 0; l < 4; ++l)
                c[l] = c[l] + a[j + l] * x[j + l];
        double acc = (c[0] + c[2]) + (c[1] + c[3]);
        for (; j < d; ++j)
            acc = acc + a[j] * x[j];
        m[s] = acc;
    }
}

/* ||M||_F^2 of a symmetric matrix from its upper part in the reference's order (the AVX2
 * specialisation of frobeniusNormSquareForSymmetricMatrixFromUpPart / frobeniusNormFor...,
 * MatrixNMD_SIMD_double.h:1068-1253): eight lane accumulators shared by all columns; in column j the
 * strictly upper rows i < 8 floor(j/8) go to lane i mod 8, the rows 8 floor(j/8) <= i < j to one
 * running scalar, the diagonal to another; at the end out = (0 + h(c0..c3)) + h(c4..c7) with
 * h(c) = (c0 + c2) + (c1 + c3), out += rest, and the result is (out + out) + diagonal. */
double orc_frob_ref(const double* m, int32_t d, int32_t lda)
{
    double c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    double rest = 0.0, diag = 0.0;
    for (int32_t j = 0; j < d; ++j) {
        const double* col = m + (size_t)j * lda;
        int32_t items = j & ~7;
        int32_t i = 0;
        for (; i < items; i += 8)
            for (int l = 0; l < 8; ++l)
                c[l] = c[l] + col[i + l] * col[i + l];
        for (; i < j; ++i)
            rest = rest + col[i] * col[i];
        diag = diag + col[j] * col[j];
    }
    double out = 0.0;
    out = out + ((c[0] + c[2]) + (c[1] + c[3]));
    out = out + ((c[4] + c[6]) + (c[5] + c[7]));
    out = out + rest;
    return (out + out) + diag;
}

/* elementwiseSigmoid (VectorND_Raw_SIMD_double.h:1596-1650): the SIMD lanes s < 8 floor(n/8) use the
 * vectorclass exp, the tail libm's exp (here: the correctly rounded one) */
void orc_sigmoid_ref(const double* m, int32_t n, double* sig)
{
    int32_t items = n & ~7;
    for (int32_t s = 0; s < n; ++s)
        sig[s] = 1.0 / (1.0 + (s < items ? orc_exp_vcl(-m[s]) : orc_exp_cr(-m[s])));
}

/* logisticUnweightedLossFromMarginSigmoid (VectorND_Raw_SIMD_double.h:1464-1532): lanes c_l -= log
 * (vectorclass log), the two Vec4d reduced and added as in orc_ref_dot, the tail rest -= log (libm;
 * here the own log), (fin + rest) / n; plus lambda/2 ||x||^2 in lane order
 * (evaluateFunction(x, margin, sigmoid), logistic_regression.h:119-123) */
double orc_client_function_ref(const double* sig, int32_t n, const double* x, int32_t d, double lambda)
{
    double c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int32_t items = n & ~7;
    int32_t i = 0;
    for (; i < items; i += 8)
        for (int l = 0; l < 8; ++l)
            c[l] = c[l] - orc_log_vcl(sig[i + l]);
    double r0 = (c[0] + c[2]) + (c[1] + c[3]);
    double r1 = (c[4] + c[6]) + (c[5] + c[7]);
    double fin = 0.0;
    fin = fin + r0;
    fin = fin + r1;
    double rest = 0.0;
    for (; i < n; ++i)
        rest = rest - orc_log(sig[i]);
    double loss = (fin + rest) / (double)n;
    return loss + (lambda * 0.5) * orc_ref_norm2(x, (size_t)d);
}

/* choleskyFactorization<Mat, fill_L_factor_in_lower_part=true, in_input_symmetric=true>
 * (CholeskyFactorization.h:153-272) in its own order: column i, rows j < i:
 * R_ji = (1 / R_jj) (H_ji - R[0:j, i] . R[0:j, j]) with the lane-ordered dot product, mirrored into
 * the lower part; then R_ii = sqrt((H_ii + l) - ||R[0:i, i]||^2) (a negative radicand fails). */
int orc_cholesky_ref(const double* h, int32_t d, int32_t lda, double l, double* ltr)
{
    memset(ltr, 0, (size_t)d * (size_t)lda * sizeof(double));
    for (int32_t i = 0; i < d; ++i) {
        double* ci = ltr + (size_t)i * lda;
        for (int32_t j = 0; j < i; ++j) {
            const double* cj = ltr + (size_t)j * lda;
            double squares = orc_ref_dot(ci, cj, (size_t)j);
            double ljj = cj[j];
            double res = (1.0 / ljj) * (h[(size_t)i * lda + j] - squares);
            ci[j] = res;
            ltr[(size_t)j * lda + i] = res;
        }
        double squares = orc_ref_norm2(ci, (size_t)i);
        double res = (h[(size_t)i * lda + i] + l) - squares;
        if (res < 0) {
            if (res > -0.0)
                res = 0.0;
            else
                return 0;
        }
        ci[i] = sqrt(res);
    }
    return 1;
}

/* forwardSubstitutionWithATranspose then backwardSubstitutionWithATranspose
 * (ElementarySolvers.h:186-224, :71-128) in their own order: y_0 = b_0 / R_00,
 * y_i = (b_i - R[0:i, i] . y[0:i]) / R_ii; x_i = (y_i - L[i+1:d, i] . x[i+1:d]) / R_ii with the
 * lane-ordered dot product over the stored lower column (the mirror of row i of R). */
void orc_solve_chol_ref(const double* ltr, int32_t d, int32_t lda, const double* b, double* x)
{
    double* y = (double*)malloc((size_t)d * sizeof(double));
    y[0] = b[0] / ltr[0];
    for (int32_t i = 1; i < d; ++i)
        y[i] = (b[i] - orc_ref_dot(ltr + (size_t)i * lda, y, (size_t)i)) / ltr[(size_t)i * lda + i];
    for (int32_t i = d - 1; i >= 0; --i) {
        size_t len = (size_t)(d - 1 - i);
        double acc = y[i] - orc_ref_dot(ltr + (size_t)i * lda + i + 1, x + i + 1, len);
        x[i] = acc / ltr[(size_t)i * lda + i];
    }
    free(y);
}

double orc_client_function(const double* sig, int32_t n, const double* x, int32_t d, double lambda)
{
    double* t = (double*)malloc((size_t)(n > 0 ? n : 1) * sizeof(double));
    for (int32_t s = 0; s < n; ++s)
        t[s] = -orc_log(sig[s]);
    double loss = chunked_sum(t, (size_t)n) / (double)n;
    free(t);
    return loss + (lambda * 0.5) * orc_l2sq(x, (size_t)d);
}

/* elementwiseSigmoid, dopt/dopt/linalg_vectors/include_internal/VectorND_Raw_SIMD_double.h:1596-1650 */
void orc_sigmoid(const double* m, int32_t n, double* sig)
{
    for (int32_t s = 0; s < n; ++s)
        sig[s] = 1.0 / (1.0 + orc_exp(-m[s]));
}

/* evaluateGradient(x, margin, sigmoid), :148-161:
 * q_s = (1 - sigma_s) * (-1/n); g = lambda x + sum_s Atr[:,s] q_s (samples in order) */
void orc_gradient(const double* atr, int32_t d, int32_t lda, int32_t n, const double* x,
                  const double* sig, double lambda, double* g)
{
    double inv_m = 1.0 / (double)n;
    double minus_inv_m = -inv_m;
    for (int32_t i = 0; i < d; ++i)
        g[i] = x[i] * lambda;
    for (int32_t s = 0; s < n; ++s) {
        double q = (1.0 - sig[s]) * minus_inv_m;
        const double* col = atr + (size_t)s * lda;
        for (int32_t i = 0; i < d; ++i)
            g[i] += col[i] * q;
    }
}

/* evaluateHessian<true, 4>, :163-547 (algorithm 4 :365-547): per entry (i <= j) the sum over
 * samples in order of u_i * (D_s * v_j), D_s = (1/n) * ((1 - sigma_s) * sigma_s); then the
 * lower triangle is mirrored and lambda is added to the diagonal. */
void orc_hessian(const double* atr, int32_t d, int32_t lda, int32_t n, const double* sig,
                 double lambda, double* h)
{
    double inv_m = 1.0 / (double)n;
    memset(h, 0, (size_t)d * (size_t)lda * sizeof(double));
    for (int32_t s = 0; s < n; ++s) {
        double z1 = 1.0 - sig[s];
        double z2 = z1 * sig[s];
        double d_s = inv_m * z2;
        const double* u = atr + (size_t)s * lda;
        for (int32_t j = 0; j < d; ++j) {
            double vj = d_s * u[j];
            double* col = h + (size_t)j * lda;
            for (int32_t i = 0; i <= j; ++i)
                col[i] += u[i] * vj;
        }
    }
    for (int32_t j = 0; j < d; ++j)
        for (int32_t i = 0; i < j; ++i)
            h[(size_t)i * lda + j] = h[(size_t)j * lda + i];
    for (int32_t j = 0; j < d; ++j)
        h[(size_t)j * lda + j] += lambda;
}

/* ================================================================================== */
/* Option-B solve                                                                     */
/* ================================================================================== */

/* The fixed-order Option-B solve (x = (H + l I)^{-1} b, the reference's choleskyFactorization and
 * triangular solves, CholeskyFactorization.h:153-272 and ElementarySolvers.h:71-224, in an order
 * with a short dependency chain per column pair): a square-root-free block LDL^T factorization,
 * H + l I = L D L^T with L unit lower triangular and D block diagonal, its 2x2 blocks on the column
 * pairs (0,1), (2,3), ... (a 1x1 block last when d is odd), right-looking.  a_ij starts at h_ij
 * (+ l on the diagonal).  Pair (k, k+1) with a = a_kk, b = a_k,k+1, c = a_k+1,k+1:
 *   det = fma(a, c, -(b b)); rejected when a or det is negative (as the reference rejects a
 *   negative radicand); rdet = 1 / det; D^{-1} = [[p, q], [q, r]] with p = c rdet, q = -(b rdet),
 *   r = a rdet; the multipliers of column j > k+1 are l1_j = fma(p, w1_j, q w2_j) and
 *   l2_j = fma(q, w1_j, r w2_j) (w1_j = a_kj, w2_j = a_k+1,j unscaled); every a_ij with
 *   k+1 < i <= j receives a_ij = fma(-l1_i, w1_j, a_ij), then a_ij = fma(-l2_i, w2_j, a_ij).
 * A 1x1 block k: pivot a = a_kk (rejected when negative), inv = 1 / a, l_kj = a_kj inv.
 * ltr's upper triangle receives the multipliers (rows k and k+1 of L^T; 0 between the two rows of a
 * pair), its diagonal p and r (a pair) or the pivot a (1x1), and q goes below the diagonal at
 * (k+1, k).  The GB300 kernel follows this order; the reference's own order is orc_cholesky_ref. */
static int orc_neg(double v) { return v < 0; }

int orc_ldlt(const double* h, int32_t d, int32_t lda, double l, double* ltr)
{
    memset(ltr, 0, (size_t)d * (size_t)lda * sizeof(double));
    for (int32_t j = 0; j < d; ++j)
        for (int32_t i = 0; i <= j; ++i)
            ltr[(size_t)j * lda + i] = (i == j) ? h[(size_t)j * lda + i] + l : h[(size_t)j * lda + i];
#define A_(i, j) ltr[(size_t)(j) * lda + (i)]
    double* w1 = (double*)malloc((size_t)d * sizeof(double));
    double* w2 = (double*)malloc((size_t)d * sizeof(double));
    for (int32_t k = 0; k < d; k += 2) {
        if (k + 1 == d) {
            const double a = A_(k, k);
            if (orc_neg(a)) {
                free(w1);
                free(w2);
                return 0;
            }
            break;          /* nothing right of the last column */
        }
        const double a = A_(k, k), b = A_(k, k + 1), c = A_(k + 1, k + 1);
        if (orc_neg(a)) {
            free(w1);
            free(w2);
            return 0;
        }
        const double det = fma(a, c, -(b * b));
        if (orc_neg(det)) {
            free(w1);
            free(w2);
            return 0;
        }
        const double rdet = 1.0 / det;
        const double p = c * rdet, q = -(b * rdet), r = a * rdet;
        for (int32_t j = k + 2; j < d; ++j) {
            w1[j] = A_(k, j);
            w2[j] = A_(k + 1, j);
            A_(k, j) = fma(p, w1[j], q * w2[j]);
            A_(k + 1, j) = fma(q, w1[j], r * w2[j]);
        }
        for (int32_t j = k + 2; j < d; ++j)
            for (int32_t i = k + 2; i <= j; ++i) {
                double v = fma(-A_(k, i), w1[j], A_(i, j));
                A_(i, j) = fma(-A_(k + 1, i), w2[j], v);
            }
        A_(k, k) = p;
        A_(k + 1, k + 1) = r;
        A_(k, k + 1) = 0.0;
        A_(k + 1, k) = q;
    }
#undef A_
    free(w1);
    free(w2);
    return 1;
}

/* L y = b, z = D^{-1} y, L^T x = z, column-oriented: for each block in order, y_i =
 * fma(-l1_i, y_k, y_i) then fma(-l2_i, y_k+1, y_i) for i > k+1 (a 1x1 block: fma(-l_i, y_k, y_i));
 * z_k = fma(p, y_k, q y_k+1), z_k+1 = fma(q, y_k, r y_k+1) (1x1: z_k = y_k (1 / a)); then
 * x_i = fma(-l_it, x_t, x_i) for t descending and every i < t (unit diagonal, no division; the
 * zero between the rows of a pair takes part like any other entry). */
void orc_solve_ldlt(const double* ltr, int32_t d, int32_t lda, const double* b, double* x)
{
#define A_(i, j) ltr[(size_t)(j) * lda + (i)]
    for (int32_t i = 0; i < d; ++i)
        x[i] = b[i];
    for (int32_t k = 0; k < d; k += 2) {
        if (k + 1 == d) {
            x[k] = x[k] * (1.0 / A_(k, k));
            break;
        }
        const double y1 = x[k], y2 = x[k + 1];
        for (int32_t i = k + 2; i < d; ++i) {
            double v = fma(-A_(k, i), y1, x[i]);
            x[i] = fma(-A_(k + 1, i), y2, v);
        }
        const double p = A_(k, k), q = A_(k + 1, k), r = A_(k + 1, k + 1);
        x[k] = fma(p, y1, q * y2);
        x[k + 1] = fma(q, y1, r * y2);
    }
    for (int32_t t = d - 1; t >= 0; --t) {
        const double xt = x[t];
        for (int32_t i = 0; i < t; ++i)
            x[i] = fma(-A_(i, t), xt, x[i]);
    }
#undef A_
}

/* ================================================================================== */
/* Whole FedNL run                                                                    */
/* dopt/bin_fednl_local/include/TrainLoop.h:103-1863 with --debug forcesequpdate      */
/* ================================================================================== */

typedef struct {
    double* atr;        /* d x n, lda */
    int32_t n;
    double* shift;      /* d x lda */
    double* grad;       /* d */
    double lk;
    uint32_t rng;       /* RandK / RandSeqK generator (seed_base + c) */
    uint32_t draws;     /* RandK-Philox: draws made so far */
    uint32_t* msg_idx;  /* flat indices */
    double* msg_val;    /* values exactly as the master adds them to H */
    int32_t msg_count;
    double fi;          /* f_i at the round's starting iterate (tracking / line search) */
    double* dir;        /* FedNL-PP: localGradient = x Lk + shift x - grad (d) */
    double* ddir;       /* FedNL-PP: the difference last sent to the master (d) */
    double dlk;         /* FedNL-PP: the Lk difference last sent */
    int32_t icpt;       /* the last attribute is 1 in every sample (an intercept column) */
} orc_client;

struct orc_state {
    orc_problem p;
    int32_t blocked;    /* {0,1} features in the fixed order: attribute sums in 64-sample words */
    size_t U;
    uint32_t* upper;
    orc_client* clients;
    uint32_t* worker_rng;  /* TopLEK thread_local generator per logical worker */
    double* x;
    double* H;             /* master, d x lda, upper current */
    double* g;
    double l;
    double* ltr;
    double prescale;       /* alpha / n (TrainLoop.h:531) */
    int32_t k_eff;
    /* FedNL-PP */
    double* g_prev;        /* prev_global_gradient_estimation */
    double l_prev;         /* prev_global_Li_fednl */
    double* true_grad;     /* computeFullGradient at the round's starting iterate */
    uint32_t sampler;      /* clientSampler (RandomGenIntegerLinear) */
    uint32_t* perm;        /* [n] the sampler's permutation buffer */
    uint8_t* is_sel;       /* [n] selected this round */
    int32_t* selected;     /* [tau] ascending */
    int32_t tau;
    double f_k;            /* f at the round's starting iterate */
    int32_t ls_steps;      /* function evaluations of the last line search */
};

/* The GPU engine's fixed order for the attribute sums of {0,1} features (its default feature format
 * takes the bit-packed kernels for them): acc + the terms of the samples holding attribute i, taken
 * in 64-sample words; a word's terms are summed in sample order (its first term exactly) and the
 * word sums are added to acc in word order.  signed_terms: the term is column i of Atr (b_s = +-1)
 * times v_s, else v_s. */
static double blocked_attr_sum(const double* atr, int32_t lda, int32_t n, int32_t i, const double* v,
                               int32_t signed_terms, double acc)
{
    for (int32_t w0 = 0; w0 < n; w0 += 64) {
        int32_t w1 = w0 + 64 < n ? w0 + 64 : n;
        int32_t have = 0;
        double part = 0.0;
        for (int32_t s = w0; s < w1; ++s) {
            double a = atr[(size_t)s * lda + i];
            if (a == 0.0)
                continue;
            double t = signed_terms ? a * v[s] : v[s];
            part = have ? part + t : t;
            have = 1;
        }
        if (have)
            acc = acc + part;
    }
    return acc;
}

/* Gradient (grad) and Hessian (h) of one client at the sigmoid values sig: orc_gradient and
 * orc_hessian, whose per-entry sample order the reference fixes; in the blocked order (S->blocked)
 * the attribute sums -- the gradient, the Hessian diagonal and, when the client's last attribute
 * is an intercept, the Hessian's last column -- are taken by blocked_attr_sum. */
static void client_grad_hess(const orc_state* S, const orc_client* C, const double* sig, double* grad, double* h)
{
    const orc_problem* P = &S->p;
    int32_t d = P->d, lda = P->lda, n = C->n;
    if (grad)
        orc_gradient(C->atr, d, lda, n, S->x, sig, P->lambda, grad);
    if (h)
        orc_hessian(C->atr, d, lda, n, sig, P->lambda, h);
    if (!S->blocked)
        return;
    double inv_m = 1.0 / (double)n;
    double minus_inv_m = -inv_m;
    double* q = (double*)malloc((size_t)n * sizeof(double));
    double* dv = (double*)malloc((size_t)n * sizeof(double));
    for (int32_t s = 0; s < n; ++s) {
        double z1 = 1.0 - sig[s];
        q[s] = z1 * minus_inv_m;              /* orc_gradient's q_s */
        dv[s] = inv_m * (z1 * sig[s]);        /* orc_hessian's D_s */
    }
    for (int32_t i = 0; i < d; ++i) {
        if (grad)
            grad[i] = blocked_attr_sum(C->atr, lda, n, i, q, 1, S->x[i] * P->lambda);
        if (h) {
            double ds = blocked_attr_sum(C->atr, lda, n, i, dv, 0, 0.0);
            h[(size_t)i * lda + i] = ds + P->lambda;
            if (C->icpt && i < d - 1) {
                h[(size_t)(d - 1) * lda + i] = ds;
                h[(size_t)i * lda + (d - 1)] = ds;
            }
        }
    }
    free(q);
    free(dv);
}

/* Worker side of one client, first half: the compressor's index draw, margins, sigmoid, gradient,
 * Hessian and difference (LocalWorkerForFedNL_*.h, bodies of the per-context loops).  Returns
 * ||diff||_F^2. */
/* margins and sigmoid of one client at x in the selected arithmetic order */
static void margin_sigmoid(const orc_problem* P, const double* atr, int32_t n, const double* x, double* m,
                           double* sig)
{
    if (P->ref_order) {
        orc_margin_ref(atr, P->d, P->lda, n, x, m);
        orc_sigmoid_ref(m, n, sig);
    } else {
        orc_margin(atr, P->d, P->lda, n, x, m);
        orc_sigmoid(m, n, sig);
    }
}

/* mean of per-client scalars: the fixed chunked order, or the reference's running sum in client
 * order times 1/n (function_aggregation, TrainLoop.h:1511-1541) */
static double client_mean(const orc_problem* P, const double* v, int32_t nc)
{
    double inv_n = 1.0 / (double)nc;
    if (!P->ref_order)
        return chunked_sum(v, (size_t)nc) * inv_n;
    double s = 0.0;
    for (int32_t c = 0; c < nc; ++c)
        s = s + v[c];
    return s * inv_n;
}

static double client_prepare(orc_state* S, int32_t c, double* hbuf, double* diff, double* mtmp, double* stmp)
{
    const orc_problem* P = &S->p;
    orc_client* C = &S->clients[c];
    int32_t d = P->d, lda = P->lda, n = C->n;
    size_t full = (size_t)d * (size_t)lda;
    size_t U = S->U;

    /* RandK / RandSeqK draw their indices before the round starts (RandK.h:46-62, RandSeqK.h:46-62;
     * FedNL-PP: only when the client is selected, bin_fednl_local_pp/.../RandSeqK.h:90-110) */
    if (P->compressor == ORC_RANDK)
        orc_randk(&C->rng, S->k_eff, U, S->upper, C->msg_idx);
    else if (P->compressor == ORC_RANDSEQK)
        orc_randseqk(&C->rng, S->k_eff, U, S->upper, C->msg_idx);
    else if (P->compressor == ORC_RANDK_PHILOX)
        orc_randk_philox(P->seed_base, (uint32_t)c, C->draws++, S->k_eff, U, S->upper, C->msg_idx);

    margin_sigmoid(P, C->atr, n, S->x, mtmp, stmp);
    if (P->line_search || P->track_f)      /* "Put fi" (TopK.h:132-137) */
        C->fi = P->ref_order ? orc_client_function_ref(stmp, n, S->x, d, P->lambda)
                             : orc_client_function(stmp, n, S->x, d, P->lambda);
    client_grad_hess(S, C, stmp, C->grad, hbuf);
    for (size_t t = 0; t < full; ++t)           /* difference = H_i - shift_i (TopK.h:70-71) */
        diff[t] = hbuf[t] - C->shift[t];
    return P->ref_order ? orc_frob_ref(diff, d, lda) : orc_frob_sym(diff, d, lda);
}

/* Worker side, second half: compression, message and shift update (TopK.h:80-129, TopLEK.h,
 * RandK.h:86-162, Identical.h:80-94, Natural.h:79-147; the FedNL-PP workers are the same) */
static void client_compress(orc_state* S, int32_t c, uint32_t* toplek_rng, const double* diff, double frob_sq)
{
    const orc_problem* P = &S->p;
    orc_client* C = &S->clients[c];
    int32_t d = P->d, lda = P->lda;
    size_t U = S->U;
    double alpha = P->alpha, pre = S->prescale;
    int32_t k = S->k_eff;

    if (P->compressor == ORC_TOPK || P->compressor == ORC_TOPLEK) {
        int32_t cnt;
        if (P->compressor == ORC_TOPK) {
            cnt = orc_topk(diff, k, U, S->upper, C->msg_idx);
        } else {
            double delta = (double)k * (1.0 / (double)U);   /* TopLEK.h:205, :244 */
            cnt = P->ref_order ? orc_toplek_ref(diff, lda, k, U, S->upper, delta, frob_sq, toplek_rng, C->msg_idx)
                               : orc_toplek(diff, lda, k, U, S->upper, delta, frob_sq, toplek_rng, C->msg_idx);
        }
        C->msg_count = cnt;
        for (int32_t t = 0; t < cnt; ++t) {     /* TopK.h:94-129 */
            uint32_t idx = C->msg_idx[t];
            double item = diff[idx];
            C->msg_val[t] = item * pre;
            uint32_t jc = idx / (uint32_t)lda, ir = idx - jc * (uint32_t)lda;
            C->shift[idx] += alpha * item;
            if (ir != jc)
                C->shift[(size_t)ir * lda + jc] += alpha * item;
        }
    } else if (P->compressor == ORC_RANDK || P->compressor == ORC_RANDSEQK || P->compressor == ORC_RANDK_PHILOX) {
        double mult = (double)U / (double)k;    /* RandK.h:90 */
        C->msg_count = k;
        for (int32_t t = 0; t < k; ++t) {       /* RandK.h:127-162 */
            uint32_t idx = C->msg_idx[t];
            double item = diff[idx] * mult;
            C->msg_val[t] = item * pre;
            uint32_t jc = idx / (uint32_t)lda, ir = idx - jc * (uint32_t)lda;
            C->shift[idx] += alpha * item;
            if (ir != jc)
                C->shift[(size_t)ir * lda + jc] += alpha * item;
        }
    } else if (P->compressor == ORC_IDENTITY) {
        /* Identical.h:80-94: message = diff * preScale over the upper part; shift += alpha * sym(diff) */
        C->msg_count = (int32_t)U;
        for (size_t t = 0; t < U; ++t) {
            C->msg_idx[t] = S->upper[t];
            C->msg_val[t] = diff[S->upper[t]] * pre;
        }
        for (int32_t j = 0; j < d; ++j)
            for (int32_t i = 0; i <= j; ++i) {
                double item = diff[(size_t)j * lda + i];
                double upd = alpha * item;
                C->shift[(size_t)j * lda + i] += upd;
                if (i != j)
                    C->shift[(size_t)i * lda + j] += upd;
            }
    } else { /* ORC_NATURAL, Natural.h:79-147: master adds preScale * trunc(diff) (TrainLoop.h:1169-1196) */
        C->msg_count = (int32_t)U;
        for (size_t t = 0; t < U; ++t) {
            C->msg_idx[t] = S->upper[t];
            C->msg_val[t] = pre * orc_natural(diff[S->upper[t]]);
        }
        for (int32_t j = 0; j < d; ++j)         /* learningHessian += alpha * trunc(diff), full matrix */
            for (int32_t i = 0; i < d; ++i) {
                size_t t = (size_t)j * lda + i;
                C->shift[t] += alpha * orc_natural(diff[t]);
            }
    }
}

/* FedNL: Lk = ||diff||_F before the update (TopK.h:74-78) */
static void client_round(orc_state* S, int32_t c, uint32_t* toplek_rng, double* hbuf, double* diff,
                         double* mtmp, double* stmp)
{
    double frob_sq = client_prepare(S, c, hbuf, diff, mtmp, stmp);
    S->clients[c].lk = sqrt(frob_sq);
    client_compress(S, c, toplek_rng, diff, frob_sq);
}

/* y = M x for a full d x lda matrix, columns swept in order (MatrixNMD::matrixVectorMultiply,
 * MatrixNMD.h:1299-1325): y_i = ((0 + m_i0 x_0) + m_i1 x_1) + ... */
static void matvec_cols(const double* m, int32_t d, int32_t lda, const double* x, double* y)
{
    for (int32_t i = 0; i < d; ++i)
        y[i] = 0.0;
    for (int32_t j = 0; j < d; ++j) {
        double xj = x[j];
        const double* col = m + (size_t)j * lda;
        for (int32_t i = 0; i < d; ++i)
            y[i] += col[i] * xj;
    }
}

/* FedNL-PP worker (bin_fednl_local_pp/include/LocalWorkerForFedNL_*.h, e.g. RandSeqK.h:90-190):
 * the same compression and shift update, then Lk = ||shift - H_i||_F after the update (sent as a
 * difference) and the direction dir = x Lk + shift x - grad (sent as a difference). */
static void client_round_pp(orc_state* S, int32_t c, uint32_t* toplek_rng, double* hbuf, double* diff,
                            double* mtmp, double* stmp)
{
    const orc_problem* P = &S->p;
    orc_client* C = &S->clients[c];
    int32_t d = P->d, lda = P->lda;
    size_t full = (size_t)d * (size_t)lda;
    double frob_sq = client_prepare(S, c, hbuf, diff, mtmp, stmp);
    client_compress(S, c, toplek_rng, diff, frob_sq);
    for (size_t t = 0; t < full; ++t)
        diff[t] = C->shift[t] - hbuf[t];
    double lk_new = sqrt(P->ref_order ? orc_frob_ref(diff, d, lda) : orc_frob_sym(diff, d, lda));
    C->dlk = lk_new - C->lk;
    C->lk = lk_new;
    matvec_cols(C->shift, d, lda, S->x, mtmp);
    for (int32_t i = 0; i < d; ++i) {
        double dir = (S->x[i] * C->lk + mtmp[i]) - C->grad[i];
        C->ddir[i] = dir - C->dir[i];
        C->dir[i] = dir;
    }
}

typedef struct {
    orc_state* S;
    int32_t tid, nthreads;
} orc_job;

static void* client_phase_thread(void* arg)
{
    orc_job* J = (orc_job*)arg;
    orc_state* S = J->S;
    int32_t d = S->p.d, lda = S->p.lda;
    size_t full = (size_t)d * (size_t)lda;
    int32_t nmax = d;                           /* the sample buffers also hold d-vectors */
    for (int32_t c = 0; c < S->p.n_clients; ++c)
        if (S->clients[c].n > nmax)
            nmax = S->clients[c].n;
    double* hbuf = (double*)malloc(full * sizeof(double));
    double* diff = (double*)malloc(full * sizeof(double));
    double* mtmp = (double*)malloc((size_t)nmax * sizeof(double));
    double* stmp = (double*)malloc((size_t)nmax * sizeof(double));
    int32_t W = S->p.workers;
    /* logical workers w = tid, tid + nthreads, ...; each processes its clients c = w, w + W, ... in order
     * (static round-robin distribution, TrainLoop.h:664-686) */
    for (int32_t w = J->tid; w < W; w += J->nthreads)
        for (int32_t c = w; c < S->p.n_clients; c += W) {
            if (!S->p.pp)
                client_round(S, c, &S->worker_rng[w], hbuf, diff, mtmp, stmp);
            else if (S->is_sel[c])                 /* clientHasBeenSelected, UsedTypes.h:169-182 */
                client_round_pp(S, c, &S->worker_rng[w], hbuf, diff, mtmp, stmp);
        }
    free(hbuf);
    free(diff);
    free(mtmp);
    free(stmp);
    return NULL;
}

orc_state* orc_create(const orc_problem* p, const double* x0)
{
    orc_state* S = (orc_state*)calloc(1, sizeof(orc_state));
    S->p = *p;
    int32_t d = p->d, lda = p->lda, nc = p->n_clients;
    if (S->p.workers > nc)                      /* TrainLoop.h:194-199 */
        S->p.workers = nc;
    if (S->p.workers < 1)
        S->p.workers = 1;
    if (S->p.threads < 1 || S->p.threads > S->p.workers)
        S->p.threads = S->p.workers;
    size_t full = (size_t)d * (size_t)lda;
    S->U = orc_upper_count(d);
    S->upper = (uint32_t*)malloc(S->U * sizeof(uint32_t));
    orc_upper_indices(d, lda, S->upper);
    S->k_eff = (p->compressor == ORC_IDENTITY || p->compressor == ORC_NATURAL) ? (int32_t)S->U : p->k;
    {
        size_t tot = 0;
        for (int32_t c = 0; c < nc; ++c)
            tot += (size_t)p->n_samples[c];
        S->blocked = !p->ref_order;
        for (size_t t = 0; S->blocked && t < tot * (size_t)d; ++t)
            if (p->features[t] != 0.0 && p->features[t] != 1.0)
                S->blocked = 0;
    }
    S->prescale = (1.0 / (double)nc) * p->alpha;
    S->x = (double*)malloc((size_t)d * sizeof(double));
    memcpy(S->x, x0, (size_t)d * sizeof(double));
    S->H = (double*)calloc(full, sizeof(double));
    S->ltr = (double*)calloc(full, sizeof(double));
    S->g = (double*)calloc((size_t)d, sizeof(double));
    S->worker_rng = (uint32_t*)malloc((size_t)S->p.workers * sizeof(uint32_t));
    for (int32_t w = 0; w < S->p.workers; ++w)
        S->worker_rng[w] = p->toplek_seed;
    S->clients = (orc_client*)calloc((size_t)nc, sizeof(orc_client));

    size_t msg_cap = S->U;
    size_t off = 0;
    int32_t nmax = d;
    for (int32_t c = 0; c < nc; ++c)
        if (p->n_samples[c] > nmax)
            nmax = p->n_samples[c];
    double* mtmp = (double*)malloc((size_t)nmax * sizeof(double));
    double* stmp = (double*)malloc((size_t)nmax * sizeof(double));
    for (int32_t c = 0; c < nc; ++c) {
        orc_client* C = &S->clients[c];
        int32_t n = p->n_samples[c];
        C->n = n;
        /* L2RegulirizeLogisticRegression ctor stores column s = b_s * a_s (logistic_regression.h:26-76) */
        C->atr = (double*)calloc((size_t)n * (size_t)lda, sizeof(double));
        for (int32_t s = 0; s < n; ++s) {
            double b = p->labels[off + s];
            const double* a = p->features + (off + (size_t)s) * (size_t)d;
            double* col = C->atr + (size_t)s * lda;
            for (int32_t i = 0; i < d; ++i)
                col[i] = (b == 1.0) ? a[i] : a[i] * -1.0;
        }
        C->icpt = 1;
        for (int32_t s = 0; s < n; ++s)
            if (p->features[(off + (size_t)s) * (size_t)d + (size_t)(d - 1)] != 1.0)
                C->icpt = 0;
        off += (size_t)n;
        C->shift = (double*)malloc(full * sizeof(double));
        C->grad = (double*)calloc((size_t)d, sizeof(double));
        C->msg_idx = (uint32_t*)malloc(msg_cap * sizeof(uint32_t));
        C->msg_val = (double*)malloc(msg_cap * sizeof(double));
        C->rng = p->seed_base + (uint32_t)c;    /* TrainLoop.h:632 */
        /* learningHessian = H_i(x0); H += learningHessian (TrainLoop.h:639-643) */
        margin_sigmoid(p, C->atr, n, S->x, mtmp, stmp);
        client_grad_hess(S, C, stmp, NULL, C->shift);
        for (size_t t = 0; t < full; ++t)
            S->H[t] += C->shift[t];
        if (p->pp) {
            /* FedNL-PP init (bin_fednl_local_pp/.../LocalWorkerForFedNL_RandSeqK.h:22-31): Lk = 0,
             * localGradient = shift x0 - grad(x0) */
            C->dir = (double*)calloc((size_t)d, sizeof(double));
            C->ddir = (double*)calloc((size_t)d, sizeof(double));
            client_grad_hess(S, C, stmp, C->grad, NULL);
            matvec_cols(C->shift, d, lda, S->x, mtmp);
            for (int32_t i = 0; i < d; ++i)
                C->dir[i] = mtmp[i] - C->grad[i];
            C->lk = 0.0;
        }
    }
    free(mtmp);
    free(stmp);
    double inv_n = 1.0 / (double)nc;
    for (size_t t = 0; t < full; ++t)           /* H *= 1/n (TrainLoop.h:732-735) */
        S->H[t] *= inv_n;
    if (p->pp) {
        /* master (bin_fednl_local_pp/include/TrainLoop.h:1064-1080): H, g_prev and l_prev are the
         * client means in client order */
        S->g_prev = (double*)calloc((size_t)d, sizeof(double));
        S->true_grad = (double*)calloc((size_t)d, sizeof(double));
        for (int32_t c = 0; c < nc; ++c) {
            for (int32_t i = 0; i < d; ++i)
                S->g_prev[i] += S->clients[c].dir[i];
            S->l_prev += S->clients[c].lk;
        }
        for (int32_t i = 0; i < d; ++i)
            S->g_prev[i] *= inv_n;
        S->l_prev *= inv_n;
        S->tau = p->clients_per_round;
        if (S->tau < 1 || S->tau > nc)
            S->tau = nc;
        S->sampler = p->client_seed;
        S->perm = (uint32_t*)malloc((size_t)nc * sizeof(uint32_t));
        S->is_sel = (uint8_t*)calloc((size_t)nc, 1);
        S->selected = (int32_t*)malloc((size_t)S->tau * sizeof(int32_t));
    }
    return S;
}

void orc_destroy(orc_state* S)
{
    if (!S)
        return;
    for (int32_t c = 0; c < S->p.n_clients; ++c) {
        orc_client* C = &S->clients[c];
        free(C->atr);
        free(C->shift);
        free(C->grad);
        free(C->msg_idx);
        free(C->msg_val);
        free(C->dir);
        free(C->ddir);
    }
    free(S->g_prev);
    free(S->true_grad);
    free(S->perm);
    free(S->is_sel);
    free(S->selected);
    free(S->clients);
    free(S->upper);
    free(S->worker_rng);
    free(S->x);
    free(S->H);
    free(S->ltr);
    free(S->g);
    free(S);
}

static int orc_round_pp_master(orc_state* S, double* grad_norm);

/* f(x) = mean of the clients' objectives at x (clients' sums in the fixed chunked order) */
static double objective_at(orc_state* S, const double* x)
{
    const orc_problem* P = &S->p;
    int32_t d = P->d, nc = P->n_clients;
    int32_t nmax = 1;
    for (int32_t c = 0; c < nc; ++c)
        if (S->clients[c].n > nmax)
            nmax = S->clients[c].n;
    double* mtmp = (double*)malloc((size_t)nmax * sizeof(double));
    double* stmp = (double*)malloc((size_t)nmax * sizeof(double));
    double* fs = (double*)malloc((size_t)nc * sizeof(double));
    for (int32_t c = 0; c < nc; ++c) {
        orc_client* C = &S->clients[c];
        margin_sigmoid(P, C->atr, C->n, x, mtmp, stmp);
        fs[c] = P->ref_order ? orc_client_function_ref(stmp, C->n, x, d, P->lambda)
                             : orc_client_function(stmp, C->n, x, d, P->lambda);
    }
    double f = client_mean(P, fs, nc);
    free(mtmp);
    free(stmp);
    free(fs);
    return f;
}

/* FedNL-LS backtracking (TrainLoop.h:1543-1640): t = 1; x = x_k - t dx until
 * f(x) <= f(x_k) + (c t) (-(dx . g)), t *= gamma after each failure, at most ls_max_steps
 * evaluations; the last trial point stays when none passes.  The dot product uses the chunked
 * order. */
static void orc_line_search(orc_state* S, const double* dx)
{
    const orc_problem* P = &S->p;
    int32_t d = P->d;
    double* t_dg = (double*)malloc((size_t)d * sizeof(double));
    double* xprev = (double*)malloc((size_t)d * sizeof(double));
    for (int32_t i = 0; i < d; ++i) {
        t_dg[i] = dx[i] * S->g[i];
        xprev[i] = S->x[i];
    }
    double dxg = P->ref_order ? -orc_ref_dot(dx, S->g, (size_t)d) : -chunked_sum(t_dg, (size_t)d);
    double t = 1.0;
    for (int32_t it = 0; it < P->ls_max_steps; ++it) {
        for (int32_t i = 0; i < d; ++i)
            S->x[i] = xprev[i] - t * dx[i];
        double fr = objective_at(S, S->x);
        S->ls_steps = it + 1;
        if (fr <= S->f_k + (P->ls_c * t) * dxg)
            break;
        t = t * P->ls_gamma;
    }
    free(t_dg);
    free(xprev);
}
static void pp_select_and_track(orc_state* S);

int orc_round(orc_state* S, double* grad_norm)
{
    const orc_problem* P = &S->p;
    int32_t d = P->d, lda = P->lda, nc = P->n_clients;
    int32_t T = S->p.threads;
    if (P->pp)
        pp_select_and_track(S);

    /* client phase */
    pthread_t* th = (pthread_t*)malloc((size_t)T * sizeof(pthread_t));
    orc_job* jobs = (orc_job*)malloc((size_t)T * sizeof(orc_job));
    for (int32_t t = 0; t < T; ++t) {
        jobs[t].S = S;
        jobs[t].tid = t;
        jobs[t].nthreads = T;
    }
    if (T == 1) {
        client_phase_thread(&jobs[0]);
    } else {
        for (int32_t t = 0; t < T; ++t)
            pthread_create(&th[t], NULL, client_phase_thread, &jobs[t]);
        for (int32_t t = 0; t < T; ++t)
            pthread_join(th[t], NULL);
    }
    free(th);
    free(jobs);
    if (P->pp)
        return orc_round_pp_master(S, grad_norm);

    /* master phase, clients merged in order (TrainLoop.h:1092-1334 with forcesequpdate) */
    double inv_n = 1.0 / (double)nc;
    for (int32_t i = 0; i < d; ++i)
        S->g[i] = 0.0;
    double l = 0.0;
    for (int32_t c = 0; c < nc; ++c) {
        orc_client* C = &S->clients[c];
        for (int32_t i = 0; i < d; ++i)
            S->g[i] += C->grad[i];
        for (int32_t t = 0; t < C->msg_count; ++t)
            S->H[C->msg_idx[t]] += C->msg_val[t];
        l += C->lk;
    }
    for (int32_t i = 0; i < d; ++i)
        S->g[i] *= inv_n;
    l *= inv_n;
    S->l = l;

    /* Option B: chol(H + l I), two triangular solves, x -= dx (TrainLoop.h:1431-1508); Option A
     * regularises by mu = lambda instead (:1383-1430, computeMuStrongConvexity) */
    double* dx = (double*)malloc((size_t)d * sizeof(double));
    int ok = P->ref_order ? orc_cholesky_ref(S->H, d, lda, P->option_a ? P->lambda : l, S->ltr)
                          : orc_ldlt(S->H, d, lda, P->option_a ? P->lambda : l, S->ltr);
    S->ls_steps = 0;
    if (P->line_search || P->track_f) {       /* function_aggregation (TrainLoop.h:1511-1541) */
        double* fs = (double*)malloc((size_t)nc * sizeof(double));
        for (int32_t c = 0; c < nc; ++c)
            fs[c] = S->clients[c].fi;
        S->f_k = client_mean(P, fs, nc);
        free(fs);
    }
    if (ok) {
        if (P->ref_order)
            orc_solve_chol_ref(S->ltr, d, lda, S->g, dx);
        else
            orc_solve_ldlt(S->ltr, d, lda, S->g, dx);
        if (!P->line_search) {
            for (int32_t i = 0; i < d; ++i)
                S->x[i] -= dx[i];
        } else {
            orc_line_search(S, dx);
        }
    }
    free(dx);
    if (grad_norm) {
        double gs = 0.0;
        if (P->ref_order) {
            gs = orc_ref_norm2(S->g, (size_t)d);
        } else {
            for (int32_t i = 0; i < d; ++i)
                gs += S->g[i] * S->g[i];
        }
        *grad_norm = sqrt(gs);
    }
    return ok ? 0 : -1;
}

/* FedNL-PP round start (bin_fednl_local_pp/include/TrainLoop.h:1150-1166): the sampler shuffles a
 * fresh 0..n-1 (partial, tau steps), then the true gradient is the mean of every client's gradient
 * at the current iterate (computeFullGradient, :117-129: sum over clients, then / n).  The client
 * sum is restated in a fixed blocked order shared with the GPU: in-order sums over blocks of 32
 * consecutive clients, then the block sums in order (a few ulps from the reference's running sum;
 * the value is only reported). */
static void pp_select_and_track(orc_state* S)
{
    const orc_problem* P = &S->p;
    int32_t d = P->d, lda = P->lda, nc = P->n_clients;
    for (int32_t c = 0; c < nc; ++c) {
        S->perm[c] = (uint32_t)c;
        S->is_sel[c] = 0;
    }
    orc_shuffle_partial(S->perm, (size_t)nc, (size_t)S->tau, &S->sampler);
    for (int32_t t = 0; t < S->tau; ++t)
        S->is_sel[S->perm[t]] = 1;
    int32_t w = 0;
    for (int32_t c = 0; c < nc; ++c)
        if (S->is_sel[c])
            S->selected[w++] = c;
    int32_t nmax = 1;
    for (int32_t c = 0; c < nc; ++c)
        if (S->clients[c].n > nmax)
            nmax = S->clients[c].n;
    double* mtmp = (double*)malloc((size_t)nmax * sizeof(double));
    double* stmp = (double*)malloc((size_t)nmax * sizeof(double));
    double* gtmp = (double*)malloc((size_t)d * sizeof(double));
    double* bsum = (double*)calloc((size_t)d, sizeof(double));
    for (int32_t i = 0; i < d; ++i)
        S->true_grad[i] = 0.0;
    for (int32_t c = 0; c < nc; ++c) {
        orc_client* C = &S->clients[c];
        orc_margin(C->atr, d, lda, C->n, S->x, mtmp);
        orc_sigmoid(mtmp, C->n, stmp);
        client_grad_hess(S, C, stmp, gtmp, NULL);
        for (int32_t i = 0; i < d; ++i)
            bsum[i] = (c % 32 == 0) ? gtmp[i] : bsum[i] + gtmp[i];
        if (c % 32 == 31 || c == nc - 1)
            for (int32_t i = 0; i < d; ++i)
                S->true_grad[i] = (c < 32) ? bsum[i] : S->true_grad[i] + bsum[i];
    }
    for (int32_t i = 0; i < d; ++i)
        S->true_grad[i] /= (double)nc;
    free(bsum);
    free(mtmp);
    free(stmp);
    free(gtmp);
}

/* FedNL-PP master (bin_fednl_local_pp/include/TrainLoop.h:1168-1560 with forcesequpdate): the
 * selected clients' direction and Lk differences and Hessian messages are merged in client order;
 * g = sum(ddir) / n + g_prev, l = sum(dLk) / n + l_prev; x = (H + l I)^-1 g by Cholesky. */
static int orc_round_pp_master(orc_state* S, double* grad_norm)
{
    const orc_problem* P = &S->p;
    int32_t d = P->d, lda = P->lda;
    double inv_n = 1.0 / (double)P->n_clients;
    for (int32_t i = 0; i < d; ++i)
        S->g[i] = 0.0;
    double l = 0.0;
    for (int32_t t = 0; t < S->tau; ++t) {
        orc_client* C = &S->clients[S->selected[t]];
        for (int32_t i = 0; i < d; ++i)
            S->g[i] += C->ddir[i];
        for (int32_t q = 0; q < C->msg_count; ++q)
            S->H[C->msg_idx[q]] += C->msg_val[q];
        l += C->dlk;
    }
    for (int32_t i = 0; i < d; ++i) {
        S->g[i] = S->g[i] * inv_n + S->g_prev[i];
        S->g_prev[i] = S->g[i];
    }
    l = l * inv_n + S->l_prev;
    S->l_prev = l;
    S->l = l;
    int ok = orc_ldlt(S->H, d, lda, l, S->ltr);
    if (ok)
        orc_solve_ldlt(S->ltr, d, lda, S->g, S->x);
    if (grad_norm) {
        double gs = 0.0;
        for (int32_t i = 0; i < d; ++i)
            gs += S->true_grad[i] * S->true_grad[i];
        *grad_norm = sqrt(gs);
    }
    return ok ? 0 : -1;
}

double orc_get_f(const orc_state* S) { return S->f_k; }
int32_t orc_get_ls_steps(const orc_state* S) { return S->ls_steps; }

void orc_get_true_grad(const orc_state* S, double* g)
{
    if (S->true_grad)
        memcpy(g, S->true_grad, (size_t)S->p.d * sizeof(double));
}
int32_t orc_get_selected(const orc_state* S, int32_t* out)
{
    if (!S->selected)
        return 0;
    memcpy(out, S->selected, (size_t)S->tau * sizeof(int32_t));
    return S->tau;
}
void orc_get_dir(const orc_state* S, int32_t c, double* dir, double* ddir)
{
    const orc_client* C = &S->clients[c];
    if (C->dir && dir)
        memcpy(dir, C->dir, (size_t)S->p.d * sizeof(double));
    if (C->ddir && ddir)
        memcpy(ddir, C->ddir, (size_t)S->p.d * sizeof(double));
}

void orc_get_x(const orc_state* S, double* x) { memcpy(x, S->x, (size_t)S->p.d * sizeof(double)); }
void orc_get_H(const orc_state* S, double* h)
{
    memcpy(h, S->H, (size_t)S->p.d * (size_t)S->p.lda * sizeof(double));
}
void orc_get_shift(const orc_state* S, int32_t c, double* sh)
{
    memcpy(sh, S->clients[c].shift, (size_t)S->p.d * (size_t)S->p.lda * sizeof(double));
}
double orc_get_l(const orc_state* S) { return S->l; }
void orc_get_grad(const orc_state* S, double* g) { memcpy(g, S->g, (size_t)S->p.d * sizeof(double)); }
int32_t orc_get_message(const orc_state* S, int32_t c, uint32_t* idx, double* val)
{
    const orc_client* C = &S->clients[c];
    if (idx)
        memcpy(idx, C->msg_idx, (size_t)C->msg_count * sizeof(uint32_t));
    if (val)
        memcpy(val, C->msg_val, (size_t)C->msg_count * sizeof(double));
    return C->msg_count;
}
double orc_get_lk(const orc_state* S, int32_t c) { return S->clients[c].lk; }
