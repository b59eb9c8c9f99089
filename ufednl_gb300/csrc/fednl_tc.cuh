// fednl_tc.cuh -- tensor-core (tcgen05) kernels of the mixed-precision round, sm_103a.
//
// The client Hessian of the L2-logistic objective is H_i = sum_s D_s a_s a_s^T + lambda I
// (logistic_regression.h:163-547).  In the mixed-precision form the sum is a weighted Gram matrix
// X_i diag(D) X_i^T of the client's feature-major FP32 block X_i (d x n_i), computed on the 5th
// generation tensor cores in TF32 with FP32 accumulation in tensor memory:
//
//   * one CTA per 128 x 128 tile of the upper triangle of H_i (tiles of one client are scheduled
//     together so that the client's block stays in L2);
//   * warp 0 streams 128 x 32 FP32 slabs of the two tile rows with TMA (3-D tensor map over
//     [client][feature][sample], 128-byte swizzle) into a 3-stage ring guarded by mbarriers (two CTAs
//     fit an SM, so one CTA's epilogue overlaps the other's main loop);
//   * warps 2-5 scale the B slab by the per-sample weights D_s in shared memory (the swizzle is
//     undone to find each element's sample) and release it to the tensor cores;
//   * warp 1 (one lane) issues tcgen05.mma.kind::tf32 (M = N = 128, K = 8, four per slab) into a
//     128-column TMEM accumulator and frees each slab with tcgen05.commit;
//   * warps 2-5 read the accumulator back with tcgen05.ld (warp w owns TMEM lanes 32 (w mod 4) ..)
//     and hand each 16-column chunk to the epilogue functor.
//
// Every wait is bounded; a wait that runs out raises the CTA's abort flag, sets *err, lets the
// copies and MMAs already issued drain (bounded again), frees the TMEM and returns.
#pragma once

#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

#include "fednl_philox.cuh"

namespace fednl_tc {

constexpr int kBM = 128, kBN = 128, kBK = 32;     // tile rows, tile columns, FP32 samples per slab
constexpr int kStages = 3;
constexpr int kSlabBytes = kBM * kBK * 4;         // 16 KB (128 rows x 128 bytes)
constexpr int kThreads = 192;
constexpr long long kWaitCycles = 2000000000ll;   // ~1 s
constexpr uint32_t kTmemCols = 128;

// dynamic shared memory: 1024-byte alignment slack + A and B rings + barriers
constexpr size_t smem_bytes() { return 1024 + 2 * kStages * kSlabBytes + 256; }

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count));
}

__device__ __forceinline__ bool mbar_try(uint64_t* b, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait; false when it ran out or another role aborted
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, volatile int* abort_flag)
{
    const long long t0 = clock64();
    while (!mbar_try(b, parity)) {
        if (*abort_flag) return false;
        if (clock64() - t0 > kWaitCycles) {
            *abort_flag = 1;
            return false;
        }
    }
    return true;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* b)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

// UMMA shared-memory descriptor, K-major operand in the 128-byte swizzle layout TMA writes:
// rows of 128 bytes, 8-row atoms 1024 bytes apart (stride byte offset), descriptor version 1.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;                   // leading byte offset (unused by swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;         // stride byte offset
    d |= (uint64_t)1 << 46;                   // descriptor version
    d |= (uint64_t)2 << 61;                   // 128-byte swizzle
    return d;
}

// instruction descriptor of kind::tf32: D = F32, A = B = TF32, both K-major, N = M = 128
constexpr uint32_t kIdescTf32 = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kBN >> 3) << 17) |
                                ((uint32_t)(kBM >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t accumulate)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(kIdescTf32), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v)
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

struct GramJob {
    int d;                 // padded features (multiple of 128)
    int nc;                // clients
    int L;                 // padded samples per client (multiple of 32)
    int nbk;               // tile rows per client (d / 128)
    int tiles;             // upper tiles per client, nbk (nbk + 1) / 2
    const int* ns;         // [nc] samples per client
    const int* act;        // [n_jobs / tiles] processed clients, or nullptr (all)
    const float* w;        // [nc][L] per-sample weights D_s (0 beyond n_i)
    int* err;              // set to 1 when a bounded wait ran out
};

// upper tile t of an nb x nb tile grid, row-major over the upper triangle
__device__ __forceinline__ void upper_tile(int t, int nb, int& mi, int& ni)
{
    int i = 0, rem = t;
    while (rem >= nb - i) {
        rem -= nb - i;
        ++i;
    }
    mi = i;
    ni = i + rem;
}

// Epilogue functor: operator()(client, row m, first column n0, 16 FP32 values, acc) for every row
// of the tile (called by the 128 epilogue threads, 8 times each, acc a per-thread Epi::Acc), then
// finish(client, tile, thread 0..127, acc).
template <class Epi>
__global__ void __launch_bounds__(kThreads) k_gram_tf32(const __grid_constant__ CUtensorMap tmX, GramJob J, Epi epi)
{
    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* ringA = smem;
    unsigned char* ringB = smem + kStages * kSlabBytes;
    uint64_t* full = (uint64_t*)(smem + 2 * kStages * kSlabBytes);
    uint64_t* scaled = full + kStages;
    uint64_t* empty = scaled + kStages;
    uint64_t* done = empty + kStages;
    uint32_t* tmem_slot = (uint32_t*)(done + 1);
    volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int slot = blockIdx.x / J.tiles, t = blockIdx.x % J.tiles;
    const int c = J.act ? J.act[slot] : slot;
    int mi, ni;
    upper_tile(t, J.nbk, mi, ni);
    const int n = J.ns[c];
    const int nk = (n + kBK - 1) / kBK;

    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&scaled[s], 128);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmX)) : "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {                      // TMA producer
            int issued = 0;
            for (int kb = 0; kb < nk; ++kb) {
                const int s = kb % kStages;
                if (kb >= kStages && !mbar_wait(&empty[s], (uint32_t)((kb / kStages) - 1) & 1u, abort_flag)) break;
                mbar_expect_tx(&full[s], 2 * kSlabBytes);
                tma_load_3d(ringA + s * kSlabBytes, &tmX, kb * kBK, mi * kBM, c, &full[s]);
                tma_load_3d(ringB + s * kSlabBytes, &tmX, kb * kBK, ni * kBN, c, &full[s]);
                ++issued;
            }
            if (*abort_flag) {                // let the copies in flight land before leaving
                for (int kb = (issued > kStages ? issued - kStages : 0); kb < issued; ++kb) {
                    const int s = kb % kStages;
                    const long long t0 = clock64();
                    while (!mbar_try(&full[s], (uint32_t)(kb / kStages) & 1u) && clock64() - t0 < kWaitCycles) {
                    }
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {                      // MMA issuer
            int kb = 0;
            for (; kb < nk; ++kb) {
                const int s = kb % kStages;
                if (!mbar_wait(&scaled[s], (uint32_t)(kb / kStages) & 1u, abort_flag)) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t a0 = smem_u32(ringA + s * kSlabBytes), b0 = smem_u32(ringB + s * kSlabBytes);
#pragma unroll
                for (int kk = 0; kk < kBK / 8; ++kk)
                    mma_tf32(tmem, sw128_desc(a0 + kk * 32), sw128_desc(b0 + kk * 32), (kb > 0 || kk > 0) ? 1u : 0u);
                mma_commit(&empty[s]);
            }
            mma_commit(done);                 // arrives once every MMA issued so far has completed
        }
    } else {
        const int et = tid - 64;              // 0..127
        // Weight the B slab: sample column k of the slab by D_(k0 + k).  Thread et owns the 16-byte
        // chunks q = et + 128 i (rows r0 + 16 i, physical chunk et & 7); the 128-byte swizzle puts
        // logical sample group lc = (et & 7) ^ (r0 & 7) there for every i, so one float4 of weights
        // per slab serves all eight chunks; the next slab's is loaded before this slab is waited for.
        const int r0 = et >> 3, lc = (et & 7) ^ (r0 & 7);
        const float* wbase = J.w + (size_t)c * J.L + lc * 4;
        float4 wv = nk > 0 ? *reinterpret_cast<const float4*>(wbase) : make_float4(0.f, 0.f, 0.f, 0.f);
        for (int kb = 0; kb < nk; ++kb) {
            const int s = kb % kStages;
            const float4 wn = kb + 1 < nk ? *reinterpret_cast<const float4*>(wbase + (kb + 1) * kBK) : wv;
            if (!mbar_wait(&full[s], (uint32_t)(kb / kStages) & 1u, abort_flag)) break;
            float4* slab = (float4*)(ringB + s * kSlabBytes);
#pragma unroll
            for (int i = 0; i < kBN / 16; ++i) {
                float4 x = slab[et + 128 * i];
                x.x *= wv.x;
                x.y *= wv.y;
                x.z *= wv.z;
                x.w *= wv.w;
                slab[et + 128 * i] = x;
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_arrive(&scaled[s]);
            wv = wn;
        }
        // epilogue: the accumulator rows of this warp's TMEM lane quarter
        const bool ok = __all_sync(0xffffffffu, mbar_wait(done, 0u, abort_flag));   // warp-uniform for tcgen05.ld
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (ok) {
            const int quarter = warp & 3;
            const int m = mi * kBM + quarter * 32 + lane;
            typename Epi::Acc acc{};
#pragma unroll 1
            for (int j = 0; j < kBN / 16; ++j) {
                float v[16];
                tmem_ld16(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(j * 16), v);
                epi(c, m, ni * kBN + j * 16, v, acc);
            }
            epi.finish(c, t, quarter * 32 + lane, acc);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (*abort_flag) {
        if (tid == 0) *J.err = 1;
        if (warp == 1) {                      // MMAs issued before the abort must finish first
            const long long t0 = clock64();
            while (!mbar_try(done, 0u) && clock64() - t0 < kWaitCycles) {
            }
        }
    }
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    }
}

// Epilogue writing the raw tile (plus lambda on the diagonal) into a full row-major d x d FP32
// matrix per client: out[c][m][n]
struct EpiStore {
    struct Acc {};
    float* out;
    int d;
    float lambda;
    __device__ __forceinline__ void operator()(int c, int m, int n0, const float* v, Acc&) const
    {
        float* row = out + ((size_t)c * d + m) * d + n0;
#pragma unroll
        for (int i = 0; i < 16; ++i) row[i] = v[i] + ((m == n0 + i) ? lambda : 0.0f);
    }
    __device__ __forceinline__ void finish(int, int, int, const Acc&) const {}
};

// packed upper position of (m, n), m <= n
__device__ __forceinline__ long long upos(int m, int n) { return (long long)n * (n + 1) / 2 + m; }

// Initial shifts: shift_c = H_c(x0) in FP32, packed upper (the lanes of a warp hold consecutive
// rows m, so for each column n they touch consecutive packed positions)
struct EpiInitShift {
    struct Acc {};
    float* shift;          // [nc][Up]
    long long Up;
    float lambda;
    int d;                 // true dimension (rows and columns from d on are padding)
    __device__ __forceinline__ void operator()(int c, int m, int n0, const float* v, Acc&) const
    {
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const int n = n0 + i;
            if (m <= n && n < d) shift[(size_t)c * Up + upos(m, n)] = v[i] + (m == n ? lambda : 0.0f);
        }
    }
    __device__ __forceinline__ void finish(int, int, int, const Acc&) const {}
};

// Round epilogue: diff = H_c - shift_c on the upper triangle; per-thread weighted sum of squares
// (diagonal once, off-diagonal twice: the full symmetric matrix) into fpart[c][tile][thread]; the
// differences at the client's selected positions into dsel[c][p] (every difference when sel is
// null: TopK / TopLEK select afterwards)
struct EpiDiff {
    struct Acc {
        float sq = 0.0f;
    };
    const float* shift;    // [nc][Up]
    float* dsel;           // [nc][Up]
    const unsigned* sel;   // [nc][SW] or nullptr
    float* fpart;          // [nc][tiles][128]
    long long Up;
    int SW, tiles;
    float lambda;
    int d;
    __device__ __forceinline__ void operator()(int c, int m, int n0, const float* v, Acc& a) const
    {
        // all 16 shift values and selection words are loaded before the first store, so that the
        // loads overlap instead of waiting one by one behind the stores to dsel
        const unsigned* sc = sel ? sel + (size_t)c * SW : nullptr;
        const float* shc = shift + (size_t)c * Up;
        float sh[16];
        unsigned sw[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const int n = n0 + i;
            const bool ok = m <= n && n < d;
            const long long p = ok ? upos(m, n) : 0;
            sh[i] = ok ? __ldg(shc + p) : 0.0f;
            sw[i] = (ok && sc) ? __ldg(sc + (p >> 5)) : 0xffffffffu;
        }
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const int n = n0 + i;
            if (m <= n && n < d) {
                const long long p = upos(m, n);
                const float df = (v[i] + (m == n ? lambda : 0.0f)) - sh[i];
                a.sq = fmaf(m == n ? df : 2.0f * df, df, a.sq);
                if ((sw[i] >> (p & 31)) & 1u) dsel[(size_t)c * Up + p] = df;
            }
        }
    }
    __device__ __forceinline__ void finish(int c, int t, int th, const Acc& a) const
    {
        fpart[((size_t)c * tiles + t) * 128 + th] = a.sq;
    }
};


// ---- mixed-precision round kernels (dense FP32 features, feature-major [nc][d][L]) ------------
// Margins and gradients need FP64-grade sums (the final ||grad|| is ~1e-9 of terms of order 1), and
// GB300 issues a warp's FP64 instruction about once per 64 cycles; both are therefore formed with
// FP32 pairs ("float-float"): each product x * (y_hi + y_lo) as an exact two-product plus the small
// cross term, accumulated with two-sum (Dekker / Knuth) -- roughly 2^-44 relative, at the FP32 rate.
__device__ __forceinline__ void ff_add(float& hi, float& lo, float p, float e)
{
    const float s = __fadd_rn(hi, p);
    const float bb = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(err, e));
}

__device__ __forceinline__ void ff_mac(float& hi, float& lo, float x, float yh, float yl)
{
    const float p = __fmul_rn(x, yh);
    const float e = __fadd_rn(fmaf(x, yh, -p), __fmul_rn(x, yl));
    ff_add(hi, lo, p, e);
}

__device__ __forceinline__ void split_ff(double v, float& h, float& l)
{
    h = __double2float_rn(v);
    l = __double2float_rn(v - (double)h);
}

struct MxDev {
    int d, dp, nc, L, U, SW, tiles;     // dp: d padded to the Gram tile (feature rows of X)
    long long Up;
    double lambda, alpha, prescale, inv_n, mult;
    float alphaf, multf;    // the shift update runs in FP32 (the shifts are FP32)
    const int* ns;          // [nc]
    const float* X;         // [nc][dp][L]
    const double* lab;      // [nc][L] labels (+-1, 0 beyond n)
    double* x;              // [d]
    float* xh;              // [d] split iterate
    float* xl;
    float* Dw;              // [nc][L] Gram weights D_s
    float* qh;              // [nc][L] gradient weights b_s q_s as FP32 pairs
    float* ql;
    double* gc;             // [nc][d]
    double* g;              // [d]
    double* H;              // [U] master, packed upper
    float* Hh;              // [U] H as an FP32 pair (hi + lo) for the FP32 solve's residual
    float* Hl;
    float* Hrh;             // [U] the same pair in row-major packed order
    float* Hrl;
    float* shift;           // [nc][Up]
    float* dsel;            // [nc][Up]
    unsigned* sel;          // [nc][SW]
    unsigned* draws;        // [nc] per-client draw counters (RandK-Philox, TopLEK rounding)
    int* cnt;               // [nc] selected entries of the round (TopK / TopLEK)
    float* fpart;           // [nc][tiles][128]
    double* lk;             // [nc]
    double* stats;          // [4]: ||g||, l
};

__global__ void k_mx_split_x(MxDev P)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P.d) split_ff(P.x[i], P.xh[i], P.xl[i]);
}

// margin m_s = b_s a_s^T x, sigmoid (FP64), D_s (Gram weight, FP32) and b_s q_s (FP32 pair)
__device__ __forceinline__ double mx_sigmoid(double m) { return 1.0 / (1.0 + exp(-m)); }

// A block covers 64 samples; its four warp rows split each sample's features in quarters (eight
// loads in flight each, two float-float accumulators), and the quarters are added in order.
__global__ void __launch_bounds__(256) k_mx_margin(MxDev P)
{
    __shared__ float s_xh[1024], s_xl[1024];
    __shared__ float s_ph[4][64], s_pl[4][64];
    const int c = blockIdx.y, sx = threadIdx.x, q = threadIdx.y;
    const int tid = q * 64 + sx;
    for (int i = tid; i < P.d && i < 1024; i += 256) {
        s_xh[i] = P.xh[i];
        s_xl[i] = P.xl[i];
    }
    __syncthreads();
    const int n = P.ns[c];
    const int s = blockIdx.x * 64 + sx;
    const int per = (P.d + 3) / 4, i0 = q * per, i1 = min(P.d, i0 + per);
    float h0 = 0.0f, l0 = 0.0f, h1 = 0.0f, l1 = 0.0f;
    if (s < n) {
        const float* col = P.X + (size_t)c * P.dp * P.L + s;
        int i = i0;
        for (; i + 8 <= i1; i += 8) {
            float xv[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) xv[u] = __ldg(col + (size_t)(i + u) * P.L);
#pragma unroll
            for (int u = 0; u < 8; u += 2) {
                const float yh0 = i + u < 1024 ? s_xh[i + u] : P.xh[i + u];
                const float yl0 = i + u < 1024 ? s_xl[i + u] : P.xl[i + u];
                const float yh1 = i + u + 1 < 1024 ? s_xh[i + u + 1] : P.xh[i + u + 1];
                const float yl1 = i + u + 1 < 1024 ? s_xl[i + u + 1] : P.xl[i + u + 1];
                ff_mac(h0, l0, xv[u], yh0, yl0);
                ff_mac(h1, l1, xv[u + 1], yh1, yl1);
            }
        }
        for (; i < i1; ++i) {
            const float yh = i < 1024 ? s_xh[i] : P.xh[i], yl = i < 1024 ? s_xl[i] : P.xl[i];
            ff_mac(h0, l0, __ldg(col + (size_t)i * P.L), yh, yl);
        }
        ff_add(h0, l0, h1, l1);
    }
    s_ph[q][sx] = h0;
    s_pl[q][sx] = l0;
    __syncthreads();
    if (q != 0 || s >= n) return;
    float hi = s_ph[0][sx], lo = s_pl[0][sx];
#pragma unroll
    for (int t = 1; t < 4; ++t) ff_add(hi, lo, s_ph[t][sx], s_pl[t][sx]);
    const double b = P.lab[(size_t)c * P.L + s];
    const double m = b * ((double)hi + (double)lo);
    const double sig = mx_sigmoid(m);
    const double inv_n = 1.0 / (double)n;
    const double z1 = 1.0 - sig;
    P.Dw[(size_t)c * P.L + s] = (float)(inv_n * (z1 * sig));
    const double qv = b * (z1 * -inv_n);
    split_ff(qv, P.qh[(size_t)c * P.L + s], P.ql[(size_t)c * P.L + s]);
}

// client gradients: one warp per (client, feature), lanes over the samples (eight in flight, the
// last pass masked).  The warp reduces in float-float; eight lanes of the block then form the FP64
// sums of its eight features, so the FP64 pipe sees one conversion and add per block, not per warp.
__global__ void __launch_bounds__(256) k_mx_grad(MxDev P)
{
    __shared__ float s_h[8], s_l[8];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wid = blockIdx.x * 8 + w, total = P.nc * P.d;
    float hi = 0.0f, lo = 0.0f;
    if (wid < total) {
        const int c = wid / P.d, i = wid - c * P.d;
        const int n = P.ns[c];
        const float* row = P.X + ((size_t)c * P.dp + i) * P.L;
        const float* qh = P.qh + (size_t)c * P.L;
        const float* ql = P.ql + (size_t)c * P.L;
        float h1 = 0.0f, l1 = 0.0f;
        for (int s = lane; s < n; s += 256) {
            float x[8], a[8], b[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int t = s + 32 * u;
                const bool in = t < n;
                x[u] = in ? __ldg(row + t) : 0.0f;
                a[u] = in ? __ldg(qh + t) : 0.0f;
                b[u] = in ? __ldg(ql + t) : 0.0f;
            }
#pragma unroll
            for (int u = 0; u < 8; u += 2) {
                ff_mac(hi, lo, x[u], a[u], b[u]);
                ff_mac(h1, l1, x[u + 1], a[u + 1], b[u + 1]);
            }
        }
        ff_add(hi, lo, h1, l1);
        for (int o = 16; o > 0; o >>= 1) {
            const float oh = __shfl_xor_sync(0xffffffffu, hi, o), ol = __shfl_xor_sync(0xffffffffu, lo, o);
            ff_add(hi, lo, oh, ol);
        }
    }
    if (lane == 0) {
        s_h[w] = hi;
        s_l[w] = lo;
    }
    __syncthreads();
    const int t = blockIdx.x * 8 + threadIdx.x;
    if (threadIdx.x < 8 && t < total) {
        const int c = t / P.d, i = t - c * P.d;
        P.gc[(size_t)c * P.d + i] = ((double)s_h[threadIdx.x] + (double)s_l[threadIdx.x]) + P.lambda * P.x[i];
    }
}

// RandK-Philox draw of every client (the FP64 engine's stream)
__global__ void k_mx_draw(MxDev P, int k, int h, unsigned seed)
{
    const int c = blockIdx.x;
    unsigned* sc = P.sel + (size_t)c * P.SW;
    for (int w = threadIdx.x; w < P.SW; w += blockDim.x) sc[w] = 0u;
    const unsigned draw = P.draws[c];
    __syncthreads();
    for (int i = threadIdx.x; i < k; i += blockDim.x) {
        uint32_t y = fednl::philox_feistel((uint32_t)i, h, seed, (uint32_t)c, draw);
        while (y >= (uint32_t)P.U) y = fednl::philox_feistel(y, h, seed, (uint32_t)c, draw);
        atomicOr(&sc[y >> 5], 1u << (y & 31));
    }
    __syncthreads();
    if (threadIdx.x == 0) P.draws[c] = draw + 1;
}

// ---- TopK / TopLEK of the mixed-precision form -----------------------------------------------
// On the FP32 differences every entry is a candidate; the key of an entry is the magnitude bits of
// its FP32 value (ordered like |v| for finite values).  TopK keeps the k largest keys, ties at the
// threshold going to the lower packed positions.  TopLEK then applies the reference's rule
// (SpecialMathRoutinesForMatrix.h:377-511) to that set: with F = ||H_c - shift_c||_F^2 (diagonal
// once, off-diagonal twice), delta = k / U and eps = F / 10, the kept entries are removed smallest
// first (ties: higher position first) while the removed mass plus the mass outside the set stays
// below the window; the boundary entry stays with probability 1 - p, p the window fraction, drawn
// from Philox4x32-10 keyed by (seed, client) at the client's draw counter.
constexpr int kSelThreads = 1024;
constexpr int kMxMaxLek = 16384;          // TopLEK: the kept set is sorted in shared memory

__device__ __forceinline__ unsigned mag_key(float v) { return __float_as_uint(v) & 0x7fffffffu; }

// inclusive scan of one unsigned per thread over the block (1024 threads); total in *tot
__device__ __forceinline__ unsigned block_scan_u32(unsigned v, unsigned* s_w, unsigned* tot)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) s_w[warp] = v;
    __syncthreads();
    if (warp == 0) {
        unsigned w = s_w[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        s_w[lane] = w;
    }
    __syncthreads();
    const unsigned r = v + (warp ? s_w[warp - 1] : 0u);
    if (tot) *tot = s_w[31];
    __syncthreads();
    return r;
}

// inclusive float-float scan over the block (1024 threads); total in (*th, *tl)
__device__ __forceinline__ void block_scan_ff(float& h, float& l, float2* s_w, float* th, float* tl)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const float uh = __shfl_up_sync(0xffffffffu, h, o), ul = __shfl_up_sync(0xffffffffu, l, o);
        if (lane >= o) ff_add(h, l, uh, ul);
    }
    if (lane == 31) s_w[warp] = make_float2(h, l);
    __syncthreads();
    if (warp == 0) {
        float wh = s_w[lane].x, wl = s_w[lane].y;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float uh = __shfl_up_sync(0xffffffffu, wh, o), ul = __shfl_up_sync(0xffffffffu, wl, o);
            if (lane >= o) ff_add(wh, wl, uh, ul);
        }
        s_w[lane] = make_float2(wh, wl);
    }
    __syncthreads();
    if (warp) ff_add(h, l, s_w[warp - 1].x, s_w[warp - 1].y);
    if (th) {
        *th = s_w[31].x;
        *tl = s_w[31].y;
    }
    __syncthreads();
}

__device__ __forceinline__ bool packed_is_diag(long long p)
{
    long long j = (long long)((sqrtf(8.0f * (float)p + 1.0f) - 1.0f) * 0.5f);
    while (j > 0 && j * (j + 1) / 2 > p) --j;
    while ((j + 1) * (j + 2) / 2 <= p) ++j;
    return p - j * (j + 1) / 2 == j;
}

// TopLEK's term of a kept-set entry (key << 32 | ~position) in fixed point: c v^2 2^sh (c = 1 on the
// diagonal, 2 off it) for the FP32 magnitude v = m 2^(eb - 150) (biased exponent eb, significand m),
// i.e. m^2 2^(2 eb - 300 + sh), exact where the shift is not negative
__device__ __forceinline__ unsigned long long lek_fixed(unsigned long long e, int sh)
{
    const unsigned key = (unsigned)(e >> 32);
    const int eb = (int)(key >> 23);
    const unsigned long long m = eb ? (unsigned long long)((key & 0x7fffffu) | 0x800000u) : (unsigned long long)(key & 0x7fffffu);
    const long long q = (long long)(0xffffffffu - (unsigned)(e & 0xffffffffu));
    const int s = 2 * (eb ? eb : 1) - 300 + sh + (packed_is_diag(q) ? 0 : 1);
    const unsigned long long m2 = m * m;
    return s >= 0 ? m2 << s : (s > -64 ? m2 >> -s : 0ull);
}

// inclusive scan of one u64 per thread over the block (1024 threads); total in *tot
__device__ __forceinline__ unsigned long long block_scan_u64(unsigned long long v, unsigned long long* s_w,
                                                             unsigned long long* tot)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) s_w[warp] = v;
    __syncthreads();
    if (warp == 0) {
        unsigned long long w = s_w[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        s_w[lane] = w;
    }
    __syncthreads();
    const unsigned long long r = v + (warp ? s_w[warp - 1] : 0ull);
    if (tot) *tot = s_w[31];
    __syncthreads();
    return r;
}

// one CTA (1024 threads) per client: selection bitmap sel[c] from the differences dsel[c]
__global__ void __launch_bounds__(kSelThreads) k_mx_select(MxDev P, int k, int toplek, unsigned seed)
{
    extern __shared__ unsigned long long s_set[];       // TopLEK: [max(Kp, 1024)] entries, [2048] masses
    __shared__ unsigned hist[2048];
    __shared__ unsigned s_wu[32];
    __shared__ unsigned long long s_wl[32];
    __shared__ float2 s_wf[32];
    __shared__ double s_win[3];                 // TopLEK: F, (1 - k/U) F, F/10
    __shared__ unsigned long long s_rx, s_above;
    __shared__ unsigned s_bin, s_need, s_cnt[32], s_nk, s_kmax, s_qstar;
    __shared__ int s_istar;
    const int c = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int U = P.U;
    const float* v = P.dsel + (size_t)c * P.Up;
    unsigned* sc = P.sel + (size_t)c * P.SW;
    const int K = k < U ? k : U;
    unsigned T = 0, need = 0;
    if (K < U) {
        // radix select of the K-th largest key: 11 + 11 + 9 bits from the top
        unsigned prefix = 0, mask = 0;
        need = (unsigned)K;
        const int shs[3] = {20, 9, 0}, nbits[3] = {11, 11, 9};
        for (int pass = 0; pass < 3; ++pass) {
            const int sh = shs[pass], nb = 1 << nbits[pass];
            for (int b = tid; b < 2048; b += kSelThreads) hist[b] = 0u;
            __syncthreads();
            for (int q = tid; q < U; q += kSelThreads) {
                const unsigned key = mag_key(v[q]);
                if ((key & mask) == prefix) atomicAdd(&hist[(key >> sh) & (unsigned)(nb - 1)], 1u);
            }
            __syncthreads();
            // thread t owns bins nb-1-2t and nb-2-2t (descending keys)
            const int b0 = nb - 1 - 2 * tid, b1 = b0 - 1;
            const unsigned h0 = b0 >= 0 ? hist[b0] : 0u, h1 = b1 >= 0 ? hist[b1] : 0u;
            const unsigned incl = block_scan_u32(h0 + h1, s_wu, nullptr);
            const unsigned excl = incl - h0 - h1;
            if (excl < need && need <= incl) {
                if (excl + h0 >= need) {
                    s_bin = (unsigned)b0;
                    s_need = need - excl;
                } else {
                    s_bin = (unsigned)b1;
                    s_need = need - excl - h0;
                }
            }
            __syncthreads();
            prefix |= s_bin << sh;
            mask |= (unsigned)(nb - 1) << sh;
            need = s_need;
            __syncthreads();
        }
        T = prefix;
    }
    // bitmap in position order: keys above T, and the first `need` keys equal to T.  Warp w owns a
    // contiguous range of selection words (lane = bit); pass 1 counts its keys equal to T, one block
    // scan orders the warps, pass 2 forms the words (loads of eight words in flight in each pass).
    {
        const int SWn = (U + 31) >> 5, wpw = (SWn + 31) >> 5;
        const int w0 = warp * wpw, w1 = min(SWn, w0 + wpw);
        unsigned neq = 0;
        for (int wd = w0; wd < w1; wd += 8) {
            unsigned key[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int q = (wd + u) * 32 + lane;
                key[u] = (wd + u < w1 && q < U) ? mag_key(v[q]) : 0xffffffffu;
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) neq += __popc(__ballot_sync(0xffffffffu, K < U && key[u] == T));
        }
        if (lane == 0) s_cnt[warp] = neq;
        __syncthreads();
        unsigned carry = 0;
        for (int w = 0; w < warp; ++w) carry += s_cnt[w];
        for (int wd = w0; wd < w1; wd += 8) {
            unsigned key[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int q = (wd + u) * 32 + lane;
                key[u] = (wd + u < w1 && q < U) ? mag_key(v[q]) : 0xffffffffu;
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int q = (wd + u) * 32 + lane;
                const bool in = wd + u < w1 && q < U;
                const bool gt = in && (K >= U || key[u] > T), eq = in && K < U && key[u] == T;
                const unsigned be = __ballot_sync(0xffffffffu, eq);
                const unsigned rank = carry + __popc(be & ((1u << lane) - 1u));
                const unsigned word = __ballot_sync(0xffffffffu, gt || (eq && rank < need));
                if (lane == 0 && wd + u < w1) sc[wd + u] = word;
                carry += __popc(be);
            }
        }
        __syncthreads();
    }
    if (!toplek || K >= U) {
        if (tid == 0) P.cnt[c] = K;
        return;
    }
    // ---- TopLEK on the kept set ----
    // The reference's rule (SpecialMathRoutinesForMatrix.h:377-511) removes kept entries smallest
    // first (ascending key, ties: higher position first) while the mass outside plus the removed
    // mass stays below the window.  In descending order (key desc, position asc) with Top(j) the
    // mass of the first j entries (terms v^2 on the diagonal, 2 v^2 off it), the boundary entry is
    // the j*-th, Top(j*) < R <= Top(j* + 1), R = F + F/10 - (1 - k/U) F.  It is found without
    // sorting: the masses are 64-bit fixed point (exact integer products of the FP32 significands,
    // so sums are exact in any order), weighted histograms walk the key bits (11 + 11 + 9) from
    // the top, then the entries tied at the boundary key are walked in position order.
    int Kp = 1;
    while (Kp < K) Kp <<= 1;
    unsigned long long* s_mass = s_set + (Kp > kSelThreads ? Kp : kSelThreads);     // [2048]
    if (tid == 0) s_kmax = 0u;
    {   // the kept entries in position order: popcounts of the bitmap words, block-scanned
        unsigned base_cnt = 0;
        for (int w0 = 0; w0 < P.SW; w0 += kSelThreads) {
            const int w = w0 + tid;
            const unsigned word = w < P.SW ? sc[w] : 0u;
            const unsigned pc = (unsigned)__popc(word);
            unsigned tot;
            const unsigned incl = block_scan_u32(pc, s_wu, &tot);
            unsigned slot = base_cnt + incl - pc;
            unsigned wd = word;
            while (wd) {
                const int b = __ffs(wd) - 1;
                wd &= wd - 1u;
                const unsigned q = (unsigned)w * 32u + (unsigned)b;
                if (slot < (unsigned)Kp)
                    s_set[slot] = ((unsigned long long)mag_key(v[q]) << 32) | (unsigned long long)(0xffffffffu - q);
                ++slot;
            }
            base_cnt += tot;
        }
    }
    __syncthreads();
    // the fixed-point scale from the largest key; F from the Gram epilogue's partial sums
    {
        unsigned km = 0u;
        for (int m = tid; m < K; m += kSelThreads) km = max(km, (unsigned)(s_set[m] >> 32));
        km = __reduce_max_sync(0xffffffffu, km);
        if (lane == 0) atomicMax(&s_kmax, km);
    }
    float fh = 0.0f, fl = 0.0f;
    for (int t = tid; t < P.tiles * 128; t += kSelThreads) ff_add(fh, fl, P.fpart[(size_t)c * P.tiles * 128 + t], 0.0f);
    float Fh, Fl;
    block_scan_ff(fh, fl, s_wf, &Fh, &Fl);
    int lgK = 0;
    while ((1 << lgK) < K) ++lgK;
    const int ebmax = max(1, (int)(s_kmax >> 23));
    const int sh = 314 - 2 * ebmax - lgK;              // K terms of at most 2^(2 ebmax - 251 + sh) < 2^63
    unsigned long long mk = 0ull;
    for (int m = tid; m < K; m += kSelThreads) mk += lek_fixed(s_set[m], sh);
    unsigned long long total;
    block_scan_u64(mk, s_wl, &total);
    if (tid == 0) {
        const double F = (double)Fh + (double)Fl, scale = ldexp(1.0, -sh);
        const double all = (double)total * scale;
        const double delta = (double)k / (double)U;
        const double omd_f = (1.0 - delta) * F, eps = 1e-1 * F;
        s_win[0] = F;
        s_win[1] = omd_f;
        s_win[2] = eps;
        const double rr = (F + eps - omd_f) * ldexp(1.0, sh);
        unsigned long long rx = rr >= 9.2e18 ? ~0ull >> 1 : (rr > 0.0 ? (unsigned long long)rr : 0ull);
        if (rx > total) rx = total;                   // past the smallest entry: it is the boundary
        s_rx = (omd_f + eps > F - all) ? rx : 0ull;   // 0: no window (nothing kept)
        s_nk = 0u;
        s_qstar = 0u;
        s_istar = 0;
    }
    __syncthreads();
    unsigned long long rrem = s_rx;
    unsigned keep = 0u;
    if (rrem > 0ull) {
        unsigned prefix = 0u, mask = 0u;
        unsigned long long above = 0ull;               // mass of the entries above the current range
        unsigned above_n = 0u;
        const int shs[3] = {20, 9, 0}, nbits[3] = {11, 11, 9};
        for (int pass = 0; pass < 3; ++pass) {
            const int sb = shs[pass], nb = 1 << nbits[pass];
            for (int b = tid; b < 2048; b += kSelThreads) {
                hist[b] = 0u;
                s_mass[b] = 0ull;
            }
            __syncthreads();
            for (int m = tid; m < K; m += kSelThreads) {
                const unsigned long long e = s_set[m];
                const unsigned key = (unsigned)(e >> 32);
                if ((key & mask) == prefix) {
                    const unsigned b = (key >> sb) & (unsigned)(nb - 1);
                    atomicAdd(&hist[b], 1u);
                    atomicAdd(&s_mass[b], lek_fixed(e, sh));
                }
            }
            __syncthreads();
            // descending bins: thread t owns nb-1-2t and nb-2-2t
            const int b0 = nb - 1 - 2 * tid, b1 = b0 - 1;
            const unsigned long long m0 = b0 >= 0 ? s_mass[b0] : 0ull, m1 = b1 >= 0 ? s_mass[b1] : 0ull;
            const unsigned n0 = b0 >= 0 ? hist[b0] : 0u, n1 = b1 >= 0 ? hist[b1] : 0u;
            unsigned long long mtot;
            const unsigned long long mi = block_scan_u64(m0 + m1, s_wl, &mtot);
            const unsigned ni = block_scan_u32(n0 + n1, s_wu, nullptr);
            const unsigned long long me = mi - m0 - m1;
            const unsigned ne = ni - n0 - n1;
            if (me < rrem && rrem <= mi) {
                if (rrem <= me + m0) {
                    s_bin = (unsigned)b0;
                    s_above = me;
                    s_need = ne;
                } else {
                    s_bin = (unsigned)b1;
                    s_above = me + m0;
                    s_need = ne + n0;
                }
            }
            __syncthreads();
            prefix |= s_bin << sb;
            mask |= (unsigned)(nb - 1) << sb;
            above += s_above;
            above_n += s_need;
            rrem -= s_above;
            __syncthreads();
        }
        // entries tied at the boundary key, in position order (= descending order among them)
        const int per = (K + kSelThreads - 1) / kSelThreads, m0 = tid * per;
        unsigned long long tm = 0ull;
        unsigned tn = 0u;
        for (int m = m0; m < m0 + per && m < K; ++m) {
            const unsigned long long e = s_set[m];
            if ((unsigned)(e >> 32) == prefix) {
                tm += lek_fixed(e, sh);
                ++tn;
            }
        }
        const unsigned long long tmi = block_scan_u64(tm, s_wl, nullptr);
        const unsigned tni = block_scan_u32(tn, s_wu, nullptr);
        unsigned long long cum = tmi - tm;
        unsigned idx = tni - tn;
        for (int m = m0; m < m0 + per && m < K; ++m) {
            const unsigned long long e = s_set[m];
            if ((unsigned)(e >> 32) != prefix) continue;
            const unsigned long long w = lek_fixed(e, sh);
            if (cum < rrem && rrem <= cum + w) {      // the boundary entry: j* = above_n + idx
                const double scale = ldexp(1.0, -sh);
                const double F = s_win[0], omd_f = s_win[1], eps = s_win[2];
                const double pv = F - (double)(above + cum + w) * scale, nv = F - (double)(above + cum) * scale;
                const double pr = (omd_f - pv + eps) / (nv - pv + eps);
                uint32_t o;
                fednl::philox4x32(P.draws[c], 0x544C454Bu, 0u, 0u, seed, (uint32_t)c, o);
                const double u = ((double)o + 0.5) * (1.0 / 4294967296.0);
                const unsigned js = above_n + idx;
                s_nk = js + (u > pr ? 1u : 0u);
                s_qstar = 0xffffffffu - (unsigned)(e & 0xffffffffu);
                s_istar = (u > pr) ? 1 : 0;
            }
            cum += w;
            ++idx;
        }
        __syncthreads();
        keep = s_nk;
        // the kept set: keys above the boundary key, tied entries before the boundary entry, and
        // the boundary entry itself when the draw keeps it
        const unsigned kap = prefix, qs = s_qstar;
        const int inc = s_istar;
        for (int w = tid; w < P.SW; w += kSelThreads) sc[w] = 0u;
        __syncthreads();
        for (int m = tid; m < K; m += kSelThreads) {
            const unsigned long long e = s_set[m];
            const unsigned key = (unsigned)(e >> 32), q = 0xffffffffu - (unsigned)(e & 0xffffffffu);
            if (key > kap || (key == kap && (q < qs || (inc && q == qs)))) atomicOr(&sc[q >> 5], 1u << (q & 31));
        }
    } else {
        for (int w = tid; w < P.SW; w += kSelThreads) sc[w] = 0u;
    }
    if (tid == 0) {
        P.cnt[c] = (int)keep;
        P.draws[c] = P.draws[c] + 1;
    }
}

// Lk = ||H_c - shift_c||_F from the Gram epilogue's partial sums
__global__ void k_mx_lk(MxDev P)
{
    const int c = blockIdx.x;
    const float* fp = P.fpart + (size_t)c * P.tiles * 128;
    double v = 0.0;
    for (int t = threadIdx.x; t < P.tiles * 128; t += blockDim.x) v += (double)fp[t];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __shared__ double s_w[32];
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_w[w];
        P.lk[c] = sqrt(t);
    }
}

// H[p] as an FP32 pair at packed position p (column-major) and at its row-major position
__device__ __forceinline__ void store_pair(const MxDev& P, int p, double h)
{
    int n = (int)((sqrtf(8.0f * (float)p + 1.0f) - 1.0f) * 0.5f);
    while (n > 0 && n * (n + 1) / 2 > p) --n;
    while ((n + 1) * (n + 2) / 2 <= p) ++n;
    const int m = p - n * (n + 1) / 2;
    const float hh = (float)h, hl = (float)(h - (double)hh);
    P.Hh[p] = hh;
    P.Hl[p] = hl;
    const int r = m * P.d - (m * (m - 1)) / 2 + n - m;
    P.Hrh[r] = hh;
    P.Hrl[r] = hl;
}

// worker shift update (FP32) and master merge (FP64), clients in order per position
// A warp covers the 32 positions of one selection word: lane c of each batch of 32 clients loads
// that client's word, and the clients with a selected position in the word are then visited in
// increasing order, each lane updating its own position (the FP64 sum stays in client order).
__global__ void k_mx_apply(MxDev P)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x, lane = threadIdx.x & 31;
    const int word = p >> 5;                     // the same for the whole warp (blockDim % 32 == 0)
    const bool in = p < P.U;
    double h = in ? P.H[p] : 0.0;
    for (int c0 = 0; c0 < P.nc; c0 += 32) {
        const int cl = c0 + lane;
        const unsigned wv = (cl < P.nc && word < P.SW) ? __ldg(P.sel + (size_t)cl * P.SW + word) : 0u;
        if (!__any_sync(0xffffffffu, wv != 0u)) continue;
        // transpose: bit t of mine = client c0 + t selected my position
        unsigned mine = 0u;
#pragma unroll
        for (int t = 0; t < 32; ++t) {
            const unsigned b = __ballot_sync(0xffffffffu, (wv >> t) & 1u);
            if (lane == t) mine = b;
        }
        if (!in) mine = 0u;
        // loads of every selected client first, then the updates in client order
        float dv[32], sv[32];
#pragma unroll
        for (int t = 0; t < 32; ++t)
            if ((mine >> t) & 1u) {
                const size_t q = (size_t)(c0 + t) * P.Up + p;
                dv[t] = P.dsel[q];
                sv[t] = P.shift[q];
            }
#pragma unroll
        for (int t = 0; t < 32; ++t)
            if ((mine >> t) & 1u) {
                const size_t q = (size_t)(c0 + t) * P.Up + p;
                const float item = dv[t] * P.multf;
                P.shift[q] = fmaf(P.alphaf, item, sv[t]);         // FP32 shift update
                h = fma((double)item, P.prescale, h);              // FP64 master, clients in order
            }
    }
    if (in) {
        P.H[p] = h;
        store_pair(P, p, h);
    }
}

// g = mean g_c (one warp per feature: lanes over clients, then a butterfly sum), l = mean Lk
__global__ void k_mx_aggregate(MxDev P)
{
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (wid < P.d) {
        double v = 0.0;
        for (int c = lane; c < P.nc; c += 32) v += P.gc[(size_t)c * P.d + wid];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) P.g[wid] = v * P.inv_n;
    }
    if (blockIdx.x == 0 && threadIdx.x < 32) {
        double l = 0.0;
        for (int c = lane; c < P.nc; c += 32) l += P.lk[c];
        for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
        if (lane == 0) P.stats[1] = l * P.inv_n;
    }
}

// H = mean of the initial shifts (FP64 sum of the FP32 shifts, clients in order)
__global__ void k_mx_hinit(MxDev P)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.U) return;
    double h = 0.0;
    for (int c = 0; c < P.nc; ++c) h += (double)P.shift[(size_t)c * P.Up + p];
    h *= P.inv_n;
    P.H[p] = h;
    store_pair(P, p, h);
}

}  // namespace fednl_tc
