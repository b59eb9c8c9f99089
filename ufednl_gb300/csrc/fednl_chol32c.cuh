// fednl_chol32c.cuh -- the mixed-precision form's Option-B solve on many SMs: an FP32 Cholesky
// factor computed by a cooperative grid, FP64 residuals and iterative refinement, and the FP64
// solve (chol_body) taking over in the same launch when an FP32 pivot is not positive.
//
// x_new = x - dx, (H + l I) dx = g (TrainLoop.h:1451-1476, Option B).
//   1. A = lower(H) + l I in FP32, row-major [ld][ld] (row i of the lower triangle is column i of
//      the packed upper H, so the conversion reads contiguously).
//   2. Right-looking panels of 32 columns.  Every CTA loads the panel (the 32 x 32 diagonal block
//      and the rows below it) into shared memory, factors the diagonal block in one warp (lane i =
//      row i, pivots by rsqrt, the new column exchanged by shuffles) and solves ALL the panel rows
//      against it (each thread one row, x L11^T = a), so that no grid barrier separates the
//      factorisation of the panel from its trailing update.  The trailing update
//      A22 -= L21 L21^T is split over the CTAs in 32 x 32 tiles; one grid barrier per panel.  The
//      CTA that owns the panel also writes the inverse of the diagonal block (for the solves).
//   3. L L^T e = r in FP32 by CTA 0 (blocks of 32: a GEMV over the finished part, then the
//      block's inverse), dx += e in FP64, r = g - (H + l I) dx by all CTAs (float-float on H held
//      as FP32 pairs, about 2^-44 relative), repeated until
//      ||e|| <= tol ||dx||, or the next correction is predicted below that (||e||^2 / ||e_prev||),
//      or after `refine` corrections; x -= dx.
// Every CTA makes the same pivot decisions (same data, same arithmetic), so a failed FP32 pivot
// sends the whole grid into the FP64 cooperative solve, which reports a matrix that is not positive
// definite there.
#pragma once

namespace fednl {

constexpr int kC32Stride = 36;      // floats per panel row in shared memory: 16-byte rows, and the
                                    // float4 reads of 8 consecutive rows fall in distinct banks
constexpr int kC32MaxD = 1312;      // panel rows beside the FP64 solve's static shared memory

struct Chol32c {
    float* A;          // [ld][ld] row-major; the lower triangle ends as the factor L (A = L L^T)
    float* diag0;      // [d] the diagonal of A before the factorisation (pivot test)
    float* linv;       // [ld / 32][32][32] inverses of the diagonal blocks, row-major
    double* r;         // [d] residual (FP64)
    double* acc;       // [d] solution being accumulated (FP64)
    float* accp;       // [2][d] the same as FP32 pairs (hi, lo), for the float-float residual
    const float* hh;   // H as FP32 pairs (about 2^-48 relative), packed upper column-major (hh + hl)
    const float* hl;   // and row-major (rh + rl)
    const float* rh;
    const float* rl;
    int* flag;         // CTA 0's stop decision, read by every CTA after a grid barrier
    int ld;            // d rounded up to 32
    int refine;        // at most this many refinement steps after the first solve
    float tol;         // stop when the correction is at most tol of the solution (2-norms)
    int resident;      // CTA 0 keeps the factor in shared memory for the solves
    int smem_floats;   // dynamic shared memory of the launch, in floats
    int cluster;       // the launch is one thread-block cluster (cluster barriers)
};

__host__ __device__ inline int c32c_ld(int d) { return (d + 31) & ~31; }

// Dynamic shared memory, in floats: a fixed head (the factored diagonal block [32][36], the solve
// vector [ld], reduction scratch [8][32] and [32], the first trailing-update tile's entries of A
// [256][4], fetched while the panel is factored); in resident mode the factor's rows below the
// diagonal blocks, column block after column block ([rows][32], filled by CTA 0 as the panels are
// factored); and at the very end the current panel ([32 + rows below rounded up to 32][36]).
__host__ __device__ inline int c32c_head_floats(int d) { return 32 * kC32Stride + c32c_ld(d) + 8 * 32 + 32 + 1024; }
constexpr int kC32ResBlocks = 10;   // resident mode: at most 10 column blocks (d <= 320), whose
                                    // diagonal-block inverses the solves hold in registers
__host__ __device__ inline int c32c_rows_below(int d, int b)
{
    const int r = d - 32 * (b + 1);
    return r > 0 ? r : 0;
}
// first row of column block b in the resident store
__host__ __device__ inline int c32c_row0(int d, int b)
{
    int s = 0;
    for (int q = 0; q < b; ++q) s += c32c_rows_below(d, q);
    return s;
}
__host__ __device__ inline int c32c_panel_floats(int d, int p)
{
    return (32 + ((c32c_rows_below(d, p) + 31) & ~31)) * kC32Stride;
}
__host__ __device__ inline size_t c32c_smem_bytes(int d, bool resident)
{
    size_t need = 0;
    for (int p = 0; p < (d + 31) / 32; ++p) {
        const size_t f = (size_t)c32c_panel_floats(d, p) + (resident ? (size_t)c32c_row0(d, p + 1) * 32 : 0);
        need = need > f ? need : f;
    }
    return ((size_t)c32c_head_floats(d) + need) * 4;
}

// Warp: lane i holds row i of the diagonal block (a[j] = A_ij for j <= i, zero above; a block of
// nb < 32 rows is padded with rows of the identity, which factor to themselves and leave the others
// alone), dref its diagonal before the factorisation.  On return column k of the factor is in
// Lbt[k * kC32Stride + i] (i >= k) and 1 / L_kk in s_rinv[k]; false if a pivot fell to 2^-18 of its
// original value or below (or is NaN): fewer than six bits of it would be left in FP32, and the
// FP64 solve takes over.
// Step k: 1 / sqrt(pivot), every lane scales its entry of column k; the entries of rows k + 1 and
// k + 2 of the column come by shuffles (the next pivot, formed by each lane as if it were row k + 1,
// is shuffled from lane k + 1), so the chain from one pivot to the next is a multiply, an fma, a
// shuffle and an rsqrt.  The column is also stored, and its update of rows k + 3 .. 31 is applied
// one step later from shared memory (loaded at the start of that step), off the chain.
__device__ __forceinline__ float c32c_rsqrt(float x)
{
    float r;   // the MUFU approximation; pivots reaching it are above 2^-100 (never subnormal)
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ bool c32c_factor_diag(float (&a)[32], float dref, float* Lbt, float* s_rinv)
{
    const int lane = threadIdx.x & 31;
    const float thr = fmaxf(0x1p-18f * dref, 0x1p-100f);
    bool bad = false;
    float piv = __shfl_sync(0xffffffffu, a[0], 0);
    float lprev = 0.0f;                               // this lane's entry of column k - 1
#pragma unroll
    for (int k = 0; k < 32; ++k) {
        {
            float4 cp[8];                             // column k - 1, rows 4 q .. 4 q + 3
            if (k >= 1) {
#pragma unroll
                for (int q = (k + 2) / 4; q < 8; ++q)
                    cp[q] = reinterpret_cast<const float4*>(Lbt + (k - 1) * kC32Stride)[q];
            }
            bad |= lane == k && !(a[k] > thr);
            const float rk = c32c_rsqrt(piv);
            const float lik = a[k] * rk;          // lane k: sqrt(pivot); lanes below: L_ik
            a[k] = lik;
            if (k + 1 < 32) {
                piv = __shfl_sync(0xffffffffu, fmaf(-lik, lik, a[k + 1]), k + 1);
                a[k + 1] = fmaf(-lik, __shfl_sync(0xffffffffu, lik, k + 1), a[k + 1]);
            }
            if (k + 2 < 32) a[k + 2] = fmaf(-lik, __shfl_sync(0xffffffffu, lik, k + 2), a[k + 2]);
            if (k >= 1) {                         // column k - 1 on rows k + 2 .. 31
#pragma unroll
                for (int q = (k + 2) / 4; q < 8; ++q) {
                    if (4 * q + 0 >= k + 2) a[4 * q + 0] = fmaf(-lprev, cp[q].x, a[4 * q + 0]);
                    if (4 * q + 1 >= k + 2) a[4 * q + 1] = fmaf(-lprev, cp[q].y, a[4 * q + 1]);
                    if (4 * q + 2 >= k + 2) a[4 * q + 2] = fmaf(-lprev, cp[q].z, a[4 * q + 2]);
                    if (4 * q + 3 >= k + 2) a[4 * q + 3] = fmaf(-lprev, cp[q].w, a[4 * q + 3]);
                }
            }
            Lbt[k * kC32Stride + lane] = lik;
            if (lane == k) s_rinv[k] = rk;
            lprev = lik;
            __syncwarp();
        }
    }
    return !__any_sync(0xffffffffu, bad);
}

// One row against the factored diagonal block: x L11^T = a (forward substitution with the block's
// columns read as float4 broadcasts).  With a = e_t the result is column t of L11^-1.
__device__ __forceinline__ void c32c_trsm_row(float (&x)[32], const float* Lbt, const float* s_rinv)
{
#pragma unroll
    for (int k = 0; k < 32; ++k) {
        x[k] *= s_rinv[k];
        const float4* col = reinterpret_cast<const float4*>(Lbt + k * kC32Stride);
#pragma unroll
        for (int q = (k + 1) / 4; q < 8; ++q) {
            const float4 c = col[q];
            if (4 * q + 0 > k) x[4 * q + 0] = fmaf(-x[k], c.x, x[4 * q + 0]);
            if (4 * q + 1 > k) x[4 * q + 1] = fmaf(-x[k], c.y, x[4 * q + 1]);
            if (4 * q + 2 > k) x[4 * q + 2] = fmaf(-x[k], c.z, x[4 * q + 2]);
            if (4 * q + 3 > k) x[4 * q + 3] = fmaf(-x[k], c.w, x[4 * q + 3]);
        }
    }
}

// L y = v in place (v: shared, zero from d to ld), by one CTA of 256 threads: per block of 32 rows
// t = v_b - L_b,<b v_<b (eight threads per row, float4 reads of the row), then v_b = L_bb^-1 t.
// Only the factor's off-diagonal blocks (rows below each diagonal block) and the blocks' inverses
// are read.
__device__ __forceinline__ void c32c_forward(const float* __restrict__ A, int ld, const float* __restrict__ linv,
                                             float* v, int d, float* s_t)
{
    const int tid = threadIdx.x, i = tid >> 3, part = tid & 7;
    for (int b0 = 0; b0 < d; b0 += 32) {
        const float4 l4 = *reinterpret_cast<const float4*>(linv + (size_t)b0 * 32 + i * 32 + part * 4);
        const float* row = A + (size_t)(b0 + i) * ld;
        float s = 0.0f;
        for (int k = part * 4; k < b0; k += 32) {
            const float4 a4 = *reinterpret_cast<const float4*>(row + k);
            s = fmaf(a4.x, v[k], s);
            s = fmaf(a4.y, v[k + 1], s);
            s = fmaf(a4.z, v[k + 2], s);
            s = fmaf(a4.w, v[k + 3], s);
        }
        s += __shfl_xor_sync(0xffffffffu, s, 1);
        s += __shfl_xor_sync(0xffffffffu, s, 2);
        s += __shfl_xor_sync(0xffffffffu, s, 4);
        if (part == 0) s_t[i] = b0 + i < d ? v[b0 + i] - s : 0.0f;      // rows past d: not data
        __syncthreads();
        float y = l4.x * s_t[part * 4];
        y = fmaf(l4.y, s_t[part * 4 + 1], y);
        y = fmaf(l4.z, s_t[part * 4 + 2], y);
        y = fmaf(l4.w, s_t[part * 4 + 3], y);
        y += __shfl_xor_sync(0xffffffffu, y, 1);
        y += __shfl_xor_sync(0xffffffffu, y, 2);
        y += __shfl_xor_sync(0xffffffffu, y, 4);
        if (part == 0 && b0 + i < d) v[b0 + i] = y;
        __syncthreads();
    }
}

// L^T z = v in place, blocks from the bottom: t = v_b - L_>b,b^T z_>b (warp w sums rows b1 + w +
// 8 s, coalesced across the block's columns), then z_b = L_bb^-T t by warp 0.
__device__ __forceinline__ void c32c_backward(const float* __restrict__ A, int ld, const float* __restrict__ linv,
                                              float* v, int d, float* s_part, float* s_t)
{
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    for (int b0 = ((d - 1) / 32) * 32; b0 >= 0; b0 -= 32) {
        const int b1 = min(d, b0 + 32);
        float lc[32];
        if (w == 0) {
            const float* Lb = linv + (size_t)b0 * 32;
#pragma unroll
            for (int r = 0; r < 32; ++r) lc[r] = Lb[r * 32 + lane];       // column lane of L_bb^-1
        }
        float s = 0.0f;
        for (int k = b1 + w; k < d; k += 8) s = fmaf(A[(size_t)k * ld + b0 + lane], v[k], s);
        s_part[w * 32 + lane] = s;
        __syncthreads();
        if (w == 0) {
            float t = v[b0 + lane];
#pragma unroll
            for (int q = 0; q < 8; ++q) t -= s_part[q * 32 + lane];
            s_t[lane] = b0 + lane < d ? t : 0.0f;                            // columns past d: not data
            __syncwarp();
            float z = 0.0f;
#pragma unroll
            for (int r = 0; r < 32; ++r) z = fmaf(lc[r], s_t[r], z);
            if (b0 + lane < d) v[b0 + lane] = z;
        }
        __syncthreads();
    }
}

// The same two solves with the factor resident in shared memory (st: column block b's rows below
// its diagonal block from row c32c_row0(d, b), 32 floats each, the float4 chunk q of row r at
// position q ^ (r & 7) so that rows written or read together fall in different banks),
// right-looking over the blocks.  Thread (i = tid / 8, part = tid % 8) holds row i, columns
// 4 part .. 4 part + 3 of every diagonal-block inverse (lin, loaded once for all the solves).
__device__ __forceinline__ void c32c_forward_res(const float* st, const float4 (&lin)[kC32ResBlocks], float* v, int d)
{
    const int tid = threadIdx.x, i = tid >> 3, part = tid & 7;
    const int nblk = (d + 31) / 32;
#pragma unroll
    for (int b = 0; b < kC32ResBlocks; ++b) {
        if (b < nblk) {
            const int b0 = 32 * b, b1 = b0 + 32, m = c32c_rows_below(d, b);
            const float4 vb = *reinterpret_cast<const float4*>(v + b0 + part * 4);
            float y = lin[b].x * vb.x;
            y = fmaf(lin[b].y, vb.y, y);
            y = fmaf(lin[b].z, vb.z, y);
            y = fmaf(lin[b].w, vb.w, y);
            y += __shfl_xor_sync(0xffffffffu, y, 1);
            y += __shfl_xor_sync(0xffffffffu, y, 2);
            y += __shfl_xor_sync(0xffffffffu, y, 4);
            __syncthreads();
            if (part == 0 && b0 + i < d) v[b0 + i] = y;
            __syncthreads();
            // rows below the block, one thread per row
            const float* blk = st + (size_t)c32c_row0(d, b) * 32;
            const float4* yv = reinterpret_cast<const float4*>(v + b0);
            for (int rr = tid; rr < m; rr += kCoopThreads) {
                const float4* row = reinterpret_cast<const float4*>(blk + (size_t)rr * 32);
                float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const float4 a4 = row[q ^ (rr & 7)], y4 = yv[q];
                    s0 = fmaf(a4.x, y4.x, s0);
                    s1 = fmaf(a4.y, y4.y, s1);
                    s2 = fmaf(a4.z, y4.z, s2);
                    s3 = fmaf(a4.w, y4.w, s3);
                }
                v[b1 + rr] -= (s0 + s1) + (s2 + s3);
            }
            __syncthreads();
        }
    }
}

// s_part: [8][32] scratch
__device__ __forceinline__ void c32c_backward_res(const float* st, const float4 (&lin)[kC32ResBlocks], float* v, int d,
                                                  float* s_part)
{
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, i = tid >> 3;
    const int nblk = (d + 31) / 32;
#pragma unroll
    for (int b = kC32ResBlocks - 1; b >= 0; --b) {
        if (b < nblk) {
            const int b0 = 32 * b, b1 = b0 + 32, m = c32c_rows_below(d, b);
            // t = v_b - L_>b,b^T z_>b: warp w sums the rows r = w + 8 s (r & 7 == w, so this lane's
            // column sits at one swizzled position)
            const float* blk = st + (size_t)c32c_row0(d, b) * 32;
            const int col = (((lane >> 2) ^ w) << 2) | (lane & 3);
            float s0 = 0.0f, s1 = 0.0f;
            int r = w;
            for (; r + 8 < m; r += 16) {
                s0 = fmaf(blk[(size_t)r * 32 + col], v[b1 + r], s0);
                s1 = fmaf(blk[(size_t)(r + 8) * 32 + col], v[b1 + r + 8], s1);
            }
            if (r < m) s0 = fmaf(blk[(size_t)r * 32 + col], v[b1 + r], s0);
            s_part[w * 32 + lane] = s0 + s1;
            __syncthreads();
            float t = v[b0 + i];
#pragma unroll
            for (int q = 0; q < 8; ++q) t -= s_part[q * 32 + i];
            if (b0 + i >= d) t = 0.0f;
            // z_j = sum_i (L_bb^-1)_ij t_i: this thread's four columns, summed over the warp's four
            // rows (lanes 8 apart), then over the eight warps
            float z0 = lin[b].x * t, z1 = lin[b].y * t, z2 = lin[b].z * t, z3 = lin[b].w * t;
#pragma unroll
            for (int o = 8; o < 32; o <<= 1) {
                z0 += __shfl_xor_sync(0xffffffffu, z0, o);
                z1 += __shfl_xor_sync(0xffffffffu, z1, o);
                z2 += __shfl_xor_sync(0xffffffffu, z2, o);
                z3 += __shfl_xor_sync(0xffffffffu, z3, o);
            }
            __syncthreads();
            if (lane < 8) {
                s_part[w * 32 + 4 * lane + 0] = z0;
                s_part[w * 32 + 4 * lane + 1] = z1;
                s_part[w * 32 + 4 * lane + 2] = z2;
                s_part[w * 32 + 4 * lane + 3] = z3;
            }
            __syncthreads();
            if (tid < 32 && b0 + tid < d) {
                float z = 0.0f;
#pragma unroll
                for (int q = 0; q < 8; ++q) z += s_part[q * 32 + tid];
                v[b0 + tid] = z;
            }
            __syncthreads();
        }
    }
}

// float-float accumulation (Dekker / Knuth two-sum, unnormalised low part): hi + lo += p + e
__device__ __forceinline__ void c32c_ff_add(float& hi, float& lo, float p, float e)
{
    const float s = __fadd_rn(hi, p);
    const float bb = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(err, e));
}

// hi + lo += (ah + al) (bh + bl): the exact product of the high parts plus the cross terms
__device__ __forceinline__ void c32c_ff_mac(float& hi, float& lo, float ah, float al, float bh, float bl)
{
    const float p = __fmul_rn(ah, bh);
    const float e = __fadd_rn(fmaf(ah, bh, -p), fmaf(ah, bl, __fmul_rn(al, bh)));
    c32c_ff_add(hi, lo, p, e);
}

__device__ __forceinline__ void c32c_timeout(const Dev& P, unsigned bid, int record)
{
    if (bid == 0 && threadIdx.x == 0) {
        *P.status = -5;
        if (record) *P.round_ctr += 1;
    }
}

// The solve of one problem by G cooperating CTAs of kCoopThreads threads (this is CTA bid).
__device__ __forceinline__ void chol32c_body(const Dev& P, const Chol32c& C, const double* __restrict__ H,
                                             const double* lptr, const double* __restrict__ g, double* dxout,
                                             double* xupd, int record, unsigned G, unsigned bid, GridSync& gs)
{
    extern __shared__ float4 c32c_smem4[];
    float* sm = reinterpret_cast<float*>(c32c_smem4);
    const int d = P.d, ld = C.ld;
    float* Lbt = sm;
    float* v = Lbt + 32 * kC32Stride;
    float* s_part = v + ld;
    float* s_t = s_part + 8 * 32;
    float* s_pre = s_t + 32;                    // [256][4]
    float* st = s_pre + 1024;                   // resident factor (CTA 0, resident mode)
    float* const top = sm + C.smem_floats;
    __shared__ float s_rinv[32];
    __shared__ int s_fail;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const double l = *lptr;

    // 1. A = lower(H) + l I, one warp per row over the grid (from the FP32 high parts)
    const float lf = (float)l;
    for (int i = (int)bid * 8 + warp; i < d; i += (int)G * 8) {
        const size_t c0i = (size_t)i * (i + 1) / 2;
        float* row = C.A + (size_t)i * ld;
        for (int j = lane; j <= i; j += 32) {
            const float a = j == i ? C.hh[c0i + j] + lf : C.hh[c0i + j];
            row[j] = a;
            if (j == i) C.diag0[i] = a;
        }
    }
    if (tid == 0) s_fail = 0;
    if (!gs.sync()) return c32c_timeout(P, bid, record);

    // 2. panels
    int p = 0;
    for (int c0 = 0; c0 < d; c0 += 32, ++p) {
        const int nb = min(32, d - c0), c1 = c0 + nb, m = d - c1, mp = (m + 31) & ~31;
        // the panel, from the diagonal block down (Ls row r = row c0 + r; zero rows past d up to a
        // multiple of 32 below the block), at the end of shared memory
        float* Ls = top - c32c_panel_floats(d, p);
        float* Lp = Ls + 32 * kC32Stride;          // the rows below the block
        const bool keep = C.resident && bid == 0;
        float* stp = st + (size_t)c32c_row0(d, p) * 32;
        for (int t = tid; t < (32 + mp) * 8; t += kCoopThreads) {
            const int r = t >> 3, q = t & 7;
            const float4 val = r < nb + m ? *reinterpret_cast<const float4*>(C.A + (size_t)(c0 + r) * ld + c0 + 4 * q)
                                          : make_float4(0.f, 0.f, 0.f, 0.f);
            *reinterpret_cast<float4*>(Ls + r * kC32Stride + 4 * q) = val;
        }
        const float dref = (warp == 0 && lane < nb) ? C.diag0[c0 + lane] : 1.0f;
        // this CTA's first tile of the trailing update: its four entries of A per thread, fetched
        // now (asynchronously) so that the update itself only computes and stores
        const int nt = mp / 32, ntiles = nt * (nt + 1) / 2, ty = tid >> 3, tx = tid & 7;
        int ti = 0, tj = (int)bid;
        while (ti < nt && tj > ti) {
            tj -= ti + 1;
            ++ti;
        }
        if ((int)bid < ntiles) {
            const float* arow = C.A + (size_t)(c1 + ti * 32 + ty) * ld + c1 + tj * 32 + tx;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint32_t sa = (uint32_t)__cvta_generic_to_shared(s_pre + tid * 4 + u);
                asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(arow + 8 * u) : "memory");
            }
            asm volatile("cp.async.commit_group;" ::: "memory");
        }
        __syncthreads();
        if (warp == 0) {
            float a[32];
            const float4* src = reinterpret_cast<const float4*>(Ls + min(lane, nb - 1) * kC32Stride);
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const float4 t4 = src[q];
                a[4 * q + 0] = t4.x;
                a[4 * q + 1] = t4.y;
                a[4 * q + 2] = t4.z;
                a[4 * q + 3] = t4.w;
            }
#pragma unroll
            for (int j = 0; j < 32; ++j)
                if (lane >= nb) a[j] = j == lane ? 1.0f : 0.0f;
                else if (j > lane) a[j] = 0.0f;
            const bool ok = c32c_factor_diag(a, dref, Lbt, s_rinv);
            if (lane == 0 && !ok) s_fail = 1;
        }
        __syncthreads();
        if (s_fail) break;
        // every panel row against the block (all CTAs, all rows); the block's owner also inverts it
        const bool owner = (unsigned)p % G == bid;
        const int nrows = m + (owner ? 32 : 0);
        for (int r = tid; r < nrows; r += kCoopThreads) {
            float x[32];
            if (r < m) {
                const float4* src = reinterpret_cast<const float4*>(Lp + r * kC32Stride);
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const float4 t4 = src[q];
                    x[4 * q + 0] = t4.x;
                    x[4 * q + 1] = t4.y;
                    x[4 * q + 2] = t4.z;
                    x[4 * q + 3] = t4.w;
                }
            } else {
#pragma unroll
                for (int j = 0; j < 32; ++j) x[j] = (j == r - m) ? 1.0f : 0.0f;
            }
            c32c_trsm_row(x, Lbt, s_rinv);
            if (r < m) {
                float4* dst = reinterpret_cast<float4*>(Lp + r * kC32Stride);
#pragma unroll
                for (int q = 0; q < 8; ++q) dst[q] = make_float4(x[4 * q], x[4 * q + 1], x[4 * q + 2], x[4 * q + 3]);
                if (keep) {
                    float4* sd = reinterpret_cast<float4*>(stp + (size_t)r * 32);
#pragma unroll
                    for (int q = 0; q < 8; ++q) sd[q ^ (r & 7)] = make_float4(x[4 * q], x[4 * q + 1], x[4 * q + 2], x[4 * q + 3]);
                } else if (!C.resident && (unsigned)r % G == bid) {
                    float4* gd = reinterpret_cast<float4*>(C.A + (size_t)(c1 + r) * ld + c0);
#pragma unroll
                    for (int q = 0; q < 8; ++q) gd[q] = make_float4(x[4 * q], x[4 * q + 1], x[4 * q + 2], x[4 * q + 3]);
                }
            } else {
                float* Lv = C.linv + (size_t)c0 * 32 + (r - m);
#pragma unroll
                for (int j = 0; j < 32; ++j) Lv[j * 32] = x[j];
            }
        }
        if (m == 0) break;
        __syncthreads();
        // trailing update A22 -= L21 L21^T over lower 32 x 32 tiles (ti, tj), tj <= ti; thread
        // (row ty, columns tx + 8 q)
        {
            asm volatile("cp.async.wait_all;" ::: "memory");
            for (int t = (int)bid; t < ntiles; t += (int)G) {
                const float4* ri = reinterpret_cast<const float4*>(Lp + (ti * 32 + ty) * kC32Stride);
                float xr[32];
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const float4 t4 = ri[q];
                    xr[4 * q + 0] = t4.x;
                    xr[4 * q + 1] = t4.y;
                    xr[4 * q + 2] = t4.z;
                    xr[4 * q + 3] = t4.w;
                }
                float acc[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const float4* rj = reinterpret_cast<const float4*>(Lp + (tj * 32 + tx + 8 * u) * kC32Stride);
                    float s = 0.0f;
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const float4 c = rj[q];
                        s = fmaf(xr[4 * q + 0], c.x, s);
                        s = fmaf(xr[4 * q + 1], c.y, s);
                        s = fmaf(xr[4 * q + 2], c.z, s);
                        s = fmaf(xr[4 * q + 3], c.w, s);
                    }
                    acc[u] = s;
                }
                float* arow = C.A + (size_t)(c1 + ti * 32 + ty) * ld + c1 + tj * 32 + tx;
                if (t == (int)bid) {
#pragma unroll
                    for (int u = 0; u < 4; ++u) arow[8 * u] = s_pre[tid * 4 + u] - acc[u];
                } else {
#pragma unroll
                    for (int u = 0; u < 4; ++u) arow[8 * u] -= acc[u];
                }
                // next tile of this CTA
                tj += (int)G;
                while (ti < nt && tj > ti) {
                    tj -= ti + 1;
                    ++ti;
                }
            }
        }
        if (!gs.sync()) return c32c_timeout(P, bid, record);
    }
    __syncthreads();
    if (s_fail) {                 // an FP32 pivot was not positive: the FP64 solve decides
        asm volatile("cp.async.wait_all;" ::: "memory");
        chol_body(P, H, 0, lptr, 0.0, g, dxout, xupd, record, G, bid, gs);
        return;
    }
    if (!gs.sync()) return c32c_timeout(P, bid, record);

    // 3. solves and refinement
    __shared__ double s_red[2][kCoopThreads / 32];
    double en_prev = 0.0;
    float4 lin[kC32ResBlocks];            // resident mode: this thread's part of every block inverse
    if (C.resident && bid == 0) {
        const int i = tid >> 3, part = tid & 7;
#pragma unroll
        for (int b = 0; b < kC32ResBlocks; ++b)
            lin[b] = b < (d + 31) / 32 ? *reinterpret_cast<const float4*>(C.linv + (size_t)b * 1024 + i * 32 + part * 4)
                                       : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    for (int it = 0;; ++it) {
        if (bid == 0) {
            for (int i = tid; i < ld; i += kCoopThreads) v[i] = i < d ? (float)(it == 0 ? g[i] : C.r[i]) : 0.0f;
            __syncthreads();
            if (C.resident) {
                c32c_forward_res(st, lin, v, d);
                c32c_backward_res(st, lin, v, d, s_part);
            } else {
                c32c_forward(C.A, ld, C.linv, v, d, s_t);
                c32c_backward(C.A, ld, C.linv, v, d, s_part, s_t);
            }
            double en = 0.0, an = 0.0;
            for (int i = tid; i < d; i += kCoopThreads) {
                const double e = (double)v[i], a = (it == 0 ? 0.0 : C.acc[i]) + e;
                C.acc[i] = a;
                const float ah = (float)a;
                C.accp[i] = ah;
                C.accp[d + i] = (float)(a - (double)ah);
                en = fma(e, e, en);
                an = fma(a, a, an);
            }
            for (int o = 16; o > 0; o >>= 1) {
                en += __shfl_xor_sync(0xffffffffu, en, o);
                an += __shfl_xor_sync(0xffffffffu, an, o);
            }
            if (lane == 0) {
                s_red[0][warp] = en;
                s_red[1][warp] = an;
            }
            __syncthreads();
            if (tid == 0) {
                en = an = 0.0;
                for (int w = 0; w < kCoopThreads / 32; ++w) {
                    en += s_red[0][w];
                    an += s_red[1][w];
                }
                // stop once the correction is small, or once the next one is predicted to be (the
                // error after this correction is about ||e_k|| ||e_k|| / ||e_k-1||)
                const double t2 = (double)C.tol * (double)C.tol;
                *C.flag = (it > 0 && (en <= t2 * an || en * en <= t2 * an * en_prev)) ? 1 : 0;
                en_prev = en;
            }
        }
        if (it >= C.refine) break;
        if (!gs.sync()) return c32c_timeout(P, bid, record);
        if (*(volatile int*)C.flag) break;
        // residual in float-float on the FP32 pairs (the FP32 pipes run 64x the FP64 one)
        for (int i = (int)bid * 8 + warp; i < d; i += (int)G * 8) {
            const size_t c0i = (size_t)i * (i + 1) / 2, r0i = (size_t)i * d - (size_t)i * (i - 1) / 2;
            float sh = 0.0f, sl = 0.0f;
            for (int j = lane; j <= i; j += 32) c32c_ff_mac(sh, sl, C.hh[c0i + j], C.hl[c0i + j], C.accp[j], C.accp[d + j]);
            for (int j = i + 1 + lane; j < d; j += 32)
                c32c_ff_mac(sh, sl, C.rh[r0i + j - i], C.rl[r0i + j - i], C.accp[j], C.accp[d + j]);
            for (int o = 16; o > 0; o >>= 1) {
                const float oh = __shfl_xor_sync(0xffffffffu, sh, o), ol = __shfl_xor_sync(0xffffffffu, sl, o);
                c32c_ff_add(sh, sl, oh, ol);
            }
            if (lane == 0) C.r[i] = g[i] - fma(l, C.acc[i], (double)sh + (double)sl);
        }
        if (!gs.sync()) return c32c_timeout(P, bid, record);
    }
    if (bid != 0) return;
    __syncthreads();
    double gn = 0.0;
    for (int i = tid; i < d; i += kCoopThreads) {
        const double dxi = C.acc[i];
        if (dxout) dxout[i] = dxi;
        if (xupd) xupd[i] = __dsub_rn(xupd[i], dxi);
        gn = fma(g[i], g[i], gn);
    }
    if (record) {   // ||g|| for the round statistics
        for (int o = 16; o > 0; o >>= 1) gn += __shfl_down_sync(0xffffffffu, gn, o);
        __shared__ double s_gs[kCoopThreads / 32];
        if (lane == 0) s_gs[warp] = gn;
        __syncthreads();
        if (tid == 0) {
            double t = 0.0;
            for (int w = 0; w < kCoopThreads / 32; ++w) t += s_gs[w];
            P.stats[0] = sqrt(t);
            const int r = *P.round_ctr;
            if (r < P.hist_cap) P.hist[r] = P.stats[0];
            *P.round_ctr = r + 1;
        }
    }
}

// H (packed upper, column-major) as FP32 pairs in column-major and row-major packed order
__global__ void k_split_pairs(const double* __restrict__ H, int d, float* hh, float* hl, float* rh, float* rl)
{
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (long long)d * (d + 1) / 2) return;
    int i, j;
    upper_ij((int)p, i, j);
    const double h = H[p];
    const float a = (float)h, b = (float)(h - (double)a);
    hh[p] = a;
    hl[p] = b;
    const size_t r = (size_t)i * d - (size_t)i * (i - 1) / 2 + j - i;
    rh[r] = a;
    rl[r] = b;
}

__global__ void __launch_bounds__(kCoopThreads, 1) k_chol32c(Dev P, Chol32c C, const double* __restrict__ H,
                                                          const double* lptr, const double* __restrict__ g,
                                                          double* dxout, double* xupd, int record)
{
    GridSync gs(P.bar, gridDim.x, C.cluster != 0);
    chol32c_body(P, C, H, lptr, g, dxout, xupd, record, gridDim.x, blockIdx.x, gs);
    gs.finish();
}

}  // namespace fednl
