// fednl_chol32.cuh -- the Option-B Newton solve of the mixed-precision round: an FP32 Cholesky
// factor in shared memory with one step of iterative refinement on a float-float residual.
//
// x_new = x - dx, (H + l I) dx = g (TrainLoop.h:1451-1476, Option B).  One CTA per system:
//   1. the augmented matrix [H + l I | g] (upper triangle, row-major packed) is loaded into shared
//      memory in FP32 and factored R^T R right-looking in panels of 32 rows: warp 0 factors the
//      32 x 32 diagonal block in registers (lane j holds column j; pivots by rsqrt, rows exchanged
//      by shuffles), every thread then solves one column of the panel rows right of the block
//      against it (R_b,rest = R_bb^-T A_b,rest), and a rank-32 update of the trailing triangle in
//      4 x 4 register tiles follows.  The augmented column becomes y = R^-T g;
//   2. R dx0 = y (blocks of 32 rows from the bottom, warp 0 solving the block in registers);
//   3. r = g - (H + l I) dx0 with H as an FP32 pair (hi + lo, kept beside the FP64 master H in
//      column-major and row-major packed order so that every row reads contiguously), accumulated
//      in float-float (about 2^-44 relative);
//   4. R^T z = r, R e = z, dx = dx0 + e in FP64; x -= dx.
// A pivot that is not positive marks the system not positive definite (status FEDNL_ENOTPD).
#pragma once

#include <cstdint>

namespace fednl_c32 {

constexpr int kT = 512;        // threads per system (128 registers a thread for the 32-wide panels)
constexpr int kNB = 32;        // panel rows

struct Job {
    int d;
    const float* Hh;       // H hi, packed upper (column-major packed: position j (j + 1) / 2 + i)
    const float* Hl;       // H lo
    const float* Hrh;      // H hi, row-major packed upper: (i, j) at i d - i (i - 1) / 2 + j - i
    const float* Hrl;      // H lo, row-major packed
    const double* lptr;    // Option-B l
    const double* g;       // [d]
    double* dx;            // [d] solution
    double* x;             // [d] x -= dx, or nullptr
    double* stats;         // stats[0] = ||g||
    double* hist;          // ||g|| per round
    int* round_ctr;
    int hist_cap;
    int* status;           // FEDNL_ENOTPD (-4) when a pivot is not positive
};

__host__ __device__ inline int pk_stride(int D) { return (D + 6) & ~3; }   // >= D + 3, multiple of 4
// floats before the panel-row buffer: the packed triangle, rounded up so that the buffer (read as
// float4) starts on a 16-byte boundary
__host__ __device__ inline int pk_offset(int D) { return (D * (D + 1) / 2 + 3) & ~3; }

// dynamic shared memory of a system of dimension d
__host__ __device__ inline size_t smem_bytes(int d)
{
    const int D = d + 1;
    return ((size_t)pk_offset(D) + (size_t)kNB * pk_stride(D) + 4 * (size_t)D + 16) * 4;
}

__device__ __forceinline__ int rp(int i, int j, int D) { return i * D - (i * (i - 1)) / 2 + j - i; }
__device__ __forceinline__ int cp(int i, int j) { return j * (j + 1) / 2 + i; }

__device__ __forceinline__ void ffa(float& hi, float& lo, float p, float e)
{
    const float s = __fadd_rn(hi, p);
    const float bb = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(err, e));
}

// acc -= (ah + al) * b, b an FP32 value
__device__ __forceinline__ void ff_sub_prod(float& hi, float& lo, float ah, float al, float b)
{
    const float p = __fmul_rn(ah, b);
    const float e = __fadd_rn(fmaf(ah, b, -p), __fmul_rn(al, b));
    ffa(hi, lo, -p, -e);
}

// R v = rhs in place (v: shared [d]), blocks of 32 rows from the bottom
__device__ __forceinline__ void back_solve(const float* A, const float* rinv, float* v, int d, int D)
{
    const int tid = threadIdx.x, lane = tid & 31;
    for (int b1 = d; b1 > 0; b1 -= 32) {
        const int b0 = b1 > 32 ? b1 - 32 : 0, nbk = b1 - b0;
        if (tid < 32) {
            float ar[32];
#pragma unroll
            for (int s = 0; s < 32; ++s) ar[s] = (lane < s && s < nbk) ? A[rp(b0 + lane, b0 + s, D)] : 0.0f;
            const float inv = lane < nbk ? rinv[b0 + lane] : 0.0f;
            float w = lane < nbk ? v[b0 + lane] : 0.0f;
#pragma unroll
            for (int s = 31; s >= 0; --s) {
                if (s < nbk) {
                    if (lane == s) w = __fmul_rn(w, inv);
                    const float xs = __shfl_sync(0xffffffffu, w, s);
                    if (lane < s) w = fmaf(-ar[s], xs, w);
                }
            }
            if (lane < nbk) v[b0 + lane] = w;
        }
        __syncthreads();
        for (int i = tid; i < b0; i += blockDim.x) {
            const float* row = A + rp(i, b0, D);
            float rv[32], w = v[i];
#pragma unroll
            for (int s = 0; s < 32; ++s) rv[s] = s < nbk ? row[s] : 0.0f;
#pragma unroll
            for (int s = 0; s < 32; ++s)
                if (s < nbk) w = fmaf(-rv[s], v[b0 + s], w);
            v[i] = w;
        }
        __syncthreads();
    }
}

// R^T v = rhs in place, blocks of 32 rows from the top
__device__ __forceinline__ void fwd_solve(const float* A, const float* rinv, float* v, int d, int D)
{
    const int tid = threadIdx.x, lane = tid & 31;
    for (int b0 = 0; b0 < d; b0 += 32) {
        const int b1 = b0 + 32 < d ? b0 + 32 : d, nbk = b1 - b0;
        if (tid < 32) {
            float ac[32];
#pragma unroll
            for (int s = 0; s < 32; ++s) ac[s] = (s < lane && lane < nbk) ? A[rp(b0 + s, b0 + lane, D)] : 0.0f;
            const float inv = lane < nbk ? rinv[b0 + lane] : 0.0f;
            float w = lane < nbk ? v[b0 + lane] : 0.0f;
#pragma unroll
            for (int s = 0; s < 32; ++s) {
                if (s < nbk) {
                    if (lane == s) w = __fmul_rn(w, inv);
                    const float zs = __shfl_sync(0xffffffffu, w, s);
                    if (lane > s) w = fmaf(-ac[s], zs, w);
                }
            }
            if (lane < nbk) v[b0 + lane] = w;
        }
        __syncthreads();
        for (int i = b1 + tid; i < d; i += blockDim.x) {
            float rv[32], w = v[i];
            int pos = rp(b0, i, D);                       // (b0 + s, i): + D - (b0 + s) - 1 per s
#pragma unroll
            for (int s = 0; s < 32; ++s) {
                rv[s] = s < nbk ? A[pos] : 0.0f;
                pos += D - (b0 + s) - 1;
            }
#pragma unroll
            for (int s = 0; s < 32; ++s)
                if (s < nbk) w = fmaf(-rv[s], v[b0 + s], w);
            v[i] = w;
        }
        __syncthreads();
    }
}

// (i, j), i <= j, of packed column-major upper position p
__device__ __forceinline__ void cp_ij(int p, int& i, int& j)
{
    int jj = (int)((sqrtf(8.0f * (float)p + 1.0f) - 1.0f) * 0.5f);
    while (jj > 0 && jj * (jj + 1) / 2 > p) --jj;
    while ((jj + 1) * (jj + 2) / 2 <= p) ++jj;
    j = jj;
    i = p - jj * (jj + 1) / 2;
}

__global__ void __launch_bounds__(kT, 1) k_chol32(const Job* __restrict__ jobs)
{
    extern __shared__ __align__(16) float sm[];
    __shared__ int s_fail;
    __shared__ double s_gn;
    __shared__ __align__(16) float s_row[kNB];
    const Job J = jobs[blockIdx.x];
    const int d = J.d, D = d + 1;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int S4 = pk_stride(D);
    float* A = sm;                                   // row-major packed upper, D (D + 1) / 2
    float* Pk = A + pk_offset(D);                    // [kNB][S4] finished panel rows (16-byte aligned)
    float* rinv = Pk + kNB * S4;                     // [D] 1 / r_ii
    float* vy = rinv + D;                            // [D] solve vector
    float* vdx = vy + D;                             // [D] dx0
    float* vr = vdx + D;                             // [D] residual / correction

    const double l = *J.lptr;
    const float lf = (float)l;
    // load [H + l I | g]: the augmented matrix's column-major packed positions coincide with H's for
    // the first d columns, so the global reads are contiguous
    const int UA = D * (D + 1) / 2;
#pragma unroll 4
    for (int p = tid; p < UA; p += kT) {
        int i, j;
        cp_ij(p, i, j);
        float v = 0.0f;
        if (j < d) {
            v = J.Hh[p];
            if (i == j) v = __fadd_rn(v, lf);
        } else if (i < d) {
            v = (float)J.g[i];
        }
        A[rp(i, j, D)] = v;
    }
    if (tid == 0) s_fail = 0;
    if (warp == 0) {
        double gs = 0.0;
        for (int i = lane; i < d; i += 32) gs = fma(J.g[i], J.g[i], gs);
        for (int o = 16; o > 0; o >>= 1) gs += __shfl_xor_sync(0xffffffffu, gs, o);
        if (lane == 0) s_gn = sqrt(gs);
    }
    __syncthreads();

    for (int c0 = 0; c0 < d; c0 += kNB) {
        const int nb = d - c0 < kNB ? d - c0 : kNB, c1 = c0 + nb;
        // 1. the diagonal block R_bb by warp 0 in registers: lane j holds column c0 + j, its rows
        //    from the current pivot row down in a[0..]; after each step the rows move up one
        //    register, so that one rolled loop body serves every step
        if (warp == 0) {
            float a[kNB];
#pragma unroll
            for (int m = 0; m < kNB; ++m) a[m] = (m <= lane && lane < nb) ? A[rp(c0 + m, c0 + lane, D)] : 0.0f;
            bool bad = false;
#pragma unroll 1
            for (int k = 0; k < nb; ++k) {
                float inv = 0.0f;
                if (lane == k) {
                    const float t = a[0];
                    bad = !(t > 0.0f);
                    inv = rsqrtf(t);
                    a[0] = __fmul_rn(t, inv);
                    rinv[c0 + k] = inv;
                }
                inv = __shfl_sync(0xffffffffu, inv, k);
                if (lane > k) a[0] = __fmul_rn(a[0], inv);             // r_{k, lane}
                s_row[lane] = a[0];
                if (lane >= k && lane < nb) A[rp(c0 + k, c0 + lane, D)] = a[0];
                __syncwarp();
#pragma unroll
                for (int m = 1; m < kNB; ++m) {
                    const int i = k + m;                                 // row of a[m]
                    const float rki = i < kNB ? s_row[i < kNB ? i : 0] : 0.0f;
                    if (lane >= i && i < nb) a[m] = fmaf(-rki, a[0], a[m]);
                }
#pragma unroll
                for (int m = 0; m + 1 < kNB; ++m) a[m] = a[m + 1];
                a[kNB - 1] = 0.0f;
                __syncwarp();
            }
            if (__any_sync(0xffffffffu, bad) && lane == 0) s_fail = 1;
        }
        __syncthreads();
        if (s_fail) break;
        // 2. the panel rows right of the block: R_b,rest = R_bb^-T A_b,rest, one column per thread
        //    (forward substitution with the same register rotation)
        for (int j = c1 + tid; j < D; j += kT) {
            float acc[kNB];
#pragma unroll
            for (int m = 0; m < kNB; ++m) acc[m] = m < nb ? A[rp(c0 + m, j, D)] : 0.0f;
#pragma unroll 1
            for (int k = 0; k < nb; ++k) {
                const float x = __fmul_rn(acc[0], rinv[c0 + k]);
                A[rp(c0 + k, j, D)] = x;
                Pk[k * S4 + j] = x;
                const float* rowk = A + rp(c0 + k, c0 + k, D);         // row k of the block: rowk[m]
#pragma unroll
                for (int m = 1; m < kNB; ++m)
                    if (k + m < nb) acc[m] = fmaf(-rowk[m], x, acc[m]);
#pragma unroll
                for (int m = 0; m + 1 < kNB; ++m) acc[m] = acc[m + 1];
                acc[kNB - 1] = 0.0f;
            }
        }
        __syncthreads();
        if (c1 >= d) break;
        // 3. trailing update: rows [c1, d), columns [c1, D), rank nb, 4 x 4 register tiles
        const int mc = D - c1, mr = d - c1;
        const int TR = (mr + 3) >> 2, TC = (mc + 3) >> 2;
        const int ntiles = TR * TC - (TR * (TR - 1)) / 2;
        for (int t = tid; t < ntiles; t += kT) {
            // tile row a holds TC - a tiles; cum(a) = a TC - a (a - 1) / 2
            int a = (int)((2.0f * TC + 1.0f - sqrtf((2.0f * TC + 1.0f) * (2.0f * TC + 1.0f) - 8.0f * t)) * 0.5f);
            if (a < 0) a = 0;
            if (a > TR - 1) a = TR - 1;
            while (a > 0 && a * TC - (a * (a - 1)) / 2 > t) --a;
            while (a + 1 < TR && (a + 1) * TC - ((a + 1) * a) / 2 <= t) ++a;
            const int b = a + (t - (a * TC - (a * (a - 1)) / 2));
            const int i0 = c1 + 4 * a, j0 = c1 + 4 * b;
            float acc[4][4];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const int i = i0 + r, j = j0 + c;
                    acc[r][c] = (i < d && j < D && j >= i) ? A[rp(i, j, D)] : 0.0f;
                }
#pragma unroll 4
            for (int q = 0; q < nb; ++q) {
                const float4 ri = *reinterpret_cast<const float4*>(Pk + q * S4 + i0);
                const float4 rj = *reinterpret_cast<const float4*>(Pk + q * S4 + j0);
                const float rv[4] = {ri.x, ri.y, ri.z, ri.w}, cv[4] = {rj.x, rj.y, rj.z, rj.w};
#pragma unroll
                for (int r = 0; r < 4; ++r)
#pragma unroll
                    for (int c = 0; c < 4; ++c) acc[r][c] = fmaf(-rv[r], cv[c], acc[r][c]);
            }
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const int i = i0 + r, j = j0 + c;
                    if (i < d && j < D && j >= i) A[rp(i, j, D)] = acc[r][c];
                }
        }
        __syncthreads();
    }
    if (s_fail) {
        if (tid == 0) {
            *J.status = -4;
            *J.round_ctr += 1;
        }
        return;
    }
    // dx0 = R^-1 y
    for (int i = tid; i < d; i += kT) vy[i] = A[rp(i, d, D)];
    __syncthreads();
    back_solve(A, rinv, vy, d, D);
    for (int i = tid; i < d; i += kT) vdx[i] = vy[i];
    __syncthreads();
    // r = g - (H + l I) dx0 in float-float, one warp per row: row i of H is column i of the
    // column-major packed upper (j < i) followed by row i of the row-major copy (j >= i)
    {
        const float lh = lf, ll = (float)(l - (double)lf);
        for (int i = warp; i < d; i += kT / 32) {
            float hi = 0.0f, lo = 0.0f;
            const int cb = i * (i + 1) / 2;                        // cp(j, i) = cb + j
            const int rb = i * d - (i * (i - 1)) / 2 - i;          // row-major (i, j) = rb + j
#pragma unroll 4
            for (int j = lane; j < d; j += 32) {
                const float hh = j < i ? J.Hh[cb + j] : J.Hrh[rb + j];
                const float hl = j < i ? J.Hl[cb + j] : J.Hrl[rb + j];
                ff_sub_prod(hi, lo, hh, hl, vdx[j]);
            }
            for (int o = 16; o > 0; o >>= 1) {
                const float oh = __shfl_xor_sync(0xffffffffu, hi, o), ol = __shfl_xor_sync(0xffffffffu, lo, o);
                ffa(hi, lo, oh, ol);
            }
            if (lane == 0) {
                const double gi = J.g[i];
                const float gh = (float)gi, gl = (float)(gi - (double)gh);
                ffa(hi, lo, gh, gl);
                ff_sub_prod(hi, lo, lh, ll, vdx[i]);
                vr[i] = __fadd_rn(hi, lo);
            }
        }
    }
    __syncthreads();
    fwd_solve(A, rinv, vr, d, D);
    back_solve(A, rinv, vr, d, D);
    for (int i = tid; i < d; i += kT) {
        const double dxi = (double)vdx[i] + (double)vr[i];
        J.dx[i] = dxi;
        if (J.x) J.x[i] = J.x[i] - dxi;
    }
    if (tid == 0) {
        J.stats[0] = s_gn;
        const int r = *J.round_ctr;
        if (r < J.hist_cap) J.hist[r] = s_gn;
        *J.round_ctr = r + 1;
    }
}

}  // namespace fednl_c32
