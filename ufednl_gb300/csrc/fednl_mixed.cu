// fednl_mixed.cu -- host side of the tensor-core (tcgen05) path: tensor maps, the feature-major
// layout of dense FP32 client data, and the operator-level weighted Gram entry point.
//
// Layout: client c's features are stored feature-major, X[c][i][s] (d rows, L columns, L = the
// largest n_i rounded up to 32, zero beyond n_c), so that a TMA box of 32 samples x 128 features is
// one 128-byte-swizzled K-major UMMA operand slab.  The per-sample weights D_s live in W[c][s]
// (zero beyond n_c, so the padding contributes nothing).

#include "fednl_gpu.h"
#include "fednl_tc.cuh"
#include "fednl_solve.h"
#include "fednl_smem.h"
#include "fednl_chol32.cuh"

#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <vector>

extern "C" const char* fednl_gpu_last_error(void);
int fednl_set_error(int code, const char* msg);   // fednl_gpu.cu

namespace {

int fail_m(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    return fednl_set_error(code, buf);
}

#define CKM(call)                                                                                  \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return fail_m(FEDNL_ECUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void* p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

// [nc][d][L] FP32, box = 32 samples x 128 features x 1 client, 128-byte swizzle
int make_feature_map(CUtensorMap* map, const float* X, int L, int d, int nc)
{
    auto fn = encode_fn();
    if (!fn) return fail_m(FEDNL_ECUDA, "cuTensorMapEncodeTiled is not available");
    cuuint64_t dims[3] = {(cuuint64_t)L, (cuuint64_t)d, (cuuint64_t)nc};
    cuuint64_t strides[2] = {(cuuint64_t)L * 4, (cuuint64_t)L * d * 4};
    cuuint32_t box[3] = {(cuuint32_t)fednl_tc::kBK, (cuuint32_t)fednl_tc::kBM, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)X, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail_m(FEDNL_ECUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return FEDNL_OK;
}

// sample-major [sum n][d] (clients in order) -> feature-major [nc][d][L], zero padding
__global__ void k_to_feature_major(const float* __restrict__ A, const int* __restrict__ soff, int d, int dp, int L,
                                   int nc, float* __restrict__ X)
{
    __shared__ float tile[32][33];
    const int c = blockIdx.z;
    const int s0 = blockIdx.x * 32, i0 = blockIdx.y * 32;
    const int n = soff[c + 1] - soff[c];
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int s = s0 + r, i = i0 + threadIdx.x;
        tile[r][threadIdx.x] = (s < n && i < d) ? A[(size_t)(soff[c] + s) * d + i] : 0.0f;
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int i = i0 + r, s = s0 + threadIdx.x;
        if (i < d && s < L) X[((size_t)c * dp + i) * L + s] = tile[threadIdx.x][r];
    }
}

__global__ void k_pad_weights(const float* __restrict__ w, const int* __restrict__ soff, int L, int nc,
                              float* __restrict__ W)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
    const int n = soff[c + 1] - soff[c];
    if (s < L) W[(size_t)c * L + s] = s < n ? w[soff[c] + s] : 0.0f;
}

}  // namespace

extern "C" int fednl_gpu_weighted_gram_tf32(const float* features, const float* weights, const int32_t* n_samples,
                                            int32_t n_clients, int32_t d, float lambda, float* out)
{
    if (!features || !weights || !n_samples || !out || n_clients < 1 || d < 128 || d % 128)
        return fail_m(FEDNL_EINVAL, "bad argument (d must be a positive multiple of 128)");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail_m(FEDNL_ENODEV, "no CUDA device available");
    std::vector<int> soff(n_clients + 1, 0);
    int maxn = 0;
    for (int c = 0; c < n_clients; ++c) {
        if (n_samples[c] < 1) return fail_m(FEDNL_EINVAL, "client %d has no samples", c);
        soff[c + 1] = soff[c] + n_samples[c];
        maxn = std::max(maxn, n_samples[c]);
    }
    const int S = soff[n_clients];
    const int L = (maxn + 31) / 32 * 32;
    float *dA = nullptr, *dw = nullptr, *dX = nullptr, *dW = nullptr, *dout = nullptr;
    int *dsoff = nullptr, *dns = nullptr, *derr = nullptr;
    auto cleanup = [&]() {
        cudaFree(dA);
        cudaFree(dw);
        cudaFree(dX);
        cudaFree(dW);
        cudaFree(dout);
        cudaFree(dsoff);
        cudaFree(dns);
        cudaFree(derr);
    };
    const size_t outN = (size_t)n_clients * d * d;
    if (cudaMalloc(&dA, (size_t)S * d * 4) != cudaSuccess || cudaMalloc(&dw, (size_t)S * 4) != cudaSuccess ||
        cudaMalloc(&dX, (size_t)n_clients * d * L * 4) != cudaSuccess ||
        cudaMalloc(&dW, (size_t)n_clients * L * 4) != cudaSuccess || cudaMalloc(&dout, outN * 4) != cudaSuccess ||
        cudaMalloc(&dsoff, (n_clients + 1) * 4) != cudaSuccess || cudaMalloc(&dns, n_clients * 4) != cudaSuccess ||
        cudaMalloc(&derr, 4) != cudaSuccess) {
        cleanup();
        return fail_m(FEDNL_ENOMEM, "device allocation failed");
    }
    int rc = FEDNL_OK;
    do {
        if (cudaMemcpy(dA, features, (size_t)S * d * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(dw, weights, (size_t)S * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(dsoff, soff.data(), (n_clients + 1) * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(dns, n_samples, n_clients * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemset(dout, 0, outN * 4) != cudaSuccess || cudaMemset(derr, 0, 4) != cudaSuccess) {
            rc = fail_m(FEDNL_ECUDA, "copies failed");
            break;
        }
        k_to_feature_major<<<dim3(L / 32, (d + 31) / 32, n_clients), dim3(32, 8)>>>(dA, dsoff, d, d, L, n_clients, dX);
        k_pad_weights<<<dim3((L + 255) / 256, n_clients), 256>>>(dw, dsoff, L, n_clients, dW);
        CUtensorMap map;
        rc = make_feature_map(&map, dX, L, d, n_clients);
        if (rc) break;
        fednl_tc::GramJob J;
        J.d = d;
        J.nc = n_clients;
        J.L = L;
        J.nbk = d / fednl_tc::kBM;
        J.tiles = J.nbk * (J.nbk + 1) / 2;
        J.ns = dns;
        J.act = nullptr;
        J.w = dW;
        J.err = derr;
        fednl_tc::EpiStore epi{dout, d, lambda};
        const size_t smem = fednl_tc::smem_bytes();
        if (cudaFuncSetAttribute(fednl_tc::k_gram_tf32<fednl_tc::EpiStore>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess) {
            rc = fail_m(FEDNL_ECUDA, "shared-memory attribute refused");
            break;
        }
        fednl_tc::k_gram_tf32<fednl_tc::EpiStore><<<n_clients * J.tiles, fednl_tc::kThreads, smem>>>(map, J, epi);
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) {
            rc = fail_m(FEDNL_ECUDA, "Gram kernel failed: %s", cudaGetErrorString(e));
            break;
        }
        int err = 0;
        cudaMemcpy(&err, derr, 4, cudaMemcpyDeviceToHost);
        if (err) {
            rc = fail_m(FEDNL_ETIMEOUT, "a bounded wait of the Gram kernel ran out");
            break;
        }
        if (cudaMemcpy(out, dout, outN * 4, cudaMemcpyDeviceToHost) != cudaSuccess) rc = fail_m(FEDNL_ECUDA, "readback failed");
    } while (0);
    cleanup();
    return rc;
}

// =================================================================================================
// The mixed-precision FedNL round (dense FP32 features, RandK-Philox, Option B): client Hessians on
// the tensor cores (TF32 x TF32 -> FP32 in TMEM) fused with the shift difference, FP32 shifts,
// float-float margins and gradients, FP64 master H, aggregation and Cholesky solve.

int fednl_device_optionb_solve(const double* H, int d, const double* lptr, const double* g, double* dx, double* xupd,
                               double* work, double* ybuf, double* rinv, unsigned* bar, int* status, double* stats,
                               double* hist, int* round_ctr, int hist_cap, int record, cudaStream_t st, int grid);

struct fednl_mx_handle_s {
    fednl_problem_desc desc{};
    std::vector<int32_t> ns, soff;
    int d = 0, dp = 0, nc = 0, L = 0, U = 0, SW = 0, k = 0, S = 0, tiles = 0, comp = 0;
    long long Up = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;       // the round graph's branch: client gradients and the aggregation
    cudaEvent_t ev_margin = nullptr, ev_lk = nullptr, ev_join = nullptr;
    std::vector<void*> allocs;
    fednl_tc::MxDev P{};
    CUtensorMap map;
    int* ns_dev = nullptr;
    int* err = nullptr;
    double *dx = nullptr, *work = nullptr, *ybuf = nullptr, *rinv = nullptr, *hist = nullptr;
    unsigned* bar = nullptr;
    int *status = nullptr, *round_ctr = nullptr;
    int hist_cap = 1 << 16;
    bool ready = false;
    int rounds_done = 0;
    size_t select_smem = 0;
    bool chol32 = false;               // the round solves with the FP32 factor + refinement
    bool chol32_ok = false;            // the system fits one CTA's shared memory
    bool coop32 = false;               // the round solves with the FP32 cooperative factor (fednl_chol32c.cuh)
    bool coop32_ok = false;            // d within that solve's shared-memory limit
    int coop32_grid = 0;               // its CTAs (0: default)
    FednlSolve32 s32{};                // its buffers
    int coop_grid = 0;                 // CTAs of the FP64 cooperative solve (0: the default heuristic)
    fednl_c32::Job* cjob = nullptr;    // device copy of the solve's job
    void* flush_buf = nullptr;
    int64_t flush_bytes = 0;
    cudaGraphExec_t gexec = nullptr;
    cudaGraph_t graph = nullptr;
    size_t dry = 0;            // footprint only: bytes the allocations would take
    bool dry_run = false;
    template <class T> int alloc(T** p, size_t n)
    {
        if (dry_run) {
            dry += (std::max<size_t>(n, 1) * sizeof(T) + 511) / 512 * 512;
            *p = nullptr;
            return FEDNL_OK;
        }
        void* q = nullptr;
        if (cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess)
            return fail_m(FEDNL_ENOMEM, "device allocation of %zu bytes failed", n * sizeof(T));
        allocs.push_back(q);
        *p = (T*)q;
        return FEDNL_OK;
    }
};

namespace {

// the round's launches; with ev, an event is recorded before each kernel and after the last
const char* const kMxKernelNames[] = {"k_mx_split_x", "k_mx_margin", "k_mx_grad", "k_mx_draw",
                                      "k_gram_tf32", "k_mx_lk", "k_mx_apply", "k_mx_aggregate", "k_chol_coop"};
const char* const kMxKernelNamesTop[] = {"k_mx_split_x", "k_mx_margin", "k_mx_grad", "k_gram_tf32",
                                         "k_mx_lk", "k_mx_select", "k_mx_apply", "k_mx_aggregate", "k_chol_coop"};
constexpr int kMxKernels = 9;

// the handle's Option-B system as a solve descriptor (dx, x -= dx, statistics of the round)
FednlSolveDesc mx_solve_desc(fednl_mx_handle h)
{
    const fednl_tc::MxDev& P = h->P;
    FednlSolveDesc S{};
    S.H = P.H;
    S.d = h->d;
    S.lptr = P.stats + 1;
    S.g = P.g;
    S.dx = h->dx;
    S.xupd = P.x;
    S.work = h->work;
    S.ybuf = h->ybuf;
    S.rinv = h->rinv;
    S.bar = h->bar;
    S.status = h->status;
    S.stats = P.stats;
    S.hist = h->hist;
    S.round_ctr = h->round_ctr;
    S.hist_cap = h->hist_cap;
    S.record = 1;
    return S;
}

int mx_launch_round(fednl_mx_handle h, cudaEvent_t* ev = nullptr, bool client_phase_only = false)
{
    using namespace fednl_tc;
    MxDev& P = h->P;
    cudaStream_t st = h->stream;
    int e = 0;
    auto mark = [&]() {
        if (ev) cudaEventRecord(ev[e++], st);
    };
    mark();
    k_mx_split_x<<<(h->d + 255) / 256, 256, 0, st>>>(P);
    mark();
    k_mx_margin<<<dim3((h->L + 63) / 64, h->nc), dim3(64, 4), 0, st>>>(P);
    mark();
    // The client gradients and the master's aggregation read only the margins' weights and Lk: in
    // a graph they run on a branch beside the Gram tiles, the selection and the shift update (kept
    // in line when the round is profiled kernel by kernel)
    const bool fork = !ev && h->side;
    if (fork) {
        CKM(cudaEventRecord(h->ev_margin, st));
        CKM(cudaStreamWaitEvent(h->side, h->ev_margin, 0));
    }
    k_mx_grad<<<(h->nc * h->d + 7) / 8, 256, 0, fork ? h->side : st>>>(P);
    mark();
    const bool randk = h->comp == FEDNL_RANDK_PHILOX;
    if (randk) {
        k_mx_draw<<<h->nc, 256, 0, st>>>(P, h->k, fednl::philox_half_bits(h->U), h->desc.seed_base);
        mark();
    }
    GramJob J{h->dp, h->nc, h->L, h->dp / kBM, h->tiles, h->ns_dev, nullptr, P.Dw, h->err};
    EpiDiff epi{P.shift, P.dsel, randk ? P.sel : nullptr, P.fpart, h->Up, h->SW, h->tiles, (float)P.lambda, h->d};
    k_gram_tf32<EpiDiff><<<h->nc * h->tiles, kThreads, smem_bytes(), st>>>(h->map, J, epi);
    mark();
    k_mx_lk<<<h->nc, 256, 0, st>>>(P);
    mark();
    if (fork) {
        CKM(cudaEventRecord(h->ev_lk, st));
        CKM(cudaStreamWaitEvent(h->side, h->ev_lk, 0));
        k_mx_aggregate<<<(h->d + 7) / 8, 256, 0, h->side>>>(P);
        CKM(cudaEventRecord(h->ev_join, h->side));
    }
    if (!randk) {
        const int toplek = h->comp == FEDNL_TOPLEK;
        k_mx_select<<<h->nc, kSelThreads, h->select_smem, st>>>(P, h->k, toplek, h->desc.toplek_seed);
        mark();
    }
    k_mx_apply<<<(h->U + 255) / 256, 256, 0, st>>>(P);
    mark();
    if (fork) {
        CKM(cudaStreamWaitEvent(st, h->ev_join, 0));
    } else {
        k_mx_aggregate<<<(h->d + 7) / 8, 256, 0, st>>>(P);
        mark();
    }
    CKM(cudaGetLastError());
    if (client_phase_only) return FEDNL_OK;
    if (h->chol32) {
        fednl_c32::k_chol32<<<1, fednl_c32::kT, fednl_c32::smem_bytes(h->d), st>>>(h->cjob);
        mark();
        CKM(cudaGetLastError());
        return FEDNL_OK;
    }
    if (h->coop32) {
        int rc = fednl_device_optionb_solve32(mx_solve_desc(h), h->s32, st, h->coop32_grid);
        mark();
        return rc;
    }
    int rc = fednl_device_optionb_solve(P.H, h->d, P.stats + 1, P.g, h->dx, P.x, h->work, h->ybuf, h->rinv, h->bar,
                                        h->status, P.stats, h->hist, h->round_ctr, h->hist_cap, 1, st, h->coop_grid);
    mark();
    return rc;
}

}  // namespace

extern "C" {

}  // extern "C"

static int mx_create_impl(const fednl_problem_desc* desc, fednl_mx_handle* out, int64_t* footprint)
{
    if (!desc || (!out && !footprint)) return fail_m(FEDNL_EINVAL, "null argument");
    if (out) *out = nullptr;
    const fednl_problem_desc& D = *desc;
    int ndev = 0;
    if (!footprint && (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0))
        return fail_m(FEDNL_ENODEV, "no CUDA device available");
    if (D.d < 1) return fail_m(FEDNL_EINVAL, "d must be >= 1");
    if (D.n_clients < 1 || !D.n_samples) return fail_m(FEDNL_EINVAL, "no clients");
    if (D.compressor != FEDNL_RANDK_PHILOX && D.compressor != FEDNL_TOPK && D.compressor != FEDNL_TOPLEK)
        return fail_m(FEDNL_EINVAL, "the mixed-precision form runs TopK, TopLEK or RandK-Philox");
    if (D.reserved) return fail_m(FEDNL_EINVAL, "reserved fields must be zero");
    if (D.arith_order != FEDNL_ORDER_FIXED)
        return fail_m(FEDNL_EINVAL, "the mixed-precision form has no reference arithmetic order");
    if (D.option_a || D.line_search || D.clients_per_round)
        return fail_m(FEDNL_EINVAL, "the mixed-precision form runs plain FedNL with Option B");
    const long long U = (long long)D.d * (D.d + 1) / 2;
    if (D.k < 1 || (D.compressor == FEDNL_RANDK_PHILOX && D.k > U)) return fail_m(FEDNL_EINVAL, "k outside [1, U]");
    if (D.compressor == FEDNL_TOPLEK && D.k < U && D.k > fednl_tc::kMxMaxLek)
        return fail_m(FEDNL_EINVAL, "TopLEK k %d above the shared-memory limit %d", D.k, fednl_tc::kMxMaxLek);
    fednl_mx_handle h = new fednl_mx_handle_s();
    h->dry_run = footprint != nullptr;
    h->desc = D;
    h->d = D.d;
    h->dp = (D.d + fednl_tc::kBM - 1) / fednl_tc::kBM * fednl_tc::kBM;
    h->comp = D.compressor;
    h->nc = D.n_clients;
    h->U = (int)U;
    h->Up = (U + 31) / 32 * 32;
    h->SW = (int)((U + 31) / 32);
    h->k = D.k;
    h->tiles = (h->dp / fednl_tc::kBM) * (h->dp / fednl_tc::kBM + 1) / 2;
    h->ns.assign(D.n_samples, D.n_samples + D.n_clients);
    h->soff.assign(h->nc + 1, 0);
    int maxn = 0;
    for (int c = 0; c < h->nc; ++c) {
        if (h->ns[c] < 1) {
            delete h;
            return fail_m(FEDNL_EINVAL, "client %d has no samples", c);
        }
        h->soff[c + 1] = h->soff[c] + h->ns[c];
        maxn = std::max(maxn, h->ns[c]);
    }
    h->S = h->soff[h->nc];
    h->L = (maxn + 31) / 32 * 32;
    fednl_tc::MxDev& P = h->P;
    P.d = h->d;
    P.dp = h->dp;
    P.nc = h->nc;
    P.L = h->L;
    P.U = h->U;
    P.Up = h->Up;
    P.SW = h->SW;
    P.tiles = h->tiles;
    P.lambda = D.lambda;
    P.alpha = D.alpha;
    P.inv_n = 1.0 / (double)h->nc;
    P.prescale = P.inv_n * D.alpha;
    P.mult = D.compressor == FEDNL_RANDK_PHILOX ? (double)U / (double)h->k : 1.0;     // RandK.h:90 / TopK
    P.multf = (float)P.mult;
    P.alphaf = (float)D.alpha;
    const size_t ncL = (size_t)h->nc * h->L, ncUp = (size_t)h->nc * h->Up;
    int rc = 0;
    float* X;
    double* lab;
    rc |= h->alloc(&h->ns_dev, h->nc);
    rc |= h->alloc(&X, (size_t)h->nc * h->dp * h->L);
    rc |= h->alloc(&lab, ncL);
    rc |= h->alloc(&P.x, h->d);
    rc |= h->alloc(&P.xh, h->d);
    rc |= h->alloc(&P.xl, h->d);
    rc |= h->alloc(&P.Dw, ncL);
    rc |= h->alloc(&P.qh, ncL);
    rc |= h->alloc(&P.ql, ncL);
    rc |= h->alloc(&P.gc, (size_t)h->nc * h->d);
    rc |= h->alloc(&P.g, h->d);
    rc |= h->alloc(&P.H, h->U);
    rc |= h->alloc(&P.Hh, h->U);
    rc |= h->alloc(&P.Hl, h->U);
    rc |= h->alloc(&P.Hrh, h->U);
    rc |= h->alloc(&P.Hrl, h->U);
    rc |= h->alloc(&h->cjob, 1);
    rc |= h->alloc(&P.shift, ncUp);
    rc |= h->alloc(&P.dsel, ncUp);
    rc |= h->alloc(&P.sel, (size_t)h->nc * h->SW);
    rc |= h->alloc(&P.draws, h->nc);
    rc |= h->alloc(&P.fpart, (size_t)h->nc * h->tiles * 128);
    rc |= h->alloc(&P.lk, h->nc);
    rc |= h->alloc(&P.cnt, h->nc);
    rc |= h->alloc(&P.stats, 4);
    rc |= h->alloc(&h->err, 1);
    rc |= h->alloc(&h->dx, h->d);
    rc |= h->alloc(&h->work, fednl_chol_work_elems(h->d));
    rc |= h->alloc(&h->ybuf, h->d);
    rc |= h->alloc(&h->rinv, h->d);
    rc |= h->alloc(&h->hist, h->hist_cap);
    rc |= h->alloc(&h->bar, 4);
    rc |= h->alloc(&h->status, 1);
    rc |= h->alloc(&h->round_ctr, 1);
    h->coop32_ok = h->d <= fednl_solve32_max_d();
    if (h->coop32_ok) {
        const size_t ld = (size_t)((h->d + 31) & ~31);
        rc |= h->alloc(&h->s32.a, ld * ld);
        rc |= h->alloc(&h->s32.diag0, h->d);
        rc |= h->alloc(&h->s32.linv, ld * 32);
        rc |= h->alloc(&h->s32.r, h->d);
        rc |= h->alloc(&h->s32.acc, h->d);
        rc |= h->alloc(&h->s32.accp, 2 * (size_t)h->d);
        h->s32.hh = P.Hh;
        h->s32.hl = P.Hl;
        h->s32.rh = P.Hrh;
        h->s32.rl = P.Hrl;
        rc |= h->alloc(&h->s32.flag, 1);
        h->s32.refine = 6;
        h->s32.tol = 0x1p-30f;
    }
    if (footprint) {     // plus the upload's staging copy of the sample-major features
        *footprint = (int64_t)h->dry + (int64_t)h->S * h->d * 4 + (int64_t)(h->nc + 1) * 4 + 4096;
        delete h;
        return FEDNL_OK;
    }
    if (rc || cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_margin, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_lk, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming) != cudaSuccess) {
        fednl_mx_destroy(h);
        return rc ? rc : fail_m(FEDNL_ECUDA, "stream creation failed");
    }
    P.X = X;
    P.lab = lab;
    P.ns = h->ns_dev;
    if (cudaMemcpy(h->ns_dev, h->ns.data(), h->nc * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(X, 0, (size_t)h->nc * h->dp * h->L * 4) != cudaSuccess || cudaMemset(lab, 0, ncL * 8) != cudaSuccess ||
        cudaMemset(P.Dw, 0, ncL * 4) != cudaSuccess || cudaMemset(P.qh, 0, ncL * 4) != cudaSuccess ||
        cudaMemset(P.ql, 0, ncL * 4) != cudaSuccess || cudaMemset(P.dsel, 0, ncUp * 4) != cudaSuccess ||
        cudaMemset(P.draws, 0, h->nc * 4) != cudaSuccess || cudaMemset(h->err, 0, 4) != cudaSuccess ||
        cudaMemset(h->bar, 0, 16) != cudaSuccess || cudaMemset(h->status, 0, 4) != cudaSuccess ||
        cudaMemset(h->round_ctr, 0, 4) != cudaSuccess || cudaMemset(P.stats, 0, 32) != cudaSuccess) {
        fednl_mx_destroy(h);
        return fail_m(FEDNL_ECUDA, "initial copies failed");
    }
    rc = make_feature_map(&h->map, X, h->L, h->dp, h->nc);
    if (rc || cudaFuncSetAttribute(fednl_tc::k_gram_tf32<fednl_tc::EpiDiff>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)fednl_tc::smem_bytes()) != cudaSuccess ||
        cudaFuncSetAttribute(fednl_tc::k_gram_tf32<fednl_tc::EpiInitShift>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fednl_tc::smem_bytes()) != cudaSuccess) {
        fednl_mx_destroy(h);
        return rc ? rc : fail_m(FEDNL_ECUDA, "shared-memory attribute refused");
    }
    {   // the FP32 solve when the augmented system fits in one CTA's shared memory
        int dev = 0, optin = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        const size_t need = fednl_c32::smem_bytes(h->d);
        if (need + 1024 <= (size_t)optin &&
            fednl_raise_dyn_smem((const void*)fednl_c32::k_chol32, need) == cudaSuccess) {
            fednl_c32::Job J{};
            J.d = h->d;
            J.Hh = P.Hh;
            J.Hl = P.Hl;
            J.Hrh = P.Hrh;
            J.Hrl = P.Hrl;
            J.lptr = P.stats + 1;
            J.g = P.g;
            J.dx = h->dx;
            J.x = P.x;
            J.stats = P.stats;
            J.hist = h->hist;
            J.round_ctr = h->round_ctr;
            J.hist_cap = h->hist_cap;
            J.status = h->status;
            if (cudaMemcpy(h->cjob, &J, sizeof(J), cudaMemcpyHostToDevice) != cudaSuccess) {
                fednl_mx_destroy(h);
                return fail_m(FEDNL_ECUDA, "initial copies failed");
            }
            h->chol32_ok = true;
        }
    }
    if (h->comp == FEDNL_TOPLEK && h->k < h->U) {     // TopLEK sorts its kept set in shared memory
        int kp = 1;
        while (kp < h->k) kp <<= 1;
        h->select_smem = ((size_t)std::max(kp, fednl_tc::kSelThreads) + 2048) * 8;
        if (fednl_raise_dyn_smem((const void*)fednl_tc::k_mx_select, h->select_smem) != cudaSuccess) {
            fednl_mx_destroy(h);
            return fail_m(FEDNL_ECUDA, "shared-memory attribute refused");
        }
    }
    *out = h;
    return FEDNL_OK;
}

extern "C" {

int fednl_mx_create(const fednl_problem_desc* desc, fednl_mx_handle* out)
{
    if (!out) return fail_m(FEDNL_EINVAL, "null argument");
    return mx_create_impl(desc, out, nullptr);
}

int fednl_mx_footprint(const fednl_problem_desc* desc, int64_t* bytes)
{
    if (!bytes) return fail_m(FEDNL_EINVAL, "null argument");
    return mx_create_impl(desc, nullptr, bytes);
}

int fednl_mx_destroy(fednl_mx_handle h)
{
    if (!h) return FEDNL_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    if (h->graph) cudaGraphDestroy(h->graph);
    for (void* p : h->allocs) cudaFree(p);
    if (h->flush_buf) cudaFree(h->flush_buf);
    if (h->stream) cudaStreamDestroy(h->stream);
    if (h->side) cudaStreamDestroy(h->side);
    for (cudaEvent_t e : {h->ev_margin, h->ev_lk, h->ev_join})
        if (e) cudaEventDestroy(e);
    delete h;
    return FEDNL_OK;
}

int fednl_mx_upload_client_data(fednl_mx_handle h, const float* features, const double* labels)
{
    if (!h || !features || !labels) return fail_m(FEDNL_EINVAL, "null argument");
    for (int s = 0; s < h->S; ++s)
        if (labels[s] != 1.0 && labels[s] != -1.0) return fail_m(FEDNL_EINVAL, "label %d is not +-1", s);
    // stream-ordered staging on the handle's own stream: the upload neither waits for nor stalls
    // other handles' work (a serving loop admits problems while others run)
    cudaStream_t st = h->stream;
    float* dA = nullptr;
    int* dsoff = nullptr;
    if (cudaMallocAsync((void**)&dA, (size_t)h->S * h->d * 4, st) != cudaSuccess ||
        cudaMallocAsync((void**)&dsoff, (h->nc + 1) * 4, st) != cudaSuccess) {
        if (dA) cudaFreeAsync(dA, st);
        cudaStreamSynchronize(st);
        return fail_m(FEDNL_ENOMEM, "staging allocation failed");
    }
    std::vector<double> labp((size_t)h->nc * h->L, 0.0);
    for (int c = 0; c < h->nc; ++c)
        for (int s = 0; s < h->ns[c]; ++s) labp[(size_t)c * h->L + s] = labels[h->soff[c] + s];
    int rc = FEDNL_OK;
    if (cudaMemcpyAsync(dA, features, (size_t)h->S * h->d * 4, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(dsoff, h->soff.data(), (h->nc + 1) * 4, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync((void*)h->P.lab, labp.data(), labp.size() * 8, cudaMemcpyHostToDevice, st) != cudaSuccess) {
        rc = fail_m(FEDNL_ECUDA, "upload failed");
    } else {
        k_to_feature_major<<<dim3(h->L / 32, (h->d + 31) / 32, h->nc), dim3(32, 8), 0, st>>>(
            dA, dsoff, h->d, h->dp, h->L, h->nc, (float*)h->P.X);
        if (cudaGetLastError() != cudaSuccess) rc = fail_m(FEDNL_ECUDA, "layout kernel failed");
    }
    cudaFreeAsync(dA, st);
    cudaFreeAsync(dsoff, st);
    if (cudaStreamSynchronize(st) != cudaSuccess && rc == FEDNL_OK) rc = fail_m(FEDNL_ECUDA, "upload failed");
    return rc;
}

int fednl_mx_init_shifts(fednl_mx_handle h, const double* x0)
{
    using namespace fednl_tc;
    if (!h) return fail_m(FEDNL_EINVAL, "null handle");
    MxDev& P = h->P;
    cudaStream_t st = h->stream;
    if (x0) CKM(cudaMemcpyAsync(P.x, x0, h->d * 8, cudaMemcpyHostToDevice, st));
    else CKM(cudaMemsetAsync(P.x, 0, h->d * 8, st));
    k_mx_split_x<<<(h->d + 255) / 256, 256, 0, st>>>(P);
    k_mx_margin<<<dim3((h->L + 63) / 64, h->nc), dim3(64, 4), 0, st>>>(P);
    GramJob J{h->dp, h->nc, h->L, h->dp / kBM, h->tiles, h->ns_dev, nullptr, P.Dw, h->err};
    EpiInitShift epi{P.shift, h->Up, (float)P.lambda, h->d};
    k_gram_tf32<EpiInitShift><<<h->nc * h->tiles, kThreads, smem_bytes(), st>>>(h->map, J, epi);
    k_mx_hinit<<<(h->U + 255) / 256, 256, 0, st>>>(P);
    CKM(cudaGetLastError());
    CKM(cudaStreamSynchronize(st));
    int err = 0;
    CKM(cudaMemcpy(&err, h->err, 4, cudaMemcpyDeviceToHost));
    if (err) return fail_m(FEDNL_ETIMEOUT, "a bounded wait of the Gram kernel ran out");
    h->ready = true;
    h->rounds_done = 0;
    return FEDNL_OK;
}

int fednl_mx_run(fednl_mx_handle h, int32_t rounds, double* grad_norms)
{
    if (!h || !h->ready) return fail_m(FEDNL_EINVAL, "call fednl_mx_init_shifts first");
    if (!h->gexec) {
        CKM(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        int rc = mx_launch_round(h);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(h->stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return fail_m(FEDNL_ECUDA, "graph capture failed: %s", cudaGetErrorString(e));
        h->graph = g;
        CKM(cudaGraphInstantiate(&h->gexec, g, 0));
    }
    for (int r = 0; r < rounds; ++r) CKM(cudaGraphLaunch(h->gexec, h->stream));
    CKM(cudaStreamSynchronize(h->stream));
    const int first = h->rounds_done;
    h->rounds_done += rounds;
    if (grad_norms && rounds > 0) {
        const int have = std::max(0, std::min(rounds, h->hist_cap - first));
        if (have) CKM(cudaMemcpy(grad_norms, h->hist + first, (size_t)have * 8, cudaMemcpyDeviceToHost));
    }
    int err = 0, status = 0;
    CKM(cudaMemcpy(&err, h->err, 4, cudaMemcpyDeviceToHost));
    CKM(cudaMemcpy(&status, h->status, 4, cudaMemcpyDeviceToHost));
    if (err) return fail_m(FEDNL_ETIMEOUT, "a bounded wait of the Gram kernel ran out");
    if (status == FEDNL_ETIMEOUT) return fail_m(status, "grid barrier of the Cholesky timed out");
    if (status) return fail_m(status, "Option-B matrix not positive definite in one of the rounds");
    return FEDNL_OK;
}

int fednl_mx_time_rounds(fednl_mx_handle h, int32_t rounds, int64_t flush_bytes, double* total_ms,
                         double* per_round_ms)
{
    if (!h || rounds < 1 || !total_ms || flush_bytes < 0) return fail_m(FEDNL_EINVAL, "bad argument");
    int rc = fednl_mx_run(h, 0, nullptr);      // builds the graph
    if (rc) return rc;
    if (flush_bytes > h->flush_bytes) {        // a buffer larger than L2, written before every round
        if (h->flush_buf) cudaFree(h->flush_buf);
        h->flush_buf = nullptr;
        h->flush_bytes = 0;
        CKM(cudaMalloc(&h->flush_buf, (size_t)flush_bytes));
        h->flush_bytes = flush_bytes;
    }
    std::vector<cudaEvent_t> ev(2 * (size_t)rounds);
    for (auto& e : ev) CKM(cudaEventCreate(&e));
    for (int r = 0; r < rounds; ++r) {
        if (flush_bytes) CKM(cudaMemsetAsync(h->flush_buf, r & 0xFF, (size_t)flush_bytes, h->stream));
        CKM(cudaEventRecord(ev[2 * r], h->stream));
        CKM(cudaGraphLaunch(h->gexec, h->stream));
        CKM(cudaEventRecord(ev[2 * r + 1], h->stream));
    }
    CKM(cudaStreamSynchronize(h->stream));
    double tot = 0.0;
    for (int r = 0; r < rounds; ++r) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev[2 * r], ev[2 * r + 1]);
        tot += ms;
        if (per_round_ms) per_round_ms[r] = ms;
    }
    *total_ms = tot;
    for (auto& e : ev) cudaEventDestroy(e);
    h->rounds_done += rounds;
    int err = 0, status = 0;
    CKM(cudaMemcpy(&err, h->err, 4, cudaMemcpyDeviceToHost));
    CKM(cudaMemcpy(&status, h->status, 4, cudaMemcpyDeviceToHost));
    if (err) return fail_m(FEDNL_ETIMEOUT, "a bounded wait of the Gram kernel ran out");
    if (status) return fail_m(status, "Option-B solve failed in one of the timed rounds");
    return FEDNL_OK;
}

int fednl_mx_profile_kernels(fednl_mx_handle h, int32_t rounds, double* kernel_ms, char* names, int32_t names_len)
{
    if (!h || !h->ready || rounds < 1 || !kernel_ms) return fail_m(FEDNL_EINVAL, "bad argument");
    std::vector<cudaEvent_t> ev((size_t)rounds * (kMxKernels + 1));
    for (auto& e : ev) CKM(cudaEventCreate(&e));
    int rc = FEDNL_OK;
    for (int r = 0; r < rounds && !rc; ++r) rc = mx_launch_round(h, &ev[(size_t)r * (kMxKernels + 1)]);
    CKM(cudaStreamSynchronize(h->stream));
    for (int t = 0; t < kMxKernels; ++t) {
        double acc = 0.0;
        for (int r = 0; r < rounds; ++r) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev[(size_t)r * (kMxKernels + 1) + t], ev[(size_t)r * (kMxKernels + 1) + t + 1]);
            acc += ms;
        }
        kernel_ms[t] = acc / rounds;
    }
    for (auto& e : ev) cudaEventDestroy(e);
    if (names && names_len > 0) {
        std::string all;
        const char* const* nm = h->comp == FEDNL_RANDK_PHILOX ? kMxKernelNames : kMxKernelNamesTop;
        for (int t = 0; t < kMxKernels; ++t)
            all += std::string(t ? ";" : "") +
                   (t == kMxKernels - 1 && h->chol32 ? "k_chol32" : t == kMxKernels - 1 && h->coop32 ? "k_chol32c" : nm[t]);
        snprintf(names, (size_t)names_len, "%s", all.c_str());
    }
    h->rounds_done += rounds;
    return rc;
}

int fednl_mx_set_solver(fednl_mx_handle h, int32_t solver)
{
    if (!h || solver < 0 || solver > 2) return fail_m(FEDNL_EINVAL, "bad argument");
    if (solver == 1 && !h->chol32_ok) return fail_m(FEDNL_EINVAL, "d %d too large for the shared-memory solve", h->d);
    if (solver == 2 && !h->coop32_ok)
        return fail_m(FEDNL_EINVAL, "d %d above the FP32 cooperative solve's limit %d", h->d, fednl_solve32_max_d());
    if ((solver == 1) != h->chol32 || (solver == 2) != h->coop32) {
        if (h->gexec) {
            cudaGraphExecDestroy(h->gexec);
            cudaGraphDestroy(h->graph);
            h->gexec = nullptr;
            h->graph = nullptr;
        }
    }
    h->chol32 = solver == 1;
    h->coop32 = solver == 2;
    return FEDNL_OK;
}

int fednl_mx_autotune(fednl_mx_handle h, int32_t* solver_out, int32_t* grid_out, double* solve_ms)
{
    if (!h || !h->ready) return fail_m(FEDNL_EINVAL, "call fednl_mx_init_shifts first");
    static std::mutex mu;
    struct Choice {
        int solver, grid, grid32;
        double ms;
    };
    static std::map<int, Choice> cache;                    // per d
    CKM(cudaStreamSynchronize(h->stream));
    int solver = 0, grid = 0, grid32 = 0;
    double best = 0.0;
    bool cached = false;
    {
        std::lock_guard<std::mutex> g(mu);
        auto it = cache.find(h->d);
        if (it != cache.end()) {
            solver = it->second.solver;
            grid = it->second.grid;
            grid32 = it->second.grid32;
            best = it->second.ms;
            cached = true;
        }
    }
    if (!cached) {
        // scratch outputs: the handle's iterate, statistics and history stay as they are
        double *sdx = nullptr, *sstats = nullptr, *shist = nullptr;
        int *sstatus = nullptr, *sctr = nullptr;
        fednl_c32::Job* sjob = nullptr;
        if (cudaMalloc(&sdx, (size_t)h->d * 8) || cudaMalloc(&sstats, 32) || cudaMalloc(&shist, 8) ||
            cudaMalloc(&sstatus, 4) || cudaMalloc(&sctr, 4) || cudaMalloc(&sjob, sizeof(fednl_c32::Job))) {
            cudaFree(sdx);
            cudaFree(sstats);
            cudaFree(shist);
            cudaFree(sstatus);
            cudaFree(sctr);
            return fail_m(FEDNL_ENOMEM, "tuning scratch allocation failed");
        }
        cudaMemset(sctr, 0, 4);
        const fednl_tc::MxDev& P = h->P;
        cudaStream_t st = h->stream;
        auto launch = [&](int G) -> int {
            return fednl_device_optionb_solve(P.H, h->d, P.stats + 1, P.g, sdx, nullptr, h->work, h->ybuf, h->rinv,
                                              h->bar, sstatus, sstats, shist, sctr, 1, 0, st, G);
        };
        double coop_ms = 0.0;
        int rc = fednl_tune_chol_grid(h->d, launch, st, &grid, &coop_ms);
        solver = 0;
        best = coop_ms;
        if (!rc && h->chol32_ok) {
            fednl_c32::Job J{};
            cudaMemcpy(&J, h->cjob, sizeof(J), cudaMemcpyDeviceToHost);
            J.dx = sdx;
            J.x = nullptr;
            J.stats = sstats;
            J.hist = shist;
            J.round_ctr = sctr;
            J.hist_cap = 1;
            J.status = sstatus;
            cudaMemcpy(sjob, &J, sizeof(J), cudaMemcpyHostToDevice);
            cudaEvent_t e0, e1;
            cudaEventCreate(&e0);
            cudaEventCreate(&e1);
            float b32 = 1e30f;
            for (int rep = 0; rep < 4; ++rep) {
                cudaEventRecord(e0, st);
                fednl_c32::k_chol32<<<1, fednl_c32::kT, fednl_c32::smem_bytes(h->d), st>>>(sjob);
                cudaEventRecord(e1, st);
                cudaEventSynchronize(e1);
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (rep) b32 = std::min(b32, ms);
            }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            if (cudaGetLastError() != cudaSuccess) rc = fail_m(FEDNL_ECUDA, "tuning launch failed");
            else if (b32 < best) {
                solver = 1;
                best = b32;
            }
        }
        if (!rc && h->coop32_ok) {
            FednlSolveDesc S = mx_solve_desc(h);
            S.dx = sdx;
            S.xupd = nullptr;
            S.stats = sstats;
            S.hist = shist;
            S.round_ctr = sctr;
            S.hist_cap = 1;
            S.status = sstatus;
            auto launch32 = [&](int G) -> int { return fednl_device_optionb_solve32(S, h->s32, st, G); };
            double ms32 = 0.0;
            rc = fednl_tune_chol32_grid(h->d, launch32, st, &grid32, &ms32);
            if (!rc && cudaStreamSynchronize(st) != cudaSuccess) rc = fail_m(FEDNL_ECUDA, "tuning launch failed");
            if (!rc && ms32 < best) {
                solver = 2;
                best = ms32;
            }
        }
        cudaFree(sdx);
        cudaFree(sstats);
        cudaFree(shist);
        cudaFree(sstatus);
        cudaFree(sctr);
        cudaFree(sjob);
        if (rc) return rc;
        std::lock_guard<std::mutex> g(mu);
        cache[h->d] = {solver, grid, grid32, best};
    }
    h->coop32_grid = grid32;
    if (grid != h->coop_grid && h->gexec) {
        cudaGraphExecDestroy(h->gexec);
        cudaGraphDestroy(h->graph);
        h->gexec = nullptr;
        h->graph = nullptr;
    }
    h->coop_grid = grid;
    int rc = fednl_mx_set_solver(h, solver);
    if (rc) return rc;
    if (solver_out) *solver_out = solver;
    if (grid_out) *grid_out = solver == 2 ? grid32 : grid;
    if (solve_ms) *solve_ms = best;
    return FEDNL_OK;
}

int fednl_mx_client_phase(fednl_mx_handle h)
{
    if (!h || !h->ready) return fail_m(FEDNL_EINVAL, "call fednl_mx_init_shifts first");
    CKM(cudaMemsetAsync(h->status, 0, 4, h->stream));
    return mx_launch_round(h, nullptr, true);
}

int fednl_mx_round_result(fednl_mx_handle h, fednl_round_stats* stats)
{
    if (!h || !h->ready) return fail_m(FEDNL_EINVAL, "call fednl_mx_init_shifts first");
    CKM(cudaStreamSynchronize(h->stream));
    double st[2] = {0, 0};
    int err = 0, status = 0;
    CKM(cudaMemcpy(st, h->P.stats, 16, cudaMemcpyDeviceToHost));
    CKM(cudaMemcpy(&err, h->err, 4, cudaMemcpyDeviceToHost));
    CKM(cudaMemcpy(&status, h->status, 4, cudaMemcpyDeviceToHost));
    if (stats) {
        stats->round = h->rounds_done - 1;
        stats->status = status == FEDNL_ENOTPD ? FEDNL_ENOTPD : FEDNL_OK;
        stats->grad_norm = st[0];
        stats->l = st[1];
    }
    if (err) return fail_m(FEDNL_ETIMEOUT, "a bounded wait of the Gram kernel ran out");
    if (status == FEDNL_ETIMEOUT) return fail_m(status, "grid barrier of the Cholesky timed out");
    if (status) return fail_m(status, "Option-B matrix not positive definite");
    return FEDNL_OK;
}

}  // extern "C"

int fednl_mx_uses_chol32(fednl_mx_handle h) { return h && h->chol32 ? 1 : 0; }

extern "C" int fednl_gpu_optionb_solve_mixed(const double* H, int32_t d, int32_t lda, double l, const double* g,
                                             double* dx)
{
    if (!H || !g || !dx || d < 1 || lda < d) return fail_m(FEDNL_EINVAL, "bad argument");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail_m(FEDNL_ENODEV, "no CUDA device available");
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const size_t need = fednl_c32::smem_bytes(d);
    if (need + 1024 > (size_t)optin) return fail_m(FEDNL_EINVAL, "d %d too large for the shared-memory solve", d);
    CKM(fednl_raise_dyn_smem((const void*)fednl_c32::k_chol32, need));
    const size_t U = (size_t)d * (d + 1) / 2;
    std::vector<float> hh(U), hl(U), rh(U), rl(U);
    for (int j = 0; j < d; ++j)
        for (int i = 0; i <= j; ++i) {
            const double v = H[(size_t)j * lda + i];
            const float a = (float)v, b = (float)(v - (double)a);
            hh[(size_t)j * (j + 1) / 2 + i] = a;
            hl[(size_t)j * (j + 1) / 2 + i] = b;
            const size_t r = (size_t)i * d - (size_t)i * (i - 1) / 2 + j - i;
            rh[r] = a;
            rl[r] = b;
        }
    float *dHh = nullptr, *dHl = nullptr, *dRh = nullptr, *dRl = nullptr;
    double *dl = nullptr, *dg = nullptr, *ddx = nullptr, *dst = nullptr, *dhist = nullptr;
    int *dctr = nullptr, *dstatus = nullptr;
    fednl_c32::Job* dj = nullptr;
    int rc = FEDNL_OK;
    if (cudaMalloc(&dHh, U * 4) || cudaMalloc(&dHl, U * 4) || cudaMalloc(&dRh, U * 4) || cudaMalloc(&dRl, U * 4) ||
        cudaMalloc(&dl, 8) || cudaMalloc(&dg, d * 8) ||
        cudaMalloc(&ddx, d * 8) || cudaMalloc(&dst, 32) || cudaMalloc(&dhist, 8) || cudaMalloc(&dctr, 4) ||
        cudaMalloc(&dstatus, 4) || cudaMalloc(&dj, sizeof(fednl_c32::Job))) {
        rc = fail_m(FEDNL_ENOMEM, "device allocation failed");
    } else {
        fednl_c32::Job J{};
        J.d = d;
        J.Hh = dHh;
        J.Hl = dHl;
        J.Hrh = dRh;
        J.Hrl = dRl;
        J.lptr = dl;
        J.g = dg;
        J.dx = ddx;
        J.x = nullptr;
        J.stats = dst;
        J.hist = dhist;
        J.round_ctr = dctr;
        J.hist_cap = 1;
        J.status = dstatus;
        if (cudaMemcpy(dHh, hh.data(), U * 4, cudaMemcpyHostToDevice) ||
            cudaMemcpy(dHl, hl.data(), U * 4, cudaMemcpyHostToDevice) ||
            cudaMemcpy(dRh, rh.data(), U * 4, cudaMemcpyHostToDevice) ||
            cudaMemcpy(dRl, rl.data(), U * 4, cudaMemcpyHostToDevice) || cudaMemcpy(dl, &l, 8, cudaMemcpyHostToDevice) ||
            cudaMemcpy(dg, g, d * 8, cudaMemcpyHostToDevice) || cudaMemset(dctr, 0, 4) || cudaMemset(dstatus, 0, 4) ||
            cudaMemcpy(dj, &J, sizeof(J), cudaMemcpyHostToDevice)) {
            rc = fail_m(FEDNL_ECUDA, "copies failed");
        } else {
            fednl_c32::k_chol32<<<1, fednl_c32::kT, need>>>(dj);
            int status = 0;
            if (cudaDeviceSynchronize() != cudaSuccess ||
                cudaMemcpy(&status, dstatus, 4, cudaMemcpyDeviceToHost) != cudaSuccess)
                rc = fail_m(FEDNL_ECUDA, "solve kernel failed");
            else if (status)
                rc = fail_m(status, "matrix not positive definite");
            else if (cudaMemcpy(dx, ddx, d * 8, cudaMemcpyDeviceToHost) != cudaSuccess)
                rc = fail_m(FEDNL_ECUDA, "copy back failed");
        }
    }
    cudaFree(dHh);
    cudaFree(dHl);
    cudaFree(dRh);
    cudaFree(dRl);
    cudaFree(dl);
    cudaFree(dg);
    cudaFree(ddx);
    cudaFree(dst);
    cudaFree(dhist);
    cudaFree(dctr);
    cudaFree(dstatus);
    cudaFree(dj);
    return rc;
}

int fednl_mx_solve32_batch(fednl_mx_handle const* hs, int n, void* stream)
{
    if (n <= 0) return FEDNL_OK;
    cudaStream_t st = (cudaStream_t)stream;
    static fednl_c32::Job* djobs = nullptr;
    static int cap = 0;
    std::vector<fednl_c32::Job> jobs(n);
    size_t smem = 0;
    for (int i = 0; i < n; ++i) {
        CKM(cudaMemcpy(&jobs[i], hs[i]->cjob, sizeof(fednl_c32::Job), cudaMemcpyDeviceToHost));
        smem = std::max(smem, fednl_c32::smem_bytes(hs[i]->d));
    }
    if (cap < n) {
        if (djobs) cudaFree(djobs);
        djobs = nullptr;
        cap = 0;
        CKM(cudaMalloc(&djobs, sizeof(fednl_c32::Job) * n));
        cap = n;
    }
    CKM(cudaMemcpyAsync(djobs, jobs.data(), sizeof(fednl_c32::Job) * n, cudaMemcpyHostToDevice, st));
    fednl_c32::k_chol32<<<n, fednl_c32::kT, smem, st>>>(djobs);
    CKM(cudaGetLastError());
    CKM(cudaStreamSynchronize(st));
    return FEDNL_OK;
}

extern "C" {

void* fednl_mx_stream(fednl_mx_handle h) { return h ? (void*)h->stream : nullptr; }

int fednl_mx_solve_desc(fednl_mx_handle h, FednlSolveDesc* S, void** stream)
{
    if (!h || !h->ready || !S) return FEDNL_EINVAL;
    *S = mx_solve_desc(h);
    if (stream) *stream = (void*)h->stream;
    h->rounds_done += 1;
    return FEDNL_OK;
}

int fednl_mx_get_x(fednl_mx_handle h, double* x)
{
    if (!h || !x) return fail_m(FEDNL_EINVAL, "null argument");
    CKM(cudaStreamSynchronize(h->stream));
    CKM(cudaMemcpy(x, h->P.x, h->d * 8, cudaMemcpyDeviceToHost));
    return FEDNL_OK;
}

int fednl_mx_get_diff(fednl_mx_handle h, int32_t client, float* diff)
{
    if (!h || !diff || client < 0 || client >= h->nc) return fail_m(FEDNL_EINVAL, "bad argument");
    CKM(cudaStreamSynchronize(h->stream));
    CKM(cudaMemcpy(diff, h->P.dsel + (size_t)client * h->Up, (size_t)h->U * 4, cudaMemcpyDeviceToHost));
    return FEDNL_OK;
}

int fednl_mx_get_selection(fednl_mx_handle h, int32_t client, uint32_t* pos, int32_t* count)
{
    if (!h || !count || client < 0 || client >= h->nc) return fail_m(FEDNL_EINVAL, "bad argument");
    CKM(cudaStreamSynchronize(h->stream));
    std::vector<unsigned> w(h->SW);
    CKM(cudaMemcpy(w.data(), h->P.sel + (size_t)client * h->SW, (size_t)h->SW * 4, cudaMemcpyDeviceToHost));
    int n = 0;
    for (int q = 0; q < h->U; ++q)
        if ((w[q >> 5] >> (q & 31)) & 1u) {
            if (pos) pos[n] = (uint32_t)q;
            ++n;
        }
    *count = n;
    return FEDNL_OK;
}

int fednl_mx_get_shift(fednl_mx_handle h, int32_t client, float* shift)
{
    if (!h || !shift || client < 0 || client >= h->nc) return fail_m(FEDNL_EINVAL, "bad argument");
    CKM(cudaStreamSynchronize(h->stream));
    CKM(cudaMemcpy(shift, h->P.shift + (size_t)client * h->Up, (size_t)h->U * 4, cudaMemcpyDeviceToHost));
    return FEDNL_OK;
}

int fednl_mx_get_grad(fednl_mx_handle h, double* g)
{
    if (!h || !g) return fail_m(FEDNL_EINVAL, "null argument");
    CKM(cudaStreamSynchronize(h->stream));
    CKM(cudaMemcpy(g, h->P.g, h->d * 8, cudaMemcpyDeviceToHost));
    return FEDNL_OK;
}

double fednl_mx_get_l(fednl_mx_handle h)
{
    if (!h) return NAN;
    double st[2] = {NAN, NAN};
    cudaStreamSynchronize(h->stream);
    cudaMemcpy(st, h->P.stats, 16, cudaMemcpyDeviceToHost);
    return st[1];
}

}  // extern "C"
