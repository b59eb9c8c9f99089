// fednl_gpu.cu -- host side of the GB300 FedNL round engine behind the C ABI of
// include/fednl_gpu.h.  One handle = one FedNL problem resident in HBM, one CUDA stream; a round
// is a fixed sequence of kernel launches that is captured once into a CUDA graph and replayed.
//
// The host code replaces the reference's train() driver (dopt/bin_fednl_local/include/
// TrainLoop.h:103-1863): client setup, the round loop and the master update; the worker
// threads and message buffers of the reference become device kernels and device buffers.

#include "fednl_gpu.h"
#include "fednl_kernels.cuh"
#include "fednl_refmode.cuh"
#include "fednl_chol32c.cuh"
#include "fednl_solve.h"
#include "fednl_smem.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <condition_variable>
#include <cstring>
#include <exception>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <unistd.h>

using namespace fednl;
static_assert(kCholNB == 32, "fednl_chol_work_elems sizes the panel buffer for 32-row panels");

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return fail(FEDNL_ECUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                        __LINE__);                                                                 \
    } while (0)

#define CKL()                                                                                      \
    do {                                                                                           \
        cudaError_t e_ = cudaGetLastError();                                                       \
        if (e_ != cudaSuccess)                                                                     \
            return fail(FEDNL_ECUDA, "kernel launch failed: %s (%s:%d)", cudaGetErrorString(e_),   \
                        __FILE__, __LINE__);                                                       \
    } while (0)

// device arena: one cudaMalloc, 256-byte aligned sub-buffers
struct Arena {
    char* base = nullptr;
    size_t cap = 0, used = 0;
    std::vector<std::pair<void**, size_t>> plan;
    template <class T> void want(T** p, size_t count) { plan.push_back({(void**)p, count * sizeof(T)}); }
    size_t planned() const
    {
        size_t total = 0;
        for (auto& q : plan) total += (q.second + 255) / 256 * 256;
        return total;
    }
    int commit()
    {
        size_t total = planned();
        if (total == 0) total = 256;
        cudaError_t e = cudaMalloc((void**)&base, total);
        if (e != cudaSuccess) return fail(FEDNL_ENOMEM, "cudaMalloc(%zu) failed: %s", total, cudaGetErrorString(e));
        cap = total;
        size_t off = 0;
        for (auto& q : plan) {
            *q.first = q.second ? (void*)(base + off) : nullptr;
            off += (q.second + 255) / 256 * 256;
        }
        plan.clear();
        return FEDNL_OK;
    }
    void release()
    {
        if (base) cudaFree(base);
        base = nullptr;
    }
};

int ensure_device()
{
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) return fail(FEDNL_ENODEV, "no CUDA device available");
    return FEDNL_OK;
}

size_t select_smem(int k) { return select_smem_bytes(k); }

// CTAs of the cooperative Cholesky: enough threads for the first trailing update, at most one
// resident CTA per SM
int chol_grid(int d)
{
    int dev = 0, sms = 1, bps = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_chol_coop, kCoopThreads, 0);
    long long m = d + 1 > kCholNB ? d + 1 - kCholNB : 1;
    long long want = (m * (m + 1) / 2 + kCoopThreads - 1) / kCoopThreads;
    long long g = std::min<long long>(want, (long long)sms * std::max(bps, 1));
    g = std::min<long long>(g, sms);
    return (int)std::max<long long>(1, g);
}

cudaError_t launch_chol(const Dev& P, int grid, cudaStream_t st, const double* Hin, int hin_lda, const double* lptr,
                        double lval, const double* gin, double* dxout, double* xupd, int record, int apply_first = 0)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kCoopThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_chol_coop, P, Hin, hin_lda, lptr, lval, gin, dxout, xupd, record, apply_first);
}

// the reference-order solve of the master's system (k_chol_ref, one cooperative launch)
cudaError_t launch_chol_ref(const Dev& P, int grid, cudaStream_t st, const double* lptr, double lval, double* dxout,
                            double* xupd, int record)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kRefCholThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_chol_ref, P, (const double*)P.H, lptr, lval, (const double*)P.g, dxout, xupd,
                              record);
}

// CTAs of the reference-order solve: its trailing updates are light, its cost is the per-block
// barriers and the pivot rows, so a modest grid
int ref_grid()
{
    int dev = 0, sms = 1, bps = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_chol_ref, kRefCholThreads, 0);
    return std::max(1, std::min(32, sms * std::max(1, bps)));
}

}  // namespace

// One cooperative launch solving several problems' systems: job j gets a contiguous group of CTAs
// (its share of the SMs, at least one) and its own barrier words.  More jobs than resident CTAs
// are solved in successive launches.
int fednl_solve_batch_launch(const FednlSolveDesc* descs, int n, void* stream)
{
    if (n <= 0) return FEDNL_OK;
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0, sms = 1, bps = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_chol_batched, kCoopThreads, 0);
    const int cap = std::max(1, sms * std::max(1, bps));
    // the device job table is kept per device and reused launch after launch; one host thread at a
    // time fills and launches it
    static std::mutex tables_mu;
    static std::map<int, std::pair<CholJob*, int>> tables;
    std::lock_guard<std::mutex> lock(tables_mu);
    CholJob*& djobs = tables[dev].first;
    int& djobs_cap = tables[dev].second;
    for (int first = 0; first < n; first += cap) {
        const int m = std::min(cap, n - first);
        std::vector<CholJob> jobs(m);
        std::vector<long long> want(m);
        long long tot = 0;
        for (int j = 0; j < m; ++j) {
            want[j] = chol_grid(descs[first + j].d);
            tot += want[j];
        }
        int cta = 0;
        for (int j = 0; j < m; ++j) {
            const FednlSolveDesc& S = descs[first + j];
            int g = tot <= cap ? (int)want[j] : (int)std::max<long long>(1, want[j] * (cap - m) / tot + 1);
            g = std::min(g, cap - cta - (m - 1 - j));
            CholJob& J = jobs[j];
            J = CholJob{};
            J.P.d = S.d;
            J.P.U = S.d * (S.d + 1) / 2;
            J.P.work = S.work;
            J.P.ybuf = S.ybuf;
            J.P.rinv = S.rinv;
            J.P.bar = S.bar;
            J.P.status = S.status;
            J.P.stats = S.stats;
            J.P.hist = S.hist;
            J.P.ls = S.ls;
            J.P.round_ctr = S.round_ctr;
            J.P.hist_cap = S.hist_cap;
            J.Hin = S.H;
            J.hin_lda = 0;
            J.lptr = S.lptr;
            J.lval = S.lval;
            J.gin = S.g;
            J.dxout = S.dx;
            J.xupd = S.xupd;
            J.record = S.record;
            J.cta0 = cta;
            J.ncta = g;
            cta += g;
        }
        if (djobs_cap < m) {
            if (djobs) cudaFree(djobs);
            djobs = nullptr;
            CK(cudaMalloc(&djobs, sizeof(CholJob) * cap));
            djobs_cap = cap;
        }
        CK(cudaMemcpyAsync(djobs, jobs.data(), sizeof(CholJob) * m, cudaMemcpyHostToDevice, st));
        for (int j = 0; j < m; ++j)     // barrier words start at zero (a timed-out launch leaves its flag set)
            CK(cudaMemsetAsync(jobs[j].P.bar, 0, 4 * sizeof(unsigned), st));
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(cta);
        cfg.blockDim = dim3(kCoopThreads);
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        CK(cudaLaunchKernelEx(&cfg, k_chol_batched, (const CholJob*)djobs, m));
        CK(cudaStreamSynchronize(st));       // the job table is reused by the next launch
    }
    return FEDNL_OK;
}

// error reporting shared with the tensor-core translation unit (fednl_mixed.cu)
int fednl_set_error(int code, const char* msg) { return fail(code, "%s", msg); }

// The cooperative Option-B solve on caller-owned device buffers, for the mixed-precision
// translation unit: H packed upper FP64 [d(d+1)/2], l from *lptr, dx = (H + l I)^-1 g, x -= dx
// when xupd is given; with record, stats[0] = ||g|| and the history / round counter advance.
// work: (d+1)(d+2)/2 doubles, ybuf and rinv: d doubles, bar: 4 x u32 (zero), status: 1 int.
int fednl_device_optionb_solve(const double* H, int d, const double* lptr, const double* g, double* dx, double* xupd,
                               double* work, double* ybuf, double* rinv, unsigned* bar, int* status, double* stats,
                               double* hist, int* round_ctr, int hist_cap, int record, cudaStream_t st, int grid)
{
    Dev P{};
    P.d = d;
    P.U = d * (d + 1) / 2;
    P.work = work;
    P.ybuf = ybuf;
    P.rinv = rinv;
    P.bar = bar;
    P.status = status;
    P.stats = stats;
    P.hist = hist;
    P.round_ctr = round_ctr;
    P.hist_cap = hist_cap;
    if (grid <= 0) {
        static int grid_cache_d = -1, grid_cache = 1;
        if (grid_cache_d != d) {
            grid_cache = chol_grid(d);
            grid_cache_d = d;
        }
        grid = grid_cache;
    }
    CK(launch_chol(P, grid, st, H, 0, lptr, 0.0, g, dx, xupd, record));
    return FEDNL_OK;
}

// ---- the FP32 cooperative solve of the mixed-precision form (fednl_chol32c.cuh) ---------------
namespace {

// dynamic shared memory of k_chol32c for dimension d, and whether CTA 0 keeps the factor resident
// (when it fits beside the kernel's static shared memory)
size_t chol32c_smem(int d, int* resident)
{
    static int optin = -1;
    static size_t stat = 0;
    if (optin < 0) {
        int dev = 0, o = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&o, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaFuncAttributes fa{};
        cudaFuncGetAttributes(&fa, k_chol32c);
        stat = fa.sharedSizeBytes;
        optin = o;
    }
    const size_t rb = c32c_smem_bytes(d, true);
    *resident = (d + 31) / 32 <= kC32ResBlocks && rb + stat + 1024 <= (size_t)optin ? 1 : 0;
    return *resident ? rb : c32c_smem_bytes(d, false);
}

// resident CTAs of k_chol32c for dimension d (the cooperative launch's upper bound)
int chol32c_cap(int d)
{
    int dev = 0, sms = 1, bps = 0, res = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t smem = chol32c_smem(d, &res);
    if (fednl_raise_dyn_smem((const void*)k_chol32c, smem) != cudaSuccess) return 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_chol32c, kCoopThreads, smem);
    return std::min(sms, sms * bps);
}

// whether one cluster of n CTAs of k_chol32c can be resident for dimension d
bool chol32c_cluster_ok(int d, int n)
{
    static std::mutex mu;
    static std::map<std::pair<int, int>, bool> cache;
    std::lock_guard<std::mutex> g(mu);
    auto it = cache.find({d, n});
    if (it != cache.end()) return it->second;
    bool ok = false;
    int res = 0;
    const size_t smem = chol32c_smem(d, &res);
    if (fednl_raise_dyn_smem((const void*)k_chol32c, smem) == cudaSuccess &&
        (n <= 8 || cudaFuncSetAttribute(k_chol32c, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess)) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(n);
        cfg.blockDim = dim3(kCoopThreads);
        cfg.dynamicSmemBytes = smem;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = n;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int clusters = 0;
        ok = cudaOccupancyMaxActiveClusters(&clusters, k_chol32c, &cfg) == cudaSuccess && clusters >= 1;
    }
    cudaGetLastError();
    cache[{d, n}] = ok;
    return ok;
}

// default launch: one cluster of 16 CTAs while the trailing updates are small (d up to 512), else
// one CTA per 32 x 32 tile of the first trailing update within the resident limit (a negative
// value -n stands for one cluster of n CTAs)
int chol32c_grid(int d)
{
    if (d <= 512) {
        if (chol32c_cluster_ok(d, 16)) return -16;
        if (chol32c_cluster_ok(d, 8)) return -8;
    }
    const long long nt = d > 32 ? (d - 32 + 31) / 32 : 1;
    return (int)std::max<long long>(1, std::min<long long>(nt * (nt + 1) / 2, chol32c_cap(d)));
}

}  // namespace

int fednl_solve32_max_d() { return kC32MaxD; }

size_t fednl_solve32_bytes(int d)
{
    const size_t ld = (size_t)c32c_ld(d);
    return ld * ld * 4 + (size_t)d * 4 + ld * 32 * 4 + 2 * (size_t)d * 8 + 2 * (size_t)d * 4 + 4;
}

int fednl_device_optionb_solve32(const FednlSolveDesc& S, const FednlSolve32& E, cudaStream_t st, int grid)
{
    if (S.d < 1 || S.d > kC32MaxD || !S.lptr) return FEDNL_EINVAL;
    Dev P{};
    P.d = S.d;
    P.U = S.d * (S.d + 1) / 2;
    P.work = S.work;
    P.ybuf = S.ybuf;
    P.rinv = S.rinv;
    P.bar = S.bar;
    P.status = S.status;
    P.stats = S.stats;
    P.hist = S.hist;
    P.ls = S.ls;
    P.round_ctr = S.round_ctr;
    P.hist_cap = S.hist_cap;
    int res = 0;
    const size_t smem = chol32c_smem(S.d, &res);
    const int cap = chol32c_cap(S.d);
    if (cap < 1) return FEDNL_ECUDA;
    if (grid == 0) grid = chol32c_grid(S.d);
    const bool cl = grid < 0;
    if (cl && !chol32c_cluster_ok(S.d, -grid)) return FEDNL_EINVAL;
    grid = cl ? -grid : std::min(grid, cap);
    Chol32c C{E.a,  E.diag0, E.linv, E.r,     E.acc,   E.accp, E.hh, E.hl,         E.rh,
              E.rl, E.flag,  c32c_ld(S.d), E.refine, E.tol, res,    (int)(smem / 4), cl ? 1 : 0};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kCoopThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    if (cl) {
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = grid;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
    } else {
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
    }
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    CK(cudaLaunchKernelEx(&cfg, k_chol32c, P, C, S.H, S.lptr, S.g, S.dx, S.xupd, S.record));
    return FEDNL_OK;
}

// ---- autotuning of the solve's launch shape ----------------------------------------------------
// A cooperative solve's CTA count is measured per dimension on the caller's own system (the
// handle's current H, l and g into scratch outputs: nothing of the run changes) and cached
// process-wide per solver kind, so later handles of the same d reuse the choice.
static int tune_grid(int kind, int d, int cap, int dflt, const std::function<int(int)>& launch, cudaStream_t st,
                     int* best_grid, double* best_ms, const std::vector<int>& extra = {})
{
    static std::mutex mu;
    static std::map<std::pair<int, int>, std::pair<int, double>> cache;
    {
        std::lock_guard<std::mutex> g(mu);
        auto it = cache.find({kind, d});
        if (it != cache.end()) {
            *best_grid = it->second.first;
            *best_ms = it->second.second;
            return FEDNL_OK;
        }
    }
    if (cap < 1) return FEDNL_ECUDA;
    std::vector<int> cand = {8, 16, 24, 32, 48, 64, 96, 128, cap, dflt};
    cand.insert(cand.end(), extra.begin(), extra.end());
    std::sort(cand.begin(), cand.end());
    cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    int bg = dflt > 0 ? std::min(dflt, cap) : dflt;
    double bm = 1e30;
    for (int G : cand) {
        if (G == 0 || G > cap || (G < 0 && std::find(extra.begin(), extra.end(), G) == extra.end())) continue;
        int rc = launch(G);                                   // warm
        if (rc) return rc;
        float best = 1e30f;
        for (int rep = 0; rep < 3; ++rep) {
            CK(cudaEventRecord(e0, st));
            rc = launch(G);
            if (rc) return rc;
            CK(cudaEventRecord(e1, st));
            CK(cudaEventSynchronize(e1));
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            best = std::min(best, ms);
        }
        if (best < bm) {
            bm = best;
            bg = G;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::lock_guard<std::mutex> g(mu);
    cache[{kind, d}] = {bg, bm};
    *best_grid = bg;
    *best_ms = bm;
    return FEDNL_OK;
}

int fednl_tune_chol_grid(int d, const std::function<int(int)>& launch, cudaStream_t st, int* best_grid, double* best_ms)
{
    int dev = 0, sms = 1, bps = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_chol_coop, kCoopThreads, 0);
    return tune_grid(0, d, std::min(sms, sms * std::max(1, bps)), chol_grid(d), launch, st, best_grid, best_ms);
}

int fednl_tune_chol32_grid(int d, const std::function<int(int)>& launch, cudaStream_t st, int* best_grid,
                           double* best_ms)
{
    std::vector<int> extra;
    for (int n : {8, 16})
        if (chol32c_cluster_ok(d, n)) extra.push_back(-n);
    return tune_grid(1, d, chol32c_cap(d), chol32c_grid(d), launch, st, best_grid, best_ms, extra);
}

struct fednl_handle_s {
    fednl_problem_desc desc{};
    std::vector<int32_t> ns, soff;
    int d = 0, lda = 0, U = 0, ustr = 0, nc = 0, k = 0, comp = 0, W = 1, SW = 0, S = 0;
    int binary = 0, maxn = 0, nfpart = 0, nseg = 0, hcap = 0;
    int pp = 0, tau = 0, pp_smem_perm = 0;   // FedNL-PP: clients per round, sampler in shared memory
    bool data_ready = false, shifts_ready = false;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;       // the round graph's second branch (k_aggregate)
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    unsigned* drawctr = nullptr;       // [1] k_select's finished CTAs (TopLEK draws in the last one)
    Arena state, feat;
    Dev dev{};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    int hess_kind = 0;                 // chosen binary-Hessian kernel (kHessMasksSmem, kHessMasksGlobal, kHessHits)
    int hess_nt = kHessThreads;        // chosen: threads per block
    size_t hess_smem_sm = 0, hess_smem_gl = 0;   // bytes with the masks staged (0: they do not fit) / read from global
    bool hits_ready = false;           // common-sample lists built at upload (k_hess_hits)
    int hits_maxrec = 0;               // most multi-sample records in one segment
    double hess_ms = 0.0;              // tuned shape's measured launch time (0: not tuned)
    int chol_grid = 1;
    int ref_grid = 1;          // CTAs of the reference-order solve
    int rounds_done = 0;
    void* flush_buf = nullptr;
    void* pin = nullptr;               // [32 B] pinned: a round's statistics and status, read back together
    size_t flush_cap = 0;
};

namespace {

struct Marks {
    std::vector<cudaEvent_t>* ev = nullptr;   // one event per mark, recorded in order
    std::vector<std::string>* names = nullptr;
    size_t next = 0;
};

int mark(fednl_handle h, Marks* m, const char* name)
{
    if (!m || m->next >= m->ev->size()) return FEDNL_OK;
    if (m->names && m->names->size() <= m->next) m->names->push_back(name);
    CK(cudaEventRecord((*m->ev)[m->next], h->stream));
    m->next += 1;
    return FEDNL_OK;
}

#define MARK(name)                                                                                 \
    do {                                                                                           \
        int rc_ = mark(h, M, name);                                                                \
        if (rc_) return rc_;                                                                       \
    } while (0)

// threads of k_client_binary: a lane pair per attribute when that fits one CTA, and a warp for the
// intercept's sums
int client_threads(int d) { return std::min(1024, std::max(128, (2 * d + 31) / 32 * 32 + 32)); }

// dynamic shared memory of k_client_binary: the weights and the intercept's word sums
size_t client_smem(fednl_handle h) { return (size_t)h->maxn * 16 + (size_t)((h->maxn + 63) / 64) * 16; }

// The binary Hessian's kernels: attribute masks intersected every round (staged in shared memory
// or read from global memory), or the common-sample lists built at upload.
enum { kHessMasksSmem = 0, kHessMasksGlobal = 1, kHessHits = 2 };

// The binary Hessian in one of its launch shapes (the results do not depend on the shape: every
// warp owns the same 512 upper positions and the client's last block adds the segments in order).
template <bool SM>
cudaError_t launch_hess_binary_t(const Dev& Q, int nseg, size_t smem, int nclients, int mode, cudaStream_t st, int nt)
{
    const unsigned gx = (unsigned)((nseg + nt / 32 - 1) / (nt / 32));
    switch (nt) {
    case 128: k_hess_binary<SM, 128><<<dim3(gx, nclients), 128, smem, st>>>(Q, mode); break;
    case 512: k_hess_binary<SM, 512><<<dim3(gx, nclients), 512, smem, st>>>(Q, mode); break;
    default: k_hess_binary<SM, 256><<<dim3(gx, nclients), 256, smem, st>>>(Q, mode); break;
    }
    return cudaGetLastError();
}

// the binary Hessian's mode in the captured round: the difference only when the selection kernel
// forms the norms (TopK / TopLEK in the fixed order, Option B, not FedNL-PP), else with them
int round_hess_mode(fednl_handle h)
{
    if (h->pp) return 2;
    const bool sel = h->comp == FEDNL_TOPK || h->comp == FEDNL_TOPLEK;
    return sel && !h->dev.ref && !h->desc.option_a ? 3 : 0;
}

size_t hits_smem(fednl_handle h, int nt)
{
    return hits_stage_bytes(nt) + ((size_t)h->maxn + 2 * h->d + (size_t)(nt / 32) * h->hits_maxrec) * 8;
}

cudaError_t launch_hess_binary(fednl_handle h, const Dev& Q, int nclients, int mode, cudaStream_t st, int kind, int nt)
{
    if (kind == kHessHits) {
        const unsigned gx = (unsigned)((h->nseg + nt / 32 - 1) / (nt / 32));
        const size_t smem = hits_smem(h, nt);
        switch (nt) {
        case 128: k_hess_hits<128><<<dim3(gx, nclients), 128, smem, st>>>(Q, mode, h->hits_maxrec); break;
        case 512: k_hess_hits<512><<<dim3(gx, nclients), 512, smem, st>>>(Q, mode, h->hits_maxrec); break;
        default: k_hess_hits<256><<<dim3(gx, nclients), 256, smem, st>>>(Q, mode, h->hits_maxrec); break;
        }
        return cudaGetLastError();
    }
    if (kind == kHessMasksSmem) return launch_hess_binary_t<true>(Q, h->nseg, h->hess_smem_sm, nclients, mode, st, nt);
    return launch_hess_binary_t<false>(Q, h->nseg, h->hess_smem_gl, nclients, mode, st, nt);
}

cudaError_t raise_hess_smem(fednl_handle h)
{
    cudaError_t e = cudaSuccess;
    if (h->hits_ready) {
        if (e == cudaSuccess) e = fednl_raise_dyn_smem((const void*)k_hess_hits<128>, hits_smem(h, 128));
        if (e == cudaSuccess) e = fednl_raise_dyn_smem((const void*)k_hess_hits<256>, hits_smem(h, 256));
        if (e == cudaSuccess) e = fednl_raise_dyn_smem((const void*)k_hess_hits<512>, hits_smem(h, 512));
    }
    for (const void* k : {(const void*)k_hess_binary<false, 128>, (const void*)k_hess_binary<false, 256>,
                          (const void*)k_hess_binary<false, 512>})
        if (e == cudaSuccess) e = fednl_raise_dyn_smem(k, h->hess_smem_gl);
    if (h->hess_smem_sm)
        for (const void* k : {(const void*)k_hess_binary<true, 128>, (const void*)k_hess_binary<true, 256>,
                              (const void*)k_hess_binary<true, 512>})
            if (e == cudaSuccess) e = fednl_raise_dyn_smem(k, h->hess_smem_sm);
    return e;
}

int launch_round(fednl_handle h, Marks* M = nullptr, bool client_phase_only = false)
{
    Dev& P = h->dev;
    cudaStream_t st = h->stream;
    int S = h->S;
    if (h->pp) {
        MARK("k_pp_sample");
        k_pp_sample<<<1, kPPThreads, h->pp_smem_perm ? (size_t)h->nc * 4 : 0, st>>>(
            h->nc, h->tau, P.sampler, P.perm, (int*)P.act, P.is_sel, P.needs, h->pp_smem_perm);
        CKL();
    }
    if (h->binary && !P.ref) {       // the client oracle in one launch
        MARK("k_client_binary");
        k_client_binary<<<h->nc, client_threads(h->d), client_smem(h), st>>>(P);
        CKL();
    } else {
        if (P.ref) {
            MARK("k_margin_ref");
            k_margin_ref<<<(S + 255) / 256, 256, 0, st>>>(P, S);
        } else {
            MARK(h->binary ? "k_margin_binary" : "k_margin_dense");
            if (h->binary) k_margin_binary<<<(S + 255) / 256, 256, 0, st>>>(P, S);
            else k_margin_dense<<<(S + 255) / 256, 256, 0, st>>>(P, S);
        }
        CKL();
        MARK(h->binary ? "k_grad_binary" : "k_grad_dense");
        dim3 gg(h->binary ? (2 * h->d + 127) / 128 : (h->d + 127) / 128, h->nc);   // binary: a lane pair per attribute
        if (h->binary) k_grad_binary<<<gg, 128, (size_t)h->maxn * 16, st>>>(P);
        else k_grad_dense<<<gg, 128, 0, st>>>(P);
        CKL();
    }
    const int na = P.n_act;
    if (h->pp) {
        MARK("k_pp_truegrad");
        k_pp_truegrad<<<(h->d + 3) / 4, 128, 0, st>>>(P);
        CKL();
        MARK("k_pp_norm");
        k_pp_norm<<<1, 32, 0, st>>>(P);
        CKL();
    }
    int comp = h->comp;
    // The master's aggregation needs only the gradients and Lk.  With TopK / TopLEK it runs in the
    // selection kernel's idle warps; otherwise, in a graph, on a branch beside the compressor and the
    // shift update (kept in line when the round is profiled kernel by kernel)
    const bool agg_in_select = !h->pp && (comp == FEDNL_TOPK || comp == FEDNL_TOPLEK);
    // the master merge runs in the solve's first phase (FP64 order, not FedNL-PP, not when the
    // solve is left to a batched launch)
    const bool apply_in_solve = !h->pp && !P.ref && !client_phase_only;
    // With TopK / TopLEK in the fixed order the selection kernel's idle warps also form ||diff||_F^2
    // and Lk (the Hessian writes the difference only), and the solve forms l from Lk while it merges
    const bool norms_in_select = agg_in_select && apply_in_solve && !h->desc.option_a;
    MARK(!h->binary ? "k_hess_dense" : h->hess_kind == kHessHits ? "k_hess_hits" : "k_hess_binary");
    const int hmode = h->pp ? 2 : norms_in_select ? 3 : 0;     // round_hess_mode(h) in the captured round
    if (h->binary) {
        CK(launch_hess_binary(h, P, na, hmode, st, h->hess_kind, h->hess_nt));
    } else {
        k_hess_dense<<<dim3(h->nfpart, na), kHessThreads, 0, st>>>(P, hmode);
        CKL();
    }
    if (P.ref) {
        MARK("k_frob_ref");
        k_frob_ref<<<na, kFrobRefThreads, (size_t)kFrobRing * h->d * 8, st>>>(P);
        CKL();
    }                             // otherwise the Hessian kernel's last block per client formed F
    const bool fork = !M && h->side && !h->pp && !agg_in_select;
    if (fork) {
        CK(cudaEventRecord(h->fork_ev, st));
        CK(cudaStreamWaitEvent(h->side, h->fork_ev, 0));
        k_aggregate<<<(h->d + kAggThreads - 1) / kAggThreads + 1, kAggThreads, 0, h->side>>>(P);
        CKL();
        CK(cudaEventRecord(h->join_ev, h->side));
    }
    if (comp == FEDNL_TOPK || comp == FEDNL_TOPLEK) {
        MARK("k_select");
        double delta = (double)h->k * (1.0 / (double)h->U);
        // TopLEK's rounding draws run in the launch's last CTA
        SelectDraws dr{comp == FEDNL_TOPLEK ? h->drawctr : nullptr, h->nc, h->W, P.wstate, MasterAgg{}};
        if (agg_in_select) dr.agg = MasterAgg{P.gc, P.lk, P.g, P.stats, h->d, h->nc, P.inv_n};
        if (norms_in_select) {
            dr.agg.lk = nullptr;          // l is formed by the solve
            dr.norms = 1;
            dr.nseg = h->nseg;
            dr.fpart = P.Fpart;
            dr.lk = P.lk;
        }
        k_select<<<na, kSelThreads, h->k < h->U ? select_smem(h->k) : 0, st>>>(
            P.diff, h->ustr, h->U, h->k, comp == FEDNL_TOPLEK, delta, P.F, P.sel, h->SW, P.cnt, P.needs, P.pdraw,
            P.minidx, P.status, P.act, P.ref, dr);
        CKL();
    } else if (comp == FEDNL_RANDK) {
        MARK("k_randk");
        k_randk<<<na, 256, 0, st>>>(P.rstate, h->nc, h->U, h->k, P.hmap, h->hcap, P.sel, h->SW, P.cnt, P.act);
        CKL();
    } else if (comp == FEDNL_RANDK_PHILOX) {
        MARK("k_randk_philox");
        k_randk_philox<<<na, 256, 0, st>>>(P.rstate, h->U, h->k, philox_half_bits(h->U), h->desc.seed_base, P.sel,
                                           h->SW, P.cnt, P.act);
        CKL();
    } else if (comp == FEDNL_RANDSEQK) {
        MARK("k_randseqk");
        k_randseqk<<<na, 256, 0, st>>>(P.rstate, h->nc, h->U, h->k, P.rseq, P.sel, h->SW, P.cnt, P.act);
        CKL();
    }
    if (!apply_in_solve) {
        MARK("k_apply");
        k_apply<<<(h->U + 127) / 128, 128, 0, st>>>(P);
        CKL();
    }
    if (h->pp) {
        MARK("k_pp_lkpart");
        k_pp_lkpart<<<dim3(h->nfpart, na), kHessThreads, 0, st>>>(P);
        CKL();
        MARK("k_pp_dir");
        k_pp_dir<<<na, 128, 0, st>>>(P);
        CKL();
        MARK("k_pp_aggregate");
        k_pp_aggregate<<<(h->d + 127) / 128, 128, 0, st>>>(P);
        CKL();
        MARK("k_chol_coop");     // x = (H + l I)^-1 g (bin_fednl_local_pp TrainLoop.h:1560-1600)
        CK(cudaMemsetAsync(P.bar, 0, 4 * sizeof(unsigned), st));   // barrier words and error flag start at zero
        CK(launch_chol(P, h->chol_grid, st, P.H, 0, P.stats + 1, 0.0, P.g, P.x, nullptr, 0));
        MARK("end");
        return FEDNL_OK;
    }
    if (fork) {
        CK(cudaStreamWaitEvent(st, h->join_ev, 0));
    } else if (!agg_in_select) {
        MARK("k_aggregate");
        k_aggregate<<<(h->d + kAggThreads - 1) / kAggThreads + 1, kAggThreads, 0, st>>>(P);   // + the block for l
        CKL();
    }
    if (P.fmode) {       // f(x_k) from the round's sigmoid values
        MARK("k_fclient");
        if (P.ref) k_fclient_ref<<<(h->nc + 3) / 4, 128, 0, st>>>(P, P.x, nullptr);
        else k_fclient<<<(h->nc + 3) / 4, 128, 0, st>>>(P, P.x, nullptr);
        CKL();
        MARK("k_fmaster");
        if (P.ref) k_fmaster_ref<<<1, 32, 0, st>>>(P, P.stats + 2);
        else k_fmaster<<<1, 32, 0, st>>>(P, P.stats + 2);
        CKL();
    }
    if (client_phase_only) return FEDNL_OK;
    const fednl_problem_desc& D = h->desc;
    const double* lptr = D.option_a ? nullptr : P.stats + 1;      // Option A: H + lambda I
    // barrier words and error flag start at zero (the binary client oracle zeroes them at the round's start)
    if (!(h->binary && !P.ref)) CK(cudaMemsetAsync(P.bar, 0, 4 * sizeof(unsigned), st));
    if (P.ref) {
        MARK("k_chol_ref");
        CK(launch_chol_ref(P, h->ref_grid, st, lptr, P.lambda, P.dx, D.line_search ? nullptr : P.x, 1));
    } else {
        MARK("k_chol_coop");
        CK(launch_chol(P, h->chol_grid, st, P.H, 0, lptr, P.lambda, P.g, P.dx, D.line_search ? nullptr : P.x, 1,
                       norms_in_select ? 2 : apply_in_solve ? 1 : 0));
    }
    if (D.line_search) {
        MARK("k_ls_init");
        if (P.ref) k_ls_init_ref<<<1, 256, 0, st>>>(P);
        else k_ls_init<<<1, 256, 0, st>>>(P);
        CKL();
        for (int it = 0; it < D.ls_max_steps; ++it) {
            MARK("k_ls_trial");
            k_ls_trial<<<(h->d + 255) / 256, 256, 0, st>>>(P);
            CKL();
            MARK("k_ls_margin");
            if (P.ref) k_ls_margin_ref<<<(S + 255) / 256, 256, 0, st>>>(P, S);
            else k_ls_margin<<<(S + 255) / 256, 256, 0, st>>>(P, S);
            CKL();
            MARK("k_fclient");
            if (P.ref) k_fclient_ref<<<(h->nc + 3) / 4, 128, 0, st>>>(P, P.x, P.ls);
            else k_fclient<<<(h->nc + 3) / 4, 128, 0, st>>>(P, P.x, P.ls);
            CKL();
            MARK("k_ls_check");
            if (P.ref) k_ls_check_ref<<<1, 32, 0, st>>>(P, D.ls_c, D.ls_gamma);
            else k_ls_check<<<1, 32, 0, st>>>(P, D.ls_c, D.ls_gamma);
            CKL();
        }
    }
    MARK("end");
    return FEDNL_OK;
}

int build_graph(fednl_handle h)
{
    if (h->gexec) return FEDNL_OK;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int rc = launch_round(h);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (rc != FEDNL_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return fail(FEDNL_ECUDA, "graph capture failed: %s", cudaGetErrorString(e));
    h->graph = g;
    CK(cudaGraphInstantiate(&h->gexec, g, 0));
    return FEDNL_OK;
}

}  // namespace

// =================================================================================================
extern "C" {

const char* fednl_gpu_last_error(void) { return g_last_error.c_str(); }

}  // extern "C"

// create, or with footprint set only the device bytes a handle of this desc would hold (its state
// arena plus a dense FP64 bound on the client data)
static int create_impl(const fednl_problem_desc* desc, fednl_handle* out, int64_t* footprint)
{
    if (!desc || (!out && !footprint)) return fail(FEDNL_EINVAL, "null argument");
    if (out) *out = nullptr;
    int rc = footprint ? FEDNL_OK : ensure_device();
    if (rc) return rc;
    const fednl_problem_desc& D = *desc;
    if (D.d < 1 || D.n_clients < 1 || !D.n_samples) return fail(FEDNL_EINVAL, "d and n_clients must be >= 1");
    if (D.compressor < 0 || D.compressor > 6) return fail(FEDNL_EINVAL, "unknown compressor %d", D.compressor);
    if (D.reserved) return fail(FEDNL_EINVAL, "reserved fields must be zero");
    if (D.arith_order != FEDNL_ORDER_FIXED && D.arith_order != FEDNL_ORDER_REFERENCE)
        return fail(FEDNL_EINVAL, "unknown arith_order %d", D.arith_order);
    if (D.arith_order == FEDNL_ORDER_REFERENCE && D.clients_per_round > 0)
        return fail(FEDNL_EINVAL, "the reference arithmetic order is available for plain FedNL only");
    if (D.clients_per_round < 0 || D.clients_per_round > D.n_clients)
        return fail(FEDNL_EINVAL, "clients_per_round %d outside [0, n_clients]", D.clients_per_round);
    if (D.line_search && (D.clients_per_round > 0 || D.ls_max_steps < 1 || !(D.ls_c > 0.0) || !(D.ls_gamma > 0.0) ||
                          !(D.ls_gamma < 1.0)))
        return fail(FEDNL_EINVAL, "line search needs plain FedNL, max steps >= 1, c > 0 and 0 < gamma < 1");
    int lda = D.lda ? D.lda : (D.d + 3) / 4 * 4;
    if (lda < D.d) return fail(FEDNL_EINVAL, "lda %d < d %d", lda, D.d);
    long long U = (long long)D.d * (D.d + 1) / 2;
    if (U >= (1ll << 31) || (long long)D.d * lda >= (1ll << 32))
        return fail(FEDNL_EINVAL, "d too large for 32-bit flat indices");
    int k = (D.compressor == FEDNL_IDENTITY || D.compressor == FEDNL_NATURAL) ? (int)U : D.k;
    if (k < 1) return fail(FEDNL_EINVAL, "k must be >= 1");
    if ((D.compressor == FEDNL_RANDK || D.compressor == FEDNL_RANDSEQK || D.compressor == FEDNL_RANDK_PHILOX) && k > U)
        return fail(FEDNL_EINVAL, "k %d larger than U %lld", k, U);
    if ((D.compressor == FEDNL_TOPK || D.compressor == FEDNL_TOPLEK) && k < U && k > kMaxK)
        return fail(FEDNL_EINVAL, "TopK/TopLEK k %d above the shared-memory heap limit %d", k, kMaxK);

    fednl_handle h = new fednl_handle_s();
    h->desc = D;
    h->d = D.d;
    h->lda = lda;
    h->U = (int)U;
    h->ustr = (int)((U + 31) / 32 * 32);
    h->nc = D.n_clients;
    h->k = k;
    h->comp = D.compressor;
    h->W = std::max(1, std::min(D.workers < 1 ? 1 : D.workers, D.n_clients));  // TrainLoop.h:194-199
    h->SW = (h->U + 31) / 32;
    h->ns.assign(D.n_samples, D.n_samples + D.n_clients);
    h->soff.assign(h->nc + 1, 0);
    for (int c = 0; c < h->nc; ++c) {
        if (h->ns[c] < 1) {
            delete h;
            return fail(FEDNL_EINVAL, "client %d has no samples", c);
        }
        h->soff[c + 1] = h->soff[c] + h->ns[c];
        h->maxn = std::max(h->maxn, h->ns[c]);
    }
    h->S = h->soff[h->nc];
    h->nfpart = (h->U + kHessPerBlock - 1) / kHessPerBlock;
    h->nseg = (h->U + 511) / 512;
    h->pp = D.clients_per_round > 0;
    h->tau = h->pp ? D.clients_per_round : h->nc;
    h->pp_smem_perm = h->pp && (size_t)h->nc * 4 <= 48 * 1024;
    h->hcap = 1;
    if (h->comp == FEDNL_RANDK)
        while (h->hcap < 4 * k) h->hcap <<= 1;

    Dev& P = h->dev;
    P.d = h->d;
    P.lda = h->lda;
    P.U = h->U;
    P.ustr = h->ustr;
    P.nc = h->nc;
    P.k = h->k;
    P.comp = h->comp;
    P.W = h->W;
    P.SW = h->SW;
    P.nfpart = h->nfpart;
    P.nseg = h->nseg;
    P.hcap = h->hcap;
    P.lambda = D.lambda;
    P.alpha = D.alpha;
    P.inv_n = 1.0 / (double)h->nc;
    P.prescale = P.inv_n * D.alpha;                          // TrainLoop.h:531
    P.mult = (double)h->U / (double)h->k;                    // RandK.h:90
    P.hist_cap = 1 << 16;
    P.pp = h->pp;
    P.n_act = h->tau;
    P.fmode = (D.line_search || D.track_f) && !h->pp;
    P.ref = D.arith_order == FEDNL_ORDER_REFERENCE;
    size_t ncU = (size_t)h->nc * h->ustr;
    Arena& A = h->state;
    A.want((int**)&P.ns, h->nc);
    A.want((int**)&P.soff, h->nc + 1);
    A.want((int**)&P.client_of, h->S);
    A.want(&P.x, h->d);
    A.want(&P.H, h->U);
    A.want(&P.g, h->d);
    A.want(&P.shift, ncU);
    A.want(&P.diff, ncU);
    A.want(&P.Dv, h->S);
    A.want(&P.qb, h->S);
    A.want(&P.gc, (size_t)h->nc * h->d);
    A.want(&P.Fpart, (size_t)h->nc * h->nseg);
    A.want(&P.dsum, (size_t)h->nc * h->d);
    A.want(&P.F, h->nc);
    A.want(&P.hdone, h->nc);
    A.want(&h->drawctr, 1);
    A.want(&P.lk, h->nc);
    A.want(&P.sel, (size_t)h->nc * h->SW);
    A.want(&P.cnt, h->nc);
    A.want(&P.needs, h->nc);
    A.want(&P.pdraw, h->nc);
    A.want(&P.minidx, h->nc);
    A.want(&P.wstate, h->W);
    A.want(&P.rstate, h->nc);
    A.want(&P.rseq, h->nc);
    A.want(&P.hmap, (size_t)h->nc * h->hcap);
    A.want(&P.work, fednl_chol_work_elems(h->d));
    A.want(&P.dx, h->d);
    A.want(&P.ybuf, h->d);
    A.want(&P.rinv, h->d);
    A.want(&P.hist, P.hist_cap);
    A.want(&P.round_ctr, 1);
    A.want(&P.status, 1);
    A.want(&P.stats, 4);
    A.want(&P.bar, 4);
    if (P.ref) {
        const size_t ua = (size_t)(h->d + 1) * (h->d + 2) / 2;
        A.want(&P.rref, ua);
        A.want(&P.racc, 9 * ua);
    }
    if (P.fmode) {
        A.want(&P.fterm, h->S);
        A.want(&P.fi, h->nc);
        A.want(&P.xprev, h->d);
        A.want(&P.ls, 5);
    }
    if (h->pp) {
        A.want((int**)&P.act, h->nc);
        A.want(&P.is_sel, h->nc);
        A.want(&P.perm, h->nc);
        A.want(&P.sampler, 1);
        A.want(&P.hbuf, ncU);
        A.want(&P.dir, (size_t)h->nc * h->d);
        A.want(&P.ddir, (size_t)h->nc * h->d);
        A.want(&P.dlk, h->nc);
        A.want(&P.gprev, h->d);
        A.want(&P.lprev, 1);
        A.want(&P.tg, h->d);
    }
    if (footprint) {
        *footprint = (int64_t)A.planned() + (int64_t)h->S * (h->d + 1) * 8 + (int64_t)(h->S + 1) * 4 + 4096;
        delete h;
        return FEDNL_OK;
    }
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->fork_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->join_ev, cudaEventDisableTiming) != cudaSuccess) {
        if (h->side) cudaStreamDestroy(h->side);
        if (h->fork_ev) cudaEventDestroy(h->fork_ev);
        if (h->join_ev) cudaEventDestroy(h->join_ev);
        delete h;
        return fail(FEDNL_ECUDA, "cudaStreamCreate failed");
    }
    rc = A.commit();
    if (rc) {
        cudaStreamDestroy(h->stream);
        delete h;
        return rc;
    }
    std::vector<int> client_of(h->S);
    for (int c = 0; c < h->nc; ++c)
        for (int s = h->soff[c]; s < h->soff[c + 1]; ++s) client_of[s] = c;
    if (cudaMemcpy((void*)P.ns, h->ns.data(), h->nc * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy((void*)P.soff, h->soff.data(), (h->nc + 1) * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy((void*)P.client_of, client_of.data(), (size_t)h->S * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(P.x, 0, h->d * 8) != cudaSuccess || cudaMemset(P.round_ctr, 0, 4) != cudaSuccess ||
        cudaMemset(P.status, 0, 4) != cudaSuccess || cudaMemset(P.bar, 0, 16) != cudaSuccess ||
        cudaMemset(P.hdone, 0, (size_t)h->nc * 4) != cudaSuccess || cudaMemset(h->drawctr, 0, 4) != cudaSuccess) {
        fednl_gpu_destroy(h);
        return fail(FEDNL_ECUDA, "initial copies failed");
    }
    if (select_smem(h->k) > 48 * 1024 && h->k < h->U)
        fednl_raise_dyn_smem((const void*)k_select, select_smem(h->k));
    h->chol_grid = chol_grid(h->d);
    if (P.ref) {
        h->ref_grid = ref_grid();
        if ((size_t)kFrobRing * h->d * 8 > 48 * 1024)
            fednl_raise_dyn_smem((const void*)k_frob_ref, (size_t)kFrobRing * h->d * 8);
    }
    *out = h;
    return FEDNL_OK;
}

// Host-side exceptions (a failed host allocation in the conversion of uploaded rows) end at the C
// boundary as error codes.
template <class F>
static int host_guarded(F&& f)
{
    try {
        return f();
    } catch (const std::bad_alloc&) {
        return fail(FEDNL_ENOMEM, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(FEDNL_EINVAL, "host error: %s", e.what());
    }
}

extern "C" {

int fednl_gpu_create(const fednl_problem_desc* desc, fednl_handle* out)
{
    if (!out) return fail(FEDNL_EINVAL, "null argument");
    return create_impl(desc, out, nullptr);
}

int fednl_gpu_footprint(const fednl_problem_desc* desc, int64_t* bytes)
{
    if (!bytes) return fail(FEDNL_EINVAL, "null argument");
    return create_impl(desc, nullptr, bytes);
}

int fednl_gpu_destroy(fednl_handle h)
{
    if (!h) return FEDNL_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    if (h->graph) cudaGraphDestroy(h->graph);
    h->state.release();
    h->feat.release();
    if (h->flush_buf) cudaFree(h->flush_buf);
    if (h->pin) cudaFreeHost(h->pin);
    if (h->stream) cudaStreamDestroy(h->stream);
    if (h->side) cudaStreamDestroy(h->side);
    if (h->fork_ev) cudaEventDestroy(h->fork_ev);
    if (h->join_ev) cudaEventDestroy(h->join_ev);
    delete h;
    return FEDNL_OK;
}

// Worker threads for the conversion of uploaded rows, started on first use and kept for the
// process: an upload runs three parallel passes, and starting 16 threads for each cost more than
// a pass's own work.  One job at a time (callers are serialised); the caller runs part 0.  A
// forked child, which holds none of its parent's threads, starts a pool of its own.
class RangePool {
public:
    static RangePool& get()
    {
        static std::mutex pm;
        static RangePool* pool = nullptr;
        std::lock_guard<std::mutex> lk(pm);
        if (!pool || pool->pid_ != getpid()) pool = new RangePool();    // a parent's pool is left as is
        return *pool;
    }
    int size() const { return nworkers_ + 1; }
    // f(0 .. n-1), n <= size(), part 0 on the calling thread
    void run(int n, const std::function<void(int)>& f)
    {
        std::lock_guard<std::mutex> one(run_m_);
        {
            std::lock_guard<std::mutex> lk(m_);
            job_ = &f;
            njob_ = n;
            left_ = n - 1;
            err_ = nullptr;
            ++gen_;
        }
        go_.notify_all();
        std::exception_ptr err;
        try {
            f(0);
        } catch (...) {
            err = std::current_exception();    // the workers still finish their parts first
        }
        {
            std::unique_lock<std::mutex> lk(m_);
            done_.wait(lk, [&] { return left_ == 0; });
            if (!err) err = err_;
        }
        if (err) std::rethrow_exception(err);    // the first part's exception, on the caller's thread
    }

private:
    RangePool() : pid_(getpid())
    {
        const unsigned hc = std::thread::hardware_concurrency();
        nworkers_ = std::max(0, std::min<int>((int)(hc ? hc : 1), 32) - 1);
        for (int i = 1; i <= nworkers_; ++i) std::thread(&RangePool::work, this, i).detach();
    }
    void work(int id)
    {
        unsigned long long seen = 0;
        for (;;) {
            const std::function<void(int)>* f;
            {
                std::unique_lock<std::mutex> lk(m_);
                go_.wait(lk, [&] { return gen_ != seen; });
                seen = gen_;
                if (id >= njob_) continue;    // not a part of this job
                f = job_;
            }
            std::exception_ptr err;
            try {
                (*f)(id);
            } catch (...) {
                err = std::current_exception();
            }
            std::lock_guard<std::mutex> lk(m_);
            if (err && !err_) err_ = err;
            if (--left_ == 0) done_.notify_one();
        }
    }
    const pid_t pid_;
    int nworkers_ = 0;
    std::mutex run_m_, m_;
    std::condition_variable go_, done_;
    const std::function<void(int)>* job_ = nullptr;
    std::exception_ptr err_;
    unsigned long long gen_ = 0;
    int njob_ = 0, left_ = 0;
};

// The conversion of the uploaded rows over client ranges: clients are split into contiguous
// ranges in order (each client's CSR range and bitmap block are disjoint, so the ranges need no
// locking), of about equal work when work[c + 1] - work[c] gives client c's (a prefix over the
// clients), else of equal client counts.  f(range, first client, end client).
static void for_client_ranges(int nc, const std::function<void(int, int, int)>& f,
                              const std::vector<long long>* work = nullptr)
{
    RangePool& pool = RangePool::get();
    const int nth = std::max(1, std::min(pool.size(), nc));
    if (nth == 1) {
        f(0, 0, nc);
        return;
    }
    std::vector<int> cut(nth + 1, nc);
    cut[0] = 0;
    for (int t = 1; t < nth; ++t) {
        int c = (int)(((long long)nc * t + nth - 1) / nth);
        if (work) {
            const long long goal = (*work)[nc] * t / nth;
            c = (int)(std::lower_bound(work->begin(), work->begin() + nc + 1, goal) - work->begin());
        }
        cut[t] = std::min(nc, std::max(cut[t - 1], c));
    }
    pool.run(nth, [&](int t) {
        if (cut[t] < cut[t + 1]) f(t, cut[t], cut[t + 1]);
    });
}

// The problem's shape as the lists builder reads it (from a handle, or from the host-only entry).
struct ListShape {
    int nc, d, U, ustr, nseg, maxn;
    const int32_t* soff;    // [nc + 1] first sample of each client
};

// Common-sample lists of the binary Hessian (k_hess_hits), from the CSR rows of the upload: each
// client's samples in order, every pair a < b of a sample's attributes other than the intercept
// adds the sample to upper position b (b + 1) / 2 + a.  Built only when the lists stay small (at
// most 16 pairs per upper position in every client, 64 M in all) and the codes can hold the
// sample and attribute indices.
struct HitLists {
    std::unique_ptr<uint16_t[]> code;    // [nc][ustr]
    std::unique_ptr<uint32_t[]> seg;     // [nc][nseg + 1]
    std::unique_ptr<uint32_t[]> rec;     // [records + 1]
    std::unique_ptr<uint16_t[]> hits;
    size_t ncode = 0, nseg = 0, nrec = 0, nhits = 0;
    int maxrec = 0;
};

static bool build_hit_lists(const ListShape& h, const std::vector<int>& rowptr, const std::vector<int>& colidx,
                            const std::vector<int>& icpt, HitLists& L)
{
    const int nc = h.nc, d = h.d, U = h.U, nseg = h.nseg;
    if (h.maxn > 0x7ffe || d > 0x1fff) return false;
    std::vector<long long> pairs(nc, 0), work(nc + 1, 0);
    long long total = 0;
    for (int c = 0; c < nc; ++c) {
        for (int s = h.soff[c]; s < h.soff[c + 1]; ++s) {
            const long long m = rowptr[s + 1] - rowptr[s] - (icpt[c] ? 1 : 0);
            pairs[c] += m * (m - 1) / 2;
        }
        if (pairs[c] > 16ll * U) return false;
        total += pairs[c];
        work[c + 1] = work[c] + 8 * pairs[c] + U;     // two walks of the pairs, one of the positions
    }
    if (total > (64ll << 20)) return false;
    auto for_pairs = [&](int c, auto&& f) {   // f(local sample, position)
        const int last = icpt[c] ? d - 1 : d;
        for (int s = h.soff[c]; s < h.soff[c + 1]; ++s) {
            const int b0 = rowptr[s], b1 = rowptr[s + 1];
            for (int y = b0; y < b1; ++y) {
                const int b = colidx[y];
                if (b >= last) break;
                const int pb = b * (b + 1) / 2;
                for (int x = b0; x < y; ++x) f(s - h.soff[c], pb + colidx[x]);
            }
        }
    };
    // one pass per client range: each client's codes in place, its records (client-relative starts
    // of their samples), samples and per-segment record counts in the client's own buffers (a
    // record holds two samples or more: at most pairs / 2 records, pairs samples)
    struct Local {
        std::vector<uint32_t> rec, seg;
        std::vector<uint16_t> hits;
        int maxrec = 0;
    };
    std::vector<Local> loc(nc);
    L.ncode = (size_t)nc * h.ustr;
    L.code.reset(new uint16_t[L.ncode]);
    for_client_ranges(nc, [&](int, int c0, int c1) {
        // per position: its samples so far (high 16 bits) and the first of them (low 16 bits); after
        // the segment walk, a multi-sample position's next slot in the client's samples with bit 31
        // set, else 0
        std::vector<uint32_t> cf(U);
        for (int c = c0; c < c1; ++c) {
            Local& o = loc[c];
            std::fill(cf.begin(), cf.end(), 0u);
            for_pairs(c, [&](int ls, int p) {
                const uint32_t v = cf[p];
                cf[p] = v ? v + 0x10000u : 0x10000u | (uint32_t)ls;
            });
            uint16_t* code = L.code.get() + (size_t)c * h.ustr;
            o.seg.resize((size_t)nseg + 1);
            o.rec.resize((size_t)(pairs[c] / 2));
            uint32_t r = 0, e = 0;
            for (int g = 0; g < nseg; ++g) {
                o.seg[g] = r;
                const uint32_t rg = r;
                for (int p = g * 512; p < std::min(U, g * 512 + 512); ++p) {
                    const uint32_t v = cf[p];
                    if (v < 0x20000u) {          // no sample, or one
                        code[p] = v ? (uint16_t)(v & 0xffffu) : (uint16_t)kHitNone;
                        cf[p] = 0;
                    } else {
                        code[p] = (uint16_t)(0x8000u | (r - rg));
                        o.rec[r++] = e;
                        cf[p] = 0x80000000u | e;
                        e += v >> 16;
                    }
                }
                o.maxrec = std::max(o.maxrec, (int)(r - rg));
            }
            o.seg[nseg] = r;
            o.rec.resize(r);
            std::fill(code + U, code + h.ustr, (uint16_t)kHitNone);
            o.hits.resize(e);
            for_pairs(c, [&](int ls, int p) {
                const uint32_t v = cf[p];
                if (v >> 31) {
                    o.hits[v & 0x7fffffffu] = (uint16_t)ls;
                    cf[p] = v + 1;
                }
            });
            for (int j = 0; j < d; ++j) {
                code[j * (j + 1) / 2 + j] = (uint16_t)(0xc000u | (unsigned)j);
                if (icpt[c] && j == d - 1)
                    for (int i = 0; i < j; ++i) code[j * (j + 1) / 2 + i] = (uint16_t)(0xa000u | (unsigned)i);
            }
        }
    }, &work);
    std::vector<long long> rbase(nc + 1, 0), hbase(nc + 1, 0);
    for (int c = 0; c < nc; ++c) {
        rbase[c + 1] = rbase[c] + (long long)loc[c].rec.size();
        hbase[c + 1] = hbase[c] + (long long)loc[c].hits.size();
        L.maxrec = std::max(L.maxrec, loc[c].maxrec);
    }
    if (hbase[nc] >= 0xffffffffll) return false;
    L.maxrec = std::max(1, L.maxrec);
    L.nseg = (size_t)nc * (nseg + 1);
    L.nrec = (size_t)rbase[nc] + 1;
    L.nhits = (size_t)hbase[nc];
    L.seg.reset(new uint32_t[L.nseg]);
    L.rec.reset(new uint32_t[L.nrec]);
    L.hits.reset(new uint16_t[std::max<size_t>(1, L.nhits)]);
    L.rec[rbase[nc]] = (uint32_t)hbase[nc];
    // the clients' buffers at their global offsets (record starts and segment counts rebased)
    for_client_ranges(nc, [&](int, int c0, int c1) {
        for (int c = c0; c < c1; ++c) {
            const Local& o = loc[c];
            for (size_t r = 0; r < o.rec.size(); ++r) L.rec[rbase[c] + r] = (uint32_t)(hbase[c] + o.rec[r]);
            for (int g = 0; g <= nseg; ++g) L.seg[(size_t)c * (nseg + 1) + g] = (uint32_t)(rbase[c] + o.seg[g]);
            if (!o.hits.empty()) std::memcpy(L.hits.get() + hbase[c], o.hits.data(), o.hits.size() * 2);
        }
    }, &hbase);
    return true;
}

// The binary layout of the uploaded clients on the device: CSR columns, per-client bitmaps (from the
// host, or packed on the device by k_pack_bits when fbits_host is null), intercept flags, the
// common-sample lists when they are built, the Hessian kernels' shared-memory shapes; the labels'
// device buffer is returned in *lab.
static int install_binary(fednl_handle h, const std::vector<int>& rowptr, const std::vector<int>& colidx,
                          const std::vector<int>& icpt, const std::vector<unsigned long long>* fbits_host, double** lab)
{
    const int d = h->d, S = h->S, nc = h->nc;
    Dev& P = h->dev;
    std::vector<long long> fboff(nc);
    long long words = 0;
    for (int c = 0; c < nc; ++c) {
        fboff[c] = words;
        words += (long long)d * ((h->ns[c] + 63) / 64);
    }
    HitLists hl;
    h->hits_ready = build_hit_lists({h->nc, h->d, h->U, h->ustr, h->nseg, h->maxn, h->soff.data()}, rowptr, colidx,
                                    icpt, hl);
    h->hits_maxrec = h->hits_ready ? hl.maxrec : 0;
    uint16_t *d_hcode = nullptr, *d_hhits = nullptr;
    uint32_t *d_hseg = nullptr, *d_hrec = nullptr;
    if (h->hits_ready) {
        h->feat.want(&d_hcode, hl.ncode);
        h->feat.want(&d_hseg, hl.nseg);
        h->feat.want(&d_hrec, hl.nrec);
        h->feat.want(&d_hhits, std::max<size_t>(1, hl.nhits));
    }
    int *d_rowptr, *d_colidx, *d_icpt;
    long long* d_fboff;
    unsigned long long* d_fbits;
    h->feat.want(&d_icpt, nc);
    h->feat.want(&d_rowptr, S + 1);
    h->feat.want(&d_colidx, std::max<size_t>(1, colidx.size()));
    h->feat.want(&d_fboff, nc);
    h->feat.want(&d_fbits, std::max<long long>(1, words));
    h->feat.want(lab, S);
    int rc = h->feat.commit();
    if (rc) return rc;
    CK(cudaMemcpy(d_rowptr, rowptr.data(), (S + 1) * 4, cudaMemcpyHostToDevice));
    if (!colidx.empty()) CK(cudaMemcpy(d_colidx, colidx.data(), colidx.size() * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_fboff, fboff.data(), nc * 8, cudaMemcpyHostToDevice));
    if (fbits_host) {
        CK(cudaMemcpy(d_fbits, fbits_host->data(), words * 8, cudaMemcpyHostToDevice));
    } else {
        CK(cudaMemsetAsync(d_fbits, 0, (size_t)std::max<long long>(1, words) * 8, h->stream));
        k_pack_bits<<<(S + 127) / 128, 128, 0, h->stream>>>(d_rowptr, d_colidx, P.client_of, P.soff, P.ns, d_fboff, S,
                                                            d_fbits);
        CKL();
        CK(cudaStreamSynchronize(h->stream));
    }
    CK(cudaMemcpy(d_icpt, icpt.data(), nc * 4, cudaMemcpyHostToDevice));
    if (h->hits_ready) {
        CK(cudaMemcpy(d_hcode, hl.code.get(), hl.ncode * 2, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(d_hseg, hl.seg.get(), hl.nseg * 4, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(d_hrec, hl.rec.get(), hl.nrec * 4, cudaMemcpyHostToDevice));
        if (hl.nhits) CK(cudaMemcpy(d_hhits, hl.hits.get(), hl.nhits * 2, cudaMemcpyHostToDevice));
    }
    P.hcode = d_hcode;
    P.hseg = d_hseg;
    P.hrec = d_hrec;
    P.hhits = d_hhits;
    P.icpt = d_icpt;
    P.rowptr = d_rowptr;
    P.colidx = d_colidx;
    P.fboff = d_fboff;
    P.fbits = d_fbits;
    int maxW = (h->maxn + 63) / 64;
    // attribute masks (when they fit), D_s, and the diagonal values
    size_t need = (size_t)d * maxW * 8 + (size_t)h->maxn * 8 + (size_t)d * 8;
    h->hess_smem_gl = (size_t)h->maxn * 8 + (size_t)d * 8;
    h->hess_smem_sm = need <= 200 * 1024 ? need : 0;
    if (h->hits_ready && hits_smem(h, 512) > 200 * 1024) h->hits_ready = false;
    h->hess_kind = h->hits_ready ? kHessHits : h->hess_smem_sm ? kHessMasksSmem : kHessMasksGlobal;
    h->hess_nt = kHessThreads;
    if (h->hess_smem_gl > 200 * 1024) return fail(FEDNL_EINVAL, "client too large for the Hessian kernel (n=%d)", h->maxn);
    CK(raise_hess_smem(h));
    if ((size_t)h->maxn * 16 > 48 * 1024) CK(fednl_raise_dyn_smem((const void*)k_grad_binary, (size_t)h->maxn * 16));
    if (client_smem(h) > 48 * 1024) CK(fednl_raise_dyn_smem((const void*)k_client_binary, client_smem(h)));
    h->binary = 1;
    return FEDNL_OK;
}

// the handle's client-data pointers cleared before a new upload
static void clear_client_data(fednl_handle h)
{
    h->feat.release();
    Dev& P = h->dev;
    P.rowptr = nullptr;
    P.colidx = nullptr;
    P.fbits = nullptr;
    P.icpt = nullptr;
    P.A = nullptr;
    P.hcode = nullptr;
    P.hseg = nullptr;
    P.hrec = nullptr;
    P.hhits = nullptr;
    h->hits_ready = false;
}

// after either upload: labels, readiness, and the captured round (its launch shapes may change)
static int finish_upload(fednl_handle h, double* lab, const double* labels)
{
    CK(cudaMemcpy(lab, labels, (size_t)h->S * 8, cudaMemcpyHostToDevice));
    h->dev.lab = lab;
    h->data_ready = true;
    h->shifts_ready = false;
    if (h->gexec) {
        cudaGraphExecDestroy(h->gexec);
        cudaGraphDestroy(h->graph);
        h->gexec = nullptr;
        h->graph = nullptr;
    }
    return FEDNL_OK;
}

static int upload_client_data_impl(fednl_handle h, const double* features, const double* labels)
{
    if (!h || !features || !labels) return fail(FEDNL_EINVAL, "null argument");
    int d = h->d, S = h->S;
    for (int s = 0; s < S; ++s)
        if (labels[s] != 1.0 && labels[s] != -1.0) return fail(FEDNL_EINVAL, "label %d is not +-1", s);
    int fmt = h->desc.feature_format;
    // one pass per client range: the first value that is neither 0 nor 1 (samples in order, so the
    // earliest range holding one has the first of the whole upload), and for 0/1 data the range's
    // CSR columns (in a buffer of the range), set-attribute counts, the per-client bitmaps
    // (feature-major, 64 samples a word) and whether the last attribute is set in every sample
    const int nc = h->nc;
    std::vector<int> ones(S, 0);
    std::vector<long long> first_bad(nc, -1);
    std::vector<int> icpt(nc, 1);
    std::vector<long long> fboff(nc);
    long long words = 0;
    for (int c = 0; c < nc; ++c) {
        fboff[c] = words;
        words += (long long)d * ((h->ns[c] + 63) / 64);
    }
    std::vector<unsigned long long> fbits;
    std::vector<std::vector<int>> rcols(32);
    const std::vector<long long> rows(h->soff.begin(), h->soff.end());     // ranges of equal sample counts
    if (fmt != FEDNL_FEATURES_DENSE) {
        fbits.assign((size_t)std::max<long long>(1, words), 0ull);
        for_client_ranges(nc, [&](int t, int c0, int c1) {
            std::vector<int>& cols = rcols[t];
            for (int c = c0; c < c1; ++c) {
                const int W = (h->ns[c] + 63) / 64;
                for (int s = h->soff[c]; s < h->soff[c + 1]; ++s) {
                    const double* a = features + (size_t)s * d;
                    const int ls = s - h->soff[c];
                    int n1 = 0;
                    for (int i0 = 0; i0 < d; i0 += 4) {
                        const int i1 = std::min(d, i0 + 4);
                        if (i1 - i0 == 4) {      // four +0.0 values (all bits clear): nothing to record
                            uint64_t w[4];
                            std::memcpy(w, a + i0, sizeof w);
                            if ((w[0] | w[1] | w[2] | w[3]) == 0) continue;
                        }
                        for (int i = i0; i < i1; ++i) {
                            if (a[i] == 1.0) {
                                ++n1;
                                cols.push_back(i);
                                fbits[fboff[c] + (size_t)i * W + (ls >> 6)] |= 1ull << (ls & 63);
                            } else if (a[i] != 0.0) {
                                first_bad[c0] = (long long)s * d + i;
                                return;
                            }
                        }
                    }
                    ones[s] = n1;
                    if (a[d - 1] != 1.0) icpt[c] = 0;
                }
            }
        }, &rows);
    }
    long long bad = -1;
    for (int c = 0; c < nc && bad < 0; ++c) bad = first_bad[c];
    if (fmt == FEDNL_FEATURES_AUTO) fmt = bad < 0 ? FEDNL_FEATURES_BINARY : FEDNL_FEATURES_DENSE;
    if (fmt == FEDNL_FEATURES_BINARY && bad >= 0)
        return fail(FEDNL_EINVAL, "feature (%d,%d) is not 0/1 in binary format", (int)(bad / d), (int)(bad % d));
    clear_client_data(h);
    Dev& P = h->dev;
    double* lab = nullptr;
    if (fmt == FEDNL_FEATURES_BINARY) {
        std::vector<int> rowptr(S + 1, 0);
        for (int s = 0; s < S; ++s) rowptr[s + 1] = rowptr[s] + ones[s];
        std::vector<int> colidx(rowptr[S]);
        {
            size_t at = 0;        // the ranges' columns in range order (ranges are contiguous, ascending)
            for (auto& v : rcols) {
                if (!v.empty()) std::memcpy(colidx.data() + at, v.data(), v.size() * 4);
                at += v.size();
                std::vector<int>().swap(v);
            }
        }
        int rc = install_binary(h, rowptr, colidx, icpt, &fbits, &lab);
        if (rc) return rc;
    } else {
        double* dA;
        h->feat.want(&dA, (size_t)S * d);
        h->feat.want(&lab, S);
        int rc = h->feat.commit();
        if (rc) return rc;
        CK(cudaMemcpy(dA, features, (size_t)S * d * 8, cudaMemcpyHostToDevice));
        P.A = dA;
        h->binary = 0;
    }
    return finish_upload(h, lab, labels);
}

int fednl_gpu_upload_client_data(fednl_handle h, const double* features, const double* labels)
{
    return host_guarded([&] { return upload_client_data_impl(h, features, labels); });
}

// CSR rows of 0/1 features: rowptr from 0, non-decreasing, each row's columns ascending in [0, d).
static int check_csr_rows(int d, int S, const int32_t* rowptr, const int32_t* colidx)
{
    if (rowptr[0] != 0) return fail(FEDNL_EINVAL, "rowptr[0] is not 0");
    for (int s = 0; s < S; ++s) {
        if (rowptr[s + 1] < rowptr[s]) return fail(FEDNL_EINVAL, "rowptr decreases at sample %d", s);
        if (rowptr[s + 1] > rowptr[s] && !colidx) return fail(FEDNL_EINVAL, "null colidx");
        for (int u = rowptr[s]; u < rowptr[s + 1]; ++u)
            if (colidx[u] < 0 || colidx[u] >= d || (u > rowptr[s] && colidx[u] <= colidx[u - 1]))
                return fail(FEDNL_EINVAL, "sample %d: columns not ascending in [0, d)", s);
    }
    return FEDNL_OK;
}

// per client: 1 when the last attribute is set in every one of its samples (an intercept column)
static std::vector<int> csr_intercepts(int d, int nc, const int32_t* soff, const std::vector<int>& rp,
                                       const std::vector<int>& ci)
{
    std::vector<int> icpt(nc, 1);
    for (int c = 0; c < nc; ++c)
        for (int s = soff[c]; s < soff[c + 1] && icpt[c]; ++s)
            if (rp[s + 1] == rp[s] || ci[rp[s + 1] - 1] != d - 1) icpt[c] = 0;
    return icpt;
}

static int upload_client_csr_impl(fednl_handle h, const int32_t* rowptr, const int32_t* colidx, const double* labels)
{
    if (!h || !rowptr || !labels) return fail(FEDNL_EINVAL, "null argument");
    const int d = h->d, S = h->S, nc = h->nc;
    for (int s = 0; s < S; ++s)
        if (labels[s] != 1.0 && labels[s] != -1.0) return fail(FEDNL_EINVAL, "label %d is not +-1", s);
    if (h->desc.feature_format == FEDNL_FEATURES_DENSE)
        return fail(FEDNL_EINVAL, "the CSR upload takes binary features (the handle asks for the dense format)");
    int rc = check_csr_rows(d, S, rowptr, colidx);
    if (rc) return rc;
    std::vector<int> rp(rowptr, rowptr + S + 1), ci(colidx ? colidx : rowptr, colidx ? colidx + rowptr[S] : rowptr);
    const std::vector<int> icpt = csr_intercepts(d, nc, h->soff.data(), rp, ci);
    clear_client_data(h);
    double* lab = nullptr;
    rc = install_binary(h, rp, ci, icpt, nullptr, &lab);
    if (rc) return rc;
    return finish_upload(h, lab, labels);
}

int fednl_gpu_upload_client_csr(fednl_handle h, const int32_t* rowptr, const int32_t* colidx, const double* labels)
{
    return host_guarded([&] { return upload_client_csr_impl(h, rowptr, colidx, labels); });
}

int fednl_gpu_hit_lists(int32_t d, int32_t nclients, const int32_t* n_samples, const int32_t* rowptr,
                        const int32_t* colidx, int64_t* sizes, int32_t* maxrec, uint16_t* code, uint32_t* seg,
                        uint32_t* rec, uint16_t* hits)
{
    return host_guarded([&]() -> int {
        if (d < 1 || nclients < 1 || !n_samples || !rowptr || !sizes) return fail(FEDNL_EINVAL, "bad argument");
        std::vector<int32_t> soff(nclients + 1, 0);
        int maxn = 0;
        for (int c = 0; c < nclients; ++c) {
            if (n_samples[c] < 1) return fail(FEDNL_EINVAL, "client %d has no samples", c);
            if ((long long)soff[c] + n_samples[c] > 0x7fffffff) return fail(FEDNL_EINVAL, "too many samples");
            soff[c + 1] = soff[c] + n_samples[c];
            maxn = std::max(maxn, n_samples[c]);
        }
        const int S = soff[nclients];
        int rc = check_csr_rows(d, S, rowptr, colidx);
        if (rc) return rc;
        if (d > 0x1fff) return fail(FEDNL_EINVAL, "the common-sample lists are not built for d > %d", 0x1fff);
        std::vector<int> rp(rowptr, rowptr + S + 1), ci(colidx ? colidx : rowptr, colidx ? colidx + rowptr[S] : rowptr);
        const std::vector<int> icpt = csr_intercepts(d, nclients, soff.data(), rp, ci);
        const int U = d * (d + 1) / 2;
        HitLists L;
        if (!build_hit_lists({nclients, d, U, (U + 31) / 32 * 32, (U + 511) / 512, maxn, soff.data()}, rp, ci, icpt, L))
            return fail(FEDNL_EINVAL, "the common-sample lists are not built for this problem (size limits)");
        sizes[0] = (int64_t)L.ncode;
        sizes[1] = (int64_t)L.nseg;
        sizes[2] = (int64_t)L.nrec;
        sizes[3] = (int64_t)L.nhits;
        if (maxrec) *maxrec = L.maxrec;
        if (code) std::memcpy(code, L.code.get(), L.ncode * 2);
        if (seg) std::memcpy(seg, L.seg.get(), L.nseg * 4);
        if (rec) std::memcpy(rec, L.rec.get(), L.nrec * 4);
        if (hits && L.nhits) std::memcpy(hits, L.hits.get(), L.nhits * 2);
        return FEDNL_OK;
    });
}

int fednl_gpu_init_shifts(fednl_handle h, const double* x0)
{
    if (!h) return fail(FEDNL_EINVAL, "null handle");
    if (!h->data_ready) return fail(FEDNL_EINVAL, "upload client data first");
    Dev& P = h->dev;
    cudaStream_t st = h->stream;
    if (x0) CK(cudaMemcpyAsync(P.x, x0, h->d * 8, cudaMemcpyHostToDevice, st));
    else CK(cudaMemsetAsync(P.x, 0, h->d * 8, st));
    int S = h->S;
    if (P.ref) k_margin_ref<<<(S + 255) / 256, 256, 0, st>>>(P, S);
    else if (h->binary) k_margin_binary<<<(S + 255) / 256, 256, 0, st>>>(P, S);
    else k_margin_dense<<<(S + 255) / 256, 256, 0, st>>>(P, S);
    CKL();
    if (h->binary) {    // gradient pass also forms the diagonal sums the Hessian kernel reuses
        k_grad_binary<<<dim3((2 * h->d + 127) / 128, h->nc), 128, (size_t)h->maxn * 16, st>>>(P);
        CKL();
    }
    Dev Pall = P;             // every client's initial shift, whatever a round processes
    Pall.act = nullptr;
    Pall.n_act = h->nc;
    if (h->binary) {
        CK(launch_hess_binary(h, Pall, h->nc, 1, st, h->hess_kind, h->hess_nt));
    } else {
        k_hess_dense<<<dim3(h->nfpart, h->nc), kHessThreads, 0, st>>>(Pall, 1);
        CKL();
    }
    k_h_init<<<(h->U + 255) / 256, 256, 0, st>>>(P);
    CKL();
    if (h->pp) {
        if (!h->binary) {
            k_grad_dense<<<dim3((h->d + 127) / 128, h->nc), 128, 0, st>>>(P);
            CKL();
        }
        k_pp_init_dir<<<h->nc, 128, 0, st>>>(P);
        CKL();
        k_pp_init_mean<<<(h->d + 127) / 128, 128, 0, st>>>(P);
        CKL();
        const unsigned seed = h->desc.client_seed;
        CK(cudaMemcpyAsync(P.sampler, &seed, 4, cudaMemcpyHostToDevice, st));
        CK(cudaMemsetAsync(P.stats, 0, 16, st));
    }
    std::vector<unsigned> ws(h->W, h->desc.toplek_seed), rs(h->nc);
    for (int c = 0; c < h->nc; ++c)     // TrainLoop.h:632; the Philox stream counts draws instead
        rs[c] = h->comp == FEDNL_RANDK_PHILOX ? 0u : h->desc.seed_base + (unsigned)c;
    CK(cudaMemcpyAsync(P.wstate, ws.data(), h->W * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(P.rstate, rs.data(), h->nc * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(P.round_ctr, 0, 4, st));
    CK(cudaMemsetAsync(P.status, 0, 4, st));
    CK(cudaStreamSynchronize(st));
    h->shifts_ready = true;
    h->rounds_done = 0;
    return FEDNL_OK;
}

int fednl_gpu_run(fednl_handle h, int32_t rounds, double* grad_norms)
{
    if (!h) return fail(FEDNL_EINVAL, "null handle");
    if (!h->shifts_ready) return fail(FEDNL_EINVAL, "call fednl_gpu_init_shifts first");
    if (rounds < 0) return fail(FEDNL_EINVAL, "rounds < 0");
    int rc = build_graph(h);
    if (rc) return rc;
    CK(cudaMemsetAsync(h->dev.status, 0, 4, h->stream));
    for (int r = 0; r < rounds; ++r) CK(cudaGraphLaunch(h->gexec, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    int first = h->rounds_done;
    h->rounds_done += rounds;
    if (grad_norms && rounds > 0) {
        int have = std::max(0, std::min(rounds, h->dev.hist_cap - first));
        if (have > 0) CK(cudaMemcpy(grad_norms, h->dev.hist + first, (size_t)have * 8, cudaMemcpyDeviceToHost));
        for (int r = have; r < rounds; ++r) grad_norms[r] = NAN;
    }
    int status = 0;
    CK(cudaMemcpy(&status, h->dev.status, 4, cudaMemcpyDeviceToHost));
    if (status == FEDNL_ETIMEOUT) return fail(status, "grid barrier of the Cholesky timed out");
    if (status) return fail(status, "Option-B matrix not positive definite in one of the rounds");
    return FEDNL_OK;
}

// One round: the captured graph, then the round's ||g||, l and status copied into one pinned
// buffer and a single wait (fednl_gpu_run's semantics for one round).
int fednl_gpu_round(fednl_handle h, fednl_round_stats* stats)
{
    if (!h) return fail(FEDNL_EINVAL, "null handle");
    if (!h->shifts_ready) return fail(FEDNL_EINVAL, "call fednl_gpu_init_shifts first");
    int rc = build_graph(h);
    if (rc) return rc;
    if (!h->pin) CK(cudaMallocHost(&h->pin, 32));
    double* pst = static_cast<double*>(h->pin);
    int* pstatus = reinterpret_cast<int*>(pst + 2);
    CK(cudaMemsetAsync(h->dev.status, 0, 4, h->stream));
    CK(cudaGraphLaunch(h->gexec, h->stream));
    CK(cudaMemcpyAsync(pst, h->dev.stats, 16, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(pstatus, h->dev.status, 4, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->rounds_done += 1;
    const int status = *pstatus;
    if (status == FEDNL_ETIMEOUT) rc = fail(status, "grid barrier of the Cholesky timed out");
    else if (status) rc = fail(status, "Option-B matrix not positive definite in one of the rounds");
    if (stats) {
        stats->round = h->rounds_done - 1;
        stats->status = rc == FEDNL_ENOTPD ? FEDNL_ENOTPD : FEDNL_OK;
        stats->grad_norm = pst[0];
        stats->l = pst[1];
    }
    return rc;
}

double fednl_gpu_get_f(fednl_handle h)
{
    if (!h || !h->dev.fmode) return NAN;
    double v = NAN;
    cudaStreamSynchronize(h->stream);
    cudaMemcpy(&v, h->dev.stats + 2, 8, cudaMemcpyDeviceToHost);
    return v;
}

int32_t fednl_gpu_get_ls_steps(fednl_handle h)
{
    if (!h || !h->desc.line_search) return 0;
    double v = 0.0;
    cudaStreamSynchronize(h->stream);
    cudaMemcpy(&v, h->dev.ls + 3, 8, cudaMemcpyDeviceToHost);
    return (int32_t)v;
}

int fednl_gpu_get_selected(fednl_handle h, int32_t* clients, int32_t* count)
{
    if (!h || !count) return fail(FEDNL_EINVAL, "null argument");
    if (!h->pp) return fail(FEDNL_EINVAL, "handle without FedNL-PP");
    CK(cudaStreamSynchronize(h->stream));
    *count = h->tau;
    if (clients) CK(cudaMemcpy(clients, h->dev.act, (size_t)h->tau * 4, cudaMemcpyDeviceToHost));
    return FEDNL_OK;
}

int fednl_gpu_get_true_grad(fednl_handle h, double* g)
{
    if (!h || !g) return fail(FEDNL_EINVAL, "null argument");
    if (!h->pp) return fail(FEDNL_EINVAL, "handle without FedNL-PP");
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaMemcpy(g, h->dev.tg, h->d * 8, cudaMemcpyDeviceToHost));
    return FEDNL_OK;
}

int fednl_gpu_get_dir(fednl_handle h, int32_t client, double* dir, double* ddir)
{
    if (!h || client < 0 || client >= h->nc) return fail(FEDNL_EINVAL, "bad argument");
    if (!h->pp) return fail(FEDNL_EINVAL, "handle without FedNL-PP");
    CK(cudaStreamSynchronize(h->stream));
    if (dir) CK(cudaMemcpy(dir, h->dev.dir + (size_t)client * h->d, h->d * 8, cudaMemcpyDeviceToHost));
    if (ddir) CK(cudaMemcpy(ddir, h->dev.ddir + (size_t)client * h->d, h->d * 8, cudaMemcpyDeviceToHost));
    return FEDNL_OK;
}

int fednl_gpu_client_phase(fednl_handle h)
{
    if (!h) return fail(FEDNL_EINVAL, "null handle");
    if (!h->shifts_ready) return fail(FEDNL_EINVAL, "call fednl_gpu_init_shifts first");
    if (h->desc.line_search || h->pp) return fail(FEDNL_EINVAL, "the split round serves plain FedNL");
    CK(cudaMemsetAsync(h->dev.status, 0, 4, h->stream));
    return launch_round(h, nullptr, true);
}

void* fednl_gpu_stream(fednl_handle h) { return h ? (void*)h->stream : nullptr; }

int fednl_gpu_round_result(fednl_handle h, fednl_round_stats* stats)
{
    if (!h) return fail(FEDNL_EINVAL, "null handle");
    CK(cudaStreamSynchronize(h->stream));
    double st[2] = {0, 0};
    int status = 0;
    CK(cudaMemcpy(st, h->dev.stats, 16, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&status, h->dev.status, 4, cudaMemcpyDeviceToHost));
    if (stats) {
        stats->round = h->rounds_done - 1;
        stats->status = status == FEDNL_ENOTPD ? FEDNL_ENOTPD : FEDNL_OK;
        stats->grad_norm = st[0];
        stats->l = st[1];
    }
    if (status == FEDNL_ETIMEOUT) return fail(status, "grid barrier of the Cholesky timed out");
    if (status) return fail(status, "Option-B matrix not positive definite");
    return FEDNL_OK;
}

int fednl_gpu_solve_batch(fednl_handle* hs, int32_t n, fednl_mx_handle* mxs, int32_t nmx)
{
    if (n < 0 || nmx < 0 || (n && !hs) || (nmx && !mxs)) return fail(FEDNL_EINVAL, "bad argument");
    static cudaStream_t bst = nullptr;
    if (!bst) CK(cudaStreamCreateWithFlags(&bst, cudaStreamNonBlocking));
    std::vector<FednlSolveDesc> descs;
    std::vector<cudaStream_t> streams;
    for (int i = 0; i < n; ++i) {
        fednl_handle h = hs[i];
        if (!h || !h->shifts_ready) return fail(FEDNL_EINVAL, "handle %d not initialised", i);
        Dev& P = h->dev;
        FednlSolveDesc S{};
        S.H = P.H;
        S.d = h->d;
        S.lptr = h->desc.option_a ? nullptr : P.stats + 1;
        S.lval = P.lambda;
        S.ls = P.ls;
        S.g = P.g;
        S.dx = P.dx;
        S.xupd = P.x;
        S.work = P.work;
        S.ybuf = P.ybuf;
        S.rinv = P.rinv;
        S.bar = P.bar;
        S.status = P.status;
        S.stats = P.stats;
        S.hist = P.hist;
        S.round_ctr = P.round_ctr;
        S.hist_cap = P.hist_cap;
        S.record = 1;
        descs.push_back(S);
        streams.push_back(h->stream);
    }
    std::vector<fednl_mx_handle> small;       // mixed handles with the FP32 shared-memory solve
    for (int i = 0; i < nmx; ++i) {
        FednlSolveDesc S{};
        cudaStream_t s2 = nullptr;
        if (fednl_mx_solve_desc(mxs[i], &S, (void**)&s2)) return fail(FEDNL_EINVAL, "mixed handle %d not initialised", i);
        streams.push_back(s2);
        if (fednl_mx_uses_chol32(mxs[i]))
            small.push_back(mxs[i]);
        else
            descs.push_back(S);
    }
    // the batch stream waits for every client phase, the problems' streams wait for the solve
    for (cudaStream_t s2 : streams) {
        cudaEvent_t e;
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        CK(cudaEventRecord(e, s2));
        CK(cudaStreamWaitEvent(bst, e, 0));
        cudaEventDestroy(e);
    }
    int rc = fednl_solve_batch_launch(descs.data(), (int)descs.size(), bst);
    if (rc) return rc;
    rc = fednl_mx_solve32_batch(small.data(), (int)small.size(), bst);
    if (rc) return rc;
    for (int i = 0; i < n; ++i) hs[i]->rounds_done += 1;
    return FEDNL_OK;
}

namespace {
// clients' sample counts bucketed by powers of two: n_i in (2^(b-1), 2^b] is bucket b
int ni_bucket_of(int n)
{
    int b = 0;
    while ((1 << b) < n && b < 30) ++b;
    return b;
}

// The binary Hessian's kernel and launch shape (common-sample lists, masks staged in shared memory
// or masks read from global memory; 128, 256 or 512 threads per block) for this d and the clients'
// largest n_i bucket: measured once per process and key on the handle's own data (round-mode
// launches between rounds: their outputs are recomputed by the next round before any use), cached
// for later handles.  Returns 1 when the handle's shape changed.
int tune_hess_shape(fednl_handle h)
{
    struct Shape {
        int kind;
        int nt;
        double ms;
    };
    static std::mutex mu;
    static std::map<std::pair<int, int>, Shape> cache;
    const std::pair<int, int> key(h->d, ni_bucket_of(h->maxn) + (h->hess_smem_sm ? 0 : 64) + (h->hits_ready ? 0 : 128) +
                                            (round_hess_mode(h) == 3 ? 256 : 0));
    Shape best{h->hess_kind, h->hess_nt, 0.0};
    bool hit = false;
    {
        std::lock_guard<std::mutex> g(mu);
        auto it = cache.find(key);
        if (it != cache.end()) {
            best = it->second;
            hit = true;
        }
    }
    if (!hit) {
        cudaStream_t st = h->stream;
        cudaEvent_t e0, e1;
        CK(cudaEventCreate(&e0));
        CK(cudaEventCreate(&e1));
        best.ms = 1e30;
        const Dev& Q = h->dev;
        for (int kind : {kHessHits, kHessMasksSmem, kHessMasksGlobal}) {
            if ((kind == kHessHits && !h->hits_ready) || (kind == kHessMasksSmem && !h->hess_smem_sm)) continue;
            for (int nt : {128, 256, 512}) {
                const int mode = round_hess_mode(h) == 3 ? 3 : 0;
                cudaError_t e = launch_hess_binary(h, Q, h->nc, mode, st, kind, nt);   // warm-up
                for (int r = 0; r < 3 && e == cudaSuccess; ++r) {
                    if (r == 1) e = cudaEventRecord(e0, st);
                    if (e == cudaSuccess) e = launch_hess_binary(h, Q, h->nc, mode, st, kind, nt);
                }
                if (e == cudaSuccess) e = cudaEventRecord(e1, st);
                if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                float t = 0.f;
                if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
                if (e != cudaSuccess) {
                    cudaEventDestroy(e0);
                    cudaEventDestroy(e1);
                    return fail(FEDNL_ECUDA, "Hessian tuning launch failed: %s", cudaGetErrorString(e));
                }
                if (t / 2.0 < best.ms) best = Shape{kind, nt, t / 2.0};
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        std::lock_guard<std::mutex> g(mu);
        cache[key] = best;
    }
    const bool changed = best.kind != h->hess_kind || best.nt != h->hess_nt;
    h->hess_kind = best.kind;
    h->hess_nt = best.nt;
    h->hess_ms = best.ms;
    return changed ? 1 : 0;
}
}  // namespace

int fednl_gpu_autotune(fednl_handle h, int32_t* chol_grid_out, double* solve_ms)
{
    if (!h) return fail(FEDNL_EINVAL, "null handle");
    if (!h->shifts_ready) return fail(FEDNL_EINVAL, "call fednl_gpu_init_shifts first");
    CK(cudaStreamSynchronize(h->stream));
    Dev Q = h->dev;                        // scratch view: no statistics, no line-search state
    Q.ls = nullptr;
    double* scratch = nullptr;
    int* sstatus = nullptr;
    CK(cudaMalloc(&scratch, (size_t)h->d * 8));
    CK(cudaMalloc(&sstatus, 4));
    Q.status = sstatus;
    const double* lptr = h->desc.option_a ? nullptr : h->dev.stats + 1;
    const double lval = h->dev.lambda;
    auto launch = [&](int G) -> int {
        cudaError_t e = launch_chol(Q, G, h->stream, Q.H, 0, lptr, lval, Q.g, scratch, nullptr, 0);
        return e == cudaSuccess ? FEDNL_OK : fail(FEDNL_ECUDA, "tuning launch failed: %s", cudaGetErrorString(e));
    };
    int grid = h->chol_grid;
    double ms = 0.0;
    int rc = fednl_tune_chol_grid(h->d, launch, h->stream, &grid, &ms);
    cudaFree(scratch);
    cudaFree(sstatus);
    if (rc) return rc;
    bool reshape = grid != h->chol_grid;
    h->chol_grid = grid;
    if (h->binary && !h->pp) {
        rc = tune_hess_shape(h);
        if (rc > 0) reshape = true;
        else if (rc < 0) return rc;
    }
    if (reshape && h->gexec) {             // the captured round holds the old launch shapes
        cudaGraphExecDestroy(h->gexec);
        cudaGraphDestroy(h->graph);
        h->gexec = nullptr;
        h->graph = nullptr;
    }
    if (chol_grid_out) *chol_grid_out = grid;
    if (solve_ms) *solve_ms = ms;
    return FEDNL_OK;
}

int fednl_gpu_autotune_shapes(fednl_handle h, int32_t* hess_threads, int32_t* hess_masks_in_smem, int32_t* ni_bucket,
                              double* hess_ms)
{
    if (!h) return fail(FEDNL_EINVAL, "null handle");
    if (hess_threads) *hess_threads = h->binary ? h->hess_nt : kHessThreads;
    if (hess_masks_in_smem) *hess_masks_in_smem = h->binary && h->hess_kind == kHessMasksSmem ? 1 : 0;
    if (ni_bucket) *ni_bucket = ni_bucket_of(h->maxn);
    if (hess_ms) *hess_ms = h->hess_ms;
    return FEDNL_OK;
}

int fednl_gpu_hess_schedule(fednl_handle h, int32_t* kind, int32_t* threads, int32_t* lists_built)
{
    if (!h) return fail(FEDNL_EINVAL, "null handle");
    if (kind) *kind = h->binary ? h->hess_kind : -1;
    if (threads) *threads = h->binary ? h->hess_nt : kHessThreads;
    if (lists_built) *lists_built = h->binary && h->hits_ready ? 1 : 0;
    return FEDNL_OK;
}

int fednl_gpu_set_hess_schedule(fednl_handle h, int32_t kind, int32_t threads)
{
    if (!h) return fail(FEDNL_EINVAL, "null handle");
    if (!h->binary) return fail(FEDNL_EINVAL, "the Hessian schedule applies to binary features only");
    if (threads != 128 && threads != 256 && threads != 512) return fail(FEDNL_EINVAL, "threads must be 128, 256 or 512");
    if (kind == kHessHits && !h->hits_ready) return fail(FEDNL_EINVAL, "no common-sample lists for this data");
    if (kind == kHessMasksSmem && !h->hess_smem_sm) return fail(FEDNL_EINVAL, "the masks do not fit in shared memory");
    if (kind < kHessMasksSmem || kind > kHessHits) return fail(FEDNL_EINVAL, "unknown Hessian kernel %d", kind);
    CK(cudaStreamSynchronize(h->stream));
    h->hess_kind = kind;
    h->hess_nt = threads;
    if (h->gexec) {                        // the captured round holds the old launch shape
        cudaGraphExecDestroy(h->gexec);
        cudaGraphDestroy(h->graph);
        h->gexec = nullptr;
        h->graph = nullptr;
    }
    return FEDNL_OK;
}

int fednl_gpu_mem_info(int64_t* free_bytes, int64_t* total_bytes)
{
    size_t f = 0, t = 0;
    CK(cudaMemGetInfo(&f, &t));
    if (free_bytes) *free_bytes = (int64_t)f;
    if (total_bytes) *total_bytes = (int64_t)t;
    return FEDNL_OK;
}

int fednl_gpu_get_x(fednl_handle h, double* x)
{
    if (!h || !x) return fail(FEDNL_EINVAL, "null argument");
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaMemcpy(x, h->dev.x, h->d * 8, cudaMemcpyDeviceToHost));
    return FEDNL_OK;
}

int fednl_gpu_set_x(fednl_handle h, const double* x)
{
    if (!h || !x) return fail(FEDNL_EINVAL, "null argument");
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaMemcpy(h->dev.x, x, h->d * 8, cudaMemcpyHostToDevice));
    return FEDNL_OK;
}

int fednl_gpu_get_grad(fednl_handle h, double* g)
{
    if (!h || !g) return fail(FEDNL_EINVAL, "null argument");
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaMemcpy(g, h->dev.g, h->d * 8, cudaMemcpyDeviceToHost));
    return FEDNL_OK;
}

static int packed_to_full(fednl_handle h, const double* dsrc, double* out)
{
    std::vector<double> up(h->U);
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaMemcpy(up.data(), dsrc, (size_t)h->U * 8, cudaMemcpyDeviceToHost));
    int d = h->d, lda = h->lda;
    std::fill(out, out + (size_t)d * lda, 0.0);
    size_t p = 0;
    for (int j = 0; j < d; ++j)
        for (int i = 0; i <= j; ++i, ++p) {
            out[(size_t)j * lda + i] = up[p];
            out[(size_t)i * lda + j] = up[p];
        }
    return FEDNL_OK;
}

int fednl_gpu_get_H(fednl_handle h, double* H)
{
    if (!h || !H) return fail(FEDNL_EINVAL, "null argument");
    return packed_to_full(h, h->dev.H, H);
}

int fednl_gpu_get_shift(fednl_handle h, int32_t client, double* shift)
{
    if (!h || !shift || client < 0 || client >= h->nc) return fail(FEDNL_EINVAL, "bad argument");
    return packed_to_full(h, h->dev.shift + (size_t)client * h->ustr, shift);
}

double fednl_gpu_get_l(fednl_handle h)
{
    if (!h) return NAN;
    double st[2] = {NAN, NAN};
    cudaStreamSynchronize(h->stream);
    cudaMemcpy(st, h->dev.stats, 16, cudaMemcpyDeviceToHost);
    return st[1];
}

double fednl_gpu_get_lk(fednl_handle h, int32_t client)
{
    if (!h || client < 0 || client >= h->nc) return NAN;
    double v = NAN;
    cudaStreamSynchronize(h->stream);
    cudaMemcpy(&v, h->dev.lk + client, 8, cudaMemcpyDeviceToHost);
    return v;
}

int fednl_gpu_get_message(fednl_handle h, int32_t client, uint32_t* idx, double* val, int32_t* count)
{
    if (!h || client < 0 || client >= h->nc || !count) return fail(FEDNL_EINVAL, "bad argument");
    CK(cudaStreamSynchronize(h->stream));
    int U = h->U, lda = h->lda;
    std::vector<double> dv(U);
    std::vector<unsigned> sel(h->SW);
    CK(cudaMemcpy(dv.data(), h->dev.diff + (size_t)client * h->ustr, (size_t)U * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(sel.data(), h->dev.sel + (size_t)client * h->SW, (size_t)h->SW * 4, cudaMemcpyDeviceToHost));
    std::vector<int> order;
    int comp = h->comp;
    if (comp == FEDNL_IDENTITY || comp == FEDNL_NATURAL) {
        order.resize(U);
        for (int p = 0; p < U; ++p) order[p] = p;
    } else if (comp == FEDNL_RANDSEQK) {
        int r = 0;
        CK(cudaMemcpy(&r, h->dev.rseq + client, 4, cudaMemcpyDeviceToHost));
        for (int t = 0; t < h->k; ++t) order.push_back((r + t) % U);
    } else {
        for (int p = 0; p < U; ++p)
            if ((sel[p >> 5] >> (p & 31)) & 1u) order.push_back(p);
    }
    const Dev& P = h->dev;
    // positions -> flat indices j * lda + i
    std::vector<int> colj(U), rowi(U);
    {
        int p = 0;
        for (int j = 0; j < h->d; ++j)
            for (int i = 0; i <= j; ++i, ++p) {
                colj[p] = j;
                rowi[p] = i;
            }
    }
    *count = (int32_t)order.size();
    for (size_t t = 0; t < order.size(); ++t) {
        int p = order[t];
        if (idx) idx[t] = (uint32_t)colj[p] * (uint32_t)lda + (uint32_t)rowi[p];
        if (val) {
            double item = dv[p];
            if (comp == FEDNL_NATURAL) {
                uint64_t b;
                memcpy(&b, &item, 8);
                b &= ~((1ull << 52) - 1);
                memcpy(&item, &b, 8);
                val[t] = P.prescale * item;
            } else {
                if (comp == FEDNL_RANDK || comp == FEDNL_RANDSEQK || comp == FEDNL_RANDK_PHILOX) item = item * P.mult;
                val[t] = item * P.prescale;
            }
        }
    }
    return FEDNL_OK;
}

// ---- wire format of the distributed client ---------------------------------------------------
// The bytes bin_fednl_distr_client sends its master for one client's round: each packet is a
// signal byte, the payload length as unsigned LEB128 and the payload
// (dopt/bin_fednl_distr_client/include/UsedTypes.h:1022-1125 with dopt::MutableData,
// dopt/copylocal/include/MutableData.h:488-536); Hessian messages in chunks of
// (1500 - 40 - 20 - 1 - 2) / 4 = 359 entries (LocalWorkerForFedNL_TopK.h:20-35).

namespace {

struct WireBuf {
    std::vector<uint8_t> b;
    void frame(uint8_t sig, const void* p, size_t n)
    {
        b.push_back(sig);
        uint64_t v = n;
        for (;;) {
            const uint8_t low = (uint8_t)(v & 0x7F);
            v >>= 7;
            if (!v) {
                b.push_back(low);
                break;
            }
            b.push_back((uint8_t)(low | 0x80));
        }
        const uint8_t* q = (const uint8_t*)p;
        b.insert(b.end(), q, q + n);
    }
};

constexpr int kWireChunk = (1500 - 40 - 20 - 1 - 2) / 4;

uint32_t natural_pack24(double a, double b)      // pack2FP64NoMantissa, FloatUtils.h:193-221
{
    uint64_t ba, bb;
    memcpy(&ba, &a, 8);
    memcpy(&bb, &b, 8);
    return ((uint32_t)(ba >> 63) << 23) | ((uint32_t)((ba >> 52) & 0x7FF) << 12) | ((uint32_t)(bb >> 63) << 11) |
           (uint32_t)((bb >> 52) & 0x7FF);
}

}  // namespace

int fednl_gpu_encode_client_round(fednl_handle h, int32_t client, int32_t flags, uint8_t* out, int64_t cap,
                                  int64_t* len)
{
    if (!h || client < 0 || client >= h->nc || !len || (flags & ~15)) return fail(FEDNL_EINVAL, "bad argument");
    if (h->pp) return fail(FEDNL_EINVAL, "FedNL-PP clients use another protocol");
    if (!h->shifts_ready) return fail(FEDNL_EINVAL, "call fednl_gpu_init_shifts first");
    const int comp = h->comp;
    if (comp == FEDNL_RANDK_PHILOX && !(flags & FEDNL_WIRE_RANDK_INDICES))
        return fail(FEDNL_EINVAL, "a reference master cannot re-derive RandK-Philox positions: send the indices");
    if ((flags & FEDNL_WIRE_FI) && !h->dev.fmode) return fail(FEDNL_EINVAL, "f_i is formed only with track_f or line_search");
    CK(cudaStreamSynchronize(h->stream));
    const Dev& P = h->dev;
    const int d = h->d, U = h->U;
    WireBuf W;
    std::vector<double> g(d);
    CK(cudaMemcpy(g.data(), P.gc + (size_t)client * d, (size_t)d * 8, cudaMemcpyDeviceToHost));
    W.frame(41, g.data(), (size_t)d * 8);                               // sig_messageGradient
    if (flags & FEDNL_WIRE_LK) {
        double lk = 0.0;
        CK(cudaMemcpy(&lk, P.lk + client, 8, cudaMemcpyDeviceToHost));
        W.frame(47, &lk, 8);                                             // sig_messageToSendLk
    }
    std::vector<double> dv(U);
    CK(cudaMemcpy(dv.data(), P.diff + (size_t)client * h->ustr, (size_t)U * 8, cudaMemcpyDeviceToHost));
    if (comp == FEDNL_NATURAL) {                                         // LocalWorkerForFedNL_Natural.h:143-201
        double packs[2] = {0.0, 0.0};
        int filled = 0, count = 0;
        std::vector<uint8_t> chunk;
        for (int p = 0; p < U; ++p) {
            packs[filled++] = dv[p];
            if (filled == 2) {
                const uint32_t w = natural_pack24(packs[0], packs[1]);
                chunk.push_back((uint8_t)w);
                chunk.push_back((uint8_t)(w >> 8));
                chunk.push_back((uint8_t)(w >> 16));
                count += 2;
                filled = 0;
            }
            if (count == kWireChunk || count == kWireChunk - 1) {
                W.frame(42, nullptr, 0);
                W.frame(44, chunk.data(), chunk.size());
                chunk.clear();
                count = 0;
            }
        }
        const uint32_t w = natural_pack24(packs[0], packs[1]);          // the trailing pair
        chunk.push_back((uint8_t)w);
        chunk.push_back((uint8_t)(w >> 8));
        chunk.push_back((uint8_t)(w >> 16));
        W.frame(43, nullptr, 0);
        W.frame(45, chunk.data(), chunk.size());
    } else if (comp == FEDNL_IDENTITY) {                                 // LocalWorkerForFedNL_Identical.h:138-167
        std::vector<double> chunk;
        for (int p = 0; p < U; ++p) {
            chunk.push_back(dv[p] * P.prescale);
            if ((int)chunk.size() == kWireChunk) {
                W.frame(42, nullptr, 0);
                W.frame(44, chunk.data(), chunk.size() * 8);
                chunk.clear();
            }
        }
        W.frame(43, nullptr, 0);
        W.frame(45, chunk.data(), chunk.size() * 8);
    } else {                                                             // TopK.h:147-189, RandK.h:171-219, RandSeqK.h:172-236
        int32_t n = 0;
        int rc = fednl_gpu_get_message(h, client, nullptr, nullptr, &n);
        if (rc) return rc;
        std::vector<uint32_t> idx((size_t)std::max(n, 1));
        rc = fednl_gpu_get_message(h, client, idx.data(), nullptr, &n);
        if (rc) return rc;
        const bool rk = comp == FEDNL_RANDK || comp == FEDNL_RANDSEQK || comp == FEDNL_RANDK_PHILOX;
        const double scale = rk ? P.prescale * ((double)U / (double)h->k) : P.prescale;
        const bool send_idx = !rk || (flags & FEDNL_WIRE_RANDK_INDICES);
        std::vector<double> items;
        for (int k = 0;;) {
            const bool last = !(k + kWireChunk < n);
            const int end = last ? n : k + kWireChunk;
            W.frame(last ? 43 : 42, send_idx ? (const void*)(idx.data() + k) : nullptr,
                    send_idx ? (size_t)(end - k) * 4 : 0);
            items.clear();
            for (int t = k; t < end; ++t) {
                const uint32_t j = idx[t] / (uint32_t)h->lda, i = idx[t] - j * (uint32_t)h->lda;
                items.push_back(dv[(size_t)j * (j + 1) / 2 + i] * scale);
            }
            W.frame(last ? 45 : 44, items.data(), items.size() * 8);
            k = end;
            if (last) break;
        }
    }
    if (flags & FEDNL_WIRE_FI) {
        double fi = 0.0;
        CK(cudaMemcpy(&fi, P.fi + client, 8, cudaMemcpyDeviceToHost));
        W.frame(48, &fi, 8);                                             // sig_messageToSendFi
    }
    if (flags & FEDNL_WIRE_FINISH) W.frame(49, nullptr, 0);              // sig_messageToSendRoundWorkHasBeenFinished
    *len = (int64_t)W.b.size();
    if (!out) return FEDNL_OK;
    if (cap < (int64_t)W.b.size()) return fail(FEDNL_EINVAL, "output buffer of %lld bytes, %zu needed", (long long)cap,
                                               W.b.size());
    memcpy(out, W.b.data(), W.b.size());
    return FEDNL_OK;
}

int fednl_gpu_get_client_grad(fednl_handle h, int32_t client, double* g)
{
    if (!h || client < 0 || client >= h->nc || !g) return fail(FEDNL_EINVAL, "bad argument");
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaMemcpy(g, h->dev.gc + (size_t)client * h->d, (size_t)h->d * 8, cudaMemcpyDeviceToHost));
    return FEDNL_OK;
}

int fednl_gpu_get_diff(fednl_handle h, int32_t client, double* diff)
{
    if (!h || client < 0 || client >= h->nc || !diff) return fail(FEDNL_EINVAL, "bad argument");
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaMemcpy(diff, h->dev.diff + (size_t)client * h->ustr, (size_t)h->U * 8, cudaMemcpyDeviceToHost));
    return FEDNL_OK;
}

// ---- operator-level entry points -------------------------------------------------------------

namespace {
struct Scratch {
    Arena a;
    cudaStream_t st = nullptr;
    ~Scratch()
    {
        if (st) cudaStreamSynchronize(st);
        a.release();
        if (st) cudaStreamDestroy(st);
    }
};

int select_common(const double* mats, int n_mat, int d, int lda, int k, bool lek, int n_workers,
                  const int32_t* worker_of, uint32_t* wstates, uint32_t* idx, int32_t* counts)
{
    int rc = ensure_device();
    if (rc) return rc;
    if (!mats || !idx || n_mat < 1 || d < 1 || lda < d || k < 1) return fail(FEDNL_EINVAL, "bad argument");
    long long U = (long long)d * (d + 1) / 2;
    if (k < U && k > kMaxK) return fail(FEDNL_EINVAL, "k above %d", kMaxK);
    int SW = (int)((U + 31) / 32);
    const long long ustr = (U + 31) / 32 * 32;
    Scratch s;
    CK(cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking));
    double *dfull, *dpack, *dF, *dp, *dcs;
    unsigned *dsel, *dws = nullptr;
    int *dcnt, *dneeds, *dmi, *dwo = nullptr, *derr;
    size_t full = (size_t)d * lda;
    s.a.want(&dfull, (size_t)n_mat * full);
    s.a.want(&dpack, (size_t)n_mat * ustr);
    s.a.want(&dF, n_mat);
    s.a.want(&dp, n_mat);
    s.a.want(&dcs, (size_t)n_mat * ((full + 31) / 32));
    s.a.want(&dsel, (size_t)n_mat * SW);
    s.a.want(&dcnt, n_mat);
    s.a.want(&dneeds, n_mat);
    s.a.want(&dmi, n_mat);
    s.a.want(&derr, 1);
    if (lek) {
        s.a.want(&dws, std::max(1, n_workers));
        s.a.want(&dwo, n_mat);
    }
    rc = s.a.commit();
    if (rc) return rc;
    CK(cudaMemcpyAsync(dfull, mats, (size_t)n_mat * full * 8, cudaMemcpyHostToDevice, s.st));
    CK(cudaMemsetAsync(derr, 0, 4, s.st));
    k_pack_upper<<<dim3((unsigned)std::min<long long>(1024, (U + 255) / 256), n_mat), 256, 0, s.st>>>(dfull, d, lda, (int)U,
                                                                                                     (int)ustr, dpack);
    CKL();
    k_l2sq_full<<<n_mat, 256, 0, s.st>>>(dfull, (long long)full, dcs, dF);
    CKL();
    if (select_smem(k) > 48 * 1024 && k < U)
        CK(fednl_raise_dyn_smem((const void*)k_select, select_smem(k)));
    double delta = (double)k * (1.0 / (double)U);
    k_select<<<n_mat, kSelThreads, k < U ? select_smem(k) : 0, s.st>>>(dpack, (int)ustr, (int)U, k, lek ? 1 : 0, delta,
                                                                      dF, dsel, SW, dcnt, dneeds, dp, dmi, derr, nullptr, 0,
                                                                      SelectDraws{nullptr, 0, 0, nullptr, MasterAgg{}});
    CKL();
    if (lek) {
        int W = std::max(1, n_workers);
        std::vector<int> wo(n_mat);
        for (int t = 0; t < n_mat; ++t) {
            wo[t] = worker_of ? worker_of[t] : 0;
            if (wo[t] < 0 || wo[t] >= W) return fail(FEDNL_EINVAL, "worker_of[%d] out of range", t);
        }
        CK(cudaMemcpyAsync(dwo, wo.data(), n_mat * 4, cudaMemcpyHostToDevice, s.st));
        CK(cudaMemcpyAsync(dws, wstates, W * 4, cudaMemcpyHostToDevice, s.st));
        k_toplek_rng<<<(W + 31) / 32, 32, 0, s.st>>>(n_mat, W, dwo, dws, dneeds, dp, dmi, dsel, SW, dcnt);
        CKL();
        CK(cudaMemcpyAsync(wstates, dws, W * 4, cudaMemcpyDeviceToHost, s.st));
    }
    std::vector<unsigned> sel((size_t)n_mat * SW);
    int errflag = 0;
    CK(cudaMemcpyAsync(sel.data(), dsel, sel.size() * 4, cudaMemcpyDeviceToHost, s.st));
    CK(cudaMemcpyAsync(&errflag, derr, 4, cudaMemcpyDeviceToHost, s.st));
    CK(cudaStreamSynchronize(s.st));
    if (errflag) return fail(FEDNL_ETIMEOUT, "bounded wait in the selection kernel ran out");
    for (int t = 0; t < n_mat; ++t) {
        int w = 0;
        long long p = 0;
        uint32_t* o = idx + (size_t)t * k;
        for (int j = 0; j < d; ++j)
            for (int i = 0; i <= j; ++i, ++p)
                if ((sel[(size_t)t * SW + (p >> 5)] >> (p & 31)) & 1u) {
                    if (w < k) o[w] = (uint32_t)j * (uint32_t)lda + (uint32_t)i;
                    ++w;
                }
        if (counts) counts[t] = w;
    }
    return FEDNL_OK;
}

int rand_common(uint32_t* states, int n_gen, int d, int lda, int k, uint32_t* idx, bool seq)
{
    int rc = ensure_device();
    if (rc) return rc;
    long long U = (long long)d * (d + 1) / 2;
    if (!states || !idx || n_gen < 1 || d < 1 || lda < d || k < 1 || k > U) return fail(FEDNL_EINVAL, "bad argument");
    int SW = (int)((U + 31) / 32);
    int hcap = 1;
    while (hcap < 4 * k) hcap <<= 1;
    Scratch s;
    CK(cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking));
    unsigned *dst, *dsel;
    int *dcnt, *drseq;
    unsigned long long* dmap = nullptr;
    s.a.want(&dst, n_gen);
    s.a.want(&dsel, (size_t)n_gen * SW);
    s.a.want(&dcnt, n_gen);
    s.a.want(&drseq, n_gen);
    if (!seq) s.a.want(&dmap, (size_t)n_gen * hcap);
    rc = s.a.commit();
    if (rc) return rc;
    CK(cudaMemcpyAsync(dst, states, n_gen * 4, cudaMemcpyHostToDevice, s.st));
    if (seq) k_randseqk<<<n_gen, 256, 0, s.st>>>(dst, n_gen, (int)U, k, drseq, dsel, SW, dcnt, nullptr);
    else k_randk<<<n_gen, 256, 0, s.st>>>(dst, n_gen, (int)U, k, dmap, hcap, dsel, SW, dcnt, nullptr);
    CKL();
    std::vector<unsigned> sel((size_t)n_gen * SW);
    std::vector<int> rseq(n_gen);
    CK(cudaMemcpyAsync(sel.data(), dsel, sel.size() * 4, cudaMemcpyDeviceToHost, s.st));
    CK(cudaMemcpyAsync(rseq.data(), drseq, n_gen * 4, cudaMemcpyDeviceToHost, s.st));
    CK(cudaMemcpyAsync(states, dst, n_gen * 4, cudaMemcpyDeviceToHost, s.st));
    CK(cudaStreamSynchronize(s.st));
    std::vector<uint32_t> flat(U);
    {
        long long p = 0;
        for (int j = 0; j < d; ++j)
            for (int i = 0; i <= j; ++i, ++p) flat[p] = (uint32_t)j * (uint32_t)lda + (uint32_t)i;
    }
    for (int t = 0; t < n_gen; ++t) {
        uint32_t* o = idx + (size_t)t * k;
        if (seq) {
            for (int q = 0; q < k; ++q) o[q] = flat[(rseq[t] + (long long)q) % U];
        } else {
            int w = 0;
            for (long long p = 0; p < U; ++p)
                if ((sel[(size_t)t * SW + (p >> 5)] >> (p & 31)) & 1u) o[w++] = flat[p];
        }
    }
    return FEDNL_OK;
}
}  // namespace

int fednl_gpu_topk(const double* mats, int32_t n_mat, int32_t d, int32_t lda, int32_t k, uint32_t* idx)
{
    return select_common(mats, n_mat, d, lda, k, false, 1, nullptr, nullptr, idx, nullptr);
}

int fednl_gpu_toplek(const double* mats, int32_t n_mat, int32_t d, int32_t lda, int32_t k, int32_t n_workers,
                     const int32_t* worker_of, uint32_t* worker_states, uint32_t* idx, int32_t* counts)
{
    if (!worker_states || n_workers < 1) return fail(FEDNL_EINVAL, "worker states required");
    return select_common(mats, n_mat, d, lda, k, true, n_workers, worker_of, worker_states, idx, counts);
}

int fednl_gpu_randk(uint32_t* states, int32_t n_gen, int32_t d, int32_t lda, int32_t k, uint32_t* idx)
{
    return rand_common(states, n_gen, d, lda, k, idx, false);
}

int fednl_gpu_randseqk(uint32_t* states, int32_t n_gen, int32_t d, int32_t lda, int32_t k, uint32_t* idx)
{
    return rand_common(states, n_gen, d, lda, k, idx, true);
}

int fednl_gpu_natural(const double* in, int64_t n, double* out, uint8_t* packed)
{
    int rc = ensure_device();
    if (rc) return rc;
    if (!in || !out || n < 1) return fail(FEDNL_EINVAL, "bad argument");
    Scratch s;
    CK(cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking));
    double *din, *dout;
    unsigned char* dpk = nullptr;
    long long nb = n / 2 + 1;
    s.a.want(&din, n);
    s.a.want(&dout, n);
    if (packed) s.a.want(&dpk, 3 * nb);
    rc = s.a.commit();
    if (rc) return rc;
    CK(cudaMemcpyAsync(din, in, n * 8, cudaMemcpyHostToDevice, s.st));
    k_natural<<<(unsigned)((n + 255) / 256), 256, 0, s.st>>>(din, n, dout);
    CKL();
    if (packed) {
        k_natural_pack<<<(unsigned)((nb + 255) / 256), 256, 0, s.st>>>(din, n, dpk);
        CKL();
        CK(cudaMemcpyAsync(packed, dpk, 3 * nb, cudaMemcpyDeviceToHost, s.st));
    }
    CK(cudaMemcpyAsync(out, dout, n * 8, cudaMemcpyDeviceToHost, s.st));
    CK(cudaStreamSynchronize(s.st));
    return FEDNL_OK;
}

int fednl_gpu_shift_update(double* shifts, const double* diffs, int32_t n_mat, int32_t d, int32_t lda,
                           const uint32_t* idx, const int32_t* counts, int32_t k_stride, double alpha,
                           double value_mult)
{
    int rc = ensure_device();
    if (rc) return rc;
    if (!shifts || !diffs || !idx || !counts || n_mat < 1 || d < 1 || lda < d || k_stride < 1)
        return fail(FEDNL_EINVAL, "bad argument");
    const size_t full = (size_t)d * lda;
    int kmax = 0;
    for (int m = 0; m < n_mat; ++m) {
        if (counts[m] < 0 || counts[m] > k_stride) return fail(FEDNL_EINVAL, "count %d outside [0, k_stride]", counts[m]);
        for (int t = 0; t < counts[m]; ++t) {
            const uint32_t f = idx[(size_t)m * k_stride + t];
            const uint32_t jc = f / (uint32_t)lda, ir = f - jc * (uint32_t)lda;
            if (jc >= (uint32_t)d || ir > jc) return fail(FEDNL_EINVAL, "index %u is not an upper entry", f);
        }
        kmax = std::max(kmax, counts[m]);
    }
    Scratch s;
    CK(cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking));
    double *dsh, *ddf;
    unsigned* didx;
    int* dcnt;
    s.a.want(&dsh, (size_t)n_mat * full);
    s.a.want(&ddf, (size_t)n_mat * full);
    s.a.want(&didx, (size_t)n_mat * k_stride);
    s.a.want(&dcnt, n_mat);
    rc = s.a.commit();
    if (rc) return rc;
    CK(cudaMemcpyAsync(dsh, shifts, (size_t)n_mat * full * 8, cudaMemcpyHostToDevice, s.st));
    CK(cudaMemcpyAsync(ddf, diffs, (size_t)n_mat * full * 8, cudaMemcpyHostToDevice, s.st));
    CK(cudaMemcpyAsync(didx, idx, (size_t)n_mat * k_stride * 4, cudaMemcpyHostToDevice, s.st));
    CK(cudaMemcpyAsync(dcnt, counts, (size_t)n_mat * 4, cudaMemcpyHostToDevice, s.st));
    if (kmax > 0) {
        k_op_shift_update<<<dim3((kmax + 255) / 256, n_mat), 256, 0, s.st>>>(dsh, ddf, n_mat, lda, full, didx, dcnt,
                                                                          k_stride, alpha, value_mult);
        CKL();
    }
    CK(cudaMemcpyAsync(shifts, dsh, (size_t)n_mat * full * 8, cudaMemcpyDeviceToHost, s.st));
    CK(cudaStreamSynchronize(s.st));
    return FEDNL_OK;
}

int fednl_gpu_aggregate(int32_t n_clients, int32_t d, int32_t lda, const double* grads, const double* lks,
                        const uint32_t* idx, const double* vals, const int32_t* counts, int32_t k_stride, double* H,
                        double* g, double* l)
{
    int rc = ensure_device();
    if (rc) return rc;
    if (!grads || !lks || !H || !g || !l || n_clients < 1 || d < 1 || lda < d || k_stride < 0 ||
        (k_stride > 0 && (!idx || !vals || !counts)))
        return fail(FEDNL_EINVAL, "bad argument");
    const long long U = (long long)d * (d + 1) / 2;
    const size_t full = (size_t)d * lda;
    for (int c = 0; c < n_clients && k_stride > 0; ++c) {
        if (counts[c] < 0 || counts[c] > k_stride || counts[c] > U)
            return fail(FEDNL_EINVAL, "count %d outside [0, min(k_stride, U)]", counts[c]);
        std::vector<char> seen((size_t)U, 0);
        for (int t = 0; t < counts[c]; ++t) {
            const uint32_t f = idx[(size_t)c * k_stride + t];
            const uint32_t jc = f / (uint32_t)lda, ir = f - jc * (uint32_t)lda;
            if (jc >= (uint32_t)d || ir > jc) return fail(FEDNL_EINVAL, "index %u is not an upper entry", f);
            const size_t p = (size_t)jc * (jc + 1) / 2 + ir;
            if (seen[p]) return fail(FEDNL_EINVAL, "client %d sends entry %u twice", c, f);
            seen[p] = 1;
        }
    }
    Scratch s;
    CK(cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking));
    double *dgr, *dlk, *dH, *dg, *dl, *dval = nullptr;
    unsigned* didx = nullptr;
    int *dcnt = nullptr, *dslot = nullptr;
    s.a.want(&dgr, (size_t)n_clients * d);
    s.a.want(&dlk, n_clients);
    s.a.want(&dH, full);
    s.a.want(&dg, d);
    s.a.want(&dl, 1);
    if (k_stride > 0) {
        s.a.want(&didx, (size_t)n_clients * k_stride);
        s.a.want(&dval, (size_t)n_clients * k_stride);
        s.a.want(&dcnt, n_clients);
        s.a.want(&dslot, (size_t)n_clients * U);
    }
    rc = s.a.commit();
    if (rc) return rc;
    CK(cudaMemcpyAsync(dgr, grads, (size_t)n_clients * d * 8, cudaMemcpyHostToDevice, s.st));
    CK(cudaMemcpyAsync(dlk, lks, (size_t)n_clients * 8, cudaMemcpyHostToDevice, s.st));
    CK(cudaMemcpyAsync(dH, H, full * 8, cudaMemcpyHostToDevice, s.st));
    k_op_aggregate_g<<<(d + 127) / 128, 128, 0, s.st>>>(dgr, dlk, n_clients, d, 1.0 / (double)n_clients, dg, dl);
    CKL();
    if (k_stride > 0) {
        CK(cudaMemcpyAsync(didx, idx, (size_t)n_clients * k_stride * 4, cudaMemcpyHostToDevice, s.st));
        CK(cudaMemcpyAsync(dval, vals, (size_t)n_clients * k_stride * 8, cudaMemcpyHostToDevice, s.st));
        CK(cudaMemcpyAsync(dcnt, counts, (size_t)n_clients * 4, cudaMemcpyHostToDevice, s.st));
        CK(cudaMemsetAsync(dslot, 0xff, (size_t)n_clients * U * 4, s.st));
        k_op_message_slots<<<dim3((k_stride + 255) / 256, n_clients), 256, 0, s.st>>>(didx, dcnt, k_stride, n_clients,
                                                                                     lda, dslot, (int)U);
        CKL();
        k_op_aggregate_h<<<(unsigned)((U + 127) / 128), 128, 0, s.st>>>(dH, d, lda, (int)U, dval, dslot, k_stride,
                                                                        n_clients);
        CKL();
    }
    CK(cudaMemcpyAsync(H, dH, full * 8, cudaMemcpyDeviceToHost, s.st));
    CK(cudaMemcpyAsync(g, dg, (size_t)d * 8, cudaMemcpyDeviceToHost, s.st));
    CK(cudaMemcpyAsync(l, dl, 8, cudaMemcpyDeviceToHost, s.st));
    CK(cudaStreamSynchronize(s.st));
    return FEDNL_OK;
}

int fednl_gpu_compress_identity(const double* diffs, int32_t n_mat, int32_t d, int32_t lda, double alpha,
                                double prescale, double* shifts, uint32_t* idx_out, double* val_out)
{
    int rc = ensure_device();
    if (rc) return rc;
    if (!diffs || n_mat < 1 || d < 1 || lda < d) return fail(FEDNL_EINVAL, "bad argument");
    const long long U = (long long)d * (d + 1) / 2;
    const size_t full = (size_t)d * lda;
    Scratch s;
    CK(cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking));
    double *ddf, *dsh = nullptr, *dval = nullptr;
    unsigned* didx = nullptr;
    s.a.want(&ddf, (size_t)n_mat * full);
    if (shifts) s.a.want(&dsh, (size_t)n_mat * full);
    if (idx_out) s.a.want(&didx, (size_t)n_mat * U);
    if (val_out) s.a.want(&dval, (size_t)n_mat * U);
    rc = s.a.commit();
    if (rc) return rc;
    CK(cudaMemcpyAsync(ddf, diffs, (size_t)n_mat * full * 8, cudaMemcpyHostToDevice, s.st));
    if (shifts) CK(cudaMemcpyAsync(dsh, shifts, (size_t)n_mat * full * 8, cudaMemcpyHostToDevice, s.st));
    k_op_identity<<<dim3((unsigned)((U + 255) / 256), n_mat), 256, 0, s.st>>>(ddf, dsh, n_mat, lda, full, (int)U, alpha,
                                                                             prescale, didx, dval);
    CKL();
    if (shifts) CK(cudaMemcpyAsync(shifts, dsh, (size_t)n_mat * full * 8, cudaMemcpyDeviceToHost, s.st));
    if (idx_out) CK(cudaMemcpyAsync(idx_out, didx, (size_t)n_mat * U * 4, cudaMemcpyDeviceToHost, s.st));
    if (val_out) CK(cudaMemcpyAsync(val_out, dval, (size_t)n_mat * U * 8, cudaMemcpyDeviceToHost, s.st));
    CK(cudaStreamSynchronize(s.st));
    return FEDNL_OK;
}

int fednl_gpu_logreg_oracle(const double* features, const double* labels, int32_t n, int32_t d, int32_t lda,
                            double lambda, const double* x, double* grad, double* hess)
{
    if (!features || !labels || !x || n < 1 || d < 1) return fail(FEDNL_EINVAL, "bad argument");
    fednl_problem_desc D{};
    D.d = d;
    D.lda = lda;
    D.n_clients = 1;
    D.n_samples = &n;
    D.lambda = lambda;
    D.compressor = FEDNL_IDENTITY;
    D.k = 1;
    D.alpha = 1.0;
    D.workers = 1;
    fednl_handle h = nullptr;
    int rc = fednl_gpu_create(&D, &h);
    if (rc) return rc;
    rc = fednl_gpu_upload_client_data(h, features, labels);
    if (!rc) rc = fednl_gpu_init_shifts(h, x);      // shift_0 = H(x)
    if (!rc && grad) {
        Dev& P = h->dev;
        if (h->binary) k_grad_binary<<<dim3((2 * d + 127) / 128, 1), 128, (size_t)h->maxn * 16, h->stream>>>(P);
        else k_grad_dense<<<dim3((d + 127) / 128, 1), 128, 0, h->stream>>>(P);
        cudaError_t e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) rc = fail(FEDNL_ECUDA, "gradient kernel failed: %s", cudaGetErrorString(e));
        else if (cudaMemcpy(grad, P.gc, d * 8, cudaMemcpyDeviceToHost) != cudaSuccess) rc = fail(FEDNL_ECUDA, "copy failed");
    }
    if (!rc && hess) rc = fednl_gpu_get_shift(h, 0, hess);
    fednl_gpu_destroy(h);
    return rc;
}

int fednl_gpu_optionb_solve(const double* H, int32_t d, int32_t lda, double l, const double* g, double* dx)
{
    int rc = ensure_device();
    if (rc) return rc;
    if (!H || !g || !dx || d < 1 || lda < d) return fail(FEDNL_EINVAL, "bad argument");
    long long U = (long long)d * (d + 1) / 2;
    Scratch s;
    CK(cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking));
    Dev P{};
    double *dfull, *dpack, *dg;
    s.a.want(&dfull, (size_t)d * lda);
    s.a.want(&dpack, U);
    s.a.want(&dg, d);
    s.a.want(&P.work, fednl_chol_work_elems(d));
    s.a.want(&P.dx, d);
    s.a.want(&P.ybuf, d);
    s.a.want(&P.rinv, d);
    s.a.want(&P.status, 1);
    s.a.want(&P.bar, 4);
    rc = s.a.commit();
    if (rc) return rc;
    P.d = d;
    P.U = (int)U;
    CK(cudaMemsetAsync(P.bar, 0, 16, s.st));
    CK(cudaMemcpyAsync(dfull, H, (size_t)d * lda * 8, cudaMemcpyHostToDevice, s.st));
    CK(cudaMemcpyAsync(dg, g, d * 8, cudaMemcpyHostToDevice, s.st));
    CK(cudaMemsetAsync(P.status, 0, 4, s.st));
    k_pack_upper<<<dim3((unsigned)std::min<long long>(1024, (U + 255) / 256), 1), 256, 0, s.st>>>(dfull, d, lda, (int)U,
                                                                                                (int)U, dpack);
    CKL();
    CK(launch_chol(P, chol_grid(d), s.st, dpack, 0, nullptr, l, dg, P.dx, nullptr, 0));
    int status = 0;
    CK(cudaMemcpyAsync(&status, P.status, 4, cudaMemcpyDeviceToHost, s.st));
    CK(cudaStreamSynchronize(s.st));
    if (status == FEDNL_ETIMEOUT) return fail(FEDNL_ETIMEOUT, "grid barrier of the Cholesky timed out");
    if (status) return fail(FEDNL_ENOTPD, "H + l I is not positive definite");
    CK(cudaMemcpy(dx, P.dx, d * 8, cudaMemcpyDeviceToHost));
    return FEDNL_OK;
}

int fednl_gpu_optionb_solve32(const double* H, int32_t d, int32_t lda, double l, const double* g, double* dx,
                              int32_t refine, int32_t grid)
{
    int rc = ensure_device();
    if (rc) return rc;
    if (!H || !g || !dx || d < 1 || lda < d || refine < 0 || refine > 8 || grid < -16) return fail(FEDNL_EINVAL, "bad argument");
    if (d > kC32MaxD) return fail(FEDNL_EINVAL, "d %d above the FP32 cooperative solve's limit %d", d, kC32MaxD);
    long long U = (long long)d * (d + 1) / 2;
    const size_t ld = (size_t)c32c_ld(d);
    Scratch s;
    CK(cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking));
    double *dfull, *dpack, *dg, *dl, *ddx, *work, *ybuf, *rinv, *stats;
    unsigned* bar;
    int* status;
    FednlSolve32 E{};
    s.a.want(&dfull, (size_t)d * lda);
    s.a.want(&dpack, U);
    s.a.want(&dg, d);
    s.a.want(&dl, 1);
    s.a.want(&ddx, d);
    s.a.want(&work, fednl_chol_work_elems(d));
    s.a.want(&ybuf, d);
    s.a.want(&rinv, d);
    s.a.want(&stats, 4);
    s.a.want(&status, 1);
    s.a.want(&bar, 4);
    s.a.want(&E.a, ld * ld);
    s.a.want(&E.diag0, d);
    s.a.want(&E.linv, ld * 32);
    s.a.want(&E.r, d);
    s.a.want(&E.acc, d);
    s.a.want(&E.accp, 2 * (size_t)d);
    s.a.want(&E.flag, 1);
    float *phh, *phl, *prh, *prl;
    s.a.want(&phh, U);
    s.a.want(&phl, U);
    s.a.want(&prh, U);
    s.a.want(&prl, U);
    rc = s.a.commit();
    if (rc) return rc;
    E.refine = refine;
    E.tol = 0x1p-30f;
    CK(cudaMemsetAsync(bar, 0, 16, s.st));
    CK(cudaMemsetAsync(status, 0, 4, s.st));
    CK(cudaMemcpyAsync(dfull, H, (size_t)d * lda * 8, cudaMemcpyHostToDevice, s.st));
    CK(cudaMemcpyAsync(dg, g, d * 8, cudaMemcpyHostToDevice, s.st));
    CK(cudaMemcpyAsync(dl, &l, 8, cudaMemcpyHostToDevice, s.st));
    k_pack_upper<<<dim3((unsigned)std::min<long long>(1024, (U + 255) / 256), 1), 256, 0, s.st>>>(dfull, d, lda, (int)U,
                                                                                                (int)U, dpack);
    k_split_pairs<<<(unsigned)((U + 255) / 256), 256, 0, s.st>>>(dpack, d, phh, phl, prh, prl);
    CKL();
    E.hh = phh;
    E.hl = phl;
    E.rh = prh;
    E.rl = prl;
    FednlSolveDesc S{};
    S.H = dpack;
    S.d = d;
    S.lptr = dl;
    S.g = dg;
    S.dx = ddx;
    S.work = work;
    S.ybuf = ybuf;
    S.rinv = rinv;
    S.bar = bar;
    S.status = status;
    S.stats = stats;
    S.record = 0;
    rc = fednl_device_optionb_solve32(S, E, s.st, grid);
    if (rc) return fail(rc, "FP32 cooperative solve launch failed");
    int st = 0;
    CK(cudaMemcpyAsync(&st, status, 4, cudaMemcpyDeviceToHost, s.st));
    CK(cudaStreamSynchronize(s.st));
    if (st == FEDNL_ETIMEOUT) return fail(FEDNL_ETIMEOUT, "grid barrier of the Cholesky timed out");
    if (st) return fail(FEDNL_ENOTPD, "H + l I is not positive definite");
    CK(cudaMemcpy(dx, ddx, d * 8, cudaMemcpyDeviceToHost));
    return FEDNL_OK;
}

// ---- self-test of the integer square root and reciprocal --------------------------------------
namespace {
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// inputs: random bit patterns (every exponent, both signs), significands near 0 and near 1, and
// squares of random doubles and their neighbours
__global__ void k_selftest_rn(unsigned long long seed, long long n, unsigned long long* bad)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long z = splitmix64(seed ^ (unsigned long long)i), w = splitmix64(z);
        unsigned long long u;
        switch (i & 3) {
        case 0: u = z; break;
        case 1: u = (z & 0x7FF0000000000000ull) | (w & 0xFFFFull); break;
        case 2: u = (z & 0x7FF0000000000000ull) | (0xFFFFFFFFFFFFFull - (w & 0xFFFFull)); break;
        default: {
            const double x = __longlong_as_double((long long)((z & 0x000FFFFFFFFFFFFFull) | (0x3FF0000000000000ull + ((w & 0x3FFull) << 52) - (0x200ull << 52))));
            u = (unsigned long long)__double_as_longlong(x * x) + (w >> 62) - 1ull;
        }
        }
        const double a = __longlong_as_double((long long)u);
        if (__double_as_longlong(sqrt_rn_int(a)) != __double_as_longlong(sqrt(a))) atomicAdd(&bad[0], 1ull);
        if (__double_as_longlong(rcp_rn_int(a)) != __double_as_longlong(1.0 / a)) atomicAdd(&bad[1], 1ull);
        // the pivot's fused pair: r against sqrt(a), 1 / r against the division of 1 by sqrt(a)
        double inv;
        const double r = sqrt_rcp_rn_int(a, inv);
        const double rh = sqrt(a);
        if (__double_as_longlong(r) != __double_as_longlong(rh)) atomicAdd(&bad[0], 1ull);
        if (rh > 0.0 && __double_as_longlong(inv) != __double_as_longlong(1.0 / rh)) atomicAdd(&bad[1], 1ull);
    }
}
}  // namespace

int fednl_gpu_selftest_rn(int64_t n, uint64_t seed, int64_t* sqrt_mismatches, int64_t* rcp_mismatches)
{
    int rc = ensure_device();
    if (rc) return rc;
    if (n < 1 || !sqrt_mismatches || !rcp_mismatches) return fail(FEDNL_EINVAL, "bad argument");
    unsigned long long* d = nullptr;
    CK(cudaMalloc(&d, 16));
    unsigned long long h[2] = {0, 0};
    cudaError_t e = cudaMemset(d, 0, 16);
    if (e == cudaSuccess) {
        k_selftest_rn<<<1216, 256>>>(seed, n, d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(h, d, 16, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return fail(FEDNL_ECUDA, "self-test kernel failed: %s", cudaGetErrorString(e));
    *sqrt_mismatches = (int64_t)h[0];
    *rcp_mismatches = (int64_t)h[1];
    return FEDNL_OK;
}

// ---- FP64 pipe rate and latency ------------------------------------------------------------------
// Throughput: every thread runs 8 independent chains of `iters` dependent FP64 operations (fma, or
// add), all SMs full of warps; lane operations per second.  Latency: one warp, one dependent chain
// of adds, clock64 cycles per add.  The values never leave registers except one store per thread,
// so the kernels measure the FP64 pipe alone.
__global__ void __launch_bounds__(256) k_fp64_rate(long long iters, int use_fma, double b, double* sink)
{
    double a0 = threadIdx.x * 1e-9, a1 = a0 + 1e-9, a2 = a0 + 2e-9, a3 = a0 + 3e-9;
    double a4 = a0 + 4e-9, a5 = a0 + 5e-9, a6 = a0 + 6e-9, a7 = a0 + 7e-9;
    if (use_fma) {
        for (long long t = 0; t < iters; ++t) {
            a0 = __fma_rn(a0, b, 1e-12); a1 = __fma_rn(a1, b, 1e-12); a2 = __fma_rn(a2, b, 1e-12);
            a3 = __fma_rn(a3, b, 1e-12); a4 = __fma_rn(a4, b, 1e-12); a5 = __fma_rn(a5, b, 1e-12);
            a6 = __fma_rn(a6, b, 1e-12); a7 = __fma_rn(a7, b, 1e-12);
        }
    } else {
        for (long long t = 0; t < iters; ++t) {
            a0 = __dadd_rn(a0, b); a1 = __dadd_rn(a1, b); a2 = __dadd_rn(a2, b); a3 = __dadd_rn(a3, b);
            a4 = __dadd_rn(a4, b); a5 = __dadd_rn(a5, b); a6 = __dadd_rn(a6, b); a7 = __dadd_rn(a7, b);
        }
    }
    sink[blockIdx.x * blockDim.x + threadIdx.x] = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
}

__global__ void k_fp64_latency(long long iters, double b, double* sink, long long* cycles)
{
    double a = threadIdx.x * 1e-9;
    __syncwarp();
    const long long t0 = clock64();
    for (long long t = 0; t < iters; ++t) a = __dadd_rn(a, b);
    const long long t1 = clock64();
    sink[threadIdx.x] = a;
    if (threadIdx.x == 0) *cycles = t1 - t0;
}

int fednl_gpu_fp64_rate(int64_t iters, double* fma_gops, double* add_gops, double* add_latency_cycles)
{
    int rc = ensure_device();
    if (rc) return rc;
    if (iters < 1 || !fma_gops || !add_gops || !add_latency_cycles) return fail(FEDNL_EINVAL, "bad argument");
    int dev = 0, sms = 1;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * 8, threads = 256;
    Scratch s;
    CK(cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking));
    double* sink;
    long long* cyc;
    s.a.want(&sink, (size_t)blocks * threads);
    s.a.want(&cyc, 1);
    rc = s.a.commit();
    if (rc) return rc;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    double out[2];
    for (int f = 0; f < 2; ++f) {
        k_fp64_rate<<<blocks, threads, 0, s.st>>>(iters / 16 + 1, 1 - f, 1.0000001, sink);   // warm-up
        CKL();
        CK(cudaEventRecord(e0, s.st));
        k_fp64_rate<<<blocks, threads, 0, s.st>>>(iters, 1 - f, 1.0000001, sink);
        CKL();
        CK(cudaEventRecord(e1, s.st));
        CK(cudaEventSynchronize(e1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        out[f] = (double)blocks * threads * 8.0 * (double)iters / (ms * 1e-3) / 1e9;
    }
    k_fp64_latency<<<1, 32, 0, s.st>>>(iters, 1e-7, sink, cyc);
    CKL();
    long long cycles = 0;
    CK(cudaMemcpyAsync(&cycles, cyc, 8, cudaMemcpyDeviceToHost, s.st));
    CK(cudaStreamSynchronize(s.st));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *fma_gops = out[0];
    *add_gops = out[1];
    *add_latency_cycles = (double)cycles / (double)iters;
    return FEDNL_OK;
}

// ---- instrumentation ---------------------------------------------------------------------------

static int flush_l2(fednl_handle h, int64_t bytes)
{
    if (bytes <= 0) return FEDNL_OK;
    if ((size_t)bytes > h->flush_cap) {
        if (h->flush_buf) cudaFree(h->flush_buf);
        h->flush_buf = nullptr;
        h->flush_cap = 0;
        CK(cudaMalloc(&h->flush_buf, (size_t)bytes));
        h->flush_cap = (size_t)bytes;
    }
    CK(cudaMemsetAsync(h->flush_buf, h->rounds_done & 0xFF, (size_t)bytes, h->stream));
    return FEDNL_OK;
}

int fednl_gpu_time_rounds(fednl_handle h, int32_t rounds, int64_t flush_bytes, double* total_ms, double* per_round_ms)
{
    if (!h || rounds < 1 || !total_ms) return fail(FEDNL_EINVAL, "bad argument");
    if (!h->shifts_ready) return fail(FEDNL_EINVAL, "call fednl_gpu_init_shifts first");
    int rc = build_graph(h);
    if (rc) return rc;
    std::vector<cudaEvent_t> ev(2 * (size_t)rounds, nullptr);
    for (auto& e : ev) CK(cudaEventCreate(&e));
    CK(cudaMemsetAsync(h->dev.status, 0, 4, h->stream));
    for (int r = 0; r < rounds; ++r) {
        rc = flush_l2(h, flush_bytes);
        if (rc) break;
        if ((rc = cudaEventRecord(ev[2 * r], h->stream)) != cudaSuccess) break;
        if ((rc = cudaGraphLaunch(h->gexec, h->stream)) != cudaSuccess) break;
        if ((rc = cudaEventRecord(ev[2 * r + 1], h->stream)) != cudaSuccess) break;
    }
    cudaError_t e = cudaStreamSynchronize(h->stream);
    double tot = 0.0;
    if (rc == 0 && e == cudaSuccess) {
        for (int r = 0; r < rounds; ++r) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev[2 * r], ev[2 * r + 1]);
            tot += ms;
            if (per_round_ms) per_round_ms[r] = ms;
        }
    }
    for (auto& x : ev) cudaEventDestroy(x);
    if (rc) return fail(FEDNL_ECUDA, "timed replay failed (%d)", rc);
    if (e != cudaSuccess) return fail(FEDNL_ECUDA, "timed replay failed: %s", cudaGetErrorString(e));
    h->rounds_done += rounds;
    *total_ms = tot;
    return FEDNL_OK;
}

int fednl_gpu_profile_kernels(fednl_handle h, int32_t rounds, int64_t flush_bytes, int32_t* n_kernels,
                              double* kernel_ms, char* names, int32_t names_len)
{
    if (!h || rounds < 1 || !n_kernels || !kernel_ms) return fail(FEDNL_EINVAL, "bad argument");
    if (!h->shifts_ready) return fail(FEDNL_EINVAL, "call fednl_gpu_init_shifts first");
    const int kMaxMarks = 65;
    std::vector<std::vector<cudaEvent_t>> ev(rounds, std::vector<cudaEvent_t>(kMaxMarks, nullptr));
    for (auto& v : ev)
        for (auto& e : v) CK(cudaEventCreate(&e));
    std::vector<std::string> nm;
    size_t nmarks = 0;
    int rc = FEDNL_OK;
    for (int r = 0; r < rounds && rc == FEDNL_OK; ++r) {
        rc = flush_l2(h, flush_bytes);
        if (rc) break;
        Marks M;
        M.ev = &ev[r];
        M.names = &nm;
        rc = launch_round(h, &M);
        nmarks = M.next;
    }
    cudaError_t e = cudaStreamSynchronize(h->stream);
    int nk = (int)nmarks - 1;
    if (rc == FEDNL_OK && e == cudaSuccess) {
        for (int t = 0; t < nk && t < 64; ++t) {
            double acc = 0.0;
            for (int r = 0; r < rounds; ++r) {
                float ms = 0.f;
                cudaEventElapsedTime(&ms, ev[r][t], ev[r][t + 1]);
                acc += ms;
            }
            kernel_ms[t] = acc / rounds;
        }
        *n_kernels = std::min(nk, 64);
        if (names && names_len > 0) {
            std::string all;
            for (int t = 0; t < nk && t < 64; ++t) {
                if (t) all += ";";
                all += nm[t];
            }
            snprintf(names, (size_t)names_len, "%s", all.c_str());
        }
    }
    for (auto& v : ev)
        for (auto& x : v) cudaEventDestroy(x);
    if (rc) return rc;
    if (e != cudaSuccess) return fail(FEDNL_ECUDA, "profiled rounds failed: %s", cudaGetErrorString(e));
    h->rounds_done += rounds;
    return FEDNL_OK;
}

// ---- allocation-free Option-B solve -------------------------------------------------------------
// For callers that may not allocate device memory: a host framework that owns every byte of device
// memory through its own allocator (a cudaMalloc beside it fails or fragments its pool), a process
// under a fixed device-memory budget, or a latency-critical loop in which cudaMalloc and cudaFree
// would synchronise the device.  The solve's scratch (the packed factor, two d-vectors, the
// grid-barrier counters and the status word) lives in one fixed device array of this file, which
// every device that loads the library holds until the process exits.  In host code the array's
// name is not a device address: the first call on a device, with that device current, looks the
// address up with cudaGetSymbolAddress (which can load the library's device code on that device)
// and keeps it; every call passes that address to the kernels.  Every call shares the array and
// finds the previous call's contents there: the barrier counters and the status word are cleared
// before each launch, the factor is overwritten.  Calls that overlap on the GPU race.
namespace {
constexpr int kNoAllocMaxD = 512;
constexpr size_t kNoAllocMaxUA = (size_t)(kNoAllocMaxD + 1) * (kNoAllocMaxD + 2) / 2 +
                                  (size_t)kCholNB * (kNoAllocMaxD + 1);   // factor with y column, panel rows
constexpr size_t kNoAllocDoubles = kNoAllocMaxUA + 2 * kNoAllocMaxD + 4;   // factor, y, 1/r, barrier+status
constexpr int kNoAllocMaxDevices = 64;
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];
static double* g_noalloc_ptr[kNoAllocMaxDevices];
static int g_noalloc_grid[kNoAllocMaxDevices];
}  // namespace

int fednl_gpu_optionb_solve_noalloc(const double* H, int32_t d, int32_t lda, double l, const double* g, double* dx,
                                    void* stream)
{
    if (!H || !g || !dx || d < 1 || lda < d) return fail(FEDNL_EINVAL, "bad argument");
    if (d > kNoAllocMaxD)
        return fail(FEDNL_EINVAL, "d = %d exceeds the allocation-free solve's maximum of %d", d, kNoAllocMaxD);
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(FEDNL_EINVAL, "device ordinal %d out of range", dev);
    if (!g_noalloc_ptr[dev]) {          // once per device, with that device current
        void* ptr = nullptr;
        CK(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
        g_noalloc_grid[dev] = chol_grid(kNoAllocMaxD);
        g_noalloc_ptr[dev] = (double*)ptr;
    }
    double* base = g_noalloc_ptr[dev];
    const long long U = (long long)d * (d + 1) / 2;
    Dev P{};
    P.d = d;
    P.U = (int)U;
    P.work = base;
    P.ybuf = base + kNoAllocMaxUA;
    P.rinv = base + kNoAllocMaxUA + kNoAllocMaxD;
    P.bar = (unsigned*)(base + kNoAllocMaxUA + 2 * kNoAllocMaxD);       // 4 x u32 = 2 doubles
    P.status = (int*)(base + kNoAllocMaxUA + 2 * kNoAllocMaxD + 2);
    cudaStream_t st = (cudaStream_t)stream;
    // barrier counters and status must start at zero; the factor is overwritten by every call
    CK(cudaMemsetAsync(P.bar, 0, 4 * sizeof(double), st));
    int grid = std::min(g_noalloc_grid[dev], chol_grid(d));
    CK(launch_chol(P, grid, st, H, lda, nullptr, l, g, dx, nullptr, 0));
    int status = 0;
    CK(cudaMemcpyAsync(&status, P.status, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (status == FEDNL_ETIMEOUT) return fail(FEDNL_ETIMEOUT, "grid barrier of the Cholesky timed out");
    if (status) return fail(FEDNL_ENOTPD, "H + l I is not positive definite");
    return FEDNL_OK;
}

}  // extern "C"
