// fednl_serve.cpp -- the serving loop: independent FedNL problems arrive at any time, are admitted
// in arrival order as device memory and slots allow, and then advance together one round per tick.
//
// Admission runs on the server's own host thread, beside the ticks: the queue head is admitted
// while its footprint (fednl_gpu_footprint / fednl_mx_footprint: state arena plus client data) fits
// in the device's free memory less the reserve, within the optional byte budget and the live-slot
// limit.  Admission creates the handle, uploads the queued client data and forms the initial shifts
// on the handle's own stream, then hands the problem to the next tick; the host copy of the data is
// released.  Arrival order is kept (a head that does not fit blocks the rest).  The same thread
// destroys retired problems, whose device memory release (cudaFree) waits for the device.
//
// A tick (fednl_server_tick):
//   1. the problems admitted since the last tick join the live set;
//   2. every live problem's client phase (oracle, compressor, shift update, aggregation) is
//      launched on the problem's own stream, so problems of different d overlap on the device;
//   3. one cooperative launch solves all live problems' Option-B Newton systems
//      (fednl_gpu_solve_batch), each problem on its own group of CTAs;
//   4. each problem's round is read back; a problem whose ||g|| reached its tolerance or that has
//      run its round limit retires: its iterate is kept in the record and its handle goes to the
//      admission thread for release.
// A tick's device time runs from an event the problems' streams wait on before their client phases
// to an event after the batched solve.
//
// The per-problem arithmetic does not depend on the mix (each problem's kernels read only its own
// state and the batched solve's result does not depend on the CTA count), so a problem's iterates
// are the same bit for bit alone and served among others.
//
// Threading: fednl_server_submit may be called from any thread; the other calls of one server
// from one thread at a time.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "fednl_gpu.h"

namespace {

double now_ms()
{
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

struct Pending {
    int64_t id = 0;
    fednl_problem_desc desc{};
    std::vector<int32_t> ns;
    int precision = 0;
    std::vector<double> feat64;
    std::vector<float> feat32;
    std::vector<double> labels;
    const void* fref = nullptr;    // borrowed caller buffers (fednl_server_submit_ref), else null
    const double* lref = nullptr;
    double tol = 0.0;
    int max_rounds = 0;
    int64_t bytes = 0;
};

struct Live {
    int64_t id = 0;
    int precision = 0;
    fednl_handle h = nullptr;
    fednl_mx_handle mh = nullptr;
    int d = 0;
    double tol = 0.0;
    int max_rounds = 0;
    int rounds = 0;
    int64_t bytes = 0;
};

struct Record {
    fednl_problem_status st{};
    std::vector<double> x;
};

}  // namespace

struct fednl_server_s {
    int64_t budget = 0, reserve = 0;
    int max_live = 0;
    std::mutex mu;                 // guards queue, records, next_id, ready, dead, admitting, held
    std::condition_variable cv;    // wakes the admission thread
    std::deque<Pending> queue;
    std::vector<Live> live;        // the tick thread's
    int live_n = 0;                // live.size(), published under mu for the admission thread
    std::vector<Live> ready;       // admitted, joining at the next tick
    std::vector<Live> dead;        // retired, to be released by the admission thread
    int admitting = 0;             // taken from the queue, being admitted
    std::map<int64_t, Record> records;
    int64_t next_id = 1;
    int64_t held = 0;              // footprints of the admitted problems not yet released
    double t0 = 0.0;
    std::vector<double> latencies; // one per (problem, round): ms from the tick's first launch to its result
    std::vector<double> device_ms; // one per tick with live problems: the tick's device time
    bool stop = false;
    std::thread admitter;
    cudaStream_t tick_stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

static void release(const Live& L)
{
    if (L.precision)
        fednl_mx_destroy(L.mh);
    else
        fednl_gpu_destroy(L.h);
}

static void retire(fednl_server_s* s, Live& L, int err)
{
    std::vector<double> x(L.d);
    int rc = L.precision ? fednl_mx_get_x(L.mh, x.data()) : fednl_gpu_get_x(L.h, x.data());
    std::lock_guard<std::mutex> g(s->mu);
    Record& R = s->records[L.id];
    R.st.state = err ? FEDNL_PROBLEM_FAILED : FEDNL_PROBLEM_DONE;
    R.st.error = err ? err : rc;
    R.st.rounds = L.rounds;
    R.st.t_done_ms = now_ms() - s->t0;
    if (!rc) R.x = std::move(x);
    s->dead.push_back(L);          // the admission thread releases its device memory
    s->cv.notify_one();
}

// admit the queue head if it fits; 1 = admitted (or failed and dropped), 0 = it waits
static int admit_one(fednl_server_s* s)
{
    Pending P;
    {
        std::lock_guard<std::mutex> g(s->mu);
        if (s->queue.empty()) return 0;
        if (s->max_live > 0 && s->live_n + (int)s->ready.size() + s->admitting >= s->max_live) return 0;
        const Pending& head = s->queue.front();
        int64_t fr = 0, tot = 0;
        if (fednl_gpu_mem_info(&fr, &tot)) return 0;
        if ((s->budget > 0 && head.bytes > s->budget) || head.bytes + s->reserve > tot) {
            // can never be admitted: refused with FEDNL_ENOMEM
            Record& R = s->records[head.id];
            R.st.state = FEDNL_PROBLEM_FAILED;
            R.st.error = FEDNL_ENOMEM;
            R.st.t_done_ms = now_ms() - s->t0;
            s->queue.pop_front();
            return 1;
        }
        if (s->budget > 0 && s->held + head.bytes > s->budget) return 0;
        if (head.bytes + s->reserve > fr) return 0;
        P = std::move(s->queue.front());
        s->queue.pop_front();
        s->admitting += 1;
        s->held += P.bytes;
    }
    P.desc.n_samples = P.ns.data();
    Live L;
    L.id = P.id;
    L.precision = P.precision;
    L.d = P.desc.d;
    L.tol = P.tol;
    L.max_rounds = P.max_rounds;
    L.bytes = P.bytes;
    int rc;
    const double* lab = P.lref ? P.lref : P.labels.data();
    if (P.precision) {
        const float* f = P.fref ? (const float*)P.fref : P.feat32.data();
        rc = fednl_mx_create(&P.desc, &L.mh);
        if (!rc) rc = fednl_mx_upload_client_data(L.mh, f, lab);
        if (!rc) rc = fednl_mx_init_shifts(L.mh, nullptr);
        if (rc && L.mh) fednl_mx_destroy(L.mh);
    } else {
        const double* f = P.fref ? (const double*)P.fref : P.feat64.data();
        rc = fednl_gpu_create(&P.desc, &L.h);
        if (!rc) rc = fednl_gpu_upload_client_data(L.h, f, lab);
        if (!rc) rc = fednl_gpu_init_shifts(L.h, nullptr);
        if (rc && L.h) fednl_gpu_destroy(L.h);
    }
    std::lock_guard<std::mutex> g(s->mu);
    s->admitting -= 1;
    if (rc == FEDNL_ENOMEM) {      // another user took the memory meanwhile: back to the head
        s->held -= P.bytes;
        P.desc.n_samples = nullptr;
        s->queue.push_front(std::move(P));
        return 0;
    }
    Record& R = s->records[P.id];
    R.st.t_admit_ms = now_ms() - s->t0;
    if (rc) {
        s->held -= P.bytes;
        R.st.state = FEDNL_PROBLEM_FAILED;
        R.st.error = rc;
        R.st.t_done_ms = R.st.t_admit_ms;
        return 1;
    }
    R.st.state = FEDNL_PROBLEM_LIVE;
    s->ready.push_back(L);
    return 1;
}

// the admission thread: releases retired problems, admits while the queue head fits, and otherwise
// waits for a submission or a release (polling every few ms: another user may free memory)
static void admission_loop(fednl_server_s* s)
{
    for (;;) {
        std::vector<Live> kill;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv.wait_for(lk, std::chrono::milliseconds(4),
                           [s] { return s->stop || !s->dead.empty() || !s->queue.empty(); });
            if (s->stop) return;
            kill.swap(s->dead);
        }
        for (const Live& L : kill) {
            release(L);
            std::lock_guard<std::mutex> g(s->mu);
            s->held -= L.bytes;
        }
        while (admit_one(s)) {
            std::lock_guard<std::mutex> g(s->mu);
            if (s->stop) return;
        }
        std::unique_lock<std::mutex> lk(s->mu);
        if (!s->queue.empty() && s->dead.empty())       // the head waits for memory: do not spin
            s->cv.wait_for(lk, std::chrono::milliseconds(2), [s] { return s->stop || !s->dead.empty(); });
    }
}

extern "C" {

int fednl_server_create(int64_t budget_bytes, int64_t reserve_bytes, int32_t max_live, fednl_server* out)
{
    if (!out || budget_bytes < 0 || reserve_bytes < 0 || max_live < 0) return FEDNL_EINVAL;
    fednl_server_s* s = new (std::nothrow) fednl_server_s();
    if (!s) return FEDNL_ENOMEM;
    s->budget = budget_bytes;
    s->reserve = reserve_bytes;
    s->max_live = max_live;
    s->t0 = now_ms();
    try {
        s->admitter = std::thread(admission_loop, s);
    } catch (...) {
        delete s;
        return FEDNL_ENOMEM;
    }
    *out = s;
    return FEDNL_OK;
}

int fednl_server_destroy(fednl_server s)
{
    if (!s) return FEDNL_OK;
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->stop = true;
    }
    s->cv.notify_all();
    if (s->admitter.joinable()) s->admitter.join();
    for (const Live& L : s->live) release(L);
    for (const Live& L : s->ready) release(L);
    for (const Live& L : s->dead) release(L);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->tick_stream) cudaStreamDestroy(s->tick_stream);
    delete s;
    return FEDNL_OK;
}

static int submit_impl(fednl_server s, const fednl_problem_desc* desc, int32_t precision, const void* features,
                       const double* labels, double tol, int32_t max_rounds, int64_t* id, bool borrow)
{
    if (!s || !desc || !features || !labels || !desc->n_samples || desc->d < 1 || desc->n_clients < 1 ||
        (precision != FEDNL_PRECISION_FP64 && precision != FEDNL_PRECISION_MIXED) || max_rounds < 1 || !(tol >= 0.0))
        return FEDNL_EINVAL;
    Pending P;
    P.desc = *desc;
    P.ns.assign(desc->n_samples, desc->n_samples + desc->n_clients);
    P.desc.n_samples = P.ns.data();
    P.precision = precision;
    int rc = precision ? fednl_mx_footprint(&P.desc, &P.bytes) : fednl_gpu_footprint(&P.desc, &P.bytes);
    if (rc) return rc;
    size_t S = 0;
    for (int32_t n : P.ns) S += (size_t)n;
    const size_t count = S * (size_t)desc->d;
    if (borrow) {
        P.fref = features;
        P.lref = labels;
    } else {
        try {
            if (precision)
                P.feat32.assign((const float*)features, (const float*)features + count);
            else
                P.feat64.assign((const double*)features, (const double*)features + count);
            P.labels.assign(labels, labels + S);
        } catch (const std::bad_alloc&) {
            return FEDNL_ENOMEM;
        }
    }
    P.tol = tol;
    P.max_rounds = max_rounds;
    P.desc.n_samples = nullptr;
    std::lock_guard<std::mutex> g(s->mu);
    P.id = s->next_id++;
    Record& R = s->records[P.id];
    R.st.state = FEDNL_PROBLEM_QUEUED;
    R.st.d = desc->d;
    R.st.bytes = P.bytes;
    R.st.t_submit_ms = now_ms() - s->t0;
    R.st.t_admit_ms = -1.0;
    R.st.t_done_ms = -1.0;
    R.st.grad_norm = -1.0;
    if (id) *id = P.id;
    s->queue.push_back(std::move(P));
    s->cv.notify_one();
    return FEDNL_OK;
}

int fednl_server_submit(fednl_server s, const fednl_problem_desc* desc, int32_t precision, const void* features,
                        const double* labels, double tol, int32_t max_rounds, int64_t* id)
{
    return submit_impl(s, desc, precision, features, labels, tol, max_rounds, id, false);
}

int fednl_server_submit_ref(fednl_server s, const fednl_problem_desc* desc, int32_t precision, const void* features,
                            const double* labels, double tol, int32_t max_rounds, int64_t* id)
{
    return submit_impl(s, desc, precision, features, labels, tol, max_rounds, id, true);
}

int fednl_server_tick(fednl_server s, fednl_tick_stats* st)
{
    if (!s) return FEDNL_EINVAL;
    fednl_tick_stats T{};
    {
        std::lock_guard<std::mutex> g(s->mu);
        T.admitted = (int32_t)s->ready.size();
        for (Live& L : s->ready) s->live.push_back(L);
        s->ready.clear();
        s->live_n = (int)s->live.size();
    }
    const double t_start = now_ms();
    T.live = (int32_t)s->live.size();
    if (!s->live.empty()) {
        if (!s->tick_stream) {
            cudaStreamCreateWithFlags(&s->tick_stream, cudaStreamNonBlocking);
            cudaEventCreate(&s->ev0);
            cudaEventCreate(&s->ev1);
        }
        // the tick's device clock: every problem's stream waits on ev0 before its client phase
        const bool timed = s->tick_stream && s->ev0 && s->ev1 && cudaEventRecord(s->ev0, s->tick_stream) == cudaSuccess;
        std::vector<int> ok(s->live.size(), 0);
        std::vector<fednl_handle> hs;
        std::vector<fednl_mx_handle> ms;
        std::vector<size_t> order;     // live index of hs[...] then ms[...]
        for (size_t i = 0; i < s->live.size(); ++i) {
            Live& L = s->live[i];
            if (timed) {
                cudaStream_t st = L.precision ? (cudaStream_t)fednl_mx_stream(L.mh) : (cudaStream_t)fednl_gpu_stream(L.h);
                if (st) cudaStreamWaitEvent(st, s->ev0, 0);
            }
            const int rc = L.precision ? fednl_mx_client_phase(L.mh) : fednl_gpu_client_phase(L.h);
            ok[i] = rc;
        }
        for (size_t i = 0; i < s->live.size(); ++i)
            if (!ok[i] && !s->live[i].precision) {
                hs.push_back(s->live[i].h);
                order.push_back(i);
            }
        for (size_t i = 0; i < s->live.size(); ++i)
            if (!ok[i] && s->live[i].precision) {
                ms.push_back(s->live[i].mh);
                order.push_back(i);
            }
        int brc = fednl_gpu_solve_batch(hs.data(), (int32_t)hs.size(), ms.data(), (int32_t)ms.size());
        if (brc)
            for (size_t i : order) ok[i] = brc;
        if (timed) {
            // after the batched solve (which waits for every client phase and returns when it is done)
            for (size_t i = 0; i < s->live.size(); ++i) {
                Live& L = s->live[i];
                cudaStream_t st = L.precision ? (cudaStream_t)fednl_mx_stream(L.mh) : (cudaStream_t)fednl_gpu_stream(L.h);
                cudaEvent_t e;
                if (st && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess) {
                    cudaEventRecord(e, st);
                    cudaStreamWaitEvent(s->tick_stream, e, 0);
                    cudaEventDestroy(e);
                }
            }
            float ms_dev = 0.f;
            if (cudaEventRecord(s->ev1, s->tick_stream) == cudaSuccess && cudaEventSynchronize(s->ev1) == cudaSuccess &&
                cudaEventElapsedTime(&ms_dev, s->ev0, s->ev1) == cudaSuccess) {
                T.device_ms = ms_dev;
                s->device_ms.push_back(ms_dev);
            }
        }
        std::vector<Live> keep;
        for (size_t i = 0; i < s->live.size(); ++i) {
            Live& L = s->live[i];
            fednl_round_stats R{};
            int rc = ok[i];
            if (!rc) rc = L.precision ? fednl_mx_round_result(L.mh, &R) : fednl_gpu_round_result(L.h, &R);
            const double t_end = now_ms();
            L.rounds += 1;
            {
                std::lock_guard<std::mutex> g(s->mu);
                Record& Rec = s->records[L.id];
                Rec.st.rounds = L.rounds;
                if (!rc) Rec.st.grad_norm = R.grad_norm;
            }
            if (!rc) s->latencies.push_back(t_end - t_start);
            if (rc || R.grad_norm <= L.tol || L.rounds >= L.max_rounds) {
                retire(s, L, rc);
                ++T.retired;
            } else {
                keep.push_back(L);
            }
        }
        s->live.swap(keep);
    }
    T.tick_ms = now_ms() - t_start;
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->live_n = (int)s->live.size();
        T.pending = (int32_t)(s->queue.size() + s->ready.size()) + s->admitting;
        T.held_bytes = s->held;
    }
    fednl_gpu_mem_info(&T.device_free, &T.device_total);
    if (st) *st = T;
    return FEDNL_OK;
}

int fednl_server_status(fednl_server s, int64_t id, fednl_problem_status* out, double* x)
{
    if (!s || !out) return FEDNL_EINVAL;
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->records.find(id);
    if (it == s->records.end()) return FEDNL_EINVAL;
    *out = it->second.st;
    if (x && !it->second.x.empty()) std::memcpy(x, it->second.x.data(), it->second.x.size() * 8);
    return FEDNL_OK;
}

int fednl_server_latencies(fednl_server s, double* out, int64_t cap, int64_t* count)
{
    if (!s || !count) return FEDNL_EINVAL;
    *count = (int64_t)s->latencies.size();
    if (out) std::memcpy(out, s->latencies.data(), (size_t)std::min<int64_t>(cap, *count) * 8);
    return FEDNL_OK;
}

int fednl_server_device_times(fednl_server s, double* out, int64_t cap, int64_t* count)
{
    if (!s || !count) return FEDNL_EINVAL;
    *count = (int64_t)s->device_ms.size();
    if (out) std::memcpy(out, s->device_ms.data(), (size_t)std::min<int64_t>(cap, *count) * 8);
    return FEDNL_OK;
}

}  // extern "C"
