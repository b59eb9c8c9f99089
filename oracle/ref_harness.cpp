// ref_harness.cpp -- drives the REFERENCE implementation (u-FedNL / dopt headers, compiled from
// the reference source tree by oracle/Makefile into oracle/_ref/) to produce golden vectors for
// tests/golden/.  TEST INFRASTRUCTURE ONLY: it is never part of the product library.
//
// The per-client step restates the worker loop of dopt/bin_fednl_local/include/
// LocalWorkerForFedNL_{TopK,TopLEK,RandK,RandSeqK,Natural,Identical}.h and the master merge of
// dopt/bin_fednl_local/include/TrainLoop.h:1092-1508 (with --debug forcesequpdate, i.e. the
// master merges clients in order), calling the reference's own operators for every computation.
// Worker threads are real std::threads that persist across rounds, so the TopLEK generator
// (thread_local in SpecialMathRoutinesForMatrix.h:383) has exactly the reference's per-worker
// streams.
//
// Binary formats are little-endian; see tests/golden/make_golden.py for the writer/reader.

#include "dopt/linalg_vectors/include/VectorND_Raw.h"
#include "dopt/linalg_matrices/include/MatrixNMD.h"
#include "dopt/optimization_problems/include/ml/logistic_regression.h"
#include "dopt/math_routines/include/SpecialMathRoutinesForMatrix.h"
#include "dopt/linalg_matrices/include/factorization/CholeskyFactorization.h"
#include "dopt/linalg_linsolvers/include/ElementarySolvers.h"
#include "dopt/random/include/RandomGenIntegerLinear.h"
#include "dopt/random/include/Shuffle.h"
#include "dopt/system/include/FloatUtils.h"
#include "dopt/optimization_problems/include/ml/dataset_loader_fs.h"
#include "dopt/copylocal/include/Data.h"
#include "dopt/copylocal/include/MutableData.h"

#include <atomic>
#include <chrono>
#include <barrier>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <cstdint>
#include <functional>
#include <thread>
#include <vector>

// the oracle's correctly rounded exp (oracle/fednl_oracle.c), linked in to check the reference's
// scalar libm exp calls
extern "C" double orc_exp_cr(double x);

// The reference's sigmoid evaluates its scalar tail (samples 8 floor(n/8) .. n-1) with libm's exp
// (VectorND_Raw_SIMD_double.h:1596-1650).  glibc's exp is within 0.51 ulp but not correctly rounded:
// for a few inputs in ten thousand it returns the other neighbour, and sometimes that changes the
// sigmoid value 1 / (1 + exp(-m)).  This records the first round in which a tail sigmoid differs
// from the one formed with the correctly rounded exp, so an oracle that uses a correctly rounded exp
// knows from which round on it cannot reproduce the reference's bits.
static std::atomic<int32_t> g_first_misround{-1};

static void note_tail_sigmoid(const dopt::VectorNDRaw_d& margin, const dopt::VectorNDRaw_d& sig, int32_t round)
{
    size_t n = margin.size();
    for (size_t s = n & ~size_t(7); s < n; ++s) {
        if (1.0 / (1.0 + orc_exp_cr(-margin.get(s))) != sig.get(s)) {
            int32_t cur = g_first_misround.load();
            while ((cur < 0 || round < cur) && !g_first_misround.compare_exchange_weak(cur, round)) {
            }
        }
    }
}

typedef dopt::VectorNDRaw_d Vec;
typedef dopt::MatrixNMD<Vec> Mat;
typedef dopt::L2RegulirizeLogisticRegression<Mat, Vec, double> Problem;

enum { kIdentity = 0, kRandK = 1, kTopK = 2, kRandSeqK = 3, kTopLEK = 4, kNatural = 5 };

struct Reader {
    FILE* f;
    template <class T> T get() { T v; if (fread(&v, sizeof(T), 1, f) != 1) { fprintf(stderr, "short read\n"); exit(2); } return v; }
    template <class T> void get(T* p, size_t n) { if (n && fread(p, sizeof(T), n, f) != n) { fprintf(stderr, "short read\n"); exit(2); } }
};
struct Writer {
    FILE* f;
    template <class T> void put(T v) { fwrite(&v, sizeof(T), 1, f); }
    template <class T> void put(const T* p, size_t n) { if (n) fwrite(p, sizeof(T), n, f); }
};

struct Client {
    Problem* prob = nullptr;
    Mat shift;
    Vec grad;
    double lk = 0.0;
    std::vector<uint32_t> idx;
    std::vector<double> val;
    dopt::RandomGenIntegerLinear rng;
    Vec dir, ddir;          // FedNL-PP: localGradient and the last sent difference
    double dlk = 0.0;       // FedNL-PP: the last sent Lk difference
    double fi = 0.0;        // f_i at the round's iterate (tracking / line search)
};

// compression, message and shift update of one client (LocalWorkerForFedNL_{TopK,TopLEK,RandK,
// RandSeqK,Identical,Natural}.h; the FedNL-PP workers are the same), on the reference's operators
static void compress_client(Client& C, const Mat& diff, int32_t comp, int32_t k, size_t U,
                            const std::vector<uint32_t>& upper, double alpha, double prescale, int32_t d)
{
    C.val.clear();
    if (comp == kTopK || comp == kTopLEK) {
        if (comp == kTopK) {
            C.idx = dopt::getTopKFromUpperDiagonalPart<true>(diff, k, upper);
        } else {
            double delta = double(k) * (1.0 / double(U));
            C.idx = dopt::getTopLEKFromUpperDiagonalPart<true>(diff, k, upper, delta);
        }
        for (uint32_t index : C.idx) {
            double item = diff.matrixByCols.get(index);
            C.val.push_back(item * prescale);
            size_t ir = 0, jc = 0;
            diff.getPositionFromFlatternIndex(ir, jc, index);
            C.shift.matrixByCols[index] += alpha * item;
            if (ir != jc) C.shift.matrixByCols[diff.getFlattenIndexFromPosition(jc, ir)] += alpha * item;
        }
    } else if (comp == kRandK || comp == kRandSeqK) {
        double mult = double(U) / double(k);
        for (uint32_t index : C.idx) {
            double item = diff.matrixByCols.get(index) * mult;
            C.val.push_back(item * prescale);
            size_t ir = 0, jc = 0;
            diff.getPositionFromFlatternIndex(ir, jc, index);
            C.shift.matrixByCols[index] += alpha * item;
            if (ir != jc) C.shift.matrixByCols[diff.getFlattenIndexFromPosition(jc, ir)] += alpha * item;
        }
    } else if (comp == kIdentity) {
        C.idx = upper;
        Mat sp = Mat::getZeroSquareMatrix(d);
        for (int32_t j = 0; j < d; ++j)
            for (int32_t i = 0; i <= j; ++i) {
                double item = diff.get(i, j);
                C.val.push_back(item * prescale);
                sp.set(i, j, item);
                sp.set(j, i, item);
            }
        C.shift += alpha * sp;
    } else {  // natural: the master adds preScale * unpacked value
        C.idx = upper;
        Mat sp = diff;
        sp.applyNaturalCompressor();
        for (int32_t j = 0; j < d; ++j)
            for (int32_t i = 0; i <= j; ++i) {
                auto pa = dopt::getFloatPointPack<DOPT_ARCH_LITTLE_ENDIAN>(sp.get(i, j));
                auto pb = pa;
                uint32_t packed = dopt::pack2FP64NoMantissa(pa, pb);
                dopt::FPComponentsPack<DOPT_ARCH_LITTLE_ENDIAN, double> un[2];
                dopt::unpack2FP64NoMantissa(un, packed);
                C.val.push_back(prescale * un[0].real_value_repr);
            }
        C.shift += alpha * sp;
    }
}

// ---- run: whole FedNL (Option B) ---------------------------------------------------------
// ext: the header carries Option A, FedNL-LS and tracking switches, and every round also reports
// f(x_k) and the number of line-search evaluations (TrainLoop.h:1383-1430, 1511-1640)
static int cmd_run(const char* in_path, const char* out_path, bool ext, bool timed = false)
{
    FILE* fi = fopen(in_path, "rb");
    FILE* fo = fopen(out_path, "wb");
    if (!fi || !fo) return 1;
    Reader R{fi};
    Writer W{fo};
    int32_t d = R.get<int32_t>(), nc = R.get<int32_t>(), comp = R.get<int32_t>(), k = R.get<int32_t>();
    int32_t nworkers = R.get<int32_t>(), rounds = R.get<int32_t>(), dump_rounds = R.get<int32_t>();
    double lambda = R.get<double>(), alpha = R.get<double>();
    int32_t option_a = 0, line_search = 0, ls_max = 5, track_f = 0;
    double ls_c = 0.5, ls_gamma = 0.5;
    if (ext) {
        option_a = R.get<int32_t>();
        line_search = R.get<int32_t>();
        ls_max = R.get<int32_t>();
        track_f = R.get<int32_t>();
        ls_c = R.get<double>();
        ls_gamma = R.get<double>();
    }
    std::vector<int32_t> ns(nc);
    R.get(ns.data(), nc);
    size_t S = 0;
    for (int32_t c = 0; c < nc; ++c) S += ns[c];
    std::vector<double> feat(S * d), lab(S);
    R.get(feat.data(), feat.size());
    R.get(lab.data(), lab.size());

    if (nworkers > nc) nworkers = nc;
    size_t U = ((size_t)d * (d + 1)) / 2;
    if (comp == kIdentity || comp == kNatural) k = (int32_t)U;
    double inv_n = 1.0 / double(nc);
    double prescale = inv_n * alpha;

    Vec x(d);                                   // x0 = 0 (RuntimeCfg x0 generator on [0,0])
    Mat H = Mat::getZeroSquareMatrix(d);
    std::vector<Client> cl(nc);
    size_t off = 0;
    for (int32_t c = 0; c < nc; ++c) {
        Mat xt(d, ns[c]);
        Vec b(ns[c]);
        for (int32_t s = 0; s < ns[c]; ++s) {
            for (int32_t i = 0; i < d; ++i) xt.set(i, s, feat[(off + s) * d + i]);
            b.set(s, lab[off + s]);
        }
        off += ns[c];
        cl[c].prob = new Problem(xt, b, lambda);
        cl[c].rng.setSeed(uint32_t(123 + c));
        cl[c].shift = cl[c].prob->evaluateHessian(x);
        H += cl[c].shift;
    }
    H *= inv_n;
    std::vector<uint32_t> upper = dopt::indiciesForUpperTriangularPart(H);
    W.put<int32_t>((int32_t)H.LDA);

    int32_t cur_round = 0;
    g_first_misround = -1;
    auto client_step = [&](Client& C) {
        Problem* P = C.prob;
        if (comp == kRandK)
            C.idx = dopt::generateRandKItemsInUpperTriangularPart(C.rng, k, C.shift, upper);
        else if (comp == kRandSeqK)
            C.idx = dopt::generateRandSeqKItemsInUpperTriangularPart(C.rng, k, C.shift, upper);
        Vec margin = P->evaluateClassificationMargin(x);
        Vec sig = P->evaluateClassificationMarginSigmoid(margin);
        note_tail_sigmoid(margin, sig, cur_round);
        C.grad = P->evaluateGradient(x, margin, sig);
        if (line_search || track_f) C.fi = P->evaluateFunction(x, margin, sig);
        Mat hess = P->evaluateHessian(x, margin, sig);
        Mat diff = hess - C.shift;
        C.lk = diff.frobeniusNormForSymmetricMatrixFromUpPart();
        compress_client(C, diff, comp, k, U, upper, alpha, prescale, d);
    };

    // persistent worker threads, clients round-robin c -> c mod W (TrainLoop.h:664-686)
    std::barrier start_bar(nworkers + 1), done_bar(nworkers + 1);
    bool stop = false;
    std::vector<std::thread> th;
    for (int32_t w = 0; w < nworkers; ++w)
        th.emplace_back([&, w]() {
            for (;;) {
                start_bar.arrive_and_wait();
                if (stop) {
                    // dopt vectors come from a thread_local pool: free them on the thread that made them
                    for (int32_t c = w; c < nc; c += nworkers) cl[c].grad = Vec();
                    return;
                }
                for (int32_t c = w; c < nc; c += nworkers) client_step(cl[c]);
                done_bar.arrive_and_wait();
            }
        });

    Mat Ltr;
    const auto t_start = std::chrono::steady_clock::now();
    std::vector<double> round_end_s;
    for (int32_t r = 0; r < rounds; ++r) {
        cur_round = r;
        start_bar.arrive_and_wait();
        done_bar.arrive_and_wait();
        Vec g(d);
        double l = 0.0;
        for (int32_t c = 0; c < nc; ++c) {
            g += cl[c].grad;
            for (size_t t = 0; t < cl[c].idx.size(); ++t) H.matrixByCols[cl[c].idx[t]] += cl[c].val[t];
            l += cl[c].lk;
        }
        g *= inv_n;
        l *= inv_n;
        bool ok = dopt::cholFactorization::choleskyFactorization<Mat, true, true>(Ltr, H, option_a ? lambda : l);
        Vec dx(d);
        if (ok) {
            Vec y = dopt::forwardSubstitutionWithATranspose(Ltr, g);
            dx = dopt::backwardSubstitutionWithATranspose(Ltr, y);
        }
        double f_k = 0.0;
        int32_t ls_steps = 0;
        if (line_search || track_f) {
            for (int32_t c = 0; c < nc; ++c) f_k += cl[c].fi;
            f_k *= inv_n;
        }
        if (!line_search) {
            x -= dx;
        } else {
            double t = 1.0;
            double dxg = -(dx & g);
            Vec xprev = x;
            for (int32_t it = 0; it < ls_max; ++it) {
                x = xprev - (t * dx);
                double fr = 0.0;
                for (int32_t c = 0; c < nc; ++c) {
                    Vec mg = cl[c].prob->evaluateClassificationMargin(x);
                    Vec sg = cl[c].prob->evaluateClassificationMarginSigmoid(mg);
                    note_tail_sigmoid(mg, sg, cur_round);
                    fr += cl[c].prob->evaluateFunction(x, mg, sg);
                }
                fr *= inv_n;
                ls_steps = it + 1;
                if (fr <= f_k + (ls_c * t) * dxg) break;
                t *= ls_gamma;
            }
        }
        round_end_s.push_back(std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count());
        W.put<int32_t>(ok ? 1 : 0);
        W.put<double>(g.vectorL2Norm());
        W.put<double>(l);
        W.put(x.dataConst(), (size_t)d);
        if (ext) {
            W.put<double>(f_k);
            W.put<int32_t>(ls_steps);
        }
        if (r < dump_rounds) {
            for (int32_t c = 0; c < nc; ++c) {
                W.put<int32_t>((int32_t)cl[c].idx.size());
                W.put(cl[c].idx.data(), cl[c].idx.size());
                W.put(cl[c].val.data(), cl[c].val.size());
                W.put<double>(cl[c].lk);
            }
        }
    }
    stop = true;
    start_bar.arrive_and_wait();
    for (auto& t : th) t.join();
    for (auto& c : cl) delete c.prob;
    W.put<int32_t>(g_first_misround.load());   // trailer: first round whose sigmoid a libm misrounding changed
    if (timed) W.put(round_end_s.data(), round_end_s.size());   // "time": wall seconds at the end of each round
    fclose(fi);
    fclose(fo);
    return 0;
}

// ---- pp: whole FedNL-PP (Option B), dopt/bin_fednl_local_pp -----------------------------
// Workers: LocalWorkerForFedNL_*.h of bin_fednl_local_pp (selected clients only; Lk after the shift
// update, sent as a difference; direction x Lk + shift x - grad, sent as a difference).  Master:
// TrainLoop.h:1064-1080 (init means), :1150-1166 (sampler: partial shuffle of a fresh 0..n-1 with
// the --client-selection-seed generator; true gradient), :1168-1450 (merge in client order with
// forcesequpdate; g and l as running means), :1560-1600 (x = Cholesky solve).  Single-threaded:
// one reference worker, so the TopLEK generator is the main thread's.
static int cmd_pp(const char* in_path, const char* out_path)
{
    FILE* fi = fopen(in_path, "rb");
    FILE* fo = fopen(out_path, "wb");
    if (!fi || !fo) return 1;
    Reader R{fi};
    Writer W{fo};
    int32_t d = R.get<int32_t>(), nc = R.get<int32_t>(), comp = R.get<int32_t>(), k = R.get<int32_t>();
    int32_t tau = R.get<int32_t>(), rounds = R.get<int32_t>(), dump_rounds = R.get<int32_t>();
    uint32_t sel_seed = R.get<uint32_t>();
    double lambda = R.get<double>(), alpha = R.get<double>();
    std::vector<int32_t> ns(nc);
    R.get(ns.data(), nc);
    size_t S = 0;
    for (int32_t c = 0; c < nc; ++c) S += ns[c];
    std::vector<double> feat(S * d), lab(S);
    R.get(feat.data(), feat.size());
    R.get(lab.data(), lab.size());

    size_t U = ((size_t)d * (d + 1)) / 2;
    if (comp == kIdentity || comp == kNatural) k = (int32_t)U;
    double inv_n = 1.0 / double(nc);
    double prescale = inv_n * alpha;

    Vec x(d);
    Mat H = Mat::getZeroSquareMatrix(d);
    Vec g_prev(d);
    double l_prev = 0.0;
    std::vector<Client> cl(nc);
    size_t off = 0;
    for (int32_t c = 0; c < nc; ++c) {
        Mat xt(d, ns[c]);
        Vec b(ns[c]);
        for (int32_t s = 0; s < ns[c]; ++s) {
            for (int32_t i = 0; i < d; ++i) xt.set(i, s, feat[(off + s) * d + i]);
            b.set(s, lab[off + s]);
        }
        off += ns[c];
        cl[c].prob = new Problem(xt, b, lambda);
        cl[c].rng.setSeed(uint32_t(123 + c));
        cl[c].shift = cl[c].prob->evaluateHessian(x);
        cl[c].lk = 0.0;
        cl[c].dir = Mat::matrixVectorMultiply(cl[c].shift, x) - cl[c].prob->evaluateGradient(x);
        H += cl[c].shift;
        g_prev += cl[c].dir;
        l_prev += cl[c].lk;
    }
    H *= inv_n;
    g_prev *= inv_n;
    l_prev *= inv_n;
    std::vector<uint32_t> upper = dopt::indiciesForUpperTriangularPart(H);
    W.put<int32_t>((int32_t)H.LDA);

    dopt::RandomGenIntegerLinear sampler;
    sampler.setSeed(sel_seed);
    std::vector<uint32_t> all(nc);
    for (int32_t c = 0; c < nc; ++c) all[c] = (uint32_t)c;
    std::vector<char> is_sel(nc);
    Mat Ltr;
    for (int32_t r = 0; r < rounds; ++r) {
        std::vector<uint32_t> selv = all;
        dopt::shuffle(selv, (size_t)tau, sampler);
        std::fill(is_sel.begin(), is_sel.end(), 0);
        for (int32_t t = 0; t < tau; ++t) is_sel[selv[t]] = 1;
        Vec tg(d);
        for (int32_t c = 0; c < nc; ++c) tg += cl[c].prob->evaluateGradient(x);
        tg = tg / double(nc);
        for (int32_t c = 0; c < nc; ++c) {
            if (!is_sel[c]) continue;
            Client& C = cl[c];
            Problem* P = C.prob;
            if (comp == kRandK)
                C.idx = dopt::generateRandKItemsInUpperTriangularPart(C.rng, k, C.shift, upper);
            else if (comp == kRandSeqK)
                C.idx = dopt::generateRandSeqKItemsInUpperTriangularPart(C.rng, k, C.shift, upper);
            Vec margin = P->evaluateClassificationMargin(x);
            Vec sig = P->evaluateClassificationMarginSigmoid(margin);
            Mat hess = P->evaluateHessian(x, margin, sig);
            Mat diff = hess - C.shift;
            compress_client(C, diff, comp, k, U, upper, alpha, prescale, d);
            double lk_new = (C.shift - hess).frobeniusNormForSymmetricMatrixFromUpPart();
            C.dlk = lk_new - C.lk;
            C.lk = lk_new;
            Vec dir = (x * C.lk) + Mat::matrixVectorMultiply(C.shift, x) - P->evaluateGradient(x, margin, sig);
            C.ddir = dir - C.dir;
            C.dir = dir;
        }
        Vec g(d);
        double l = 0.0;
        for (int32_t c = 0; c < nc; ++c) {
            if (!is_sel[c]) continue;
            g += cl[c].ddir;
            for (size_t t = 0; t < cl[c].idx.size(); ++t) H.matrixByCols[cl[c].idx[t]] += cl[c].val[t];
            l += cl[c].dlk;
        }
        g *= inv_n;
        g += g_prev;
        g_prev = g;
        l *= inv_n;
        l += l_prev;
        l_prev = l;
        bool ok = dopt::cholFactorization::choleskyFactorization<Mat, true, true>(Ltr, H, l);
        if (ok) {
            Vec y = dopt::forwardSubstitutionWithATranspose(Ltr, g);
            x = dopt::backwardSubstitutionWithATranspose(Ltr, y);
        }
        W.put<int32_t>(ok ? 1 : 0);
        W.put<double>(tg.vectorL2Norm());
        W.put<double>(l);
        W.put(x.dataConst(), (size_t)d);
        for (int32_t c = 0; c < nc; ++c)
            if (is_sel[c]) W.put<int32_t>(c);
        if (r < dump_rounds) {
            for (int32_t c = 0; c < nc; ++c) {
                if (!is_sel[c]) continue;
                W.put<int32_t>((int32_t)cl[c].idx.size());
                W.put(cl[c].idx.data(), cl[c].idx.size());
                W.put(cl[c].val.data(), cl[c].val.size());
                W.put<double>(cl[c].lk);
                W.put(cl[c].dir.dataConst(), (size_t)d);
            }
        }
    }
    for (auto& c : cl) delete c.prob;
    fclose(fi);
    fclose(fo);
    return 0;
}

// ---- libsvm: the reference's text loader (dataset_loader_fs.h) as bin_fednl_local drives it
// (TrainLoop.h:124-180): statistics pass, then createDataset with label remapping and optional
// intercept.  Output: status, d, n, then features [n][d] and labels [n].
static int cmd_libsvm(const char* in_path, const char* out_path, int add_intercept)
{
    FILE* fi = fopen(in_path, "rb");
    FILE* fo = fopen(out_path, "wb");
    if (!fi || !fo) return 1;
    std::string text;
    char buf[65536];
    size_t got;
    while ((got = fread(buf, 1, sizeof(buf), fi)) > 0) text.append(buf, got);
    fclose(fi);
    Writer W{fo};
    auto line_sep = [](char c) { return c == '\n' || c == '\r'; };
    auto field_sep = [](char c) { return c == '\t' || c == ' '; };
    auto attr_sep = [](char c) { return c == ':'; };
    auto skip = [](char c) { return false; };
    dopt::Data raw(text.data(), text.size(), dopt::Data::MemInitializedType::eGiftWholeMemoryPleaseNotFree);
    dopt::TextFileDataSetLoader loader(raw, line_sep, field_sep, attr_sep, skip);
    auto stats = loader.computeStatisticsWithOneDataPass<false, true, int32_t, int32_t>();
    if (!stats.ok) {
        W.put<int32_t>(0);
        fclose(fo);
        return 0;
    }
    typedef dopt::DataSet<Mat, Vec, dopt::VectorNDRaw_b, Vec> DS;
    DS ds;
    int flags = (add_intercept ? dopt::CreateDatasetFlags::eAddInterceptTerm : dopt::CreateDatasetFlags::eNone) |
                dopt::CreateDatasetFlags::eMakeRemappingForBinaryLogisticLoss;
    size_t n = loader.createDataset<true, true>(ds, stats, flags);
    int32_t d = (int32_t)ds.train_samples_tr.rows();
    W.put<int32_t>(1);
    W.put<int32_t>(d);
    W.put<int32_t>((int32_t)n);
    for (size_t s = 0; s < n; ++s)
        for (int32_t i = 0; i < d; ++i) W.put<double>(ds.train_samples_tr.get(i, s));
    for (size_t s = 0; s < n; ++s) W.put<double>(ds.train_outputs.get(s));
    fclose(fo);
    return 0;
}

// ---- topk / toplek on given matrices (one OS thread => one TopLEK stream) ------------------
static int cmd_select(const char* in_path, const char* out_path, bool lek)
{
    FILE* fi = fopen(in_path, "rb");
    FILE* fo = fopen(out_path, "wb");
    if (!fi || !fo) return 1;
    Reader R{fi};
    Writer W{fo};
    int32_t d = R.get<int32_t>(), k = R.get<int32_t>(), nm = R.get<int32_t>();
    Mat m(d, d);
    size_t U = ((size_t)d * (d + 1)) / 2;
    std::vector<uint32_t> upper = dopt::indiciesForUpperTriangularPart(m);
    W.put<int32_t>((int32_t)m.LDA);
    std::vector<double> buf((size_t)d * d);
    for (int32_t t = 0; t < nm; ++t) {
        R.get(buf.data(), buf.size());          // column-major d x d (unpadded)
        for (int32_t j = 0; j < d; ++j)
            for (int32_t i = 0; i < d; ++i) m.set(i, j, buf[(size_t)j * d + i]);
        std::vector<uint32_t> idx;
        if (lek) idx = dopt::getTopLEKFromUpperDiagonalPart<true>(m, k, upper, double(k) * (1.0 / double(U)));
        else idx = dopt::getTopKFromUpperDiagonalPart<true>(m, k, upper);
        W.put<int32_t>((int32_t)idx.size());
        W.put(idx.data(), idx.size());
    }
    fclose(fi);
    fclose(fo);
    return 0;
}

// ---- randk / randseqk draws for one client generator -------------------------------------
static int cmd_rand(const char* out_path, int32_t d, int32_t k, uint32_t seed, int32_t draws, bool seq)
{
    FILE* fo = fopen(out_path, "wb");
    if (!fo) return 1;
    Writer W{fo};
    Mat m(d, d);
    std::vector<uint32_t> upper = dopt::indiciesForUpperTriangularPart(m);
    dopt::RandomGenIntegerLinear g;
    g.setSeed(seed);
    W.put<int32_t>((int32_t)m.LDA);
    for (int32_t t = 0; t < draws; ++t) {
        std::vector<uint32_t> idx = seq ? dopt::generateRandSeqKItemsInUpperTriangularPart(g, k, m, upper)
                                        : dopt::generateRandKItemsInUpperTriangularPart(g, k, m, upper);
        W.put(idx.data(), idx.size());
    }
    fclose(fo);
    return 0;
}

// ---- Cholesky Option-B solve on a given matrix --------------------------------------------
static int cmd_chol(const char* in_path, const char* out_path)
{
    FILE* fi = fopen(in_path, "rb");
    FILE* fo = fopen(out_path, "wb");
    if (!fi || !fo) return 1;
    Reader R{fi};
    Writer W{fo};
    int32_t d = R.get<int32_t>();
    double l = R.get<double>();
    std::vector<double> buf((size_t)d * d), b(d);
    R.get(buf.data(), buf.size());
    R.get(b.data(), b.size());
    Mat h(d, d);
    for (int32_t j = 0; j < d; ++j)
        for (int32_t i = 0; i < d; ++i) h.set(i, j, buf[(size_t)j * d + i]);
    Vec g(d);
    for (int32_t i = 0; i < d; ++i) g.set(i, b[i]);
    Mat Ltr;
    bool ok = dopt::cholFactorization::choleskyFactorization<Mat, true, true>(Ltr, h, l);
    Vec x(d);
    if (ok) {
        Vec y = dopt::forwardSubstitutionWithATranspose(Ltr, g);
        x = dopt::backwardSubstitutionWithATranspose(Ltr, y);
    }
    W.put<int32_t>(ok ? 1 : 0);
    W.put(x.dataConst(), (size_t)d);
    fclose(fi);
    fclose(fo);
    return 0;
}

// Packet framing of the distributed client's messages: for every record (u8 signal, u32 length,
// payload) the bytes that WorkerContextForFedNL::prepareUpdate writes with dopt::MutableData
// (dopt/bin_fednl_distr_client/include/UsedTypes.h:1022-1125): putByte(signal),
// putUnsignedVaryingInteger(length), putBytes(payload).
static int cmd_wire(const char* in_path, const char* out_path)
{
    FILE* fi = fopen(in_path, "rb");
    FILE* fo = fopen(out_path, "wb");
    if (!fi || !fo) return 1;
    Reader R{fi};
    int32_t n = R.get<int32_t>();
    dopt::MutableData buf;
    for (int32_t r = 0; r < n; ++r) {
        uint8_t sig = (uint8_t)R.get<int32_t>();
        uint32_t len = (uint32_t)R.get<int32_t>();
        std::vector<uint8_t> payload(len);
        if (len) R.get(payload.data(), len);
        buf.putByte(sig);
        buf.putUnsignedVaryingInteger(len);
        if (len) buf.putBytes(payload.data(), len);
    }
    fwrite(buf.getPtr(), 1, buf.getFilledSize(), fo);
    fclose(fi);
    fclose(fo);
    return 0;
}

int main(int argc, char** argv)
{
    if (argc < 3) {
        fprintf(stderr, "usage: ref_harness run|topk|toplek|chol IN OUT | randk|randseqk OUT d k seed draws\n");
        return 2;
    }
    if (!strcmp(argv[1], "run")) return cmd_run(argv[2], argv[3], false);
    if (!strcmp(argv[1], "runx")) return cmd_run(argv[2], argv[3], true);
    if (!strcmp(argv[1], "time")) return cmd_run(argv[2], argv[3], false, true);
    if (!strcmp(argv[1], "pp")) return cmd_pp(argv[2], argv[3]);
    if (!strcmp(argv[1], "libsvm") && argc >= 5) return cmd_libsvm(argv[2], argv[3], atoi(argv[4]));
    if (!strcmp(argv[1], "topk")) return cmd_select(argv[2], argv[3], false);
    if (!strcmp(argv[1], "toplek")) return cmd_select(argv[2], argv[3], true);
    if (!strcmp(argv[1], "chol")) return cmd_chol(argv[2], argv[3]);
    if (!strcmp(argv[1], "wire")) return cmd_wire(argv[2], argv[3]);
    if ((!strcmp(argv[1], "randk") || !strcmp(argv[1], "randseqk")) && argc >= 7)
        return cmd_rand(argv[2], atoi(argv[3]), atoi(argv[4]), (uint32_t)strtoul(argv[5], 0, 10), atoi(argv[6]),
                        !strcmp(argv[1], "randseqk"));
    fprintf(stderr, "bad command\n");
    return 2;
}
