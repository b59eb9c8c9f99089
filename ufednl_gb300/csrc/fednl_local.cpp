// fednl_local.cpp -- the reference's local-simulation driver behind one C call:
// fednl_gpu_execute_local(command, callback) takes the command line of bin_fednl_local
// (dopt/bin_fednl_local/src/mainShared.cpp:15-38, doptExecuteLocal) and runs it on the GB300 round
// engine: flag parsing (bin_fednl_local/include/Args.h), LIBSVM loading with the reference's parser
// semantics (dopt/optimization_problems/include/ml/dataset_loader_fs.h:380-885,
// dopt/fs/include/StringUtils.h:95-470), the even client split with optional reshuffle
// (TrainLoop.h:188-250), k and alpha selection (TrainLoop.h:355-521), the rounds, the tracking
// record file (TrainLoop.h:753-792, 1679-1691, 1820-1850) and the final callback (:1854-1860).
// Host code only; every round runs through the C ABI of include/fednl_gpu.h.

#include "fednl_gpu.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

// ---- command line (dopt/cmdline/src/CmdLineParser.cpp): "--name value" pairs and "--flag"s, names
// compared without their one or two leading dashes; the first occurrence counts
struct CmdLine {
    std::vector<std::string> argv;

    static std::string strip(const std::string& s)
    {
        size_t p = 0;
        if (p < s.size() && s[p] == '-') ++p;
        if (p < s.size() && s[p] == '-') ++p;
        return s.substr(p);
    }
    int index_of_value(const char* name) const
    {
        for (size_t i = 1; i < argv.size(); ++i) {
            if (argv[i].empty() || argv[i][0] != '-') continue;
            if (strip(argv[i]) == name) return i + 1 < argv.size() ? (int)(i + 1) : -1;
        }
        return -1;
    }
    bool flag(const char* name) const
    {
        for (size_t i = 1; i < argv.size(); ++i)
            if (strip(argv[i]) == name) return true;
        return false;
    }
    bool str(const char* name, std::string& v) const
    {
        int i = index_of_value(name);
        if (i < 0) return false;
        v = argv[i];
        return true;
    }
};

// ---- number parsing with the reference's semantics ------------------------------------------
// fromStringSignedInteger (StringUtils.h:171-268): optional sign, digits only, 32-bit wrap-around
bool parse_i32(const char* b, const char* e, int32_t& out)
{
    if (b == e) return false;
    bool neg = false;
    if (*b == '+' || *b == '-') {
        neg = *b == '-';
        ++b;
        if (b == e) return false;
    }
    uint32_t v = 0;
    for (; b != e; ++b) {
        if (*b < '0' || *b > '9') return false;
        v = neg ? v * 10u - (uint32_t)(*b - '0') : v * 10u + (uint32_t)(*b - '0');
    }
    out = (int32_t)v;
    return true;
}

bool parse_u32(const char* b, const char* e, uint32_t& out)
{
    if (b == e) return false;
    uint32_t v = 0;
    for (; b != e; ++b) {
        if (*b < '0' || *b > '9') return false;
        v = v * 10u + (uint32_t)(*b - '0');
    }
    out = v;
    return true;
}

// powerNatural (SimpleMathRoutines.h:179-197): recursive squaring
double power_natural(double a, uint32_t p)
{
    if (p == 0) return 1.0;
    if (p % 2 == 0) {
        double t = power_natural(a, p / 2);
        return t * t;
    }
    double t = power_natural(a, (p - 1) / 2);
    return t * t * a;
}

// fromStringFloat (StringUtils.h:270-461): integer and fraction digits in 32-bit ints, the fraction
// scaled by 1/10^len (table up to 16 digits), exponent by repeated squaring
bool parse_f64(const char* b, const char* e, double& out)
{
    if (b == e) return false;
    int sign = +1;
    if (*b == '+') ++b;
    else if (*b == '-') {
        sign = -1;
        ++b;
    }
    uint32_t ip = 0, fp = 0, flen = 0, ep = 0;
    int esign = +1;
    for (; b != e; ++b) {
        if (*b == '.' || *b == 'e' || *b == 'E') break;
        if (*b < '0' || *b > '9') return false;
        ip = ip * 10u + (uint32_t)(*b - '0');
    }
    if (b != e && *b == '.') {
        for (++b; b != e; ++b) {
            if (*b == 'e' || *b == 'E') break;
            if (*b < '0' || *b > '9') return false;
            fp = fp * 10u + (uint32_t)(*b - '0');
            ++flen;
        }
    }
    if (b != e && (*b == 'e' || *b == 'E')) {
        ++b;
        if (b != e && *b == '+') ++b;
        else if (b != e && *b == '-') {
            esign = -1;
            ++b;
        }
        for (; b != e; ++b) {
            if (*b < '0' || *b > '9') return false;
            ep = ep * 10u + (uint32_t)(*b - '0');
        }
    }
    const double I = (double)(int32_t)ip, F = (double)(int32_t)fp;
    if (ep == 0) {
        if (flen == 0) {
            out = sign > 0 ? I : -I;
        } else {
            static const double den[17] = {1.0 / 1e0,  1.0 / 1e1,  1.0 / 1e2,  1.0 / 1e3,  1.0 / 1e4,  1.0 / 1e5,
                                           1.0 / 1e6,  1.0 / 1e7,  1.0 / 1e8,  1.0 / 1e9,  1.0 / 1e10, 1.0 / 1e11,
                                           1.0 / 1e12, 1.0 / 1e13, 1.0 / 1e14, 1.0 / 1e15, 1.0 / 1e16};
            const double dn = flen < 17 ? den[flen] : 1.0 / power_natural(10.0, flen);
            const double v = I + F * dn;
            out = sign > 0 ? v : -v;
        }
    } else {
        const double dn = 1.0 / power_natural(10.0, flen);
        const double ev = power_natural(10.0, ep);
        const double v = I + F * dn;
        if (esign > 0) out = sign > 0 ? v * ev : -v * ev;
        else out = sign > 0 ? v / ev : -v / ev;
    }
    return true;
}

// ---- LIBSVM text: "label index:value ..." per line ------------------------------------------
struct Dataset {
    int d = 0;                       // attributes (+1 with the intercept row)
    int n = 0;
    std::vector<double> x;           // [n][d] row-major
    std::vector<double> y;           // +-1
    // the same rows as CSR columns of the attributes equal to 1 (ascending), valid when every
    // value of the file is 0 or 1 (binary)
    std::vector<int32_t> rp, cols;
    bool binary = true;
};

template <class F>
void split_tokens(const char* b, const char* e, F is_sep, std::vector<std::pair<const char*, const char*>>& out)
{
    out.clear();
    const char* s = b;
    for (const char* p = b; p != e; ++p)
        if (is_sep(*p)) {
            if (p > s) out.push_back({s, p});
            s = p + 1;
        }
    if (e > s) out.push_back({s, e});
}

// dataset_loader_fs.h:380-600 (statistics pass) and :607-885 (createDataset), with line separators
// '\n' and '\r', field separators ' ' and '\t', ':' between index and value (TrainLoop.h:124-134)
int load_libsvm(const std::string& path, bool add_intercept, Dataset& ds, std::string& err)
{
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) {
        err = "cannot open " + path;
        return -3;
    }
    std::string text;
    char buf[1 << 16];
    size_t got;
    while ((got = fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, got);
    fclose(f);
    std::vector<std::pair<const char*, const char*>> lines, fields, kv;
    split_tokens(text.data(), text.data() + text.size(), [](char c) { return c == '\n' || c == '\r'; }, lines);
    // statistics pass: int32 labels and indices; the first line resets min and max for each of its
    // entries, later lines update min, else max (the reference's rule, kept as is)
    long long examples = 0;
    int32_t fmin = 0, fmax = 0, lmin = 0, lmax = 0;
    int unique = 0;
    for (auto& ln : lines) {
        split_tokens(ln.first, ln.second, [](char c) { return c == ' ' || c == '\t'; }, fields);
        if (fields.empty()) continue;
        for (auto& fd : fields) {
            split_tokens(fd.first, fd.second, [](char c) { return c == ':'; }, kv);
            if (kv.size() == 1) {
                int32_t lv;
                if (!parse_i32(kv[0].first, kv[0].second, lv)) continue;
                if (examples == 0) {
                    lmin = lmax = lv;
                    unique = 1;
                } else if (lv != lmin && lv != lmax) {
                    ++unique;
                    if (lv < lmin) lmin = lv;
                    else if (lv > lmax) lmax = lv;
                }
            } else if (kv.size() == 2) {
                int32_t idx;
                if (!parse_i32(kv[0].first, kv[0].second, idx)) {
                    err = "line " + std::to_string(examples + 1) + ": cannot parse a feature index";
                    return -4;
                }
                if (examples == 0) {
                    fmin = fmax = idx;
                } else if (idx < fmin) {
                    fmin = idx;
                } else if (idx > fmax) {
                    fmax = idx;
                }
            }
        }
        ++examples;
    }
    if (unique != 2) {
        err = "the dataset has " + std::to_string(unique) + " label classes, 2 are needed";
        return -4;
    }
    const int d0 = fmax - fmin + 1;
    ds.d = d0 + (add_intercept ? 1 : 0);
    ds.n = (int)examples;
    ds.x.assign((size_t)ds.n * ds.d, 0.0);
    ds.y.assign(ds.n, 0.0);
    const double avg = ((double)lmin + (double)lmax) / 2.0;
    int s = 0;
    std::vector<int32_t> touched;
    ds.rp.assign(1, 0);
    for (auto& ln : lines) {
        split_tokens(ln.first, ln.second, [](char c) { return c == ' ' || c == '\t'; }, fields);
        if (fields.empty()) continue;
        double* row = ds.x.data() + (size_t)s * ds.d;
        touched.clear();
        for (auto& fd : fields) {
            split_tokens(fd.first, fd.second, [](char c) { return c == ':'; }, kv);
            if (kv.size() == 1) {
                double lv = 0.0;
                parse_f64(kv[0].first, kv[0].second, lv);
                ds.y[s] = lv < avg ? -1.0 : 1.0;          // eMakeRemappingForBinaryLogisticLoss
            } else if (kv.size() == 2) {
                int32_t idx = 0;
                double v = 0.0;
                parse_i32(kv[0].first, kv[0].second, idx);
                parse_f64(kv[1].first, kv[1].second, v);
                const long long r = (long long)idx - fmin;
                if (r < 0 || r >= d0) {
                    err = "line " + std::to_string(s + 1) + ": feature index outside the range the statistics pass found";
                    return -4;
                }
                row[r] = v;
                touched.push_back((int32_t)r);
            }
        }
        if (add_intercept) {
            row[ds.d - 1] = 1.0;
            touched.push_back(ds.d - 1);
        }
        // the row's final values (a repeated index keeps its last value) as ascending CSR columns
        std::sort(touched.begin(), touched.end());
        touched.erase(std::unique(touched.begin(), touched.end()), touched.end());
        for (int32_t col : touched) {
            if (row[col] == 1.0) ds.cols.push_back(col);
            else if (row[col] != 0.0) ds.binary = false;
        }
        ds.rp.push_back((int32_t)ds.cols.size());
        ++s;
    }
    return 0;
}

// RandomGenIntegerLinear (RandomGenIntegerLinear.h:49-58) and the Fisher-Yates of Shuffle.h:133-160
double lcg_unit(uint32_t& st)
{
    st = 214013u * st + 2531011u;
    return (double)st * (1.0 / 4294967295.0);
}

size_t round_to_nearest(double v)
{
    size_t t = (size_t)v;
    return v - (double)t > 0.5 ? t + 1 : t;
}

void shuffle_all(std::vector<int32_t>& a, uint32_t seed)
{
    uint32_t st = seed;
    size_t n = a.size(), nm = n - 1;
    for (size_t i = 0; i < n; ++i, --nm) {
        size_t r = round_to_nearest(lcg_unit(st) * (double)nm);
        if (r != 0) std::swap(a[i], a[i + r]);
    }
}

std::string base_name(const std::string& p)
{
    size_t s = p.find_last_of("/\\");
    std::string b = s == std::string::npos ? p : p.substr(s + 1);
    size_t dot = b.find_last_of('.');
    return dot == std::string::npos ? b : b.substr(0, dot);
}

struct Tracker {
    std::vector<unsigned char> bytes;
    void put(const void* p, size_t n)
    {
        const unsigned char* c = (const unsigned char*)p;
        bytes.insert(bytes.end(), c, c + n);
    }
    void i32(int32_t v) { put(&v, 4); }
    void f64(double v) { put(&v, 8); }
    void cstr(const std::string& s, bool zero)
    {
        put(s.data(), s.size());
        if (zero) bytes.push_back(0);
    }
};

}  // namespace

extern "C" int fednl_gpu_load_libsvm(const char* path, int32_t add_intercept, int32_t* n_samples, int32_t* d,
                                     double* features, double* labels)
{
    if (!path || !n_samples || !d) return -1;
    Dataset ds;
    std::string err;
    const int rc = load_libsvm(path, add_intercept != 0, ds, err);
    if (rc) return rc;
    *n_samples = ds.n;
    *d = ds.d;
    if (features) std::memcpy(features, ds.x.data(), ds.x.size() * sizeof(double));
    if (labels) std::memcpy(labels, ds.y.data(), ds.y.size() * sizeof(double));
    return 0;
}

// Squared L2 norm in the reference's two-Vec4d order (VectorNDRaw<double>::vectorL2NormSquare,
// VectorND_Raw_SIMD_double.h:749-800): element i < 8 floor(n/8) into lane i mod 8, lanes reduced as
// (0 + ((c0 + c2) + (c1 + c3))) + ((c4 + c6) + (c5 + c7)), the tail summed in order and added last.
static double ref_norm2(const std::vector<double>& v)
{
    double c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const size_t n = v.size(), items = n & ~(size_t)7;
    size_t i = 0;
    for (; i < items; i += 8)
        for (int l = 0; l < 8; ++l) c[l] = c[l] + v[i + l] * v[i + l];
    double fin = 0.0;
    fin = fin + ((c[0] + c[2]) + (c[1] + c[3]));
    fin = fin + ((c[4] + c[6]) + (c[5] + c[7]));
    double rest = 0.0;
    for (; i < n; ++i) rest = rest + v[i] * v[i];
    return fin + rest;
}

// bin_fednl_local's and bin_fednl_local_pp's train() on the engine.  pp: the partial-participation
// binary (--clients-per-round, Option B/A, no line search; its callback receives the dimension only).
static int execute_local_impl(const char* command, bool pp, fednl_result_callback cb, void (*cb_pp)(int))
{
    if (!command) return -1;
    CmdLine cl;
    {
        std::string all = std::string("train ") + command;    // mainShared.cpp:17-18
        std::vector<std::pair<const char*, const char*>> tok;
        split_tokens(all.data(), all.data() + all.size(), [](char c) { return c == ' '; }, tok);
        for (auto& t : tok) cl.argv.emplace_back(t.first, t.second);
    }
    auto num = [&](const char* name, double& v) {
        std::string s;
        return cl.str(name, s) && parse_f64(s.data(), s.data() + s.size(), v);
    };
    auto i32 = [&](const char* name, int32_t& v) {
        std::string s;
        return cl.str(name, s) && parse_i32(s.data(), s.data() + s.size(), v);
    };
    auto u32 = [&](const char* name, uint32_t& v) {
        std::string s;
        return cl.str(name, s) && parse_u32(s.data(), s.data() + s.size(), v);
    };
    // --debug modes (Args.h:82-127); the engine always merges clients in order (forcesequpdate)
    std::string dbg;
    if (cl.str("debug", dbg)) {
        std::vector<std::pair<const char*, const char*>> modes;
        split_tokens(dbg.data(), dbg.data() + dbg.size(), [](char c) { return c == ',' || c == ';'; }, modes);
        for (auto& m : modes) {
            std::string mode(m.first, m.second);
            if (mode != "notracingprint" && mode != "meminfo" && mode != "forcesequpdate" && mode != "crc32fordata" &&
                mode != "printtrain")
                return -8;                                   // eUnknownDebugMode
        }
    }
    const bool tracking = cl.flag("tracking");
    std::string out_path;
    if (!cl.str("out", out_path)) return -1;
    std::string path;
    if (!cl.str("train_dataset", path)) return -1;
    {
        FILE* f = fopen(path.c_str(), "rb");
        if (!f) return -3;                                   // eTrainDatasetIsNotAvailable
        fclose(f);
    }
    int32_t n_clients = 1, workers = 1, rounds = 0;
    uint32_t reshuffle_seed = 123, x0_seed = 1234;
    i32("clients", n_clients);
    const bool reshuffle = cl.flag("reshuffle_train");
    u32("reshuffle_train_seed", reshuffle_seed);
    const bool add_intercept = cl.flag("add_intercept");
    double lambda = 0.0;
    if (!num("lambda", lambda)) return -1;
    i32("workers", workers);
    if (!i32("rounds", rounds)) return -1;
    u32("x0_seed", x0_seed);
    std::string algorithm;
    if (!cl.str("algorithm", algorithm)) return -1;
    if (algorithm != "fednl1") return -2;                    // GD is outside the FedNL hot path
    double kmult = 1.0;
    if (!num("k_compressor_as_d_mult", kmult)) return -1;
    std::string comp_name;
    if (!cl.str("compressor", comp_name)) return -1;
    const bool theo = cl.flag("theoretical_alpha");
    const bool opt1 = cl.flag("use_theoretical_alpha_option_1"), opt2 = cl.flag("use_theoretical_alpha_option_2");
    double alpha = 0.0;
    if (!theo && !num("alpha_step_size", alpha)) return -1;
    const bool ls = !pp && cl.flag("line_search");          // the PP binary has no line search (its Args.h)
    double ls_c = 0.5, ls_gamma = 0.5;
    uint32_t ls_max = 5;
    int32_t per_round = 0;
    if (pp && (!i32("clients-per-round", per_round) || per_round < 1)) return -1;
    // arithmetic order of the engine: the reference's own (default; bit-identical rounds) or the
    // engine's fixed order (faster); FedNL-PP runs in the fixed order
    int32_t arith = pp ? FEDNL_ORDER_FIXED : FEDNL_ORDER_REFERENCE;
    {
        std::string o;
        if (cl.str("gpu-arith-order", o)) {
            if (o == "fixed") arith = FEDNL_ORDER_FIXED;
            else if (o == "reference" && !pp) arith = FEDNL_ORDER_REFERENCE;
            else return -1;
        }
    }
    if (ls) {
        if (!num("c_line_search", ls_c) || !num("gamma_line_search", ls_gamma)) return -1;
        u32("max_line_search_steps", ls_max);
    }
    const bool opt_a = cl.flag("fednl-option-a"), opt_b = cl.flag("fednl-option-b");
    if (!opt_a && !opt_b) return -1;

    Dataset ds;
    std::string err;
    int rc = load_libsvm(path, add_intercept, ds, err);
    if (rc) return rc;
    if (n_clients < 1 || ds.n < n_clients) return -5;
    if (pp && per_round > n_clients) return -1;
    const int d = ds.d;
    const long long U = (long long)d * (d + 1) / 2;

    // compressor, k and alpha (TrainLoop.h:355-521)
    int comp;
    int32_t k = (int32_t)(kmult * d);
    if (comp_name == "identical") { comp = FEDNL_IDENTITY; k = (int32_t)U; }
    else if (comp_name == "natural") { comp = FEDNL_NATURAL; k = (int32_t)U; }
    else if (comp_name == "randk") comp = FEDNL_RANDK;
    else if (comp_name == "topk") comp = FEDNL_TOPK;
    else if (comp_name == "toplek") comp = FEDNL_TOPLEK;
    else if (comp_name == "seqk") comp = FEDNL_RANDSEQK;
    else return -2;
    if (theo) {
        if (comp == FEDNL_IDENTITY) alpha = 1.0 / (0.0 + 1.0);
        else if (comp == FEDNL_NATURAL) alpha = 1.0 / (1.0 / 8.0 + 1.0);
        else if (comp == FEDNL_RANDK || comp == FEDNL_RANDSEQK) {
            if (k > U) return -2;
            const double w = (double)U / k - 1.0;            // computeWForRandKMatrixOperator
            alpha = 1.0 / (w + 1.0);
        } else {
            if (k > U) return -2;
            const double delta = (double)k / ((double)d * (double)d);   // computeDeltaForTopKMatrixOpeator
            if (opt1) alpha = 1.0 - std::sqrt(1.0 - delta);
            else if (opt2) alpha = 1.0;
            else return -1;
        }
    }

    // even split, residual samples dropped, optional reshuffle (TrainLoop.h:188-250)
    const int per = ds.n / n_clients;
    std::vector<int32_t> order(ds.n);
    for (int i = 0; i < ds.n; ++i) order[i] = i;
    if (reshuffle) shuffle_all(order, reshuffle_seed);
    // 0/1 data goes up as the split's CSR rows (packed into the bit layout on the device), other
    // data as dense rows
    std::vector<double> feat, lab((size_t)per * n_clients);
    std::vector<int32_t> crp, ccols;
    if (ds.binary) {
        crp.assign(1, 0);
        for (int s = 0; s < per * n_clients; ++s) {
            const int o = order[s];
            ccols.insert(ccols.end(), ds.cols.begin() + ds.rp[o], ds.cols.begin() + ds.rp[o + 1]);
            crp.push_back((int32_t)ccols.size());
            lab[s] = ds.y[o];
        }
    } else {
        feat.resize((size_t)per * n_clients * d);
        for (int s = 0; s < per * n_clients; ++s) {
            std::memcpy(&feat[(size_t)s * d], &ds.x[(size_t)order[s] * d], (size_t)d * sizeof(double));
            lab[s] = ds.y[order[s]];
        }
    }
    std::vector<int32_t> ns(n_clients, per);

    fednl_problem_desc desc = {};
    desc.d = d;
    desc.lda = 0;
    desc.n_clients = n_clients;
    desc.n_samples = ns.data();
    desc.lambda = lambda;
    desc.compressor = comp;
    desc.k = k;
    desc.alpha = alpha;
    desc.workers = workers;
    desc.seed_base = 123;       // TrainLoop.h:632
    desc.toplek_seed = 1234;    // SpecialMathRoutinesForMatrix.h:383
    desc.option_a = opt_a ? 1 : 0;                          // Option A is tested first (TrainLoop.h:1383)
    desc.line_search = ls ? 1 : 0;
    desc.ls_c = ls_c;
    desc.ls_gamma = ls_gamma;
    desc.ls_max_steps = (int32_t)ls_max;
    desc.track_f = (tracking && !pp) ? 1 : 0;
    desc.clients_per_round = pp ? per_round : 0;
    desc.client_seed = 1234;    // bin_fednl_local_pp Args.h:244 (not taken from the command line)
    desc.arith_order = arith;
    fednl_handle h = nullptr;
    if (fednl_gpu_create(&desc, &h) != 0) return -7;
    // x0 from RandomGenRealLinear(0, 0): every coordinate is 0 whatever the seed (Args.h:235)
    std::vector<double> x0(d, 0.0), x(d), g(d);
    const int up = ds.binary ? fednl_gpu_upload_client_csr(h, crp.data(), ccols.empty() ? crp.data() : ccols.data(), lab.data())
                             : fednl_gpu_upload_client_data(h, feat.data(), lab.data());
    if (up != 0 || fednl_gpu_init_shifts(h, x0.data()) != 0) {
        fednl_gpu_destroy(h);
        return -7;
    }

    Tracker tr;
    if (tracking) {
        tr.cstr(base_name(path), true);
        std::string alg = pp ? "FedNL-PP" : "FedNL";
        if (ls) alg += "-LS";
        if (opt_a) alg += " (a)";
        if (opt_b) alg += " (b)";
        tr.cstr(alg, true);
        tr.cstr(comp_name, true);
        tr.i32(per);
        tr.i32(ds.n);
        tr.i32(rounds);
        tr.i32(n_clients);
        tr.i32(d);
        tr.i32(k);
        tr.f64(kmult);
        tr.f64(0.0);            // global step size: GD only
        tr.f64(alpha);
        tr.f64(lambda);
    }
    // bytes the clients send per round (indices only for the index-sending compressors)
    const double idx_bytes = (comp == FEDNL_TOPK || comp == FEDNL_TOPLEK) ? 4.0 : 0.0;
    double sent_scalars = 0.0, sent_indices = 0.0;
    const auto t0 = std::chrono::steady_clock::now();
    int status = 0;
    std::vector<int32_t> sel(n_clients);
    for (int r = 0; r < rounds; ++r) {
        fednl_gpu_get_x(h, x.data());
        double xn = 0.0;
        if (arith == FEDNL_ORDER_REFERENCE) xn = ref_norm2(x);
        else
            for (double v : x) xn += v * v;
        fednl_round_stats st{};
        const int rr = fednl_gpu_round(h, &st);
        if (rr != 0 && rr != FEDNL_ENOTPD) {
            status = -7;
            break;
        }
        double last_scalars = 0.0, last_idx = 0.0;
        int32_t nsel = n_clients;
        if (pp) fednl_gpu_get_selected(h, sel.data(), &nsel);
        for (int t = 0; t < nsel; ++t) {
            const int c = pp ? sel[t] : t;
            int32_t cnt = 0;
            fednl_gpu_get_message(h, c, nullptr, nullptr, &cnt);
            if (comp == FEDNL_NATURAL) last_scalars += 3.0 * ((cnt + 2) / 2);
            else last_scalars += 8.0 * cnt;
            last_scalars += 8.0 * d + 8.0 + (tracking || ls ? 8.0 : 0.0);   // gradient, Lk, f_i
            last_idx += idx_bytes * cnt;
        }
        if (tracking) {
            const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            tr.i32(r);
            tr.f64(st.grad_norm);
            tr.f64(pp ? NAN : fednl_gpu_get_f(h));       // FedNL-PP: f is not formed by the engine
            tr.f64(std::sqrt(xn));
            tr.f64(sent_scalars);
            tr.f64(sent_indices);
            tr.f64(secs);
        }
        sent_scalars += last_scalars;
        sent_indices += last_idx;
    }
    fednl_gpu_get_x(h, x.data());
    fednl_gpu_get_grad(h, g.data());
    fednl_gpu_destroy(h);
    if (status) return status;

    std::string outp = out_path;      // placeholders of TrainLoop.h:1820-1840
    const char* keys[4] = {"{run_id}", "{algorithm}", "{dataset}", "{kmultiplier}"};
    char kbuf[64];
    snprintf(kbuf, sizeof(kbuf), "%g", kmult);
    const std::string vals[4] = {"0", algorithm, base_name(path), kbuf};
    for (int i = 0; i < 4; ++i) {
        size_t p = outp.find(keys[i]);
        if (p != std::string::npos) outp.replace(p, strlen(keys[i]), vals[i]);
    }
    if (!outp.empty()) {
        FILE* f = fopen(outp.c_str(), "wb");
        if (!f) return -6;                                   // eResultSavingHasBeenFailed
        if (!tr.bytes.empty()) fwrite(tr.bytes.data(), 1, tr.bytes.size(), f);
        fclose(f);
    }
    if (pp) {
        if (cb_pp) cb_pp(d);                                 // bin_fednl_local_pp TrainLoop.h:1870-1871
        return 0;
    }
    double g2 = 0.0;
    if (arith == FEDNL_ORDER_REFERENCE) g2 = ref_norm2(g);
    else
        for (double v : g) g2 += v * v;
    const double mu = lambda;                                // computeMuStrongConvexity
    if (cb) cb(d, std::sqrt(g2), g2 / (mu + mu), (g2 + g2) / mu);
    return 0;
}

extern "C" int fednl_gpu_execute_local(const char* command, fednl_result_callback cb)
{
    return execute_local_impl(command, false, cb, nullptr);
}

// The reference's exported entry points (bin_fednl_local/exported/FedNLLocalShared.h:8-17 and
// bin_fednl_local_pp/exported/FedNLPPLocalShared.h:8-16), same names, signatures and return codes.
extern "C" int doptExecuteLocal(const char* command, ResultCallbackLocal resultCallback)
{
    return execute_local_impl(command, false, resultCallback, nullptr);
}

extern "C" int doptExecuteLocalPP(const char* command, ResultCallbackLocalPP resultCallback)
{
    return execute_local_impl(command, true, nullptr, resultCallback);
}
