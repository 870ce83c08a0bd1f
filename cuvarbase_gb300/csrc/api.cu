// C ABI of libcuvgls: handle, grid planner, workspace arena, batching.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <climits>
#include <chrono>
#include <map>
#include <tuple>
#include <string>
#include <thread>
#include <vector>

#include "../../include/cuvgls.h"
#include "kernels.cuh"

using namespace cuvgls;

static_assert(CUVGLS_MAX_CURVE_POINTS + cuvgls::kSegPoints <= 0x7fffffffLL,
              "segment arithmetic of a curve stays within int");
static_assert(sizeof(cuvgls_gridfin_curve) == 72, "cuvgls_gridfin_curve layout");
static_assert(sizeof(cuvgls_raw_curve) == 48 && sizeof(cuvgls_raw_input) == 72,
              "raw input layout");

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr size_t kAlign = 256;

size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

struct PlanKey {
    int G1, G2, B, R;
    double sigma;  // oversampling the window parameter is derived from
    int m;         // window half-width (cells)
    int win = kWinGauss;
};

// Autotuner candidates (window, sigma, m): each keeps max |dP| <= 2e-5
// against FP64 direct sums on the benchmark-shaped curves (the FP32 grid,
// FFT and finish included; measured 6e-6 for the Gaussians, 1.3e-5 for the
// ES window).  Lower sigma shrinks the FFT; for the Gaussian the larger m
// keeps its truncation error at the same level.  The ES window holds that
// accuracy at sigma 1.28 with 10 taps (the Gaussian needs 18 at sigma 1.6),
// so for every nf it gives the smallest grid and is chosen.
struct SigmaM {
    int win;
    double sigma;
    int m;
};
constexpr SigmaM kAutoCandidates[] = {{kWinGauss, 2.0, 8}, {kWinGauss, 1.75, 8},
                                      {kWinGauss, 1.6, 9}, {kWinGauss, 1.5, 10},
                                      {kWinES, 1.28, 5}};
// ES shape beta = gamma pi w (1 - 1 / (2 sigma)) for w = 2m taps (the
// published choice for upsampling factors below 2, gamma = 0.97).
constexpr double kEsGamma = 0.97;

struct ClassTables {
    float2 *d = nullptr;  // FFT table of G1 | of G2 | inter-pass twiddles
    Plan plan;
};

}  // namespace

struct cuvgls_handle {
    cuvgls_opts opts;
    std::string err;
    int device = 0;
    // workspace arena (grow-only)
    char *ws = nullptr;
    size_t ws_size = 0;
    // pinned staging of the per-curve descriptors
    DevCurve *h_cv = nullptr;
    size_t h_cv_cap = 0;
    cudaEvent_t h_cv_free = nullptr;  // recorded after the descriptor H2D
    unsigned *d_flags = nullptr;
    unsigned *h_flags = nullptr;  // page-locked copy of d_flags read by cuvgls_sync
    cudaStream_t copy_stream = nullptr;   // device-to-host copies of the outputs
    cudaStream_t in_stream = nullptr;     // second-phase host-to-device input copies
    cudaStream_t table_stream = nullptr;  // builds the tables of new plan classes
    cudaEvent_t done = nullptr;       // last enqueued work of this handle
    cudaStream_t last_stream = nullptr;
    bool have_last = false;
    std::vector<cudaEvent_t> chunk_events;
    // key (ngrids*64+m, G1*4096+G2, sigma): sigma sets the window parameter b
    std::map<std::tuple<int, int, double>, ClassTables> classes;
    std::map<long long, PlanKey> nf_plan;                // (ngrids*2^40+nf) -> plan
    std::map<long long, std::pair<int, int>> pins;      // GLS nf -> pinned (G1, G2)
    std::map<int, long long> nf_max;                     // ngrids -> largest nf with a plan
    // profiling
    long long smem_optin = kSmemLimit;  // device's opt-in shared memory per block
    bool prof_on = false;
    long long launches[CUVGLS_NSTAGES] = {0, 0, 0, 0, 0};
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> prof[CUVGLS_NSTAGES];
    std::vector<cudaEvent_t> ev_pool;
};

namespace {

int fail(cuvgls_handle *h, int code, const std::string &msg) {
    if (h) h->err = msg;
    return code;
}

int cuda_fail(cuvgls_handle *h, cudaError_t e, const char *what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return fail(h, CUVGLS_ENOMEM, m);
    return fail(h, CUVGLS_ECUDA, m);
}

#define CK(call, what)                                  \
    do {                                                \
        cudaError_t _e = (call);                        \
        if (_e != cudaSuccess) return cuda_fail(h, _e, what); \
    } while (0)

cudaEvent_t prof_event(cuvgls_handle *h) {
    if (!h->ev_pool.empty()) {
        cudaEvent_t e = h->ev_pool.back();
        h->ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Launch `call` on stream s, counting it under `stage` and, with profiling
// on, bracketing it with CUDA events.
#define LAUNCH(stage, s, call, what)                                   \
    do {                                                               \
        cudaEvent_t _a = nullptr, _b = nullptr;                        \
        if (h->prof_on) { _a = prof_event(h); cudaEventRecord(_a, s); } \
        cudaError_t _e = (call);                                       \
        if (_e != cudaSuccess) return cuda_fail(h, _e, what);          \
        if (h->prof_on) {                                              \
            _b = prof_event(h);                                        \
            cudaEventRecord(_b, s);                                    \
            h->prof[stage].push_back({_a, _b});                        \
        }                                                              \
        h->launches[stage]++;                                          \
    } while (0)

// ----- planner ---------------------------------------------------------------
// Choose (G1, G2) from the compiled lengths for nf frequencies: among the
// grids G = G1 G2 >= max(sigma nf, 256) whose tiles fit and that are at most
// 5 % above the smallest such G, the one of least measured cost
// G (kPass1PsPerCell[G1] + kPass2PsPerCell[G2]); shapes with a side below 64
// (a few long columns per curve or very short rows, slow in every
// measurement) only when nothing else fits.
// Per-length tile facts (columns B, rows R and shared memory of each pass
// for 1 and 3 grids), computed once: the planner runs for every new nf of a
// serving loop.
struct LenFacts {
    int B[2][kNumLens], R[2][kNumRowLens];
    long long s1[2][kNumLens], s2[2][kNumRowLens];
};
const LenFacts &len_facts() {
    static const LenFacts lf = [] {
        LenFacts f{};
        for (int g = 0; g < 2; ++g) {
            const int ngr = g ? 3 : 1;
            for (int i = 0; i < kNumLens; ++i) {
                f.B[g][i] = pass1_cols(ngr, kLens[i]);
                f.s1[g][i] = pass1_smem(ngr, kLens[i], 0);
            }
            for (int j = 0; j < kNumRowLens; ++j) {
                f.R[g][j] = pass2_rows(ngr, kRowLens[j]);
                f.s2[g][j] = pass2_smem(ngr, kRowLens[j]);
            }
        }
        return f;
    }();
    return lf;
}

struct Shape {
    int G1, G2, B, R;
    double cost;  // modelled ps per curve (measured per-cell costs)
};

// Grid shapes G1 x G2 >= max(sigma nf, 256) whose tiles fit, at most
// slack_pct % above the smallest such G, cheapest first by the measured
// costs G (kPass1PsPerCell[G1] + kPass2PsPerCell[G2]); shapes with a side
// below 64 (a few long columns per curve or very short rows, slow in every
// measurement) count four times their cost.
std::vector<Shape> plan_shapes(long long nf, double sigma, int m, int ng, long long smem_limit,
                               int slack_pct) {
    const LenFacts &lf = len_facts();
    const int gi = ng == 3 ? 1 : 0;
    long long Gmin = (long long)ceil(sigma * (double)nf);
    if (Gmin < 256) Gmin = 256;
    auto fits = [&](int i, int j) {
        const int G1 = kLens[i], G2 = kRowLens[j];
        const int B = lf.B[gi][i], R = lf.R[gi][j];
        if (G2 % B || G1 % R) return false;
        if (G2 < 2 * m + B || G2 / B > kMaxBins) return false;
        return lf.s1[gi][i] <= smem_limit && lf.s2[gi][j] <= smem_limit;
    };
    std::vector<Shape> out;
    long long gsmall = -1;
    for (int i = 0; i < kNumLens; ++i)
        for (int j = 0; j < kNumRowLens; ++j) {
            const long long G = (long long)kLens[i] * kRowLens[j];
            if (G < Gmin || (gsmall >= 0 && G >= gsmall)) continue;
            if (fits(i, j)) gsmall = G;
        }
    if (gsmall < 0) return out;
    for (int i = 0; i < kNumLens; ++i)
        for (int j = 0; j < kNumRowLens; ++j) {
            const int G1 = kLens[i], G2 = kRowLens[j];
            const long long G = (long long)G1 * G2;
            if (G < Gmin || G * 100 > gsmall * (100 + slack_pct) || !fits(i, j)) continue;
            double cost = (double)G * (kPass1PsPerCell[i] + kPass2PsPerCell[j]);
            if (G1 < 64 || G2 < 64) cost *= 4.0;
            out.push_back(Shape{G1, G2, lf.B[gi][i], lf.R[gi][j], cost});
        }
    std::stable_sort(out.begin(), out.end(),
                     [](const Shape &a, const Shape &b) { return a.cost < b.cost; });
    return out;
}

// Choose (G1, G2) from the compiled lengths for nf frequencies: among the
// grids that fit and are at most 5 % above the smallest, the one of least
// measured cost (plan_shapes).
bool choose_plan(long long nf, double sigma, int m, int ng, int &G1o, int &G2o,
                 int &Bo, int &Ro, long long smem_limit = kSmemLimit) {
    const std::vector<Shape> sh = plan_shapes(nf, sigma, m, ng, smem_limit, 5);
    if (sh.empty()) return false;
    G1o = sh[0].G1; G2o = sh[0].G2; Bo = sh[0].B; Ro = sh[0].R;
    return true;
}

// Whether the grid G1 x G2 fits a plan for nf frequencies (any size above
// sigma nf, for a shape pinned by the caller).
bool shape_fits(long long nf, double sigma, int m, int ng, int G1, int G2, long long smem_limit,
                int &Bo, int &Ro) {
    const LenFacts &lf = len_facts();
    const int gi = ng == 3 ? 1 : 0;
    int i = -1, j = -1;
    for (int a = 0; a < kNumLens; ++a) if (kLens[a] == G1) i = a;
    for (int b = 0; b < kNumRowLens; ++b) if (kRowLens[b] == G2) j = b;
    if (i < 0 || j < 0) return false;
    long long Gmin = (long long)ceil(sigma * (double)nf);
    if (Gmin < 256) Gmin = 256;
    const int B = lf.B[gi][i], R = lf.R[gi][j];
    if ((long long)G1 * G2 < Gmin || G2 % B || G1 % R) return false;
    if (G2 < 2 * m + B || G2 / B > kMaxBins) return false;
    if (lf.s1[gi][i] > smem_limit || lf.s2[gi][j] > smem_limit) return false;
    Bo = B; Ro = R;
    return true;
}

// Plan for nf: with opts.sigma > 0 the requested (sigma, m); with
// opts.sigma < 0 (autotune) the candidate giving the smallest grid, then the
// smallest m.
bool plan_default(const cuvgls_handle *h, long long nf, int ng, PlanKey &k) {
    if (h->opts.sigma > 0) {
        k.sigma = h->opts.sigma;
        k.m = h->opts.m;
        return choose_plan(nf, k.sigma, k.m, ng, k.G1, k.G2, k.B, k.R, h->smem_optin);
    }
    bool found = false;
    for (const SigmaM &c : kAutoCandidates) {
        PlanKey t{0, 0, 0, 0, c.sigma, c.m, c.win};
        if (!choose_plan(nf, c.sigma, c.m, ng, t.G1, t.G2, t.B, t.R, h->smem_optin)) continue;
        const long long G = (long long)t.G1 * t.G2, Gk = (long long)k.G1 * k.G2;
        if (!found || G < Gk || (G == Gk && t.m < k.m)) { k = t; found = true; }
    }
    return found;
}

// The plan of plan_default with the grid shape the caller pinned for GLS
// bands of exactly nf frequencies (cuvgls_plan_pin), when it still fits.
bool plan_for(const cuvgls_handle *h, long long nf, int ng, PlanKey &k) {
    if (!plan_default(h, nf, ng, k)) return false;
    if (ng == 3) {
        auto it = h->pins.find(nf);
        int B, R;
        if (it != h->pins.end() && shape_fits(nf, k.sigma, k.m, ng, it->second.first,
                                              it->second.second, h->smem_optin, B, R)) {
            k.G1 = it->second.first; k.G2 = it->second.second; k.B = B; k.R = R;
        }
    }
    return true;
}

// Largest nf that one grid plans for ng grids (plans grow with nf), found by
// bisection once per handle.
long long max_plan_nf(cuvgls_handle *h, int ng) {
    auto it = h->nf_max.find(ng);
    if (it != h->nf_max.end()) return it->second;
    PlanKey k{0, 0, 0, 0, 0.0, 0};
    long long lo = 0, hi = 1LL << 30;  // plan_for(lo) holds (or lo == 0), plan_for(hi) fails
    while (hi - lo > 1) {
        const long long mid = lo + (hi - lo) / 2;
        if (plan_default(h, mid, ng, k)) lo = mid;
        else hi = mid;
    }
    h->nf_max[ng] = lo;
    return lo;
}

// Sub-bands a band of nf frequencies is split into, and their width.
void band_split(long long nf, long long nf_max, long long &n_sub, long long &width) {
    n_sub = (nf <= nf_max || nf_max < 1) ? 1 : (nf + nf_max - 1) / nf_max;
    width = (nf + n_sub - 1) / n_sub;
}

// A curve whose band is wider than the largest grid becomes several curves:
// the same points and consecutive slices of the band (at most nf_max wide),
// each with its own centre kc and output offset.  The centring phase and the
// NFFT output phase are computed per descriptor, so nothing else changes.
void split_bands(cuvgls_handle *h, int ng, std::vector<DevCurve> &cvs,
                 std::vector<long long> &nfs) {
    const long long mx = max_plan_nf(h, ng);
    bool wide = false;
    for (long long nf : nfs) wide = wide || nf > mx;
    if (!wide || mx < 1) return;
    std::vector<DevCurve> oc;
    std::vector<long long> on;
    for (size_t i = 0; i < cvs.size(); ++i) {
        const long long nf = nfs[i];
        long long ns, w;
        band_split(nf, mx, ns, w);
        if (ns == 1) { oc.push_back(cvs[i]); on.push_back(nf); continue; }
        // kc = base + floor(nf / 2), base = k0 (GLS) or f0 / df (NFFT)
        const double base = cvs[i].kc - (double)(nf / 2);
        for (long long lo = 0; lo < nf; lo += w) {
            DevCurve d = cvs[i];
            const long long ws = std::min(w, nf - lo);
            d.nf = (int)ws;
            d.out_off += lo;
            d.best_off += (int)lo;
            d.kc = base + (double)lo + (double)(ws / 2);
            oc.push_back(d);
            on.push_back(ws);
        }
    }
    cvs.swap(oc);
    nfs.swap(on);
}

int get_class(cuvgls_handle *h, long long nf, int ng, ClassTables **out) {
    const long long key = ((long long)ng << 40) + nf;
    auto it = h->nf_plan.find(key);
    PlanKey pk{0, 0, 0, 0, 0.0, 0};
    if (it == h->nf_plan.end()) {
        if (!plan_for(h, nf, ng, pk))
            return fail(h, CUVGLS_ENOTSUP,
                        "no grid plan for nf=" + std::to_string(nf) +
                            " (largest supported grid is 2048 x 2048 cells)");
        h->nf_plan[key] = pk;
    } else {
        pk = it->second;
    }
    const int G1 = pk.G1, G2 = pk.G2, B = pk.B, R = pk.R;
    const long long G = (long long)G1 * G2;
    const std::tuple<int, int, double> ck(pk.win * 4096 + ng * 64 + pk.m, G1 * 4096 + G2,
                                          pk.sigma);
    auto ct = h->classes.find(ck);
    if (ct != h->classes.end()) { *out = &ct->second; return CUVGLS_OK; }
    ClassTables c;
    Plan &p = c.plan;
    memset(&p, 0, sizeof(p));
    p.G1 = G1; p.G2 = G2; p.G = G; p.m = pk.m; p.B = B; p.R = R;
    p.nb = G2 / B;
    const double sig = pk.sigma;
    p.win = pk.win;
    const double b = 2.0 * sig * p.m / ((2.0 * sig - 1.0) * kPi);
    p.binv = (float)(1.0 / b);
    p.dc1 = (float)(b * kPi * kPi / ((double)G * (double)G));
    p.dc2 = (float)(1.0 / sqrt(kPi * b));
    const double beta = kEsGamma * kPi * (2.0 * p.m) * (1.0 - 1.0 / (2.0 * sig));
    p.es_beta = (float)beta;
    p.es_im2 = (float)(1.0 / ((double)p.m * p.m));
    // tables (FFT tables of G1 and G2, inter-pass twiddles, and for the ES
    // window the deconvolution of |k'| <= G / 2) built on the device
    const size_t n1 = (size_t)fft_table_len(G1), n2 = (size_t)fft_table_len(G2);
    const size_t nd = p.win == kWinES ? (size_t)(G / 2 + 2) / 2 : 0;  // in float2 units
    CK(cudaMalloc(&c.d, (n1 + n2 + (size_t)G + nd) * sizeof(float2)), "cudaMalloc(plan tables)");
    // on a stream of their own: a new class waits neither for batches nor for
    // result copies in flight
    CK(launch_plan_tables(c.d, G1, G2, B, h->table_stream), "plan tables");
    if (p.win == kWinES)
        CK(launch_es_deconv((float *)(c.d + n1 + n2 + G), G, p.m, beta, h->table_stream),
           "deconvolution table");
    CK(cudaStreamSynchronize(h->table_stream), "plan tables");
    p.st1 = c.d;
    p.st2 = c.d + n1;
    p.itw = c.d + n1 + n2;
    p.dtab = p.win == kWinES ? (const float *)(c.d + n1 + n2 + G) : nullptr;
    auto ins = h->classes.emplace(ck, c);
    *out = &ins.first->second;
    return CUVGLS_OK;
}

// ----- workspace ---------------------------------------------------------------
int ensure_ws(cuvgls_handle *h, size_t need) {
    if (need <= h->ws_size) return CUVGLS_OK;
    if ((long long)need > h->opts.workspace_bytes)
        return fail(h, CUVGLS_EBUDGET,
                    "batch needs " + std::to_string(need) +
                        " workspace bytes, budget is " +
                        std::to_string(h->opts.workspace_bytes));
    if (h->ws) {
        CK(cudaDeviceSynchronize(), "sync before workspace growth");
        cudaFree(h->ws);
        h->ws = nullptr;
        h->ws_size = 0;
    }
    size_t sz = std::max(need, (size_t)64 << 20);
    sz = std::min(sz, (size_t)h->opts.workspace_bytes);
    CK(cudaMalloc(&h->ws, sz), "cudaMalloc(workspace)");
    h->ws_size = sz;
    return CUVGLS_OK;
}

int ensure_host_cv(cuvgls_handle *h, size_t n) {
    if (n <= h->h_cv_cap) {
        CK(cudaEventSynchronize(h->h_cv_free), "wait descriptor staging");
        return CUVGLS_OK;
    }
    if (h->h_cv) {
        CK(cudaEventSynchronize(h->h_cv_free), "wait descriptor staging");
        cudaFreeHost(h->h_cv);
        h->h_cv = nullptr;
    }
    size_t cap = std::max(n, (size_t)1024);
    CK(cudaMallocHost(&h->h_cv, cap * sizeof(DevCurve)), "cudaMallocHost(descriptors)");
    h->h_cv_cap = cap;
    return CUVGLS_OK;
}

int order_stream(cuvgls_handle *h, cudaStream_t s) {
    CK(cudaSetDevice(h->device), "cudaSetDevice");
    if (h->have_last && h->last_stream != s)
        CK(cudaStreamWaitEvent(s, h->done, 0), "order streams");
    h->last_stream = s;
    h->have_last = true;
    return CUVGLS_OK;
}

// A chunk: a run of curves of one class whose records and intermediates fit.
// A prep group: curves of one class whose records and bins are built by one
// prep launch; it holds the FFT chunks (intermediate buffers) run after it.
struct Chunk {
    int first, count;          // into the reordered descriptor table
};
struct Group {
    ClassTables *cls;
    int first, count;
    long long n_pts;
    size_t rec_bytes;          // records + bins of the group
    size_t inter_bytes;        // largest intermediate of its chunks
    std::vector<Chunk> chunks;
    // Its binning, in one part per input phase that holds its curves: the
    // descriptors [first, first + count) and their segments, [seg_b, seg_m)
    // single-segment descriptors, [seg_m, seg_e) segments of longer curves.
    struct Part {
        int first, count, seg_b, seg_m, seg_e;
    };
    std::vector<Part> parts;
};

// Shared driver of the GLS and NFFT batches.
struct Work {
    int ng;
    const double *t;
    const float *ya;
    const float *wv;
    long long n_points_total;
    long long n_out_total;   // elements of the output type
    size_t out_elem;         // bytes per output element
    int flags;
    // best-power mode (GLS): no powers are written; per curve of the
    // caller's batch, the index and value of the largest valid power
    int n_best = 0;
    int64_t *best_k = nullptr;
    float *best_p = nullptr;
    // raw input (GLS): t, y, dy in FP64; yw, w and the per-curve statistics
    // of n_raw curves are prepared on the device
    const double *ry = nullptr;
    const double *rdy = nullptr;
    int n_raw = 0;
};

int run_batch(cuvgls_handle *h, const Work &wk, std::vector<DevCurve> &cvs,
              std::vector<long long> &nfs, void *out, cudaStream_t s,
              int mode, float reg) {
    split_bands(h, wk.ng, cvs, nfs);
    if (cvs.size() > 0x7fffffffULL) return fail(h, CUVGLS_ENOTSUP, "too many sub-bands");
    const int nc = (int)cvs.size();
    if (nc == 0) return CUVGLS_OK;
    int rc = order_stream(h, s);
    if (rc) return rc;
    // classes and order
    std::vector<ClassTables *> cls(nc);
    for (int i = 0; i < nc; ++i) {
        rc = get_class(h, nfs[i], wk.ng, &cls[i]);
        if (rc) return rc;
    }
    std::vector<int> order(nc);
    for (int i = 0; i < nc; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return cls[a] < cls[b]; });
    // Preparation segments, in SegEntry tables copied with the descriptors,
    // both built per input phase once the groups are known.  Binning: per
    // group, the single-segment descriptors first (binned whole by
    // k_bin_scatter), then the segments of its longer curves (counted and
    // scanned first).  Raw input: the curves of one segment first (done whole
    // by k_raw_finish), then the segments of the longer ones (summed first);
    // every band of a curve refers to its curve's first entry.
    const bool raw = wk.ry != nullptr;
    long long nseg_bin = 0;
    for (int i = 0; i < nc; ++i) {
        nseg_bin += seg_count(cvs[i].n);
        cvs[i].flags = 0;
    }
    if (nseg_bin > 0x7fffffffLL) return fail(h, CUVGLS_ENOTSUP, "too many points");
    // (the raw table itself is built once the input phases are known)
    std::vector<int> bands;
    long long nseg_raw = 0;
    bool multi_band = false;
    if (raw) {
        bands.assign(wk.n_raw, 0);
        for (const DevCurve &cv : cvs) {
            if (++bands[cv.best_slot] > 1) multi_band = true;
            if (cv.best_off == 0) nseg_raw += seg_count(cv.n);
        }
    }
    // Budget: the arena holds the staged inputs / outputs, the descriptor and
    // segment tables ("fixed"), then the records and bins of one prep group, then the
    // intermediate of one FFT chunk (at most chunk_mb).  Preparing many
    // curves per launch keeps the prep kernel's grid deep.
    const size_t npts = (size_t)wk.n_points_total;
    const size_t in_bytes =
        raw ? ((wk.flags & CUVGLS_HOST_INPUT) ? 3 * align_up(npts * 8) : 0) + align_up(npts * 8) +
                  2 * align_up(npts * 4) + 2 * align_up(nseg_raw * sizeof(double4))
            : (wk.flags & CUVGLS_HOST_INPUT) ? align_up(npts * 8) + 2 * align_up(npts * 4) : 0;
    const bool best = wk.n_best > 0;
    const size_t out_bytes = !(wk.flags & CUVGLS_HOST_OUTPUT) ? 0
        : best ? align_up(wk.n_best * 8) + align_up(wk.n_best * 4)
               : align_up(wk.n_out_total * wk.out_elem);
    const size_t best_bytes = best ? align_up(wk.n_best * sizeof(unsigned long long)) : 0;
    // descriptors, then the binning and raw segment tables, in one copy
    const size_t tab_bytes = nc * sizeof(DevCurve) + (nseg_bin + nseg_raw) * sizeof(SegEntry);
    const size_t cv_bytes = align_up(tab_bytes);
    const size_t aux_bytes = align_up(nc * sizeof(float4));
    const size_t fixed = in_bytes + out_bytes + best_bytes + cv_bytes + aux_bytes + kAlign;
    // (8 alignment slots of slack are reserved for the arena's rounding)
    if ((long long)(fixed + 16 * kAlign) > h->opts.workspace_bytes)
        return fail(h, CUVGLS_EBUDGET, "batch inputs/outputs exceed the workspace budget");
    const size_t avail = (size_t)h->opts.workspace_bytes - fixed - 8 * kAlign;
    const size_t inter_budget = std::min(avail, (size_t)h->opts.chunk_mb << 20);
    std::vector<Group> groups;
    size_t max_group_bytes = 0;
    int first_chunk = 0;  // curves of the first FFT chunk before any split
    {
        int i = 0;
        while (i < nc) {
            ClassTables *c = cls[order[i]];
            const Plan &p = c->plan;
            const size_t inter1 = (size_t)wk.ng * p.G * sizeof(float2);
            // counts / offsets and cursors of both record kinds
            const size_t bins1 = align_up((size_t)4 * (p.nb + 1) * sizeof(int));
            Group g{c, i, 0, 0, 0, 0, {}};
            while (i < nc && cls[order[i]] == c) {
                // next FFT chunk: intermediates within inter_budget
                Chunk ch{i, 0};
                size_t ib = 0, rb = 0;
                while (i + ch.count < nc && cls[order[i + ch.count]] == c && ch.count < 65535) {
                    const DevCurve &cv = cvs[order[i + ch.count]];
                    const size_t radd = align_up((size_t)cv.n * (sizeof(RecAB) + sizeof(RecC))) + bins1;
                    if (ch.count > 0 && ib + inter1 > inter_budget) break;
                    // the group keeps its records for all of its chunks
                    if ((g.count > 0 || ch.count > 0) &&
                        g.rec_bytes + rb + radd + std::max(g.inter_bytes, ib + inter1) > avail)
                        break;
                    ib += inter1;
                    rb += radd;
                    ch.count++;
                }
                if (ch.count == 0) break;  // the group is full
                for (int k = 0; k < ch.count; ++k) g.n_pts += cvs[order[i + k]].n;
                g.rec_bytes += rb;
                g.inter_bytes = std::max(g.inter_bytes, ib);
                g.count += ch.count;
                g.chunks.push_back(ch);
                i += ch.count;
            }
            groups.push_back(g);
            max_group_bytes = std::max(max_group_bytes, g.rec_bytes + g.inter_bytes);
        }
        // With host output each chunk's powers are copied back while later
        // work runs; only the last chunk's copy has nothing to hide behind.
        // Split the last chunk into pieces of 1/2, 1/4, 1/8, 1/8 so that the
        // exposed copy is an eighth of a chunk.
        first_chunk = groups.empty() || groups[0].chunks.empty() ? 0
                                                                 : groups[0].chunks[0].count;
        if ((wk.flags & CUVGLS_HOST_OUTPUT) && !best && !groups.empty() &&
            !groups.back().chunks.empty() && groups.back().chunks.back().count >= 8) {
            std::vector<Chunk> &chs = groups.back().chunks;
            const Chunk last = chs.back();
            chs.pop_back();
            const int c = last.count;
            const int parts[4] = {c / 2, c / 4, c / 8, c - c / 2 - c / 4 - c / 8};
            int f = last.first;
            for (int q = 0; q < 4; ++q) {
                chs.push_back(Chunk{f, parts[q]});
                f += parts[q];
            }
        }
    }
    // Input phases.  With host input the points of each FFT chunk's curves
    // are a phase of their own: phase 0 is copied on the work stream, the
    // others in order on the input stream, and each chunk is prepared and
    // binned just before its passes, so the preparation of later chunks
    // never stalls the output copies (the host link, not the kernels, sets
    // the pace of a step with host output).  That needs the chunks' point
    // ranges to be disjoint and in order (true when the curves are given in
    // input order and each class's curves are contiguous); otherwise the
    // first chunk is phase 0 and the rest one more phase, or, when even
    // that does not split the input, a single phase.  Raw input with
    // sub-bands stays in one phase (a curve's preparation serves all of its
    // bands).  Phase k is the reordered descriptors [pb[k], pb[k + 1]) and
    // copies the point ranges prng[k].
    std::vector<int> pb{0, nc};
    std::vector<std::vector<std::pair<long long, long long>>> prng{{{0, (long long)npts}}};
    if ((wk.flags & CUVGLS_HOST_INPUT) && !multi_band && !groups.empty()) {
        auto span = [&](int a, int b) {  // point range of descriptors [a, b)
            long long lo = LLONG_MAX, hi = 0;
            for (int i = a; i < b; ++i) {
                const DevCurve &cv = cvs[order[i]];
                lo = std::min(lo, (long long)cv.pt_off);
                hi = std::max(hi, (long long)cv.pt_off + cv.n);
            }
            return std::make_pair(lo, hi);
        };
        std::vector<int> cut{0};
        for (const Group &g : groups)
            for (const Chunk &ch : g.chunks)
                if (ch.first > 0) cut.push_back(ch.first);
        cut.push_back(nc);
        bool ordered = cut.size() > 2;
        std::vector<std::pair<long long, long long>> r;
        long long end = 0;  // end of the ranges so far (phases without points skipped)
        for (size_t k = 0; ordered && k + 1 < cut.size(); ++k) {
            r.push_back(span(cut[k], cut[k + 1]));
            if (r[k].second <= r[k].first) continue;
            if (r[k].first < end) ordered = false;
            end = r[k].second;
        }
        if (ordered) {
            pb = cut;
            prng.clear();
            for (const auto &x : r) prng.push_back({x});
        } else if (groups[0].chunks.size() >= 2) {
            // the first chunk (all of its pieces), or the first piece when the
            // group was one chunk
            const int c0 = first_chunk < groups[0].count ? first_chunk
                                                         : groups[0].chunks[0].count;
            const auto x = span(0, c0);
            if (x.second - x.first < (long long)npts) {
                pb = {0, c0, nc};
                prng = {{x}, {{0, x.first}, {x.second, (long long)npts}}};
            }
        }
    }
    const int nph = (int)pb.size() - 1;
    // Raw segment table, per phase: the curves of one segment first (done
    // whole by k_raw_finish), then the segments of the longer ones (summed
    // first); every band of a curve refers to its curve's first entry.
    // raw_ph[ph] = {first entry, first multi-segment entry, end}.
    std::vector<SegEntry> raw_tab;
    std::vector<std::array<int, 3>> raw_ph(nph, std::array<int, 3>{0, 0, 0});
    bool need_fill = false;
    if (raw) {
        raw_tab.reserve((size_t)nseg_raw);
        std::vector<int> first(wk.n_raw, 0);
        for (int ph = 0; ph < nph; ++ph) {
            const int i0 = pb[ph], i1 = pb[ph + 1];
            raw_ph[ph][0] = (int)raw_tab.size();
            for (int pass = 0; pass < 2; ++pass) {
                if (pass == 1) raw_ph[ph][1] = (int)raw_tab.size();
                for (int i = i0; i < i1; ++i) {
                    DevCurve &cv = cvs[order[i]];
                    const int ns = seg_count(cv.n);
                    if (cv.best_off != 0 || (ns > 1) != (pass == 1)) continue;
                    first[cv.best_slot] = (int)raw_tab.size();
                    for (int k = 0; k < ns; ++k) raw_tab.push_back(SegEntry{i, k * kSegPoints});
                    if (pass == 0 && bands[cv.best_slot] == 1) cv.flags = kDescFillHere;
                }
            }
            raw_ph[ph][2] = (int)raw_tab.size();
        }
        for (DevCurve &cv : cvs) {
            cv.raw_seg = first[cv.best_slot];
            if (!(cv.flags & kDescFillHere)) need_fill = true;
        }
    }
    if ((int)h->chunk_events.size() < 3 + nph) {
        // two for alternating chunk copies, the start of the later phases'
        // input copies, then the end of each later phase's copies
        while ((int)h->chunk_events.size() < 3 + nph) {
            cudaEvent_t e;
            CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
            h->chunk_events.push_back(e);
        }
    }
    // arena layout
    size_t need = fixed + max_group_bytes + 8 * kAlign;
    rc = ensure_ws(h, need);
    if (rc) return rc;
    char *base = h->ws;
    size_t off = 0;
    auto take = [&](size_t bytes) { char *p = base + off; off += align_up(bytes); return p; };
    DevCurve *d_cv = (DevCurve *)take(tab_bytes);
    SegEntry *d_bseg = reinterpret_cast<SegEntry *>(d_cv + nc);
    SegEntry *d_rseg = d_bseg + nseg_bin;
    float4 *d_aux = (float4 *)take(nc * sizeof(float4));
    const double *t = wk.t;
    const float *ya = wk.ya, *wv = wk.wv;
    const double *ry = wk.ry, *rdy = wk.rdy;
    double4 *partA = nullptr, *partB = nullptr;
    double *d_ir = nullptr;  // dy^-2 of the raw points of longer curves
    // Host input: phase 0's points on the work stream, then each later
    // phase's on the input stream (not behind the output copies), ending
    // with its event.  Those start once phase 0's copies are done, so that
    // they never delay them, and so also after the work stream's earlier
    // work, which may still read this arena; phase k waits for its event.
    struct InCopy {
        char *dst;
        const char *src;
        size_t elem;
    };
    InCopy incs[3];
    int ninc = 0;
    auto copy_in = [&](void *dst, const void *src, size_t elem) {
        incs[ninc++] = InCopy{(char *)dst, (const char *)src, elem};
    };
    auto issue_in = [&]() -> cudaError_t {
        cudaError_t r = cudaSuccess;
        auto phase = [&](int ph, cudaStream_t st) {
            for (int k = 0; k < ninc && r == cudaSuccess; ++k) {
                const InCopy &c = incs[k];
                for (const auto &x : prng[ph]) {
                    const size_t a = (size_t)x.first * c.elem, b = (size_t)x.second * c.elem;
                    if (b > a && r == cudaSuccess)
                        r = cudaMemcpyAsync(c.dst + a, c.src + a, b - a, cudaMemcpyHostToDevice,
                                            st);
                }
            }
        };
        phase(0, s);
        if (nph == 1 || ninc == 0 || r != cudaSuccess) return r;
        // after phase 0's copies (and so after the work stream's earlier work)
        r = cudaEventRecord(h->chunk_events[2], s);
        if (r == cudaSuccess) r = cudaStreamWaitEvent(h->in_stream, h->chunk_events[2], 0);
        for (int ph = 1; ph < nph && r == cudaSuccess; ++ph) {
            phase(ph, h->in_stream);
            if (r == cudaSuccess) r = cudaEventRecord(h->chunk_events[2 + ph], h->in_stream);
        }
        return r;
    };
    if (raw) {
        if (wk.flags & CUVGLS_HOST_INPUT) {
            double *dt = (double *)take(npts * 8);
            double *dy = (double *)take(npts * 8);
            double *dd = (double *)take(npts * 8);
            copy_in(dt, wk.t, 8);
            copy_in(dy, wk.ry, 8);
            copy_in(dd, wk.rdy, 8);
            t = dt; ry = dy; rdy = dd;
        }
        ya = (const float *)take(npts * 4);
        wv = (const float *)take(npts * 4);
        d_ir = (double *)take(npts * 8);
        partA = (double4 *)take(nseg_raw * sizeof(double4));
        partB = (double4 *)take(nseg_raw * sizeof(double4));
    } else if (wk.flags & CUVGLS_HOST_INPUT) {
        double *dt = (double *)take(npts * 8);
        float *dy = (float *)take(npts * 4);
        float *dw = (float *)take(npts * 4);
        copy_in(dt, wk.t, 8);
        copy_in(dy, wk.ya, 4);
        if (wk.wv) copy_in(dw, wk.wv, 4);
        t = dt; ya = dy; wv = wk.wv ? dw : nullptr;
    }
    char *dev_out = (char *)out;
    unsigned long long *keys = nullptr;
    int64_t *bk = wk.best_k;
    float *bp = wk.best_p;
    if (best) {
        dev_out = nullptr;
        keys = (unsigned long long *)take(wk.n_best * sizeof(unsigned long long));
        CK(cudaMemsetAsync(keys, 0, wk.n_best * sizeof(unsigned long long), s), "zero keys");
        if (wk.flags & CUVGLS_HOST_OUTPUT) {
            bk = (int64_t *)take(wk.n_best * 8);
            bp = (float *)take(wk.n_best * 4);
        }
    } else if (wk.flags & CUVGLS_HOST_OUTPUT) {
        dev_out = take(wk.n_out_total * wk.out_elem);
    }
    char *group_base = base + off;
    // offsets: records and bins relative to the group, intermediates relative
    // to the chunk, in the reordered table
    rc = ensure_host_cv(h, (tab_bytes + sizeof(DevCurve) - 1) / sizeof(DevCurve));
    if (rc) return rc;
    SegEntry *h_bseg = reinterpret_cast<SegEntry *>(h->h_cv + nc);
    int sidx = 0;
    for (Group &g : groups) {
        const Plan &p = g.cls->plan;
        long long rec = 0;
        for (int k = 0; k < g.count; ++k) {
            DevCurve cv = cvs[order[g.first + k]];
            cv.rec_off = rec;
            cv.bin_off = (long long)k * (p.nb + 1);
            cv.aux = g.first + k;
            rec += cv.n;
            h->h_cv[g.first + k] = cv;
        }
        for (const Chunk &ch : g.chunks)
            for (int k = 0; k < ch.count; ++k)
                h->h_cv[ch.first + k].inter_off = (long long)k * wk.ng * p.G;
        // one binning part per input phase that holds curves of the group
        g.parts.clear();
        for (int ph = 0; ph < nph; ++ph) {
            const int k0 = std::max(pb[ph], g.first) - g.first;
            const int k1 = std::min(pb[ph + 1], g.first + g.count) - g.first;
            if (k1 <= k0) continue;
            Group::Part pt{g.first + k0, k1 - k0, sidx, 0, 0};
            for (int k = k0; k < k1; ++k)
                if (h->h_cv[g.first + k].n <= kSegPoints) h_bseg[sidx++] = SegEntry{g.first + k, 0};
            pt.seg_m = sidx;
            for (int k = k0; k < k1; ++k) {
                const int ns = seg_count(h->h_cv[g.first + k].n);
                if (ns > 1)
                    for (int q = 0; q < ns; ++q)
                        h_bseg[sidx++] = SegEntry{g.first + k, q * kSegPoints};
            }
            pt.seg_e = sidx;
            g.parts.push_back(pt);
        }
    }
    if (nseg_raw > 0)
        memcpy(h_bseg + nseg_bin, raw_tab.data(), nseg_raw * sizeof(SegEntry));
    CK(cudaMemcpyAsync(d_cv, h->h_cv, tab_bytes, cudaMemcpyHostToDevice, s),
       "H2D descriptors");
    CK(cudaEventRecord(h->h_cv_free, s), "record");
    // The input copies after the descriptor table: host-to-device copies of
    // all streams share the copy engine in the order they are issued, so a
    // table issued after the later phases' input would wait for all of it
    // (1.3 ms on the bench workload) before the first chunk could start.
    CK(issue_in(), "H2D input");
    const bool in_copies = ninc > 0 && nph > 1;  // later phases wait for their copies
    // weights, yw and statistics of one phase's raw curves on the device,
    // then the descriptors' normalisation from them
    auto prep_raw = [&](int ph) -> int {
        const int b = raw_ph[ph][0], m = raw_ph[ph][1], e = raw_ph[ph][2];
        if (m < e)
            LAUNCH(CUVGLS_STAGE_PREP, s,
                   launch_raw_sums(d_rseg + m, e - m, d_cv, ry, rdy, d_ir, partA, s),
                   "k_raw_sums");
        if (b < e)
            LAUNCH(CUVGLS_STAGE_PREP, s,
                   launch_raw_finish(d_rseg + b, e - b, d_cv, ry, rdy, d_ir, (float *)ya,
                                     (float *)wv, partA, partB, mode, s),
                   "k_raw_finish");
        const int c0 = pb[ph], c1 = pb[ph + 1];
        if (need_fill && c1 > c0)
            LAUNCH(CUVGLS_STAGE_PREP, s,
                   launch_fill_desc(d_cv + c0, c1 - c0, partA, partB, mode, s), "k_fill_desc");
        return CUVGLS_OK;
    };
    // the phases up to the one of descriptor `first`, before its first
    // work: their input copied, their raw curves prepared
    int cur_ph = 0;
    auto reach = [&](int first) -> int {
        while (cur_ph + 1 < nph && pb[cur_ph + 1] <= first) {
            ++cur_ph;
            if (in_copies)
                CK(cudaStreamWaitEvent(s, h->chunk_events[2 + cur_ph], 0), "wait input");
            if (raw) {
                const int r = prep_raw(cur_ph);
                if (r) return r;
            }
        }
        return CUVGLS_OK;
    };
    if (raw) {
        rc = prep_raw(0);
        if (rc) return rc;
    }
    int evi = 0;
    for (const Group &g : groups) {
        const Plan &p = g.cls->plan;
        size_t o2 = 0;
        auto gtake = [&](size_t bytes) { char *q = group_base + o2; o2 += align_up(bytes); return q; };
        RecAB *recAB = (RecAB *)gtake(g.n_pts * sizeof(RecAB));
        RecC *recC = (RecC *)gtake(g.n_pts * sizeof(RecC));
        const size_t nbin = (size_t)g.count * (p.nb + 1);
        int *binsAB = (int *)gtake(4 * nbin * sizeof(int));
        int *binsC = binsAB + nbin, *curAB = binsC + nbin, *curC = curAB + nbin;
        float2 *inter = (float2 *)gtake(g.inter_bytes);
        const int fp32 = h->opts.precision == CUVGLS_PREC_FP32;
        float4 *gaux = wk.ng == 1 ? d_aux : nullptr;
        bool multi = false;  // curves longer than one segment
        for (const Group::Part &pt : g.parts) multi = multi || pt.seg_e > pt.seg_m;
        if (multi) CK(cudaMemsetAsync(binsAB, 0, 2 * nbin * sizeof(int), s), "zero bins");
        auto bin_part = [&](const Group::Part &pt) -> int {
            if (pt.seg_e > pt.seg_m) {
                LAUNCH(CUVGLS_STAGE_PREP, s,
                       launch_bin_count(d_bseg + pt.seg_m, pt.seg_e - pt.seg_m, d_cv, t, binsAB,
                                        binsC, p, wk.ng, fp32, s),
                       "k_bin_count");
                LAUNCH(CUVGLS_STAGE_PREP, s,
                       launch_bin_scan(d_cv + pt.first, pt.count, t, binsAB, binsC, curAB, curC,
                                       gaux, p, wk.ng, s),
                       "k_bin_scan");
            }
            LAUNCH(CUVGLS_STAGE_PREP, s,
                   launch_bin_scatter(d_bseg + pt.seg_b, pt.seg_e - pt.seg_b, d_cv, t, ya, wv,
                                      recAB, recC, binsAB, binsC, curAB, curC, gaux, p, wk.ng,
                                      fp32, h->d_flags, s),
                   "k_bin_scatter");
            return CUVGLS_OK;
        };
        size_t pi = 0;  // next binning part (each starts at a chunk)
        for (const Chunk &ch : g.chunks) {
            while (pi < g.parts.size() && g.parts[pi].first < ch.first + ch.count) {
                rc = reach(g.parts[pi].first);
                if (!rc) rc = bin_part(g.parts[pi]);
                if (rc) return rc;
                ++pi;
            }
            const DevCurve *dcv = d_cv + ch.first;
            LAUNCH(CUVGLS_STAGE_PASS1, s,
                   launch_pass1(dcv, ch.count, recAB, recC, binsAB, binsC, inter, p, wk.ng, s),
                   "k_pass1");
            // With host output, pass 2 runs in four launches over consecutive
            // curves, each followed by the copy of its powers: the copy stream
            // is nearly as long as the compute, and copying in quarter chunks
            // keeps it from falling a whole chunk behind.
            const bool hcopy = (wk.flags & CUVGLS_HOST_OUTPUT) && !best;
            const int nsub = hcopy && ch.count >= 64 ? 4 : 1;
            for (int q = 0; q < nsub; ++q) {
                const int a = (int)((long long)ch.count * q / nsub);
                const int e = (int)((long long)ch.count * (q + 1) / nsub);
                const DevCurve *dq = dcv + a;
                if (wk.ng == 3) {
                    GlsParams gp{mode, reg, keys};
                    LAUNCH(CUVGLS_STAGE_PASS2, s,
                           launch_pass2_gls(dq, e - a, inter, (float *)dev_out, p, gp, s),
                           "k_pass2_gls");
                } else {
                    LAUNCH(CUVGLS_STAGE_PASS2, s,
                           launch_pass2_nfft(dq, e - a, inter, (float2 *)dev_out, d_aux, p, s),
                           "k_pass2_nfft");
                }
                if (!hcopy) continue;
                // copy these curves' outputs on the copy stream while later work runs
                cudaEvent_t ev = h->chunk_events[evi];
                evi ^= 1;
                CK(cudaEventRecord(ev, s), "record chunk");
                CK(cudaStreamWaitEvent(h->copy_stream, ev, 0), "wait chunk");
                std::vector<std::pair<long long, long long>> rng;
                for (int k = ch.first + a; k < ch.first + e; ++k) {
                    const DevCurve &cv = h->h_cv[k];
                    rng.push_back({cv.out_off, cv.out_off + cv.nf});
                }
                std::sort(rng.begin(), rng.end());
                long long x0 = rng[0].first, x1 = rng[0].second;
                auto flush = [&](long long x, long long y) -> cudaError_t {
                    return cudaMemcpyAsync((char *)out + x * wk.out_elem,
                                           dev_out + x * wk.out_elem, (y - x) * wk.out_elem,
                                           cudaMemcpyDeviceToHost, h->copy_stream);
                };
                for (size_t r = 1; r < rng.size(); ++r) {
                    if (rng[r].first <= x1) { x1 = std::max(x1, rng[r].second); continue; }
                    CK(flush(x0, x1), "D2H out");
                    x0 = rng[r].first; x1 = rng[r].second;
                }
                CK(flush(x0, x1), "D2H out");
            }
        }
    }
    if (best) {
        CK(launch_best_finish(keys, wk.n_best, bk, bp, s), "best finish");
        if (wk.flags & CUVGLS_HOST_OUTPUT) {
            CK(cudaMemcpyAsync(wk.best_k, bk, wk.n_best * 8, cudaMemcpyDeviceToHost, s),
               "D2H best index");
            CK(cudaMemcpyAsync(wk.best_p, bp, wk.n_best * 4, cudaMemcpyDeviceToHost, s),
               "D2H best power");
        }
    } else if (wk.flags & CUVGLS_HOST_OUTPUT) {
        CK(cudaEventRecord(h->chunk_events[evi], h->copy_stream), "record copies");
        CK(cudaStreamWaitEvent(s, h->chunk_events[evi], 0), "join copies");
    }
    CK(cudaEventRecord(h->done, s), "record done");
    return CUVGLS_OK;
}

bool is_fin(double x) { return isfinite(x) != 0; }

}  // namespace

// ============================================================================
extern "C" {

int cuvgls_version(void) { return CUVGLS_VERSION; }

int cuvgls_create(cuvgls_handle **out, const cuvgls_opts *opts) {
    if (!out) return CUVGLS_EINVAL;
    *out = nullptr;
    cuvgls_opts o;
    o.sigma = 2.0; o.m = 8; o.device = 0; o.workspace_bytes = 16LL << 30;
    o.precision = CUVGLS_PREC_MIXED; o.chunk_mb = 0;
    if (opts) {
        o = *opts;
        if (o.sigma == 0) o.sigma = 2.0;
        if (o.m == 0) o.m = 8;
        if (o.workspace_bytes == 0) o.workspace_bytes = 16LL << 30;
        if (o.chunk_mb == 0) o.chunk_mb = 4096;
    } else {
        o.chunk_mb = 4096;
    }
    if (!((o.sigma >= 1.25 && o.sigma <= 16.0) || o.sigma < 0) || o.m < 2 || o.m > 16 ||
        o.workspace_bytes < (16LL << 20) ||
        (o.precision != CUVGLS_PREC_MIXED && o.precision != CUVGLS_PREC_FP32) ||
        o.chunk_mb < 1)
        return CUVGLS_EINVAL;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || o.device < 0 || o.device >= ndev)
        return CUVGLS_ECUDA;
    cuvgls_handle *h = new cuvgls_handle();
    h->opts = o;
    h->device = o.device;
    {
        int optin = 0;
        if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, o.device) ==
                cudaSuccess && optin > 0)
            h->smem_optin = std::min<long long>(optin, kSmemLimit);
    }
    if (cudaSetDevice(o.device) != cudaSuccess ||
        cudaMalloc(&h->d_flags, sizeof(unsigned)) != cudaSuccess ||
        cudaMemset(h->d_flags, 0, sizeof(unsigned)) != cudaSuccess ||
        cudaMallocHost(&h->h_flags, sizeof(unsigned)) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->in_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->table_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->done, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->h_cv_free, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventRecord(h->h_cv_free, 0) != cudaSuccess) {
        cuvgls_destroy(h);
        return CUVGLS_ECUDA;
    }
    *out = h;
    return CUVGLS_OK;
}

int cuvgls_destroy(cuvgls_handle *h) {
    if (!h) return CUVGLS_EINVAL;
    cudaSetDevice(h->device);
    cudaDeviceSynchronize();
    for (auto &kv : h->classes) cudaFree(kv.second.d);
    if (h->ws) cudaFree(h->ws);
    if (h->h_cv) cudaFreeHost(h->h_cv);
    if (h->d_flags) cudaFree(h->d_flags);
    if (h->h_flags) cudaFreeHost(h->h_flags);
    for (auto e : h->chunk_events) cudaEventDestroy(e);
    for (int st = 0; st < CUVGLS_NSTAGES; ++st)
        for (auto &pr : h->prof[st]) { cudaEventDestroy(pr.first); cudaEventDestroy(pr.second); }
    for (auto e : h->ev_pool) cudaEventDestroy(e);
    if (h->done) cudaEventDestroy(h->done);
    if (h->h_cv_free) cudaEventDestroy(h->h_cv_free);
    if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
    if (h->in_stream) cudaStreamDestroy(h->in_stream);
    if (h->table_stream) cudaStreamDestroy(h->table_stream);
    delete h;
    return CUVGLS_OK;
}

const char *cuvgls_last_error(cuvgls_handle *h) { return h ? h->err.c_str() : "null handle"; }

static int check_gls_batch(cuvgls_handle *h, const cuvgls_gls_input *b, const void *p_out,
                           bool outputs = true) {
    if (!h) return CUVGLS_EINVAL;
    h->err.clear();
    if (!b || b->n_curves < 0) return fail(h, CUVGLS_EINVAL, "null batch or negative n_curves");
    if (b->n_curves == 0) return CUVGLS_OK;
    if (!b->curves || !b->t || !b->yw || !b->w || !p_out)
        return fail(h, CUVGLS_EINVAL, "null pointer in batch");
    if (b->mode < 0 || b->mode > 2) return fail(h, CUVGLS_EINVAL, "mode must be 0, 1 or 2");
    if (b->reg[0] != b->reg[1] || b->reg[2] != 0.f || !(b->reg[0] >= 0.f))
        return fail(h, CUVGLS_EINVAL,
                    "reg must be (lambda, lambda, 0) with lambda >= 0, as "
                    "LombScargleMemory builds it");
    for (int i = 0; i < b->n_curves; ++i) {
        const cuvgls_curve &c = b->curves[i];
        if (c.n < 1 || c.nf < 1 || c.pt_off < 0 || c.out_off < 0)
            return fail(h, CUVGLS_EINVAL, "curve " + std::to_string(i) + ": empty or negative size");
        if (c.pt_off + c.n > b->n_points_total ||
            (outputs && c.out_off + c.nf > b->n_out_total))
            return fail(h, CUVGLS_EINVAL, "curve " + std::to_string(i) + ": range outside arrays");
        if (c.n > CUVGLS_MAX_CURVE_POINTS || c.nf > 0x7fffffffLL)
            return fail(h, CUVGLS_ENOTSUP, "curve " + std::to_string(i) + ": n or nf too large");
        // Non-finite YY / means are allowed: as in the reference, such a
        // curve yields invalid powers (-1) rather than an error.
        if (!(c.df > 0) || !is_fin(c.df))
            return fail(h, CUVGLS_EINVAL, "curve " + std::to_string(i) + ": df must be finite and > 0");
    }
    return CUVGLS_OK;
}

static void fill_gls_curves(const cuvgls_gls_input *b, std::vector<DevCurve> &cvs,
                            std::vector<long long> &nfs) {
    cvs.resize(b->n_curves);
    nfs.resize(b->n_curves);
    for (int i = 0; i < b->n_curves; ++i) {
        const cuvgls_curve &c = b->curves[i];
        DevCurve d;
        memset(&d, 0, sizeof(d));
        d.pt_off = c.pt_off; d.out_off = c.out_off;
        d.kc = (double)(c.k0 + c.nf / 2);
        d.n = (int)c.n; d.nf = (int)c.nf; d.df = c.df;
        double norm = 1.0;
        if (b->mode == 1) norm = 1.0 / c.yy;
        else if (b->mode == 0) norm = 1.0 / (c.yy + c.ybar * c.ybar);
        d.yy_inv = (float)norm;
        d.ybar = (float)c.ybar;
        d.yw_sum = (float)c.yw_sum;
        d.w_sum = (float)c.w_sum;
        d.best_slot = i;
        d.best_off = 0;
        cvs[i] = d;
        nfs[i] = c.nf;
    }
}

int cuvgls_gls_batch(cuvgls_handle *h, const cuvgls_gls_input *b, float *p_out,
                     void *stream) {
    int rc = check_gls_batch(h, b, p_out);
    if (rc || b->n_curves == 0) return rc;
    std::vector<DevCurve> cvs;
    std::vector<long long> nfs;
    fill_gls_curves(b, cvs, nfs);
    Work wk{3, b->t, b->yw, b->w, b->n_points_total, b->n_out_total, sizeof(float), b->flags};
    return run_batch(h, wk, cvs, nfs, p_out, (cudaStream_t)stream, b->mode, b->reg[0]);
}

int cuvgls_gls_best(cuvgls_handle *h, const cuvgls_gls_input *b, int64_t *best_k,
                    float *best_p, void *stream) {
    if (!best_k || !best_p) return h ? fail(h, CUVGLS_EINVAL, "null best output") : CUVGLS_EINVAL;
    int rc = check_gls_batch(h, b, best_k, false);
    if (rc || b->n_curves == 0) return rc;
    std::vector<DevCurve> cvs;
    std::vector<long long> nfs;
    fill_gls_curves(b, cvs, nfs);
    Work wk{3, b->t, b->yw, b->w, b->n_points_total, 0, sizeof(float), b->flags};
    wk.n_best = b->n_curves;
    wk.best_k = best_k;
    wk.best_p = best_p;
    return run_batch(h, wk, cvs, nfs, nullptr, (cudaStream_t)stream, b->mode, b->reg[0]);
}

int cuvgls_gls_raw(cuvgls_handle *h, const cuvgls_raw_input *b, float *p_out,
                   int64_t *best_k, float *best_p, void *stream) {
    if (!h) return CUVGLS_EINVAL;
    h->err.clear();
    if (!b || b->n_curves < 0) return fail(h, CUVGLS_EINVAL, "null batch or negative n_curves");
    if (b->n_curves == 0) return CUVGLS_OK;
    const bool best = best_k != nullptr || best_p != nullptr;
    if (best == (p_out != nullptr) || (best && (!best_k || !best_p)))
        return fail(h, CUVGLS_EINVAL, "give p_out, or best_k and best_p");
    if (!b->curves || !b->t || !b->y || !b->dy)
        return fail(h, CUVGLS_EINVAL, "null pointer in batch");
    if (b->mode < 0 || b->mode > 2) return fail(h, CUVGLS_EINVAL, "mode must be 0, 1 or 2");
    if (b->reg[0] != b->reg[1] || b->reg[2] != 0.f || !(b->reg[0] >= 0.f))
        return fail(h, CUVGLS_EINVAL, "reg must be (lambda, lambda, 0) with lambda >= 0");
    std::vector<DevCurve> cvs(b->n_curves);
    std::vector<long long> nfs(b->n_curves);
    for (int i = 0; i < b->n_curves; ++i) {
        const cuvgls_raw_curve &c = b->curves[i];
        if (c.n < 1 || c.nf < 1 || c.pt_off < 0 || c.out_off < 0 || c.k0 < 0 ||
            c.pt_off + c.n > b->n_points_total ||
            (!best && c.out_off + c.nf > b->n_out_total))
            return fail(h, CUVGLS_EINVAL, "curve " + std::to_string(i) + ": bad range");
        if (c.n > CUVGLS_MAX_CURVE_POINTS || c.nf > 0x7fffffffLL)
            return fail(h, CUVGLS_ENOTSUP, "curve " + std::to_string(i) + ": n or nf too large");
        if (!(c.df > 0) || !is_fin(c.df))
            return fail(h, CUVGLS_EINVAL, "curve " + std::to_string(i) + ": df must be finite and > 0");
        DevCurve d;
        memset(&d, 0, sizeof(d));
        d.pt_off = c.pt_off; d.out_off = c.out_off;
        d.kc = (double)(c.k0 + c.nf / 2);
        d.n = (int)c.n; d.nf = (int)c.nf; d.df = c.df;
        d.best_slot = i;
        d.best_off = 0;   // yy_inv, ybar, yw_sum, w_sum come from the device
        cvs[i] = d;
        nfs[i] = c.nf;
    }
    Work wk{3, b->t, nullptr, nullptr, b->n_points_total, best ? 0 : b->n_out_total,
            sizeof(float), b->flags};
    wk.ry = b->y;
    wk.rdy = b->dy;
    wk.n_raw = b->n_curves;
    if (best) {
        wk.n_best = b->n_curves;
        wk.best_k = best_k;
        wk.best_p = best_p;
    }
    return run_batch(h, wk, cvs, nfs, p_out, (cudaStream_t)stream, b->mode, b->reg[0]);
}

// ---- captured plans ---------------------------------------------------------
struct cuvgls_gls_plan {
    cuvgls_handle *h = nullptr;   // private: its arena, tables and staged
                                  // descriptors belong to the graph
    void *stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

int cuvgls_gls_plan_destroy(cuvgls_gls_plan *pl) {
    if (!pl) return CUVGLS_EINVAL;
    if (pl->stream) cudaStreamSynchronize((cudaStream_t)pl->stream);
    if (pl->exec) cudaGraphExecDestroy(pl->exec);
    if (pl->graph) cudaGraphDestroy(pl->graph);
    if (pl->stream) cuvgls_stream_destroy(pl->stream);
    if (pl->h) cuvgls_destroy(pl->h);
    delete pl;
    return CUVGLS_OK;
}

int cuvgls_gls_plan_create(cuvgls_handle *h0, const cuvgls_raw_input *b, float *p_out,
                           int64_t *best_k, float *best_p, cuvgls_gls_plan **out) {
    if (!h0 || !out) return CUVGLS_EINVAL;
    *out = nullptr;
    h0->err.clear();
    if (!b || b->n_curves < 1) return fail(h0, CUVGLS_EINVAL, "a plan needs at least one curve");
    if (b->flags != 0)
        return fail(h0, CUVGLS_EINVAL, "a plan takes device pointers only (flags 0)");
    cuvgls_gls_plan *pl = new cuvgls_gls_plan();
    int rc = cuvgls_create(&pl->h, &h0->opts);
    if (rc == CUVGLS_OK) rc = cuvgls_stream_create(&pl->stream);
    // a first, ordinary run allocates the arena, builds the plan tables and
    // stages the descriptors; the second run, captured, launches only
    if (rc == CUVGLS_OK) rc = cuvgls_gls_raw(pl->h, b, p_out, best_k, best_p, pl->stream);
    if (rc == CUVGLS_OK && cudaStreamSynchronize((cudaStream_t)pl->stream) != cudaSuccess)
        rc = CUVGLS_ECUDA;
    if (rc == CUVGLS_OK) {
        cudaStream_t cs = (cudaStream_t)pl->stream;
        if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
            rc = CUVGLS_ECUDA;
        } else {
            rc = cuvgls_gls_raw(pl->h, b, p_out, best_k, best_p, pl->stream);
            const cudaError_t e = cudaStreamEndCapture(cs, &pl->graph);
            if (rc == CUVGLS_OK && e != cudaSuccess) rc = CUVGLS_ECUDA;
        }
    }
    if (rc == CUVGLS_OK && cudaGraphInstantiate(&pl->exec, pl->graph, 0) != cudaSuccess)
        rc = CUVGLS_ECUDA;
    if (rc) {
        if (pl->h && !pl->h->err.empty()) h0->err = pl->h->err;
        else h0->err = "plan capture failed";
        cudaGetLastError();
        cuvgls_gls_plan_destroy(pl);
        return rc;
    }
    *out = pl;
    return CUVGLS_OK;
}

int cuvgls_gls_plan_launch(cuvgls_gls_plan *pl, void *stream) {
    if (!pl || !pl->exec) return CUVGLS_EINVAL;
    return cudaGraphLaunch(pl->exec, (cudaStream_t)stream) == cudaSuccess ? CUVGLS_OK
                                                                           : CUVGLS_ECUDA;
}

int cuvgls_gls_direct_batch(cuvgls_handle *h, const cuvgls_gls_input *b,
                            float *p_out, void *stream) {
    int rc = check_gls_batch(h, b, p_out);
    if (rc || b->n_curves == 0) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    rc = order_stream(h, s);
    if (rc) return rc;
    std::vector<DevCurve> cvs;
    std::vector<long long> nfs;
    fill_gls_curves(b, cvs, nfs);
    const int nc = b->n_curves;
    const bool hin = b->flags & CUVGLS_HOST_INPUT, hout = b->flags & CUVGLS_HOST_OUTPUT;
    size_t need = align_up(nc * sizeof(DevCurve)) + kAlign;
    if (hin) need += align_up(b->n_points_total * 8) + 2 * align_up(b->n_points_total * 4);
    if (hout) need += align_up(b->n_out_total * 4);
    rc = ensure_ws(h, need);
    if (rc) return rc;
    rc = ensure_host_cv(h, nc);
    if (rc) return rc;
    char *base = h->ws;
    size_t off = 0;
    auto take = [&](size_t bytes) { char *p = base + off; off += align_up(bytes); return p; };
    DevCurve *d_cv = (DevCurve *)take(nc * sizeof(DevCurve));
    const double *t = b->t;
    const float *yw = b->yw, *w = b->w;
    if (hin) {
        double *dt = (double *)take(b->n_points_total * 8);
        float *dy = (float *)take(b->n_points_total * 4);
        float *dw = (float *)take(b->n_points_total * 4);
        CK(cudaMemcpyAsync(dt, b->t, b->n_points_total * 8, cudaMemcpyHostToDevice, s), "H2D t");
        CK(cudaMemcpyAsync(dy, b->yw, b->n_points_total * 4, cudaMemcpyHostToDevice, s), "H2D yw");
        CK(cudaMemcpyAsync(dw, b->w, b->n_points_total * 4, cudaMemcpyHostToDevice, s), "H2D w");
        t = dt; yw = dy; w = dw;
    }
    float *dout = hout ? (float *)take(b->n_out_total * 4) : p_out;
    int max_nf = 0;
    for (int i = 0; i < nc; ++i) { h->h_cv[i] = cvs[i]; max_nf = std::max(max_nf, cvs[i].nf); }
    CK(cudaMemcpyAsync(d_cv, h->h_cv, nc * sizeof(DevCurve), cudaMemcpyHostToDevice, s),
       "H2D descriptors");
    CK(cudaEventRecord(h->h_cv_free, s), "record");
    GlsParams g{b->mode, b->reg[0]};
    for (int c0 = 0; c0 < nc; c0 += 65535) {
        int cnt = std::min(65535, nc - c0);
        LAUNCH(CUVGLS_STAGE_DIRECT, s,
               launch_gls_direct(d_cv + c0, cnt, max_nf, t, yw, w, dout, g, s), "k_gls_direct");
    }
    if (hout)
        CK(cudaMemcpyAsync(p_out, dout, b->n_out_total * 4, cudaMemcpyDeviceToHost, s), "D2H");
    CK(cudaEventRecord(h->done, s), "record done");
    return CUVGLS_OK;
}

int cuvgls_nfft_adjoint_batch(cuvgls_handle *h, const cuvgls_nfft_input *b,
                              float *out, void *stream) {
    if (!h) return CUVGLS_EINVAL;
    h->err.clear();
    if (!b || b->n_curves < 0) return fail(h, CUVGLS_EINVAL, "null batch");
    if (b->n_curves == 0) return CUVGLS_OK;
    if (!b->curves || !b->t || !b->y || !out) return fail(h, CUVGLS_EINVAL, "null pointer");
    std::vector<DevCurve> cvs(b->n_curves);
    std::vector<long long> nfs(b->n_curves);
    for (int i = 0; i < b->n_curves; ++i) {
        const cuvgls_nfft_curve &c = b->curves[i];
        if (c.n < 1 || c.nf < 1 || c.pt_off < 0 || c.out_off < 0 ||
            c.pt_off + c.n > b->n_points_total || c.out_off + c.nf > b->n_out_total)
            return fail(h, CUVGLS_EINVAL, "curve " + std::to_string(i) + ": bad range");
        if (c.nf > 0x7fffffffLL || c.n > CUVGLS_MAX_CURVE_POINTS)
            return fail(h, CUVGLS_ENOTSUP, "curve " + std::to_string(i) + ": n or nf too large");
        if (!(c.df > 0) || !is_fin(c.df) || !is_fin(c.f0) || !is_fin(c.f0 / c.df))
            return fail(h, CUVGLS_EINVAL, "curve " + std::to_string(i) + ": df must be > 0, f0 finite");
        DevCurve d;
        memset(&d, 0, sizeof(d));
        d.pt_off = c.pt_off; d.out_off = c.out_off;
        d.kc = c.f0 / c.df + (double)(c.nf / 2);
        d.n = (int)c.n; d.nf = (int)c.nf; d.df = c.df;
        cvs[i] = d;
        nfs[i] = c.nf;
    }
    Work wk{1, b->t, b->y, nullptr, b->n_points_total, b->n_out_total, sizeof(float2), b->flags};
    return run_batch(h, wk, cvs, nfs, out, (cudaStream_t)stream, 0, 0.f);
}

int cuvgls_mhgls_direct(cuvgls_handle *h, int32_t nharms, const double *t, const double *yw,
                        const double *w, int64_t n, const double *freqs, int64_t nf, double yy,
                        double ybar, const double *amp_d, const double *cn0, const double *sn0,
                        int32_t flags, double *out, void *stream) {
    if (!h) return CUVGLS_EINVAL;
    h->err.clear();
    if (nharms < 1 || nharms > kMaxHarm)
        return fail(h, CUVGLS_EINVAL, "nharms must be 1.." + std::to_string(kMaxHarm));
    if (n < 1 || nf < 1) return fail(h, CUVGLS_EINVAL, "n and nf must be >= 1");
    if (!t || !yw || !w || !freqs || !out) return fail(h, CUVGLS_EINVAL, "null pointer");
    if (!is_fin(yy) || !is_fin(ybar)) return fail(h, CUVGLS_EINVAL, "YY and ybar must be finite");
    MhParams mp;
    memset(&mp, 0, sizeof mp);
    mp.ybar = ybar;
    mp.yy = yy;
    for (int i = 0; i < nharms; ++i) {
        mp.d[i] = amp_d ? amp_d[i] : 0.0;
        mp.cn0[i] = cn0 ? cn0[i] : 0.0;
        mp.sn0[i] = sn0 ? sn0[i] : 0.0;
    }
    cudaStream_t s = (cudaStream_t)stream;
    int rc = order_stream(h, s);
    if (rc) return rc;
    const bool hin = flags & CUVGLS_HOST_INPUT, hout = flags & CUVGLS_HOST_OUTPUT;
    size_t need = kAlign;
    if (hin) need += 3 * align_up((size_t)n * 8) + align_up((size_t)nf * 8);
    if (hout) need += align_up((size_t)nf * 8);
    if ((long long)need > h->opts.workspace_bytes)
        return fail(h, CUVGLS_EBUDGET, "inputs/outputs exceed the workspace budget");
    rc = ensure_ws(h, need);
    if (rc) return rc;
    char *base = h->ws;
    size_t off = 0;
    auto take = [&](size_t bytes) { char *p = base + off; off += align_up(bytes); return p; };
    const double *dt = t, *dyw = yw, *dw = w, *df = freqs;
    if (hin) {
        double *a = (double *)take(n * 8), *b = (double *)take(n * 8);
        double *c = (double *)take(n * 8), *d = (double *)take(nf * 8);
        CK(cudaMemcpyAsync(a, t, n * 8, cudaMemcpyHostToDevice, s), "H2D t");
        CK(cudaMemcpyAsync(b, yw, n * 8, cudaMemcpyHostToDevice, s), "H2D yw");
        CK(cudaMemcpyAsync(c, w, n * 8, cudaMemcpyHostToDevice, s), "H2D w");
        CK(cudaMemcpyAsync(d, freqs, nf * 8, cudaMemcpyHostToDevice, s), "H2D freqs");
        dt = a; dyw = b; dw = c; df = d;
    }
    double *dout = hout ? (double *)take(nf * 8) : out;
    LAUNCH(CUVGLS_STAGE_DIRECT, s, launch_mhgls_direct(nharms, dt, dyw, dw, n, df, nf, mp, dout, s),
           "k_mhgls_direct");
    if (hout) CK(cudaMemcpyAsync(out, dout, nf * 8, cudaMemcpyDeviceToHost, s), "D2H");
    CK(cudaEventRecord(h->done, s), "record done");
    return CUVGLS_OK;
}

int cuvgls_nfft_adjoint_fp64(cuvgls_handle *h, const cuvgls_nfft_input *b, const double *y,
                             double *out, void *stream) {
    if (!h) return CUVGLS_EINVAL;
    h->err.clear();
    if (!b || b->n_curves < 0) return fail(h, CUVGLS_EINVAL, "null batch or negative n_curves");
    if (b->n_curves == 0) return CUVGLS_OK;
    if (!b->curves || !b->t || !y || !out) return fail(h, CUVGLS_EINVAL, "null pointer");
    cudaStream_t s = (cudaStream_t)stream;
    int rc = order_stream(h, s);
    if (rc) return rc;
    const int nc = b->n_curves;
    std::vector<Direct64Curve> hc(nc);
    long long max_nf = 0;
    for (int i = 0; i < nc; ++i) {
        const cuvgls_nfft_curve &c = b->curves[i];
        if (c.n < 1 || c.nf < 1 || c.pt_off < 0 || c.out_off < 0 ||
            c.pt_off + c.n > b->n_points_total || c.out_off + c.nf > b->n_out_total ||
            !(c.df > 0) || !is_fin(c.df) || !is_fin(c.f0))
            return fail(h, CUVGLS_EINVAL,
                        "curve " + std::to_string(i) + ": bad size, range or frequency grid");
        hc[i] = Direct64Curve{c.pt_off, c.n, c.nf, c.out_off, c.f0, c.df};
        max_nf = std::max(max_nf, (long long)c.nf);
    }
    const bool hin = b->flags & CUVGLS_HOST_INPUT, hout = b->flags & CUVGLS_HOST_OUTPUT;
    const size_t npts = (size_t)b->n_points_total, nout = (size_t)b->n_out_total;
    size_t need = align_up(nc * sizeof(Direct64Curve)) + kAlign;
    if (hin) need += 2 * align_up(npts * 8);
    if (hout) need += align_up(nout * 16);
    if ((long long)need > h->opts.workspace_bytes)
        return fail(h, CUVGLS_EBUDGET, "batch inputs/outputs exceed the workspace budget");
    rc = ensure_ws(h, need);
    if (rc) return rc;
    char *base = h->ws;
    size_t off = 0;
    auto take = [&](size_t bytes) { char *p = base + off; off += align_up(bytes); return p; };
    Direct64Curve *d_cv = (Direct64Curve *)take(nc * sizeof(Direct64Curve));
    // pageable table: staged by the runtime before the call returns
    CK(cudaMemcpyAsync(d_cv, hc.data(), nc * sizeof(Direct64Curve), cudaMemcpyHostToDevice, s),
       "H2D curves");
    const double *dt = b->t, *dy = y;
    if (hin) {
        double *a = (double *)take(npts * 8);
        double *c = (double *)take(npts * 8);
        CK(cudaMemcpyAsync(a, b->t, npts * 8, cudaMemcpyHostToDevice, s), "H2D t");
        CK(cudaMemcpyAsync(c, y, npts * 8, cudaMemcpyHostToDevice, s), "H2D y");
        dt = a;
        dy = c;
    }
    double2 *dout = hout ? (double2 *)take(nout * 16) : (double2 *)out;
    for (int c0 = 0; c0 < nc; c0 += 65535) {
        const int cnt = std::min(65535, nc - c0);
        LAUNCH(CUVGLS_STAGE_DIRECT, s,
               launch_nfft_direct64(d_cv + c0, cnt, max_nf, dt, dy, dout, s), "k_nfft_direct64");
    }
    if (hout) CK(cudaMemcpyAsync(out, dout, nout * 16, cudaMemcpyDeviceToHost, s), "D2H");
    CK(cudaEventRecord(h->done, s), "record done");
    return CUVGLS_OK;
}

int cuvgls_nfft_from_grid(cuvgls_handle *h, int32_t n_curves,
                          const cuvgls_gridfin_curve *curves, const double *grid,
                          int64_t n_grid_total, int64_t n_out_total, int32_t flags, double *out,
                          void *stream) {
    if (!h) return CUVGLS_EINVAL;
    h->err.clear();
    if (n_curves < 0) return fail(h, CUVGLS_EINVAL, "negative n_curves");
    if (n_curves == 0) return CUVGLS_OK;
    if (!curves || !grid || !out) return fail(h, CUVGLS_EINVAL, "null pointer");
    cudaStream_t s = (cudaStream_t)stream;
    int rc = order_stream(h, s);
    if (rc) return rc;
    std::vector<GridFinishCurve> hc(n_curves);
    long long max_nf = 0;
    for (int i = 0; i < n_curves; ++i) {
        const cuvgls_gridfin_curve &c = curves[i];
        if (c.ng < 1 || c.nf < 1 || c.grid_off < 0 || c.out_off < 0 ||
            c.grid_off + c.ng > n_grid_total || c.out_off + c.nf > n_out_total)
            return fail(h, CUVGLS_EINVAL, "curve " + std::to_string(i) + ": bad range");
        if (!(c.tmax > c.tmin) || !(c.spp > 0) || !is_fin(c.f0) || !is_fin(c.b))
            return fail(h, CUVGLS_EINVAL,
                        "curve " + std::to_string(i) + ": needs tmax > tmin, spp > 0, finite f0, b");
        // the reference's nfft_shift and normalize (cuvarbase/kernels/cunfft.cu:59-82,
        // :214-248); the shift only for |f0| > 1e-9 (cuvarbase/cunfft.py:275-285)
        const double sT = c.spp * (c.tmax - c.tmin);
        const double k0 = c.f0 * sT;
        hc[i] = GridFinishCurve{c.grid_off, c.ng, c.nf, c.out_off, k0,
                                std::fabs(c.f0) > 1e-9 ? k0 : 0.0,
                                c.tmin / sT * (double)c.ng, c.b};
        max_nf = std::max(max_nf, (long long)c.nf);
    }
    const bool hin = flags & CUVGLS_HOST_INPUT, hout = flags & CUVGLS_HOST_OUTPUT;
    const size_t ngt = (size_t)n_grid_total, nout = (size_t)n_out_total;
    size_t need = align_up(n_curves * sizeof(GridFinishCurve)) + kAlign;
    if (hin) need += align_up(ngt * 16);
    if (hout) need += align_up(nout * 16);
    if ((long long)need > h->opts.workspace_bytes)
        return fail(h, CUVGLS_EBUDGET, "grids/outputs exceed the workspace budget");
    rc = ensure_ws(h, need);
    if (rc) return rc;
    char *base = h->ws;
    size_t off = 0;
    auto take = [&](size_t bytes) { char *p = base + off; off += align_up(bytes); return p; };
    GridFinishCurve *d_cv = (GridFinishCurve *)take(n_curves * sizeof(GridFinishCurve));
    CK(cudaMemcpyAsync(d_cv, hc.data(), n_curves * sizeof(GridFinishCurve),
                       cudaMemcpyHostToDevice, s), "H2D curves");
    const double2 *dg = (const double2 *)grid;
    if (hin) {
        double2 *a = (double2 *)take(ngt * 16);
        CK(cudaMemcpyAsync(a, grid, ngt * 16, cudaMemcpyHostToDevice, s), "H2D grid");
        dg = a;
    }
    double2 *dout = hout ? (double2 *)take(nout * 16) : (double2 *)out;
    for (int c0 = 0; c0 < n_curves; c0 += 65535) {
        const int cnt = std::min(65535, n_curves - c0);
        LAUNCH(CUVGLS_STAGE_DIRECT, s, launch_grid_finish(d_cv + c0, cnt, max_nf, dg, dout, s),
               "k_grid_finish");
    }
    if (hout) CK(cudaMemcpyAsync(out, dout, nout * 16, cudaMemcpyDeviceToHost, s), "D2H");
    CK(cudaEventRecord(h->done, s), "record done");
    return CUVGLS_OK;
}

int cuvgls_spread_ref(cuvgls_handle *h, int32_t n_curves, const cuvgls_grid_curve *curves,
                      const double *t, const float *y, int64_t n_points_total,
                      int64_t n_out_total, int32_t flags, float *grid_out, void *stream) {
    if (!h) return CUVGLS_EINVAL;
    h->err.clear();
    if (n_curves < 0) return fail(h, CUVGLS_EINVAL, "negative n_curves");
    if (n_curves == 0) return CUVGLS_OK;
    if (!curves || !t || !y || !grid_out) return fail(h, CUVGLS_EINVAL, "null pointer");
    cudaStream_t s = (cudaStream_t)stream;
    int rc = order_stream(h, s);
    if (rc) return rc;
    std::vector<RefGridCurve> hc(n_curves);
    long long max_n = 0;
    for (int i = 0; i < n_curves; ++i) {
        const cuvgls_grid_curve &c = curves[i];
        if (c.n < 1 || c.ng < 1 || c.pt_off < 0 || c.out_off < 0 ||
            c.pt_off + c.n > n_points_total || c.out_off + c.ng > n_out_total)
            return fail(h, CUVGLS_EINVAL, "curve " + std::to_string(i) + ": bad range");
        if (!(c.tmax > c.tmin) || !(c.spp > 0))
            return fail(h, CUVGLS_EINVAL, "curve " + std::to_string(i) + ": needs tmax > tmin, spp > 0");
        hc[i] = RefGridCurve{c.pt_off, c.n, c.ng, c.tmin, 1.0 / (c.spp * (c.tmax - c.tmin)), c.out_off};
        max_n = std::max(max_n, (long long)c.n);
    }
    const bool hin = flags & CUVGLS_HOST_INPUT, hout = flags & CUVGLS_HOST_OUTPUT;
    size_t need = align_up(n_curves * sizeof(RefGridCurve)) + kAlign;
    if (hin) need += align_up(n_points_total * 8) + align_up(n_points_total * 4);
    if (hout) need += align_up(n_out_total * 4);
    rc = ensure_ws(h, need);
    if (rc) return rc;
    char *base = h->ws;
    size_t off = 0;
    auto take = [&](size_t bytes) { char *p = base + off; off += align_up(bytes); return p; };
    RefGridCurve *d_cv = (RefGridCurve *)take(n_curves * sizeof(RefGridCurve));
    CK(cudaMemcpyAsync(d_cv, hc.data(), n_curves * sizeof(RefGridCurve), cudaMemcpyHostToDevice, s),
       "H2D curves");
    const double *dt = t;
    const float *dy = y;
    if (hin) {
        double *a = (double *)take(n_points_total * 8);
        float *c = (float *)take(n_points_total * 4);
        CK(cudaMemcpyAsync(a, t, n_points_total * 8, cudaMemcpyHostToDevice, s), "H2D t");
        CK(cudaMemcpyAsync(c, y, n_points_total * 4, cudaMemcpyHostToDevice, s), "H2D y");
        dt = a; dy = c;
    }
    float *dg = hout ? (float *)take(n_out_total * 4) : grid_out;
    CK(cudaMemsetAsync(dg, 0, n_out_total * 4, s), "memset grid");
    const double sig = h->opts.sigma;
    const int m = h->opts.m;
    const double b = 2.0 * sig * m / ((2.0 * sig - 1.0) * kPi);
    for (int c0 = 0; c0 < n_curves; c0 += 65535) {
        int cnt = std::min(65535, n_curves - c0);
        LAUNCH(CUVGLS_STAGE_SPREAD, s,
               launch_spread_ref(d_cv + c0, cnt, max_n, dt, dy, dg, m, (float)(1.0 / b),
                                 (float)(1.0 / sqrt(kPi * b)), s), "k_spread_ref");
    }
    if (hout) CK(cudaMemcpyAsync(grid_out, dg, n_out_total * 4, cudaMemcpyDeviceToHost, s), "D2H");
    // the curve table above is pageable and copied synchronously, so no
    // staging lifetime to track here
    CK(cudaEventRecord(h->done, s), "record done");
    return CUVGLS_OK;
}

int cuvgls_sync(cuvgls_handle *h, void *stream, int32_t timeout_ms) {
    if (!h) return CUVGLS_EINVAL;
    CK(cudaSetDevice(h->device), "cudaSetDevice");
    cudaStream_t s = (cudaStream_t)stream;
    // ev[0] marks the caller's work, ev[1] the copy of the flag word queued
    // behind it into page-locked memory: nothing here blocks (a blocking
    // copy would also wait for other streams' work).  The deadline applies
    // to the work; the one-word copy then gets a bounded grace period.
    cudaEvent_t ev[2] = {nullptr, nullptr};
    auto release = [&]() {
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
    };
    cudaError_t e = cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(ev[0], s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h->h_flags, h->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaEventRecord(ev[1], s);
    if (e != cudaSuccess) { release(); return cuda_fail(h, e, "record sync"); }
    constexpr double kCopyGraceMs = 1000.0;
    auto t0 = std::chrono::steady_clock::now();
    for (int k = 0; k < 2; ++k) {
        const double limit = k == 0 ? (double)timeout_ms : (double)timeout_ms + kCopyGraceMs;
        for (;;) {
            e = cudaEventQuery(ev[k]);
            if (e == cudaSuccess) break;
            if (e != cudaErrorNotReady) { release(); return cuda_fail(h, e, "sync"); }
            const double ms =
                std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0)
                    .count();
            if (timeout_ms >= 0 && ms > limit) {
                release();
                return fail(h, CUVGLS_ETIMEOUT,
                            "sync deadline of " + std::to_string(timeout_ms) + " ms passed");
            }
            std::this_thread::sleep_for(std::chrono::microseconds(50));
        }
    }
    release();
    const unsigned f = *(volatile unsigned *)h->h_flags;
    if (f & ~(unsigned)CUVGLS_DEVERR_NONFINITE)
        return fail(h, CUVGLS_EDEVICE, "device error flags " + std::to_string(f));
    return CUVGLS_OK;
}

int cuvgls_device_flags(cuvgls_handle *h, int32_t *flags) {
    if (!h || !flags) return CUVGLS_EINVAL;
    CK(cudaSetDevice(h->device), "cudaSetDevice");
    unsigned f = 0;
    CK(cudaMemcpy(&f, h->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost), "read flags");
    CK(cudaMemset(h->d_flags, 0, sizeof(unsigned)), "clear flags");
    *flags = (int32_t)f;
    return CUVGLS_OK;
}

int cuvgls_plan(cuvgls_handle *h, int64_t nf, int64_t *G, int32_t *G1, int32_t *G2, int32_t *m) {
    if (!h || nf < 1) return CUVGLS_EINVAL;
    PlanKey k{0, 0, 0, 0, 0.0, 0};
    if (!plan_for(h, nf, 3, k))
        return fail(h, CUVGLS_ENOTSUP, "no plan for nf=" + std::to_string(nf));
    if (G) *G = (int64_t)k.G1 * k.G2;
    if (G1) *G1 = k.G1;
    if (G2) *G2 = k.G2;
    if (m) *m = k.m;
    return CUVGLS_OK;
}

int cuvgls_plan_shapes(cuvgls_handle *h, int64_t nf, int32_t max_shapes, int32_t *G1,
                       int32_t *G2, int32_t *n_shapes) {
    if (!h || nf < 1 || max_shapes < 0 || (max_shapes > 0 && (!G1 || !G2)) || !n_shapes)
        return CUVGLS_EINVAL;
    PlanKey k{0, 0, 0, 0, 0.0, 0};
    if (!plan_default(h, nf, 3, k))
        return fail(h, CUVGLS_ENOTSUP, "no plan for nf=" + std::to_string(nf));
    const std::vector<Shape> sh = plan_shapes(nf, k.sigma, k.m, 3, h->smem_optin, 10);
    for (int i = 0; i < max_shapes && i < (int)sh.size(); ++i) {
        G1[i] = sh[i].G1;
        G2[i] = sh[i].G2;
    }
    *n_shapes = (int32_t)sh.size();
    return CUVGLS_OK;
}

int cuvgls_plan_pin(cuvgls_handle *h, int64_t nf, int32_t G1, int32_t G2) {
    if (!h || nf < 1 || G1 < 0 || G2 < 0) return CUVGLS_EINVAL;
    h->err.clear();
    if (G1 == 0 && G2 == 0) {
        h->pins.erase(nf);
    } else {
        PlanKey k{0, 0, 0, 0, 0.0, 0};
        if (!plan_default(h, nf, 3, k))
            return fail(h, CUVGLS_ENOTSUP, "no plan for nf=" + std::to_string(nf));
        int B, R;
        if (!shape_fits(nf, k.sigma, k.m, 3, G1, G2, h->smem_optin, B, R))
            return fail(h, CUVGLS_EINVAL,
                        "grid " + std::to_string(G1) + " x " + std::to_string(G2) +
                            " does not fit a plan for nf=" + std::to_string(nf));
        h->pins[nf] = std::make_pair((int)G1, (int)G2);
    }
    h->nf_plan.erase((3LL << 40) + nf);  // planned again at the next use
    return CUVGLS_OK;
}

int cuvgls_plan_window(cuvgls_handle *h, int64_t nf, int32_t *window, double *sigma) {
    if (!h || nf < 1) return CUVGLS_EINVAL;
    PlanKey k{0, 0, 0, 0, 0.0, 0};
    if (!plan_for(h, nf, 3, k))
        return fail(h, CUVGLS_ENOTSUP, "no plan for nf=" + std::to_string(nf));
    if (window) *window = k.win == kWinES ? CUVGLS_WIN_ES : CUVGLS_WIN_GAUSS;
    if (sigma) *sigma = k.sigma;
    return CUVGLS_OK;
}

int cuvgls_plan_nf(double sigma, int32_t m, int64_t nf, int64_t *G, int32_t *G1,
                   int32_t *G2) {
    if (nf < 1 || !(sigma >= 1.25 && sigma <= 16.0) || m < 2 || m > 16) return CUVGLS_EINVAL;
    int a, b, B, R;
    if (!choose_plan(nf, sigma, m, 3, a, b, B, R)) return CUVGLS_ENOTSUP;
    if (G) *G = (int64_t)a * b;
    if (G1) *G1 = a;
    if (G2) *G2 = b;
    return CUVGLS_OK;
}

int cuvgls_warm(cuvgls_handle *h, int64_t nf_min, int64_t nf_max, int32_t reserve) {
    if (!h || nf_min < 1 || nf_max < nf_min) return CUVGLS_EINVAL;
    h->err.clear();
    CK(cudaSetDevice(h->device), "cudaSetDevice");
    const long long mx = max_plan_nf(h, 3);
    // bands wider than one grid run as sub-bands of at least half its width
    if (nf_max > mx) {
        nf_max = mx;
        nf_min = std::min<long long>(nf_min, std::max(1LL, mx / 2));
    }
    // plans change at a few thresholds of nf: build each one once
    auto same = [&](const PlanKey &a, const PlanKey &b) {
        return a.G1 == b.G1 && a.G2 == b.G2 && a.m == b.m && a.sigma == b.sigma &&
               a.win == b.win;
    };
    long long nf = nf_min;
    while (nf <= nf_max) {
        ClassTables *c = nullptr;
        int rc = get_class(h, nf, 3, &c);
        if (rc) return rc;
        CK(preload_pass_kernels(c->plan.G1, c->plan.G2, 3), "preload pass kernels");
        PlanKey k{0, 0, 0, 0, 0.0, 0}, q{0, 0, 0, 0, 0.0, 0};
        plan_for(h, nf, 3, k);
        long long lo = nf, hi = nf_max + 1;  // first nf with another plan
        while (hi - lo > 1) {
            const long long mid = lo + (hi - lo) / 2;
            if (plan_for(h, mid, 3, q) && same(q, k)) lo = mid;
            else hi = mid;
        }
        nf = hi;
    }
    if (reserve) return ensure_ws(h, (size_t)h->opts.workspace_bytes);
    return CUVGLS_OK;
}

int cuvgls_batch_bytes(cuvgls_handle *h, int32_t n_curves, const int64_t *n,
                       const int64_t *nf, int32_t host_io, int64_t *bytes) {
    if (!h || n_curves < 0 || (n_curves > 0 && (!n || !nf)) || !bytes) return CUVGLS_EINVAL;
    long long tot = 0;
    const long long mx = max_plan_nf(h, 3);
    for (int i = 0; i < n_curves; ++i) {
        if (nf[i] < 1 || n[i] < 0) return fail(h, CUVGLS_EINVAL, "negative size");
        long long ns, w;
        band_split(nf[i], mx, ns, w);  // bands wider than one grid run as sub-bands
        PlanKey k{0, 0, 0, 0, 0.0, 0};
        if (!plan_for(h, w, 3, k))
            return fail(h, CUVGLS_ENOTSUP, "no plan for nf=" + std::to_string(nf[i]));
        const int a = k.G1, b = k.G2, B = k.B;
        long long per = 3LL * a * b * (long long)sizeof(float2);
        per += n[i] * (long long)(sizeof(RecAB) + sizeof(RecC));
        per += 4LL * (b / B + 1) * 4 + sizeof(DevCurve) + sizeof(float4) + 64;
        // segment tables and the raw-preparation partials
        per += (n[i] + kSegPoints - 1) / kSegPoints *
               (long long)(2 * sizeof(SegEntry) + 2 * sizeof(double4));
        tot += ns * per;
        // staged host input (raw t, y, dy in FP64, dy^-2, yw and w: 40 B per
        // point; prepared input needs 16) and the staged powers
        if (host_io) tot += n[i] * 40 + nf[i] * 4;
    }
    // alignment of the arena's arrays and the per-batch tables
    if (n_curves > 0) tot += 64 * (long long)kAlign;
    *bytes = tot;
    return CUVGLS_OK;
}

int cuvgls_profile(cuvgls_handle *h, int32_t enable) {
    if (!h) return CUVGLS_EINVAL;
    CK(cudaSetDevice(h->device), "cudaSetDevice");
    for (int st = 0; st < CUVGLS_NSTAGES; ++st) {
        for (auto &pr : h->prof[st]) {
            cudaEventSynchronize(pr.second);
            h->ev_pool.push_back(pr.first);
            h->ev_pool.push_back(pr.second);
        }
        h->prof[st].clear();
        h->launches[st] = 0;
    }
    h->prof_on = enable != 0;
    return CUVGLS_OK;
}

int cuvgls_profile_read(cuvgls_handle *h, int64_t *launches, double *ms) {
    if (!h || !launches || !ms) return CUVGLS_EINVAL;
    CK(cudaSetDevice(h->device), "cudaSetDevice");
    for (int st = 0; st < CUVGLS_NSTAGES; ++st) {
        double tot = 0;
        for (auto &pr : h->prof[st]) {
            CK(cudaEventSynchronize(pr.second), "profile sync");
            float x = 0;
            CK(cudaEventElapsedTime(&x, pr.first, pr.second), "profile elapsed");
            tot += x;
        }
        launches[st] = h->launches[st];
        ms[st] = tot;
    }
    return CUVGLS_OK;
}

int cuvgls_stream_create(void **stream) {
    if (!stream) return CUVGLS_EINVAL;
    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return CUVGLS_ECUDA;
    *stream = (void *)s;
    return CUVGLS_OK;
}

int cuvgls_stream_destroy(void *stream) {
    if (!stream) return CUVGLS_EINVAL;
    return cudaStreamDestroy((cudaStream_t)stream) == cudaSuccess ? CUVGLS_OK : CUVGLS_ECUDA;
}

int cuvgls_host_alloc(void **ptr, int64_t bytes) {
    if (!ptr || bytes <= 0) return CUVGLS_EINVAL;
    cudaError_t e = cudaMallocHost(ptr, (size_t)bytes);
    if (e == cudaErrorMemoryAllocation) return CUVGLS_ENOMEM;
    return e == cudaSuccess ? CUVGLS_OK : CUVGLS_ECUDA;
}

int cuvgls_host_free(void *ptr) {
    if (!ptr) return CUVGLS_EINVAL;
    return cudaFreeHost(ptr) == cudaSuccess ? CUVGLS_OK : CUVGLS_ECUDA;
}

}  // extern "C"

// Planner entry for other translation units (same rule as the batch calls).
bool cuvgls_internal_choose_plan(long long nf, double sigma, int m, int ng, int *G1,
                                 int *G2, int *B, int *R) {
    return choose_plan(nf, sigma, m, ng, *G1, *G2, *B, *R);
}
