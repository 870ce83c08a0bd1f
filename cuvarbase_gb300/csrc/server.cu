// Continuous-batching GLS server inside libcuvgls (C ABI in cuvgls.h).
//
// Requests (one light curve and its frequency grid each) are prepared on the
// submitting thread (the host preparation of LombScargleMemory.setdata and
// normalize_light_curves, cuvarbase/lombscargle.py:235-293,
// cuvarbase/utils.py:113-146) and queued.  One loop thread admits queued
// requests under the HBM budget into the next free slot, runs them as one
// cuvgls_gls_batch call on the slot's handle and stream, and completes a
// slot's requests when its event has fired.  Each slot has its own workspace
// (hbm_budget / inflight bytes) and its own page-locked staging and result
// buffers, so batches in flight overlap on the device and together stay
// within the budget.  Results stay in the slot's result buffer until every
// request of the batch is released by the consumer; a slot is reused only
// then (the consumer's pace is the back-pressure).
//
// No counterpart in the reference: cuvarbase runs one synchronous batch per
// call.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/cuvgls.h"

static_assert(sizeof(cuvgls_server_opts) == 80, "cuvgls_server_opts layout");

namespace {

// Recycled requests: at most kPoolReqs, each holding at most kPoolPoints
// points of array capacity.
constexpr size_t kPoolReqs = 256;
constexpr size_t kPoolPoints = 1 << 20;

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

struct SrvReq {
    int64_t id = 0;
    std::vector<double> t;
    std::vector<float> yw, w;
    double yy = 0, ybar = 0, yw_sum = 0, w_sum = 0, df = 0;
    int64_t nf = 0, k0 = 0, bytes = 0;
    double arrival = 0, latency_ms = 0;
    int slot = -1;          // slot holding the result (-1: none)
    int64_t out_off = 0;    // offset of the result in the slot's buffer
    int status = CUVGLS_OK;
};

struct SrvSlot {
    cuvgls_handle *h = nullptr;
    void *stream = nullptr;
    cudaEvent_t ev = nullptr;
    bool busy = false;      // batch on the device
    int unreleased = 0;     // completed results not yet released
    std::vector<SrvReq *> reqs;
    double *pt = nullptr;   // page-locked staging of t, yw, w
    float *pyw = nullptr, *pw = nullptr;
    size_t cap_pts = 0;
    float *pout = nullptr;  // page-locked results
    size_t cap_out = 0;
    std::vector<cuvgls_curve> cv;
};

}  // namespace

struct cuvgls_server {
    cuvgls_server_opts o;
    int64_t slot_bytes = 0;
    std::vector<SrvSlot> slots;
    cuvgls_handle *planner = nullptr;  // request sizes (own lock)
    std::mutex plan_mu;
    std::mutex mu;
    std::condition_variable loop_cv, done_cv;
    std::deque<SrvReq *> queue;
    std::deque<SrvReq *> done;
    std::unordered_map<int64_t, SrvReq *> live;  // completed, not yet released
    // Released requests kept for reuse with their arrays' capacity, so that a
    // warmed-up server allocates nothing per request (large per-request
    // allocations and frees go through mmap / munmap, whose page faults and
    // TLB shootdowns stall the process's other threads)
    std::vector<SrvReq *> free_reqs;
    int64_t inflight_bytes = 0;
    bool stop = false, closed = false;
    std::thread th;
    // counters
    int64_t submitted = 0, completed = 0, rejected = 0, batches = 0, batched = 0;
    std::string err;
};

namespace {

void free_slot(SrvSlot &s) {
    if (s.pt) cudaFreeHost(s.pt);
    if (s.pyw) cudaFreeHost(s.pyw);
    if (s.pw) cudaFreeHost(s.pw);
    if (s.pout) cudaFreeHost(s.pout);
    s.pt = nullptr; s.pyw = s.pw = s.pout = nullptr;
    s.cap_pts = s.cap_out = 0;
}

// Grow-only page-locked staging for n points and nf results.
int ensure_slot(SrvSlot &s, size_t n, size_t nf) {
    if (n > s.cap_pts) {
        size_t cap = std::max(n, (size_t)1 << 20);
        if (s.pt) cudaFreeHost(s.pt);
        if (s.pyw) cudaFreeHost(s.pyw);
        if (s.pw) cudaFreeHost(s.pw);
        s.pt = nullptr; s.pyw = s.pw = nullptr; s.cap_pts = 0;
        if (cudaHostAlloc((void **)&s.pt, cap * 8, cudaHostAllocDefault) != cudaSuccess ||
            cudaHostAlloc((void **)&s.pyw, cap * 4, cudaHostAllocDefault) != cudaSuccess ||
            cudaHostAlloc((void **)&s.pw, cap * 4, cudaHostAllocDefault) != cudaSuccess)
            return CUVGLS_ENOMEM;
        s.cap_pts = cap;
    }
    if (nf > s.cap_out) {
        size_t cap = std::max(nf, (size_t)16 << 20);
        if (s.pout) cudaFreeHost(s.pout);
        s.pout = nullptr; s.cap_out = 0;
        if (cudaHostAlloc((void **)&s.pout, cap * 4, cudaHostAllocDefault) != cudaSuccess)
            return CUVGLS_ENOMEM;
        s.cap_out = cap;
    }
    return CUVGLS_OK;
}

// Launch a batch on slot k (called without the server lock; the slot is
// reserved by busy = true).
int launch(cuvgls_server *sv, int k) {
    SrvSlot &s = sv->slots[k];
    size_t n = 0, nf = 0;
    for (SrvReq *r : s.reqs) { n += r->t.size(); nf += (size_t)r->nf; }
    int rc = ensure_slot(s, n, nf);
    if (rc) return rc;
    s.cv.resize(s.reqs.size());
    size_t o = 0, fo = 0;
    for (size_t i = 0; i < s.reqs.size(); ++i) {
        SrvReq *r = s.reqs[i];
        const size_t m = r->t.size();
        memcpy(s.pt + o, r->t.data(), m * 8);
        memcpy(s.pyw + o, r->yw.data(), m * 4);
        memcpy(s.pw + o, r->w.data(), m * 4);
        cuvgls_curve &c = s.cv[i];
        c.pt_off = (int64_t)o; c.n = (int64_t)m; c.nf = r->nf; c.k0 = r->k0; c.df = r->df;
        c.yy = r->yy; c.ybar = r->ybar; c.yw_sum = r->yw_sum; c.w_sum = r->w_sum;
        c.out_off = (int64_t)fo;
        r->slot = k;
        r->out_off = (int64_t)fo;
        o += m;
        fo += (size_t)r->nf;
    }
    cuvgls_gls_input in;
    memset(&in, 0, sizeof(in));
    in.n_curves = (int32_t)s.reqs.size();
    in.mode = sv->o.mode;
    in.curves = s.cv.data();
    in.t = s.pt; in.yw = s.pyw; in.w = s.pw;
    in.reg[0] = in.reg[1] = sv->o.reg; in.reg[2] = 0.f;
    in.flags = CUVGLS_HOST_INPUT | CUVGLS_HOST_OUTPUT;
    in.n_points_total = (int64_t)n;
    in.n_out_total = (int64_t)nf;
    rc = cuvgls_gls_batch(s.h, &in, s.pout, s.stream);
    if (rc) return rc;
    if (cudaEventRecord(s.ev, (cudaStream_t)s.stream) != cudaSuccess) return CUVGLS_ECUDA;
    return CUVGLS_OK;
}

// Recycle a request (server lock held): keep it for reuse unless the pool
// is full or its arrays are large.
void recycle(cuvgls_server *sv, SrvReq *r) {
    if (sv->free_reqs.size() < kPoolReqs && r->t.capacity() <= kPoolPoints) {
        r->status = CUVGLS_OK;
        r->slot = -1;
        r->out_off = 0;
        sv->free_reqs.push_back(r);
    } else {
        delete r;
    }
}

// Move the requests of slot k to the completion queue (lock held).
void finish_slot(cuvgls_server *sv, int k, int status) {
    SrvSlot &s = sv->slots[k];
    const double t = now_s();
    int64_t freed = 0;
    for (SrvReq *r : s.reqs) {
        r->status = status;
        r->latency_ms = 1000.0 * (t - r->arrival);
        if (status != CUVGLS_OK) r->slot = -1;
        freed += r->bytes;
        sv->done.push_back(r);
        sv->completed++;
    }
    s.unreleased = status == CUVGLS_OK ? (int)s.reqs.size() : 0;
    s.reqs.clear();
    s.busy = false;
    sv->inflight_bytes -= freed;
    sv->done_cv.notify_all();
}

void loop(cuvgls_server *sv) {
    cudaSetDevice(sv->o.device);
    std::unique_lock<std::mutex> lk(sv->mu);
    while (true) {
        bool any_busy = false;
        for (size_t k = 0; k < sv->slots.size(); ++k) {
            SrvSlot &s = sv->slots[k];
            if (!s.busy) continue;
            const cudaError_t e = cudaEventQuery(s.ev);
            if (e == cudaSuccess) finish_slot(sv, (int)k, CUVGLS_OK);
            else if (e != cudaErrorNotReady) finish_slot(sv, (int)k, CUVGLS_ECUDA);
            else any_busy = true;
        }
        if (sv->stop && sv->queue.empty() && !any_busy) break;
        int free_k = -1;
        for (size_t k = 0; k < sv->slots.size(); ++k)
            if (!sv->slots[k].busy && sv->slots[k].unreleased == 0) { free_k = (int)k; break; }
        if (free_k >= 0 && !sv->queue.empty()) {
            int64_t budget = std::min<int64_t>(sv->slot_bytes,
                                               sv->o.hbm_budget - sv->inflight_bytes);
            SrvSlot &s = sv->slots[free_k];
            // also within the slot's page-locked buffers (a batch grows them
            // only when one request alone does not fit)
            size_t pts = 0, outs = 0;
            while (!sv->queue.empty() && (int)s.reqs.size() < sv->o.max_batch &&
                   sv->queue.front()->bytes <= budget) {
                SrvReq *r = sv->queue.front();
                if (!s.reqs.empty() && (pts + r->t.size() > s.cap_pts ||
                                        outs + (size_t)r->nf > s.cap_out))
                    break;
                pts += r->t.size();
                outs += (size_t)r->nf;
                sv->queue.pop_front();
                budget -= r->bytes;
                sv->inflight_bytes += r->bytes;
                s.reqs.push_back(r);
            }
            if (!s.reqs.empty()) {
                s.busy = true;
                sv->batches++;
                sv->batched += (int64_t)s.reqs.size();
                lk.unlock();
                const int rc = launch(sv, free_k);
                lk.lock();
                if (rc) {
                    sv->err = "batch launch failed";
                    finish_slot(sv, free_k, rc);
                }
                continue;
            }
        }
        // wait: poll the GPU while batches run, else until something changes
        if (any_busy) sv->loop_cv.wait_for(lk, std::chrono::microseconds(50));
        else sv->loop_cv.wait_for(lk, std::chrono::milliseconds(20));
    }
    sv->closed = true;
    sv->done_cv.notify_all();
}

// Bytes one request occupies on the device while in flight.
int request_bytes(cuvgls_server *sv, int64_t n, int64_t nf, int64_t *bytes) {
    std::lock_guard<std::mutex> g(sv->plan_mu);
    return cuvgls_batch_bytes(sv->planner, 1, &n, &nf, 1, bytes);
}

}  // namespace

extern "C" {

int cuvgls_server_create(cuvgls_server **out, const cuvgls_server_opts *opts) {
    if (!out || !opts) return CUVGLS_EINVAL;
    *out = nullptr;
    cuvgls_server_opts o = *opts;
    if (o.inflight < 1 || o.inflight > 16 || o.max_batch < 1 || o.hbm_budget < (64LL << 20) ||
        o.mode < 0 || o.mode > 2 || !(o.reg >= 0.f))
        return CUVGLS_EINVAL;
    cuvgls_server *sv = new cuvgls_server();
    sv->o = o;
    sv->slot_bytes = std::max<int64_t>(32LL << 20, o.hbm_budget / o.inflight);
    cuvgls_opts ho;
    memset(&ho, 0, sizeof(ho));
    ho.sigma = o.sigma; ho.m = o.m; ho.device = o.device; ho.precision = o.precision;
    ho.workspace_bytes = sv->slot_bytes;
    // 1 GiB chunks: a batch's result copies overlap its later chunks, which
    // keeps the tail latency of large batches down
    ho.chunk_mb = 1024;
    int rc = cuvgls_create(&sv->planner, &ho);
    sv->slots.resize(o.inflight);
    sv->free_reqs.reserve(kPoolReqs);
    for (int k = 0; rc == CUVGLS_OK && k < o.inflight; ++k) {
        SrvSlot &s = sv->slots[k];
        rc = cuvgls_create(&s.h, &ho);
        if (rc == CUVGLS_OK) rc = cuvgls_stream_create(&s.stream);
        if (rc == CUVGLS_OK &&
            cudaEventCreateWithFlags(&s.ev, cudaEventDisableTiming) != cudaSuccess)
            rc = CUVGLS_ECUDA;
        // plan tables and the whole workspace up front: nothing is allocated
        // or built while requests wait
        if (rc == CUVGLS_OK && o.warm_nf_min > 0 && o.warm_nf_max >= o.warm_nf_min)
            rc = cuvgls_warm(s.h, o.warm_nf_min, o.warm_nf_max, 1);
        if (rc == CUVGLS_OK)
            rc = ensure_slot(s, o.stage_points > 0 ? (size_t)o.stage_points : (size_t)1 << 20,
                             o.stage_results > 0 ? (size_t)o.stage_results : (size_t)16 << 20);
    }
    if (rc) {
        sv->stop = true;
        cuvgls_server_destroy(sv);
        return rc;
    }
    sv->th = std::thread(loop, sv);
    *out = sv;
    return CUVGLS_OK;
}

int cuvgls_server_submit(cuvgls_server *sv, int64_t id, const double *t, const double *y,
                         const double *dy, int64_t n, int64_t nf, double df, int64_t k0) {
    if (!sv) return CUVGLS_EINVAL;
    if (!t || !y || !dy || n < 1 || nf < 1 || nf > 0x7fffffffLL || n > CUVGLS_MAX_CURVE_POINTS ||
        !(df > 0) || !isfinite(df) || k0 < 0)
        return CUVGLS_EINVAL;
    const double arrival = now_s();
    SrvReq *r = nullptr;
    {
        std::lock_guard<std::mutex> g(sv->mu);
        if (!sv->free_reqs.empty()) {
            r = sv->free_reqs.back();
            sv->free_reqs.pop_back();
        }
    }
    if (!r) r = new SrvReq();
    r->arrival = arrival;
    r->id = id;
    r->nf = nf; r->k0 = k0; r->df = df;
    int rc = request_bytes(sv, n, nf, &r->bytes);
    if (rc || r->bytes > sv->slot_bytes) {
        std::lock_guard<std::mutex> g(sv->mu);
        recycle(sv, r);
        if (rc) return rc;
        sv->rejected++;
        return CUVGLS_EBUDGET;
    }
    // host preparation: subtract the (nan-)means of t and y, weights
    // w = dy^-2 / sum dy^-2, ybar = w.y, yw = w (y - ybar), YY = w.(y - ybar)^2
    // in FP64; yw and w cast to float32; sum(yw) as a sequential float32 sum
    double st = 0, sy = 0;
    int64_t ct = 0, cy = 0;
    for (int64_t j = 0; j < n; ++j) {
        if (!isnan(t[j])) { st += t[j]; ++ct; }
        if (!isnan(y[j])) { sy += y[j]; ++cy; }
    }
    const double mt = ct ? st / (double)ct : NAN, my = cy ? sy / (double)cy : NAN;
    r->t.resize(n);
    r->yw.resize(n);
    r->w.resize(n);
    // scratch of the submitting thread, reused across its requests
    thread_local std::vector<double> w, yc;
    if (w.size() < (size_t)n) { w.resize(n); yc.resize(n); }
    double ws = 0;
    for (int64_t j = 0; j < n; ++j) {
        r->t[j] = t[j] - mt;
        yc[j] = y[j] - my;
        w[j] = 1.0 / (dy[j] * dy[j]);
        ws += w[j];
    }
    double ybar = 0;
    for (int64_t j = 0; j < n; ++j) { w[j] /= ws; ybar += yc[j] * w[j]; }
    double yy = 0, wsum = 0;
    float ysum = 0.f;
    for (int64_t j = 0; j < n; ++j) {
        const double d = yc[j] - ybar;
        yy += w[j] * d * d;
        r->yw[j] = (float)(w[j] * d);
        r->w[j] = (float)w[j];
        ysum += r->yw[j];
        wsum += (double)r->w[j];
    }
    r->ybar = ybar; r->yy = yy; r->yw_sum = ysum; r->w_sum = wsum;
    {
        std::lock_guard<std::mutex> g(sv->mu);
        if (sv->stop) { recycle(sv, r); return CUVGLS_EINVAL; }
        sv->queue.push_back(r);
        sv->submitted++;
    }
    sv->loop_cv.notify_one();
    return CUVGLS_OK;
}

int cuvgls_server_poll(cuvgls_server *sv, int32_t max, int32_t timeout_ms, int64_t *ids,
                       int32_t *status, const float **results, int64_t *nf,
                       double *latency_ms) {
    if (!sv || max < 1 || !ids || !status || !results || !nf || !latency_ms)
        return CUVGLS_EINVAL;
    std::unique_lock<std::mutex> lk(sv->mu);
    if (sv->done.empty() && !sv->closed && timeout_ms != 0) {
        const auto until = std::chrono::steady_clock::now() +
                           std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms);
        sv->done_cv.wait_until(lk, until, [&] { return !sv->done.empty() || sv->closed; });
    }
    int32_t k = 0;
    while (k < max && !sv->done.empty()) {
        SrvReq *r = sv->done.front();
        sv->done.pop_front();
        ids[k] = r->id;
        status[k] = r->status;
        results[k] = r->slot >= 0 ? sv->slots[r->slot].pout + r->out_off : nullptr;
        nf[k] = r->nf;
        latency_ms[k] = r->latency_ms;
        sv->live[r->id] = r;
        ++k;
    }
    if (k == 0 && sv->closed) return CUVGLS_ECLOSED;
    return k;
}

int cuvgls_server_release(cuvgls_server *sv, int64_t id) {
    if (!sv) return CUVGLS_EINVAL;
    {
        std::lock_guard<std::mutex> g(sv->mu);
        auto it = sv->live.find(id);
        if (it == sv->live.end()) return CUVGLS_EINVAL;
        SrvReq *r = it->second;
        sv->live.erase(it);
        if (r->slot >= 0) sv->slots[r->slot].unreleased--;
        recycle(sv, r);
    }
    sv->loop_cv.notify_one();
    return CUVGLS_OK;
}

int cuvgls_server_release_many(cuvgls_server *sv, const int64_t *ids, int32_t n) {
    if (!sv || n < 0 || (n > 0 && !ids)) return CUVGLS_EINVAL;
    int rc = CUVGLS_OK;
    {
        std::lock_guard<std::mutex> g(sv->mu);
        for (int32_t i = 0; i < n; ++i) {
            auto it = sv->live.find(ids[i]);
            if (it == sv->live.end()) { rc = CUVGLS_EINVAL; continue; }
            SrvReq *r = it->second;
            sv->live.erase(it);
            if (r->slot >= 0) sv->slots[r->slot].unreleased--;
            recycle(sv, r);
        }
    }
    sv->loop_cv.notify_one();
    return rc;
}

int cuvgls_server_slot_buffer(cuvgls_server *sv, int32_t k, const float **ptr, int64_t *len) {
    if (!sv || !ptr || !len || k < 0 || k >= (int32_t)sv->slots.size()) return CUVGLS_EINVAL;
    std::lock_guard<std::mutex> g(sv->mu);
    *ptr = sv->slots[k].pout;
    *len = (int64_t)sv->slots[k].cap_out;
    return CUVGLS_OK;
}

int cuvgls_server_request_bytes(cuvgls_server *sv, int64_t n, int64_t nf, int64_t *bytes) {
    if (!sv || !bytes || n < 0 || nf < 1) return CUVGLS_EINVAL;
    return request_bytes(sv, n, nf, bytes);
}

int cuvgls_server_stats(cuvgls_server *sv, int64_t *counts) {
    if (!sv || !counts) return CUVGLS_EINVAL;
    std::lock_guard<std::mutex> g(sv->mu);
    counts[0] = sv->submitted;
    counts[1] = sv->completed;
    counts[2] = sv->rejected;
    counts[3] = sv->batches;
    counts[4] = sv->batched;
    counts[5] = sv->slot_bytes;
    counts[6] = (int64_t)sv->queue.size();
    counts[7] = sv->inflight_bytes;
    return CUVGLS_OK;
}

int cuvgls_server_shutdown(cuvgls_server *sv) {
    if (!sv) return CUVGLS_EINVAL;
    {
        std::lock_guard<std::mutex> g(sv->mu);
        sv->stop = true;
    }
    sv->loop_cv.notify_all();
    return CUVGLS_OK;
}

int cuvgls_server_destroy(cuvgls_server *sv) {
    if (!sv) return CUVGLS_EINVAL;
    cuvgls_server_shutdown(sv);
    if (sv->th.joinable()) {
        // the loop drains the queue; completed results need no consumer here
        {
            std::lock_guard<std::mutex> g(sv->mu);
            for (SrvSlot &s : sv->slots) s.unreleased = 0;
        }
        sv->th.join();
    }
    for (SrvReq *r : sv->free_reqs) delete r;
    for (SrvReq *r : sv->done) delete r;
    for (auto &kv : sv->live) delete kv.second;
    for (SrvReq *r : sv->queue) delete r;
    for (SrvSlot &s : sv->slots) {
        if (s.h) cuvgls_destroy(s.h);
        if (s.stream) cuvgls_stream_destroy(s.stream);
        if (s.ev) cudaEventDestroy(s.ev);
        free_slot(s);
    }
    if (sv->planner) cuvgls_destroy(sv->planner);
    delete sv;
    return CUVGLS_OK;
}

}  // extern "C"
