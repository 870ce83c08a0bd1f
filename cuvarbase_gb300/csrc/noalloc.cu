// cuvgls_gls_noalloc: the GLS batch for callers that cannot allocate memory.
//
// Some callers cannot call cudaMalloc: code that runs inside a host
// framework that owns every device allocation (a memory pool or arena that
// accounts for all of the GPU's memory and would be bypassed or starved by a
// private allocation), or a hard-real-time loop that may not touch the
// allocator, which can block or fail, once it has started.  For them this
// entry point does the same work as cuvgls_gls_batch with no allocation at
// all: the caller passes device inputs and outputs, and every temporary
// (descriptors, twiddle tables, spreading records, bin offsets, the error
// word and the intermediate FFT buffer) lives in one fixed static device
// array of CUVGLS_NOALLOC_SCRATCH_BYTES.  Every GPU that loads the library
// holds that array until the process exits.
//
// The array's name is only a host-side stand-in in host code; the device
// address comes from cudaGetSymbolAddress, called once per device (with that
// device current) by the first call made on it.  That first call should come
// before any stream capture.  The per-curve descriptors travel to the scratch
// array as kernel parameters, so no host buffer has to outlive the call.  All
// calls share the one array and it keeps the last call's contents: calls that
// overlap on the GPU (on different streams or from different threads) race
// and must be serialised by the caller.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <mutex>

#include "../../include/cuvgls.h"
#include "kernels.cuh"

using namespace cuvgls;

bool cuvgls_internal_choose_plan(long long nf, double sigma, int m, int ng, int *G1,
                                 int *G2, int *B, int *R);

namespace {

constexpr size_t kScratchBytes = (size_t)CUVGLS_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;
constexpr size_t kAlignN = 256;
constexpr double kPiN = 3.14159265358979323846;

size_t up(size_t x) { return (x + kAlignN - 1) / kAlignN * kAlignN; }

// Device address of the scratch array on each device (set up on first use).
void *g_scratch_addr[kMaxDevices];
std::mutex g_scratch_mutex;

}  // namespace

// The scratch array itself (device memory, fixed size).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Descriptors handed to the device as a kernel parameter, kDescPerLaunch at
// a time (32 x 104 bytes stays under the classic 4 KB parameter limit).
constexpr int kDescPerLaunch = 32;
struct DescChunk {
    DevCurve cv[kDescPerLaunch];
    int first, n;
};

__global__ void k_noalloc_put_desc(const DescChunk c, DevCurve *__restrict__ dst) {
    const int i = threadIdx.x;
    if (i < c.n) dst[c.first + i] = c.cv[i];
}

extern "C" int cuvgls_gls_noalloc(double sigma, int32_t m, const cuvgls_gls_input *b,
                                  float *p_out, int32_t *device_flags, void *stream,
                                  char *err, int32_t err_len) {
    auto fail = [&](int code, const char *msg) {
        if (err && err_len > 0) snprintf(err, (size_t)err_len, "%s", msg);
        return code;
    };
    char msg[256];
    if (err && err_len > 0) err[0] = 0;
    if (!b || b->n_curves < 0) return fail(CUVGLS_EINVAL, "null batch or negative n_curves");
    if (b->n_curves == 0) return CUVGLS_OK;
    const int nc = b->n_curves;
    if (nc > CUVGLS_NOALLOC_MAX_CURVES) {
        snprintf(msg, sizeof msg, "%d curves; cuvgls_gls_noalloc takes at most %d per call",
                 nc, CUVGLS_NOALLOC_MAX_CURVES);
        return fail(CUVGLS_EBUDGET, msg);
    }
    if (!b->curves || !b->t || !b->yw || !b->w || !p_out)
        return fail(CUVGLS_EINVAL, "null pointer in batch");
    if (b->flags != 0)
        return fail(CUVGLS_EINVAL, "cuvgls_gls_noalloc takes device inputs and outputs only "
                                   "(flags must be 0)");
    if (b->mode < 0 || b->mode > 2) return fail(CUVGLS_EINVAL, "mode must be 0, 1 or 2");
    if (b->reg[0] != b->reg[1] || b->reg[2] != 0.f || !(b->reg[0] >= 0.f))
        return fail(CUVGLS_EINVAL, "reg must be (lambda, lambda, 0) with lambda >= 0");
    if (!(sigma >= 1.25 && sigma <= 16.0) || m < 2 || m > 16)
        return fail(CUVGLS_EINVAL, "sigma must be in [1.25, 16] and m in [2, 16]");
    long long max_nf = 0, n_tot = 0, n_seg = 0;
    for (int i = 0; i < nc; ++i) {
        const cuvgls_curve &c = b->curves[i];
        if (c.n < 1 || c.nf < 1 || c.pt_off < 0 || c.out_off < 0 ||
            c.pt_off + c.n > b->n_points_total || c.out_off + c.nf > b->n_out_total ||
            !(c.df > 0) || !isfinite(c.df) || c.n > CUVGLS_MAX_CURVE_POINTS) {
            snprintf(msg, sizeof msg, "curve %d: bad size, range or df", i);
            return fail(CUVGLS_EINVAL, msg);
        }
        max_nf = std::max(max_nf, (long long)c.nf);
        n_tot += c.n;
        n_seg += seg_count((int)c.n);
    }
    // one plan (the one for the largest nf) serves every curve of the call
    int G1, G2, B, R;
    if (!cuvgls_internal_choose_plan(max_nf, sigma, m, 3, &G1, &G2, &B, &R)) {
        snprintf(msg, sizeof msg, "no grid plan for nf=%lld", max_nf);
        return fail(CUVGLS_ENOTSUP, msg);
    }
    const long long G = (long long)G1 * G2;
    Plan p;
    memset(&p, 0, sizeof p);
    p.G1 = G1; p.G2 = G2; p.G = G; p.m = m; p.B = B; p.R = R; p.nb = G2 / B;
    const double bw = 2.0 * sigma * m / ((2.0 * sigma - 1.0) * kPiN);
    p.binv = (float)(1.0 / bw);
    p.dc1 = (float)(bw * kPiN * kPiN / ((double)G * (double)G));
    p.dc2 = (float)(1.0 / sqrt(kPiN * bw));
    const int n1 = fft_table_len(G1), n2 = fft_table_len(G2);

    // scratch layout
    size_t off = 0;
    const size_t o_tab = off;
    off += up((size_t)(n1 + n2 + G) * sizeof(float2));
    const size_t o_cv = off;  off += up((size_t)nc * sizeof(DevCurve));
    const size_t o_flag = off; off += up(sizeof(unsigned));
    const size_t o_ra = off;  off += up((size_t)n_tot * sizeof(RecAB));
    const size_t o_rc = off;  off += up((size_t)n_tot * sizeof(RecC));
    const size_t o_seg = off; off += up((size_t)n_seg * sizeof(SegEntry));
    const size_t nbin = (size_t)nc * (p.nb + 1);
    const size_t o_bins = off; off += up(4 * nbin * sizeof(int));  // counts, cursors
    const size_t o_in = off;  off += up((size_t)nc * 3 * G * sizeof(float2));
    if (off > kScratchBytes) {
        snprintf(msg, sizeof msg,
                 "batch needs %zu bytes of scratch; cuvgls_gls_noalloc holds %zu "
                 "(use fewer curves per call or cuvgls_gls_batch)", off, kScratchBytes);
        return fail(CUVGLS_EBUDGET, msg);
    }

    // set-up: device address of the scratch array, once per device
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return fail(CUVGLS_ECUDA, "cudaGetDevice failed");
    char *base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_scratch_mutex);
        if (!g_scratch_addr[dev]) {
            void *ptr = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess || !ptr) {
                snprintf(msg, sizeof msg, "cudaGetSymbolAddress(scratch): %s",
                         cudaGetErrorString(e));
                return fail(CUVGLS_ECUDA, msg);
            }
            g_scratch_addr[dev] = ptr;
        }
        base = (char *)g_scratch_addr[dev];
    }
    float2 *tab = (float2 *)(base + o_tab);
    p.st1 = tab;
    p.st2 = tab + n1;
    p.itw = tab + n1 + n2;

    // per-curve descriptors, built kDescPerLaunch at a time on the stack and
    // passed to k_noalloc_put_desc by value (no host allocation either)
    cudaStream_t s = (cudaStream_t)stream;
    DevCurve *d_cv = (DevCurve *)(base + o_cv);
    unsigned *d_flag = (unsigned *)(base + o_flag);
    cudaError_t e = cudaSuccess;
    DescChunk chunk;
    long long rec = 0;
    int seg = 0;
    for (int i0 = 0; i0 < nc && e == cudaSuccess; i0 += kDescPerLaunch) {
        memset(&chunk, 0, sizeof chunk);
        chunk.first = i0;
        chunk.n = std::min(kDescPerLaunch, nc - i0);
        for (int j = 0; j < chunk.n; ++j) {
            const int i = i0 + j;
            const cuvgls_curve &c = b->curves[i];
            DevCurve &d = chunk.cv[j];
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
            d.rec_off = rec;
            d.bin_off = i * (p.nb + 1);
            d.seg0 = seg;
            seg += seg_count(d.n);
            d.inter_off = (long long)i * 3 * G;
            d.aux = i;
            rec += c.n;
        }
        k_noalloc_put_desc<<<1, kDescPerLaunch, 0, s>>>(chunk, d_cv);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(d_flag, 0, sizeof(unsigned), s);
    if (e == cudaSuccess) e = launch_plan_tables(tab, G1, G2, B, s);
    RecAB *recAB = (RecAB *)(base + o_ra);
    RecC *recC = (RecC *)(base + o_rc);
    SegEntry *segs = (SegEntry *)(base + o_seg);
    int *binsAB = (int *)(base + o_bins);
    int *binsC = binsAB + nbin, *curAB = binsC + nbin, *curC = curAB + nbin;
    float2 *inter = (float2 *)(base + o_in);
    // binning: the segment table is filled on the device (no host memory
    // for it here); count and scan run only when a curve is longer than one
    // segment, and skip the others
    const int ns = (int)n_seg;
    const bool multi = n_seg > nc;
    if (e == cudaSuccess) e = launch_seg_fill(d_cv, nc, segs, nullptr, s);
    if (e == cudaSuccess && multi) e = cudaMemsetAsync(binsAB, 0, 2 * nbin * sizeof(int), s);
    if (e == cudaSuccess && multi)
        e = launch_bin_count(segs, ns, d_cv, b->t, binsAB, binsC, p, 3, 0, s);
    if (e == cudaSuccess && multi)
        e = launch_bin_scan(d_cv, nc, b->t, binsAB, binsC, curAB, curC, nullptr, p, 3, s);
    if (e == cudaSuccess)
        e = launch_bin_scatter(segs, ns, d_cv, b->t, b->yw, b->w, recAB, recC, binsAB, binsC,
                               curAB, curC, nullptr, p, 3, 0, d_flag, s);
    if (e == cudaSuccess)
        e = launch_pass1(d_cv, nc, recAB, recC, binsAB, binsC, inter, p, 3, s);
    if (e == cudaSuccess)
        e = launch_pass2_gls(d_cv, nc, inter, p_out, p, GlsParams{b->mode, b->reg[0]}, s);
    // this call's device error word (CUVGLS_DEVERR_*) to the caller's word
    if (e == cudaSuccess && device_flags)
        e = cudaMemcpyAsync(device_flags, d_flag, sizeof(unsigned), cudaMemcpyDefault, s);
    if (e != cudaSuccess) {
        snprintf(msg, sizeof msg, "launch failed: %s", cudaGetErrorString(e));
        return fail(CUVGLS_ECUDA, msg);
    }
    return CUVGLS_OK;
}
