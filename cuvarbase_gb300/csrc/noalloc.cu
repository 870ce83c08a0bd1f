// cuvgls_gls_noalloc: the GLS batch for callers that cannot allocate memory.
//
// Some callers cannot call cudaMalloc: code that runs inside a host
// framework that owns every device allocation (a memory pool or arena it
// accounts for), code running while a CUDA stream is being captured, or a
// hard-real-time loop that may not touch the allocator once it has started.
// For them this entry point does the same work as cuvgls_gls_batch with no
// allocation at all: the caller passes device inputs and outputs, and every
// temporary (descriptors, twiddle tables, spreading records, bin offsets and
// the intermediate FFT buffer) lives in one fixed static device array of
// CUVGLS_NOALLOC_SCRATCH_BYTES.  Every GPU that loads the library holds that
// array until the process exits.
//
// The array's name is only a host-side stand-in in host code; the device
// address comes from cudaGetSymbolAddress, called once per device (with that
// device current) by the first call made on it.  That first call should come
// before any stream capture.  All calls share the one array and it keeps the
// last call's contents: calls that overlap on the GPU (on different streams
// or from different threads) race and must be serialised by the caller.
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

// Turns (fraction of a full turn) of entry e of the FFT table of a length-L
// transform, in the layout the pass kernels read: [qa][i] stage-A twiddles
// i qa / L of a two-level length, else [stage][r - 1][k] Stockham twiddles.
__device__ double noalloc_stage_turns(int L, int e) {
    if (two_level_la(L) > 0) {
        const int LB = L / two_level_la(L);
        const int qa = e / LB, i = e % LB;
        return (double)(i * qa) / (double)L;
    }
    const FacList f = fft_factors(L);
    int ns = 1;
    for (int s = 0; s < f.n; ++s) {
        const int R = f.r[s];
        if (ns > 1) {
            const int seg = ns * (R - 1);
            if (e < seg) {
                const int r = e / ns + 1, k = e % ns;
                return (double)(k * r) / (double)(ns * R);
            }
            e -= seg;
        }
        ns *= R;
    }
    return 0.0;
}

// Fill the twiddle tables of a plan (FP64 angles, rounded once to float).
__global__ void k_noalloc_tables(float2 *st1, int G1, int n1, float2 *st2, int G2,
                                 int n2, float2 *thi, int nthi, int shift,
                                 float2 *tlo, int nlo, float2 *ytw, int B,
                                 long long G) {
    // ytw is followed by the full inter-pass table [q1][l2] (G entries)
    const int total = n1 + n2 + nthi + nlo + G1 * B + (int)G;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += gridDim.x * blockDim.x) {
        double turns;
        float2 *dst;
        int i = e;
        if (i < n1) { turns = noalloc_stage_turns(G1, i); dst = st1 + i; }
        else if ((i -= n1) < n2) { turns = noalloc_stage_turns(G2, i); dst = st2 + i; }
        else if ((i -= n2) < nthi) { turns = (double)((long long)i << shift) / (double)G; dst = thi + i; }
        else if ((i -= nthi) < nlo) { turns = (double)i / (double)G; dst = tlo + i; }
        else if ((i -= nlo) < G1 * B) {
            const int q1 = i / B, c = i % B;
            turns = (double)((long long)q1 * c) / (double)G;
            dst = ytw + i;
        } else {
            // inter-pass table in the intermediate's [cb][q1][c] order
            i -= G1 * B;
            const int c = i % B, q1 = (i / B) % G1, cb = i / (B * G1);
            const long long l2 = (long long)cb * B + c;
            turns = (double)(((long long)q1 * l2) % G) / (double)G;
            dst = ytw + G1 * B + i;
        }
        double s, c;
        sincospi(2.0 * turns, &s, &c);
        *dst = make_float2((float)c, (float)s);
    }
}

extern "C" int cuvgls_gls_noalloc(double sigma, int32_t m, const cuvgls_gls_input *b,
                                  float *p_out, void *stream, char *err,
                                  int32_t err_len) {
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
    long long max_nf = 0, n_tot = 0;
    for (int i = 0; i < nc; ++i) {
        const cuvgls_curve &c = b->curves[i];
        if (c.n < 1 || c.nf < 1 || c.pt_off < 0 || c.out_off < 0 ||
            c.pt_off + c.n > b->n_points_total || c.out_off + c.nf > b->n_out_total ||
            !(c.df > 0) || !isfinite(c.df) || c.n > 0x7fffffffLL) {
            snprintf(msg, sizeof msg, "curve %d: bad size, range or df", i);
            return fail(CUVGLS_EINVAL, msg);
        }
        max_nf = std::max(max_nf, (long long)c.nf);
        n_tot += c.n;
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
    p.tw_shift = tw_shift_for(G);
    p.tw_mask = (1 << p.tw_shift) - 1;
    p.n_thi = (int)(((G - 1) >> p.tw_shift) + 1);
    const int n1 = fft_table_len(G1), n2 = fft_table_len(G2), nlo = p.tw_mask + 1;

    // scratch layout
    size_t off = 0;
    const size_t o_tab = off;
    off += up((size_t)(n1 + n2 + p.n_thi + nlo + G1 * B + G) * sizeof(float2));
    const size_t o_cv = off;  off += up((size_t)nc * sizeof(DevCurve));
    const size_t o_aux = off; off += up((size_t)nc * sizeof(float4));
    const size_t o_flag = off; off += up(sizeof(unsigned));
    const size_t o_ra = off;  off += up((size_t)n_tot * sizeof(RecAB));
    const size_t o_rc = off;  off += up((size_t)n_tot * sizeof(RecC));
    const size_t o_ba = off;  off += up((size_t)nc * (p.nb + 1) * sizeof(int));
    const size_t o_bc = off;  off += up((size_t)nc * (p.nb + 1) * sizeof(int));
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
    p.thi = tab + n1 + n2;
    p.tlo = p.thi + p.n_thi;
    p.ytw = p.tlo + nlo;
    p.itw = p.ytw + G1 * B;

    // per-curve descriptors, built on the stack (no host allocation either)
    DevCurve hcv[CUVGLS_NOALLOC_MAX_CURVES];
    long long rec = 0;
    for (int i = 0; i < nc; ++i) {
        const cuvgls_curve &c = b->curves[i];
        DevCurve d;
        memset(&d, 0, sizeof d);
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
        d.inter_off = (long long)i * 3 * G;
        d.aux = i;
        rec += c.n;
        hcv[i] = d;
    }
    cudaStream_t s = (cudaStream_t)stream;
    DevCurve *d_cv = (DevCurve *)(base + o_cv);
    unsigned *d_flag = (unsigned *)(base + o_flag);
    cudaError_t e = cudaMemcpyAsync(d_cv, hcv, (size_t)nc * sizeof(DevCurve),
                                    cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_flag, 0, sizeof(unsigned), s);
    if (e == cudaSuccess) {
        const int total = n1 + n2 + p.n_thi + nlo + G1 * B + (int)G;
        k_noalloc_tables<<<(total + 255) / 256, 256, 0, s>>>(
            tab, G1, n1, tab + n1, G2, n2, tab + n1 + n2, p.n_thi,
            p.tw_shift, tab + n1 + n2 + p.n_thi, nlo, tab + n1 + n2 + p.n_thi + nlo, B, G);
        e = cudaGetLastError();
    }
    RecAB *recAB = (RecAB *)(base + o_ra);
    RecC *recC = (RecC *)(base + o_rc);
    int *binsAB = (int *)(base + o_ba);
    int *binsC = (int *)(base + o_bc);
    float2 *inter = (float2 *)(base + o_in);
    if (e == cudaSuccess)
        e = launch_prep_bin(d_cv, nc, b->t, b->yw, b->w, recAB, recC, binsAB, binsC,
                            (float4 *)(base + o_aux), p, 3, 0, d_flag, s);
    if (e == cudaSuccess)
        e = launch_pass1(d_cv, nc, recAB, recC, binsAB, binsC, inter, p, 3, s);
    if (e == cudaSuccess)
        e = launch_pass2_gls(d_cv, nc, inter, p_out, p, GlsParams{b->mode, b->reg[0]}, s);
    if (e != cudaSuccess) {
        snprintf(msg, sizeof msg, "launch failed: %s", cudaGetErrorString(e));
        return fail(CUVGLS_ECUDA, msg);
    }
    return CUVGLS_OK;
}
