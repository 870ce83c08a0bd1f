// cuvgls kernels for sm_103a.
//
// This file holds the per-point and auxiliary kernels and the length
// dispatch; the pass kernels are in pass_kernels.cuh.
//
// The path per size class (G = G1 * G2 grid cells):
//   k_bin_count, k_bin_scan, k_bin_scatter
//                FP64 offsets t - t0, grid cell index and band-centring
//                phase per point; counting sort of the points by the column
//                block (cell mod G2) / B their Gaussian window starts in;
//                compact FP32 spreading records.  k_bin_scatter (one CTA
//                per segment of kSegPoints points) bins a curve of one
//                segment completely; a longer curve is counted per segment
//                and scanned per descriptor (a warp each) before it.
//   k_pass1      one CTA per (curve, column block).  Spreads the records of
//                the neighbouring bins into a G1 x B shared-memory tile per
//                grid (shared-memory float atomics), runs the length-G1 column
//                FFTs in shared memory, applies the inter-pass twiddle and
//                writes the tile to the intermediate buffer.
//   k_pass2_*    one CTA per (curve, R-row block).  Loads R rows of every
//                grid, runs the length-G2 row FFTs in shared memory and, in
//                the same kernel, deconvolves the Gaussian window and either
//                evaluates the GLS power (3 grids) or applies the output phase
//                of the adjoint NFFT (1 grid).
// The grid itself never exists in HBM: spreading is fused into pass 1.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>

#include "gls_math.cuh"
#include "kernels.cuh"

namespace cuvgls {

// ---------------------------------------------------------------------------
// point positions
// ---------------------------------------------------------------------------
struct Pos {
    int ca;    // cell of frac(x) * G
    float fa;  // fractional offset in that cell
    int cc;    // cell of frac(2x) * G
    float fc;
};

__device__ __forceinline__ void cell_of(double x, double G, int Gi, int &c, float &f) {
    double xf = x - floor(x);
    double u = xf * G;
    double fl = floor(u);
    int ci = (int)fl;
    float fr = (float)(u - fl);
    if (ci >= Gi) { ci -= Gi; }
    c = ci;
    f = fr;
}

__device__ __forceinline__ void cell_of32(float x, float G, int Gi, int &c, float &f) {
    float xf = x - floorf(x);
    float u = xf * G;
    float fl = floorf(u);
    int ci = (int)fl;
    float fr = u - fl;
    if (ci >= Gi) { ci -= Gi; }
    if (ci < 0) { ci = 0; }
    c = ci;
    f = fr;
}

// Position of one point.  Mixed precision: t - t0, frac(x) and the cell
// index in FP64, the in-cell offset in FP32.  FP32 variant: everything FP32
// (t cast to float first, as cuvarbase/lombscargle.py:259 does).
template <bool FP32POS>
__device__ __forceinline__ Pos position(double tj, double tref, double df, int G) {
    Pos p;
    if (!FP32POS) {
        double x = (tj - tref) * df;
        cell_of(x, (double)G, G, p.ca, p.fa);
        cell_of(2.0 * x, (double)G, G, p.cc, p.fc);
    } else {
        float x = ((float)tj - (float)tref) * (float)df;
        cell_of32(x, (float)G, G, p.ca, p.fa);
        cell_of32(2.0f * x, (float)G, G, p.cc, p.fc);
    }
    return p;
}

// exp(2 pi i kc x) with the product kc x range-reduced in FP64 (mixed) or
// FP32.  In the mixed variant the reduced phase th in [-1/2, 1/2) is split
// into hi + lo floats; sincospif(2 hi) is corrected to first order in lo.
template <bool FP32POS>
__device__ __forceinline__ float2 centre_phase(double tj, double tref, double df,
                                               double kc) {
    float s, c;
    if (!FP32POS) {
        double x = (tj - tref) * df;
        double th = kc * x;
        th -= floor(th);
        if (th >= 0.5) th -= 1.0;
        float hi = (float)th;
        float lo = (float)(th - (double)hi);
        sincospif(2.0f * hi, &s, &c);
        float e = 6.283185307179586f * lo;
        float c1 = fmaf(-e, s, c);
        float s1 = fmaf(e, c, s);
        return make_float2(c1, s1);
    } else {
        float x = ((float)tj - (float)tref) * (float)df;
        float th = (float)kc * x;
        th -= floorf(th);
        sincospif(2.0f * th, &s, &c);
        return make_float2(c, s);
    }
}

// ---------------------------------------------------------------------------
// binning: points of each descriptor sorted by the column block their
// Gaussian window starts in, in segments of kSegPoints points
// ---------------------------------------------------------------------------
// One CTA per descriptor: its binning segments at seg0 and, where raw is
// given, the raw-preparation segments of each curve (from the band with
// best_off == 0) at raw_seg.
__global__ void k_seg_fill(const DevCurve *__restrict__ cvs, SegEntry *__restrict__ bin,
                           SegEntry *__restrict__ raw) {
    const DevCurve &cv = cvs[blockIdx.x];
    const int ns = seg_count(cv.n), s0 = cv.seg0, r0 = cv.raw_seg;
    const bool first = raw != nullptr && cv.best_off == 0;
    for (int k = threadIdx.x; k < ns; k += blockDim.x) {
        const SegEntry e{(int)blockIdx.x, k * kSegPoints};
        bin[s0 + k] = e;
        if (first) raw[r0 + k] = e;
    }
}

// Records of one point: the x-position record (grids A and B) and the
// 2x-position record (grid C) with the column blocks they are binned by.  A
// point with a non-finite t, value or weight is kept at t0 with zero values
// and sets `bad`.
template <bool FP32POS>
__device__ __forceinline__ void point_records(double tj, float a, float w, double tref, double df,
                                              double kc, int G, int G2, int B, int ngrids,
                                              RecAB &ra, RecC &rc, int &binA, int &binC,
                                              bool &bad) {
    if (!(isfinite(tj) && isfinite(a) && isfinite(w))) {
        bad = true;
        tj = isfinite(tj) ? tj : tref;
        a = 0.f;
        w = 0.f;
    }
    const Pos ps = position<FP32POS>(tj, tref, df, G);
    const float2 ph = centre_phase<FP32POS>(tj, tref, df, kc);
    const int colA = ps.ca % G2;
    ra.rc = ((ps.ca / G2) << 16) | colA;
    ra.frac = ps.fa;
    ra.a = cscale(ph, a);
    ra.b = cscale(ph, w);
    binA = colA / B;
    binC = 0;
    if (ngrids == 3) {
        const float2 ph2 = make_float2(ph.x * ph.x - ph.y * ph.y, 2.f * ph.x * ph.y);
        const int colC = ps.cc % G2;
        rc.rc = ((ps.cc / G2) << 16) | colC;
        rc.frac = ps.fc;
        rc.c = cscale(ph2, w);
        binC = colC / B;
    }
}

// Output phase of the adjoint NFFT of a descriptor: out[k] needs
// exp(2 pi i (kc + k') df t0): base = exp(2 pi i kc df t0), alpha =
// frac(df t0) split into hi + lo floats.
__device__ __forceinline__ void write_aux(const DevCurve &cv, double tref,
                                          float4 *__restrict__ aux) {
    double v = cv.kc * cv.df * tref;
    v -= floor(v);
    double s, c;
    sincospi(2.0 * v, &s, &c);
    double al = cv.df * tref;
    al -= floor(al);
    const float ah = (float)al;
    const float alo = (float)(al - (double)ah);
    aux[cv.aux] = make_float4((float)c, (float)s, ah, alo);
}

// Exclusive scan of h[0..n) in place by one warp, h[n] = total; the scan is
// also written to cur[0..n) where cur is given.
__device__ __forceinline__ void scan_bins(int *__restrict__ h, int *__restrict__ cur, int n,
                                          int lane) {
    int carry = 0;
    for (int base = 0; base < n; base += 32) {
        const int i = base + lane;
        const int x = (i < n) ? h[i] : 0;
        int inc = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (i < n) {
            h[i] = carry + inc - x;
            if (cur != nullptr) cur[i] = carry + inc - x;
        }
        carry += __shfl_sync(0xffffffffu, inc, 31);
    }
    if (lane == 0) h[n] = carry;
}

// Count of one segment of a curve longer than one segment (CTAs of shorter
// curves return at once): shared-memory histogram of the column blocks,
// added to the descriptor's counts (zeroed before the launch).
template <bool FP32POS>
__global__ void __launch_bounds__(kSegThreads)
k_bin_count(const SegEntry *__restrict__ segs, const DevCurve *__restrict__ cvs,
            const double *__restrict__ t, int *__restrict__ binsAB, int *__restrict__ binsC,
            Plan p, int ngrids) {
    __shared__ int hA[kMaxBins];
    __shared__ int hC[kMaxBins];
    const SegEntry sg = segs[blockIdx.x];
    const DevCurve &cv = cvs[sg.desc];
    const int n = cv.n;
    if (n <= kSegPoints) return;  // uniform over the CTA
    const int tid = threadIdx.x, nb = p.nb, G2 = p.G2, B = p.B, G = (int)p.G;
    for (int i = tid; i < nb; i += kSegThreads) { hA[i] = 0; hC[i] = 0; }
    __syncthreads();
    const long long po = cv.pt_off;
    const double tref = t[po], df = cv.df;
    const int end = min(n, sg.start + kSegPoints);
    for (int j = sg.start + tid; j < end; j += kSegThreads) {
        double tj = t[po + j];
        if (!isfinite(tj)) tj = tref;
        const Pos ps = position<FP32POS>(tj, tref, df, G);
        atomicAdd(&hA[(ps.ca % G2) / B], 1);
        if (ngrids == 3) atomicAdd(&hC[(ps.cc % G2) / B], 1);
    }
    __syncthreads();
    int *bA = binsAB + cv.bin_off, *bC = binsC + cv.bin_off;
    for (int i = tid; i < nb; i += kSegThreads) {
        if (hA[i]) atomicAdd(&bA[i], hA[i]);
        if (ngrids == 3 && hC[i]) atomicAdd(&bC[i], hC[i]);
    }
}

// A curve of at most kSegPoints points binned completely by one CTA:
// shared-memory histogram, scan, bin offsets, records (slots from
// shared-memory cursors) and aux.
template <bool FP32POS>
__device__ __forceinline__ void bin_whole_curve(const DevCurve &cv, const double *__restrict__ t,
                                                const float *__restrict__ ya,
                                                const float *__restrict__ wv,
                                                RecAB *__restrict__ recAB,
                                                RecC *__restrict__ recC,
                                                int *__restrict__ binsAB,
                                                int *__restrict__ binsC,
                                                float4 *__restrict__ aux, const Plan &p,
                                                int ngrids, unsigned *__restrict__ errflag,
                                                int *hA, int *hC) {
    const int tid = threadIdx.x, nb = p.nb, G2 = p.G2, B = p.B, G = (int)p.G;
    const int n = cv.n;
    for (int i = tid; i <= nb; i += kSegThreads) { hA[i] = 0; hC[i] = 0; }
    __syncthreads();
    const long long po = cv.pt_off;
    const double tref = t[po], df = cv.df;
    for (int j = tid; j < n; j += kSegThreads) {
        double tj = t[po + j];
        if (!isfinite(tj)) tj = tref;
        const Pos ps = position<FP32POS>(tj, tref, df, G);
        atomicAdd(&hA[(ps.ca % G2) / B], 1);
        if (ngrids == 3) atomicAdd(&hC[(ps.cc % G2) / B], 1);
    }
    __syncthreads();
    if (tid < 32) {
        scan_bins(hA, nullptr, nb, tid);
        if (ngrids == 3) scan_bins(hC, nullptr, nb, tid);
    }
    __syncthreads();
    int *bA = binsAB + cv.bin_off, *bC = binsC + cv.bin_off;
    for (int i = tid; i <= nb; i += kSegThreads) {
        bA[i] = hA[i];
        if (ngrids == 3) bC[i] = hC[i];
    }
    __syncthreads();  // the offsets are read before the cursors move
    RecAB *rA = recAB + cv.rec_off;
    RecC *rC = recC + cv.rec_off;
    const double kc = cv.kc;
    bool bad = false, lost = false;
    for (int j = tid; j < n; j += kSegThreads) {
        RecAB ra;
        RecC rc;
        int binA, binC;
        point_records<FP32POS>(t[po + j], ya[po + j], (ngrids == 3) ? wv[po + j] : 0.f, tref,
                               df, kc, G, G2, B, ngrids, ra, rc, binA, binC, bad);
        // a slot outside the curve's n records would mean that the count and
        // the scatter binned a point differently: flag it, write nothing
        const int sa = atomicAdd(&hA[binA], 1);
        if ((unsigned)sa < (unsigned)n) rA[sa] = ra;
        else lost = true;
        if (ngrids == 3) {
            const int sc = atomicAdd(&hC[binC], 1);
            if ((unsigned)sc < (unsigned)n) rC[sc] = rc;
            else lost = true;
        }
    }
    if (bad) atomicOr(errflag, 1u);
    if (lost) atomicOr(errflag, 4u);
    if (aux != nullptr && tid == 0) write_aux(cv, tref, aux);
}

// One warp per descriptor of a curve longer than one segment: bin offsets
// and cursors from the counts, and the output phase of the adjoint NFFT in
// aux.  Single-segment descriptors are binned whole by k_bin_scatter.
__global__ void __launch_bounds__(128)
k_bin_scan(const DevCurve *__restrict__ cvs, int n, const double *__restrict__ t,
           int *__restrict__ binsAB, int *__restrict__ binsC, int *__restrict__ curAB,
           int *__restrict__ curC, float4 *__restrict__ aux, int nb, int ngrids) {
    const int i = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (i >= n) return;  // whole warps
    const int lane = threadIdx.x & 31;
    const DevCurve &cv = cvs[i];
    if (cv.n <= kSegPoints) return;
    scan_bins(binsAB + cv.bin_off, curAB + cv.bin_off, nb, lane);
    if (ngrids == 3) scan_bins(binsC + cv.bin_off, curC + cv.bin_off, nb, lane);
    if (aux != nullptr && lane == 0) write_aux(cv, t[cv.pt_off], aux);
}

// Last binning kernel, one CTA per segment.  A curve of one segment is
// binned here completely (bin_whole_curve).  A segment of a longer curve
// (counted and scanned before): FP64 positions and band-centring phases, a
// shared-memory rank of each point within its column block, one global
// reservation per block for the segment's run, then the records.
template <bool FP32POS>
__global__ void __launch_bounds__(kSegThreads)
k_bin_scatter(const SegEntry *__restrict__ segs, const DevCurve *__restrict__ cvs,
              const double *__restrict__ t, const float *__restrict__ ya,
              const float *__restrict__ wv, RecAB *__restrict__ recAB,
              RecC *__restrict__ recC, int *__restrict__ binsAB, int *__restrict__ binsC,
              int *__restrict__ curAB, int *__restrict__ curC, float4 *__restrict__ aux,
              Plan p, int ngrids, unsigned *__restrict__ errflag) {
    constexpr int PPT = kSegPoints / kSegThreads;
    __shared__ int hA[kMaxBins + 1];
    __shared__ int hC[kMaxBins + 1];
    const SegEntry sg = segs[blockIdx.x];
    const DevCurve &cv = cvs[sg.desc];
    const int n = cv.n;
    if (n <= kSegPoints) {  // uniform over the CTA
        bin_whole_curve<FP32POS>(cv, t, ya, wv, recAB, recC, binsAB, binsC, aux, p, ngrids,
                                 errflag, hA, hC);
        return;
    }
    const int tid = threadIdx.x, nb = p.nb, G2 = p.G2, B = p.B, G = (int)p.G;
    for (int i = tid; i < nb; i += kSegThreads) { hA[i] = 0; hC[i] = 0; }
    __syncthreads();
    const long long po = cv.pt_off;
    const double tref = t[po], df = cv.df, kc = cv.kc;
    RecAB ra[PPT];
    RecC rc[PPT];
    int binA[PPT], binC[PPT], rkA[PPT], rkC[PPT];
    bool bad = false, lost = false;
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        const int j = sg.start + q * kSegThreads + tid;
        binA[q] = -1;
        binC[q] = 0;
        rkC[q] = 0;
        if (j < n) {
            point_records<FP32POS>(t[po + j], ya[po + j], (ngrids == 3) ? wv[po + j] : 0.f,
                                   tref, df, kc, G, G2, B, ngrids, ra[q], rc[q], binA[q],
                                   binC[q], bad);
            rkA[q] = atomicAdd(&hA[binA[q]], 1);
            if (ngrids == 3) rkC[q] = atomicAdd(&hC[binC[q]], 1);
        }
    }
    __syncthreads();
    for (int i = tid; i < nb; i += kSegThreads) {
        const int ca = hA[i];
        if (ca) hA[i] = atomicAdd(&curAB[cv.bin_off + i], ca);
        if (ngrids == 3) {
            const int cc = hC[i];
            if (cc) hC[i] = atomicAdd(&curC[cv.bin_off + i], cc);
        }
    }
    __syncthreads();
    RecAB *rA = recAB + cv.rec_off;
    RecC *rC = recC + cv.rec_off;
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        if (binA[q] < 0) continue;
        // a slot outside the curve's n records would mean that the count and
        // the scatter binned a point differently: flag it, write nothing
        const int sa = hA[binA[q]] + rkA[q];
        if ((unsigned)sa < (unsigned)n) rA[sa] = ra[q];
        else lost = true;
        if (ngrids == 3) {
            const int sc = hC[binC[q]] + rkC[q];
            if ((unsigned)sc < (unsigned)n) rC[sc] = rc[q];
            else lost = true;
        }
    }
    if (bad) atomicOr(errflag, 1u);
    if (lost) atomicOr(errflag, 4u);
}

// ---------------------------------------------------------------------------
// reference-convention gridding (just_return_gridded_data)
// ---------------------------------------------------------------------------
__global__ void k_spread_ref(const RefGridCurve *__restrict__ cvs,
                             const double *__restrict__ t,
                             const float *__restrict__ y, float *__restrict__ grid,
                             int m, float binv, float norm) {
    const RefGridCurve cv = cvs[blockIdx.y];
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= cv.n) return;
    const double x = (t[cv.pt_off + j] - cv.tmin) * cv.scale;
    const double gx = (double)cv.ng * x;
    const long long u = (long long)floor(gx - (double)m);
    const float yj = y[cv.pt_off + j];
    for (int k = 0; k <= 2 * m; ++k) {
        const float d = (float)(gx - (double)(u + k));
        const float wg = expf(-d * d * binv) * norm;
        long long l = (u + k) % cv.ng;
        if (l < 0) l += cv.ng;
        atomicAdd(&grid[cv.out_off + l], yj * wg);
    }
}

// ---------------------------------------------------------------------------
// FP64 adjoint NFFT by direct summation (use_double)
// ---------------------------------------------------------------------------
// One thread per kDirBins consecutive bins of one curve.  Points are staged
// 128 at a time as (frac(f0 t), frac(df t), y); for each point the phasor of
// the thread's first bin comes from sincospi and the next bins by
// multiplication with exp(2 pi i df t) (kDirBins - 1 steps).
constexpr int kDirBins = 8;

__global__ void __launch_bounds__(128)
k_nfft_direct64(const Direct64Curve *__restrict__ cvs, const double *__restrict__ t,
                const double *__restrict__ y, double2 *__restrict__ out) {
    __shared__ double sa[128], sb[128], sy[128];
    const Direct64Curve cv = cvs[blockIdx.y];
    const long long k0 = ((long long)blockIdx.x * 128 + threadIdx.x) * kDirBins;
    double re[kDirBins], im[kDirBins];
#pragma unroll
    for (int q = 0; q < kDirBins; ++q) { re[q] = 0.0; im[q] = 0.0; }
    const double kd = (double)k0;
    for (long long base = 0; base < cv.n; base += 128) {
        const long long j = base + threadIdx.x;
        __syncthreads();  // the previous tile is consumed
        if (j < cv.n) {
            const double tj = t[cv.pt_off + j];
            double a = cv.f0 * tj;
            a -= floor(a);
            double b = cv.df * tj;
            b -= floor(b);
            sa[threadIdx.x] = a;
            sb[threadIdx.x] = b;
            sy[threadIdx.x] = y[cv.pt_off + j];
        }
        __syncthreads();
        const int cnt = (int)min((long long)128, cv.n - base);
        if (k0 < cv.nf) {
            for (int q = 0; q < cnt; ++q) {
                double ph = fma(kd, sb[q], sa[q]);
                ph -= floor(ph);
                double s, c, ss, cs;
                sincospi(2.0 * ph, &s, &c);
                sincospi(2.0 * sb[q], &ss, &cs);
                const double yq = sy[q];
#pragma unroll
                for (int r = 0; r < kDirBins; ++r) {
                    re[r] = fma(yq, c, re[r]);
                    im[r] = fma(yq, s, im[r]);
                    const double c2 = c * cs - s * ss;
                    s = fma(s, cs, c * ss);
                    c = c2;
                }
            }
        }
    }
#pragma unroll
    for (int r = 0; r < kDirBins; ++r)
        if (k0 + r < cv.nf) out[cv.out_off + k0 + r] = make_double2(re[r], im[r]);
}

cudaError_t launch_nfft_direct64(const Direct64Curve *cv, int n_curves, long long max_nf,
                                 const double *t, const double *y, double2 *out,
                                 cudaStream_t s) {
    if (n_curves <= 0 || max_nf <= 0) return cudaSuccess;
    const long long nb = (max_nf + 128LL * kDirBins - 1) / (128LL * kDirBins);
    if (nb > 0x7fffffffLL || n_curves > 65535) return cudaErrorInvalidValue;
    k_nfft_direct64<<<dim3((unsigned)nb, n_curves), 128, 0, s>>>(cv, t, y, out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// finish of a caller-given reference-convention grid (use_grid)
// ---------------------------------------------------------------------------
// One thread per output bin k; the grid is staged 128 cells at a time and
// exp(2 pi i j (ks + k) / ng) advances by multiplication along j, re-seeded
// from sincospi at every tile.
__global__ void __launch_bounds__(128)
k_grid_finish(const GridFinishCurve *__restrict__ cvs, const double2 *__restrict__ grid,
              double2 *__restrict__ out) {
    __shared__ double2 sg[128];
    const GridFinishCurve cv = cvs[blockIdx.y];
    const long long k = (long long)blockIdx.x * 128 + threadIdx.x;
    const double ng = (double)cv.ng;
    const double fr = (cv.ks + (double)k) / ng;  // cycles per grid cell
    double step_s, step_c;
    {
        double st = fr - floor(fr);
        sincospi(2.0 * st, &step_s, &step_c);
    }
    double re = 0.0, im = 0.0;
    for (long long base = 0; base < cv.ng; base += 128) {
        const long long j = base + threadIdx.x;
        __syncthreads();
        if (j < cv.ng) sg[threadIdx.x] = grid[cv.grid_off + j];
        __syncthreads();
        const int cnt = (int)min((long long)128, cv.ng - base);
        if (k < cv.nf) {
            double ph = fr * (double)base;
            ph -= floor(ph);
            double s, c;
            sincospi(2.0 * ph, &s, &c);
            for (int q = 0; q < cnt; ++q) {
                const double2 g = sg[q];
                re = fma(g.x, c, fma(-g.y, s, re));
                im = fma(g.x, s, fma(g.y, c, im));
                const double c2 = c * step_c - s * step_s;
                s = fma(s, step_c, c * step_s);
                c = c2;
            }
        }
    }
    if (k < cv.nf) {
        const double kk = cv.k0 + (double)k;
        double th = cv.n0 * kk / ng;
        th -= floor(th);
        double s, c;
        sincospi(2.0 * th, &s, &c);
        const double kh = kk / ng;  // khat / pi
        const double pk = 3.141592653589793 * kh;
        const double sc = exp(cv.b * pk * pk);
        out[cv.out_off + k] = make_double2((re * c - im * s) * sc, (re * s + im * c) * sc);
    }
}

cudaError_t launch_grid_finish(const GridFinishCurve *cv, int n_curves, long long max_nf,
                               const double2 *grid, double2 *out, cudaStream_t s) {
    if (n_curves <= 0 || max_nf <= 0) return cudaSuccess;
    const long long nb = (max_nf + 127) / 128;
    if (nb > 0x7fffffffLL || n_curves > 65535) return cudaErrorInvalidValue;
    k_grid_finish<<<dim3((unsigned)nb, n_curves), 128, 0, s>>>(cv, grid, out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// multi-harmonic floating-mean GLS by FP64 direct sums
// ---------------------------------------------------------------------------
// One thread per frequency; points staged 128 at a time.  Per point the
// phasor exp(i phi) comes from sincospi of frac(t f) and its powers
// n = 2 .. 2H by multiplication.  Then the sums of
// cuvarbase/lombscargle.py:337-400 (mhdirect_sums) with the regulariser of
// :403-447, the 2H x 2H system solved by Gaussian elimination with partial
// pivoting, and the power of :497-536.
template <int H>
__global__ void __launch_bounds__(128)
k_mhgls_direct(const double *__restrict__ t, const double *__restrict__ yw,
               const double *__restrict__ w, long long n, const double *__restrict__ freqs,
               long long nf, MhParams mp, double *__restrict__ out) {
    constexpr int NH = 2 * H;
    __shared__ double st[128], sy[128], sw[128];
    const long long k = (long long)blockIdx.x * 128 + threadIdx.x;
    const double f = (k < nf) ? freqs[k] : 0.0;
    double c[NH + 1], s[NH + 1], yc[H + 1], ys[H + 1];
#pragma unroll
    for (int m = 0; m <= NH; ++m) { c[m] = 0.0; s[m] = 0.0; }
#pragma unroll
    for (int m = 0; m <= H; ++m) { yc[m] = 0.0; ys[m] = 0.0; }
    for (long long base = 0; base < n; base += 128) {
        const long long j = base + threadIdx.x;
        __syncthreads();  // the previous tile is consumed
        if (j < n) {
            st[threadIdx.x] = t[j];
            sy[threadIdx.x] = yw[j];
            sw[threadIdx.x] = w[j];
        }
        __syncthreads();
        const int cnt = (int)min((long long)128, n - base);
        if (k < nf) {
            for (int q = 0; q < cnt; ++q) {
                double ph = st[q] * f;
                ph -= floor(ph);
                double s1, c1;
                sincospi(2.0 * ph, &s1, &c1);
                const double wq = sw[q], yq = sy[q];
                c[0] += wq;
                double cn = c1, sn = s1;
#pragma unroll
                for (int m = 1; m <= NH; ++m) {
                    c[m] = fma(wq, cn, c[m]);
                    s[m] = fma(wq, sn, s[m]);
                    if (m <= H) {
                        yc[m] = fma(yq, cn, yc[m]);
                        ys[m] = fma(yq, sn, ys[m]);
                    }
                    const double cn2 = cn * c1 - sn * s1;
                    sn = fma(cn, s1, sn * c1);
                    cn = cn2;
                }
            }
        }
    }
    if (k >= nf) return;
    // regularised blocks: M = [[CC, CS], [CS^T, SS]], rhs = [YC; YS]
    double M[NH][NH], rhs[NH];
#pragma unroll
    for (int a = 1; a <= H; ++a) {
#pragma unroll
        for (int b = 1; b <= H; ++b) {
            const int dd = a > b ? a - b : b - a;
            const double sg = (a >= b) ? 1.0 : -1.0;  // sign(a - b), 1 at a == b
            const double reg = (a == b) ? mp.d[a - 1] : 0.0;
            const double cc = 0.5 * (c[a + b] + c[dd]) - c[a] * c[b] + reg;
            const double cs = 0.5 * (s[a + b] - sg * s[dd]) - c[a] * s[b];
            const double ss = 0.5 * (c[dd] - c[a + b]) - s[a] * s[b] + reg;
            M[a - 1][b - 1] = cc;
            M[a - 1][H + b - 1] = cs;
            M[H + b - 1][a - 1] = cs;
            M[H + a - 1][H + b - 1] = ss;
        }
        rhs[a - 1] = yc[a] - mp.ybar * c[a] + mp.d[a - 1] * mp.cn0[a - 1];
        rhs[H + a - 1] = ys[a] - mp.ybar * s[a] + mp.d[a - 1] * mp.sn0[a - 1];
    }
    // Gaussian elimination with partial pivoting on a copy
    double W[NH][NH + 1];
#pragma unroll
    for (int r = 0; r < NH; ++r) {
#pragma unroll
        for (int q = 0; q < NH; ++q) W[r][q] = M[r][q];
        W[r][NH] = rhs[r];
    }
    bool singular = false;
    for (int col = 0; col < NH; ++col) {
        int piv = col;
        double best = fabs(W[col][col]);
        for (int r = col + 1; r < NH; ++r)
            if (fabs(W[r][col]) > best) { best = fabs(W[r][col]); piv = r; }
        if (!(best > 0.0)) { singular = true; break; }
        if (piv != col)
            for (int q = col; q <= NH; ++q) {
                const double tmp = W[col][q];
                W[col][q] = W[piv][q];
                W[piv][q] = tmp;
            }
        for (int r = col + 1; r < NH; ++r) {
            const double fct = W[r][col] / W[col][col];
            for (int q = col; q <= NH; ++q) W[r][q] = fma(-fct, W[col][q], W[r][q]);
        }
    }
    double th[NH];
    if (!singular) {
        for (int r = NH - 1; r >= 0; --r) {
            double v = W[r][NH];
            for (int q = r + 1; q < NH; ++q) v = fma(-W[r][q], th[q], v);
            th[r] = v / W[r][r];
        }
    }
    if (singular) {
        out[k] = nan("");
        return;
    }
    // P = (YX - sum XX) / YY with the regularised blocks
    double xx = 0.0, yx = 0.0;
#pragma unroll
    for (int a = 0; a < H; ++a) {
        yx += th[a] * rhs[a] + th[H + a] * rhs[H + a];
#pragma unroll
        for (int b = 0; b < H; ++b)
            xx += th[a] * th[b] * M[a][b] + 2.0 * th[a] * th[H + b] * M[a][H + b] +
                  th[H + a] * th[H + b] * M[H + a][H + b];
    }
    out[k] = (2.0 * yx - xx) / mp.yy;
}

cudaError_t launch_mhgls_direct(int nharms, const double *t, const double *yw, const double *w,
                                long long n, const double *freqs, long long nf,
                                const MhParams &mp, double *out, cudaStream_t s) {
    if (n <= 0 || nf <= 0) return cudaSuccess;
    const long long nb = (nf + 127) / 128;
    if (nb > 0x7fffffffLL) return cudaErrorInvalidValue;
    const dim3 g((unsigned)nb);
    switch (nharms) {
#define CUVGLS_MH(HH) \
    case HH: k_mhgls_direct<HH><<<g, 128, 0, s>>>(t, yw, w, n, freqs, nf, mp, out); break;
        CUVGLS_MH(1) CUVGLS_MH(2) CUVGLS_MH(3) CUVGLS_MH(4)
        CUVGLS_MH(5) CUVGLS_MH(6) CUVGLS_MH(7) CUVGLS_MH(8)
#undef CUVGLS_MH
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// direct sums (FP64 phases and accumulation): GPU cross-check path
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
k_gls_direct(const DevCurve *__restrict__ cvs, const double *__restrict__ t,
             const float *__restrict__ yw, const float *__restrict__ w,
             float *__restrict__ out, GlsParams gp) {
    __shared__ double st[256];
    __shared__ float syw[256], sw[256];
    const DevCurve cv = cvs[blockIdx.y];
    const int k = blockIdx.x * 256 + threadIdx.x;
    const bool act = k < cv.nf;
    const double f = (cv.kc - (double)(cv.nf / 2) + (double)k) * cv.df;
    double C = 0, S = 0, C2 = 0, S2 = 0, YC = 0, YS = 0;
    for (int base = 0; base < cv.n; base += 256) {
        const int j = base + threadIdx.x;
        __syncthreads();
        if (j < cv.n) {
            st[threadIdx.x] = t[cv.pt_off + j];
            syw[threadIdx.x] = yw[cv.pt_off + j];
            sw[threadIdx.x] = w[cv.pt_off + j];
        }
        __syncthreads();
        const int cnt = min(256, cv.n - base);
        if (act) {
            for (int jj = 0; jj < cnt; ++jj) {
                double ph = f * st[jj];
                ph -= floor(ph);
                double s, c;
                sincospi(2.0 * ph, &s, &c);
                const double c2 = c * c - s * s, s2 = 2.0 * c * s;
                const double wj = sw[jj], yj = syw[jj];
                C += wj * c; S += wj * s; C2 += wj * c2; S2 += wj * s2;
                YC += yj * c; YS += yj * s;
            }
        }
    }
    if (act) {
        const double P = gls_from_sums<double>(
            YC, YS, C, S, C2, S2, gp.mode, (double)gp.reg, (double)cv.w_sum,
            (double)cv.yw_sum, (double)cv.ybar, (double)cv.yy_inv);
        out[cv.out_off + k] = (float)P;
    }
}

// ---------------------------------------------------------------------------
// plan tables (FP64 angles, rounded once to float)
// ---------------------------------------------------------------------------
// Turns (fraction of a full turn) of entry e of the FFT table of a length-L
// transform, in the layout the pass kernels read: [qa][i] stage-A twiddles
// i qa / L of a two-level length, else [stage][r - 1][k] Stockham twiddles.
__device__ double fft_table_turns(int L, int e) {
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

__global__ void k_plan_tables(float2 *dst, int G1, int G2, int B, int n1, int n2) {
    const long long G = (long long)G1 * G2;
    const long long total = n1 + n2 + G;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        double turns;
        if (e < n1) {
            turns = fft_table_turns(G1, (int)e);
        } else if (e < n1 + n2) {
            turns = fft_table_turns(G2, (int)(e - n1));
        } else {
            // inter-pass twiddle in the intermediate's [cb][q1][c] order
            const long long i = e - n1 - n2;
            const int c = (int)(i % B);
            const long long rest = i / B;
            const int q1 = (int)(rest % G1), cb = (int)(rest / G1);
            const long long l2 = (long long)cb * B + c;
            turns = (double)(((long long)q1 * l2) % G) / (double)G;
        }
        double s, c;
        sincospi(2.0 * turns, &s, &c);
        dst[e] = make_float2((float)c, (float)s);
    }
}

// Deconvolution table of the ES window: dst[j] = 1 / phihat(j), j = 0..n-1,
// with phihat(j) = 2 int_0^m phi(s) cos(2 pi j s / G) ds the Fourier
// transform of phi(s) = exp(beta (sqrt(1 - s^2 / m^2) - 1)) at band index j,
// in FP64 by the midpoint rule over kEsNodes nodes (phi and its derivatives
// are smooth inside [0, m); at s = m phi is e^-beta, ~1e-8, so the rule's
// endpoint error is far below FP32).  The cosines come from a rotation
// recurrence re-seeded every 64 nodes.
constexpr int kEsNodes = 256;

__global__ void __launch_bounds__(256) k_es_deconv(float *dst, int n, double G, int m,
                                                   double beta) {
    __shared__ double phi[kEsNodes];
    const double h = (double)m / kEsNodes;
    for (int q = threadIdx.x; q < kEsNodes; q += blockDim.x) {
        const double z = (q + 0.5) * h / m;
        phi[q] = exp(beta * (sqrt(1.0 - z * z) - 1.0));
    }
    __syncthreads();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const double th = 2.0 * (double)j * h / G;  // rotation per node, in half turns
    double sr, cr;
    sincospi(th, &sr, &cr);
    double acc = 0.0;
    for (int q0 = 0; q0 < kEsNodes; q0 += 64) {
        double zs, zc;
        sincospi(th * (q0 + 0.5), &zs, &zc);
        for (int q = q0; q < q0 + 64; ++q) {
            acc = fma(phi[q], zc, acc);
            const double nc = zc * cr - zs * sr;
            zs = fma(zc, sr, zs * cr);
            zc = nc;
        }
    }
    dst[j] = (float)(1.0 / (2.0 * h * acc));
}

// Sum of a double over the CTA (blockDim.x a multiple of 32, <= 1024);
// every thread gets the total.
__device__ double block_sum(double v, double *red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();  // red is reused across calls
    if (lane == 0) red[wid] = v;
    __syncthreads();
    double t = 0.0;
    for (int i = 0; i < nw; ++i) t += red[i];
    return t;
}

// Sum of the partials part[first .. first + n) in a fixed order (lane
// stride, then a butterfly): every lane gets the same total, and every
// caller reducing the same range gets the same bits.
__device__ __forceinline__ double4 warp_sum_parts(const double4 *__restrict__ part, int first,
                                                  int n, int lane) {
    double4 a = make_double4(0.0, 0.0, 0.0, 0.0);
    for (int k = lane; k < n; k += 32) {
        const double4 v = part[first + k];
        a.x += v.x;
        a.y += v.y;
        a.z += v.z;
        a.w += v.w;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a.x += __shfl_xor_sync(0xffffffffu, a.x, o);
        a.y += __shfl_xor_sync(0xffffffffu, a.y, o);
        a.z += __shfl_xor_sync(0xffffffffu, a.z, o);
        a.w += __shfl_xor_sync(0xffffffffu, a.w, o);
    }
    return a;
}

// Normalisation and statistics of a descriptor from its curve's totals:
// YY, ybar (relative to the unweighted nan-mean of y, as cuvarbase's
// normalize_light_curves leaves it), sum(yw), sum(w), and the scale of the
// mode.
__device__ __forceinline__ void fill_stats(DevCurve &cv, double4 a, double4 b, int mode) {
    const double yy = b.x;
    const double ybar = a.y / a.x - a.z / a.w;
    double norm = 1.0;
    if (mode == 1) norm = 1.0 / yy;
    else if (mode == 0) norm = 1.0 / (yy + ybar * ybar);
    cv.yy_inv = (float)norm;
    cv.ybar = (float)ybar;
    cv.yw_sum = (float)b.y;
    cv.w_sum = (float)b.z;
}

// Partial sums of raw points [j0, j1) over the CTA: sum dy^-2, sum y dy^-2
// and the nan-mean parts (sum and count of the non-NaN y); each dy^-2 is kept
// in ir for the second pass (one FP64 division per point).
__device__ __forceinline__ double4 raw_sums(const double *__restrict__ y,
                                            const double *__restrict__ dy,
                                            double *__restrict__ ir, long long o, int j0,
                                            int j1, double *red) {
    double sw = 0.0, swy = 0.0, sy = 0.0, cy = 0.0;
    for (int j = j0 + threadIdx.x; j < j1; j += kSegThreads) {
        const double yj = y[o + j], dj = dy[o + j];
        const double wj = 1.0 / (dj * dj);
        ir[o + j] = wj;
        sw += wj;
        swy += wj * yj;
        if (!isnan(yj)) { sy += yj; cy += 1.0; }
    }
    sw = block_sum(sw, red);
    swy = block_sum(swy, red);
    sy = block_sum(sy, red);
    cy = block_sum(cy, red);
    return make_double4(sw, swy, sy, cy);
}

// w = dy^-2 / sw and yw = w (y - ybar_w) as FP32 for raw points [j0, j1),
// and their sums over the CTA: YY and the stored FP32 yw and w.
__device__ __forceinline__ double4 raw_weights(const double *__restrict__ y,
                                               const double *__restrict__ ir,
                                               float *__restrict__ yw, float *__restrict__ w,
                                               long long o, int j0, int j1, double sw,
                                               double ybar_w, double *red) {
    double yy = 0.0, ys = 0.0, ws = 0.0;
    const double inv_sw = 1.0 / sw;
    for (int j = j0 + threadIdx.x; j < j1; j += kSegThreads) {
        const double wj = ir[o + j] * inv_sw;  // dy^-2 from raw_sums
        const double d = y[o + j] - ybar_w;
        yy += wj * d * d;
        const float ywf = (float)(wj * d), wf = (float)wj;
        yw[o + j] = ywf;
        w[o + j] = wf;
        ys += (double)ywf;
        ws += (double)wf;
    }
    yy = block_sum(yy, red);
    ys = block_sum(ys, red);
    ws = block_sum(ws, red);
    return make_double4(yy, ys, ws, 0.0);
}

// Raw input, step 1, one CTA per segment of a curve longer than one segment
// (CTAs of shorter curves return at once): its partial sums into partA.
__global__ void __launch_bounds__(kSegThreads)
k_raw_sums(const SegEntry *__restrict__ segs, const DevCurve *__restrict__ cvs,
           const double *__restrict__ y, const double *__restrict__ dy,
           double *__restrict__ ir, double4 *__restrict__ partA) {
    __shared__ double red[32];
    const SegEntry sg = segs[blockIdx.x];
    const DevCurve &cv = cvs[sg.desc];
    const int n = cv.n;
    if (n <= kSegPoints) return;  // uniform over the CTA
    const double4 a =
        raw_sums(y, dy, ir, cv.pt_off, sg.start, min(n, sg.start + kSegPoints), red);
    if (threadIdx.x == 0) partA[cv.raw_seg + sg.start / kSegPoints] = a;
}

// Raw input, step 2, one CTA per segment.  A curve of one segment is done
// here completely: its sums (partA), w and yw, the sums of YY, yw and w
// (partB) and, for a curve of one band (kDescFillHere), the descriptor's
// statistics.  A segment of a longer curve: the curve's totals from step 1,
// then w, yw and the segment's partB.
__global__ void __launch_bounds__(kSegThreads)
k_raw_finish(const SegEntry *__restrict__ segs, DevCurve *__restrict__ cvs,
             const double *__restrict__ y, const double *__restrict__ dy,
             const double *__restrict__ ir, float *__restrict__ yw, float *__restrict__ w,
             double4 *__restrict__ partA, double4 *__restrict__ partB, int mode) {
    __shared__ double red[32];
    __shared__ double4 tot;
    const SegEntry sg = segs[blockIdx.x];
    DevCurve &cv = cvs[sg.desc];
    const long long o = cv.pt_off;
    const int n = cv.n;
    const int seg = cv.raw_seg + sg.start / kSegPoints;  // index of the partials
    if (n <= kSegPoints) {  // uniform over the CTA
        // the whole curve, kSegPoints / kSegThreads points per thread: dy^-2
        // and y kept in registers between the sums and the weights (one
        // FP64 division per point)
        constexpr int PPT = kSegPoints / kSegThreads;
        double ir[PPT], yr[PPT];
        double sw = 0.0, swy = 0.0, sy = 0.0, cy = 0.0;
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            const int j = threadIdx.x + q * kSegThreads;
            ir[q] = 0.0;
            yr[q] = 0.0;
            if (j < n) {
                const double yj = y[o + j], dj = dy[o + j];
                ir[q] = 1.0 / (dj * dj);
                yr[q] = yj;
                sw += ir[q];
                swy += ir[q] * yj;
                if (!isnan(yj)) { sy += yj; cy += 1.0; }
            }
        }
        sw = block_sum(sw, red);
        swy = block_sum(swy, red);
        sy = block_sum(sy, red);
        cy = block_sum(cy, red);
        const double4 a = make_double4(sw, swy, sy, cy);
        const double ybar_w = swy / sw, inv_sw = 1.0 / sw;
        double yy = 0.0, ys = 0.0, ws = 0.0;
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            const int j = threadIdx.x + q * kSegThreads;
            if (j < n) {
                const double wj = ir[q] * inv_sw;
                const double d = yr[q] - ybar_w;
                yy += wj * d * d;
                const float ywf = (float)(wj * d), wf = (float)wj;
                yw[o + j] = ywf;
                w[o + j] = wf;
                ys += (double)ywf;
                ws += (double)wf;
            }
        }
        yy = block_sum(yy, red);
        ys = block_sum(ys, red);
        ws = block_sum(ws, red);
        const double4 b = make_double4(yy, ys, ws, 0.0);
        if (threadIdx.x == 0) {
            partA[seg] = a;
            partB[seg] = b;
            if (cv.flags & kDescFillHere) fill_stats(cv, a, b, mode);
        }
        return;
    }
    if (threadIdx.x < 32) {
        const double4 a = warp_sum_parts(partA, cv.raw_seg, seg_count(n), threadIdx.x);
        if (threadIdx.x == 0) tot = a;
    }
    __syncthreads();
    const double4 a = tot;
    const double4 b = raw_weights(y, ir, yw, w, o, sg.start, min(n, sg.start + kSegPoints), a.x,
                                  a.y / a.x, red);
    if (threadIdx.x == 0) partB[seg] = b;
}

// Raw input, step 3, one warp per band descriptor not filled by
// k_raw_finish: its curve's totals from the segment partials, then
// fill_stats.
__global__ void __launch_bounds__(128)
k_fill_desc(DevCurve *__restrict__ cvs, int n, const double4 *__restrict__ partA,
            const double4 *__restrict__ partB, int mode) {
    const int i = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (i >= n) return;  // whole warps
    const int lane = threadIdx.x & 31;
    DevCurve &cv = cvs[i];
    if (cv.flags & kDescFillHere) return;
    const int ns = seg_count(cv.n);
    const double4 a = warp_sum_parts(partA, cv.raw_seg, ns, lane);
    const double4 b = warp_sum_parts(partB, cv.raw_seg, ns, lane);
    if (lane == 0) fill_stats(cv, a, b, mode);
}

cudaError_t launch_seg_fill(const DevCurve *cv, int n, SegEntry *bin_segs, SegEntry *raw_segs,
                            cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_seg_fill<<<n, 64, 0, s>>>(cv, bin_segs, raw_segs);
    return cudaGetLastError();
}

cudaError_t launch_raw_sums(const SegEntry *segs, int n_segs, const DevCurve *cv,
                            const double *y, const double *dy, double *ir, double4 *partA,
                            cudaStream_t s) {
    if (n_segs <= 0) return cudaSuccess;
    k_raw_sums<<<n_segs, kSegThreads, 0, s>>>(segs, cv, y, dy, ir, partA);
    return cudaGetLastError();
}

cudaError_t launch_raw_finish(const SegEntry *segs, int n_segs, DevCurve *cv, const double *y,
                              const double *dy, const double *ir, float *yw, float *w,
                              double4 *partA, double4 *partB, int mode, cudaStream_t s) {
    if (n_segs <= 0) return cudaSuccess;
    k_raw_finish<<<n_segs, kSegThreads, 0, s>>>(segs, cv, y, dy, ir, yw, w, partA, partB, mode);
    return cudaGetLastError();
}

cudaError_t launch_fill_desc(DevCurve *cv, int n, const double4 *partA, const double4 *partB,
                             int mode, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_fill_desc<<<(n + 3) / 4, 128, 0, s>>>(cv, n, partA, partB, mode);
    return cudaGetLastError();
}

__global__ void k_best_finish(const unsigned long long *__restrict__ keys, int n,
                              int64_t *__restrict__ best_k, float *__restrict__ best_p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long k = keys[i];
    if (k == 0) {
        best_k[i] = -1;
        best_p[i] = -1.f;
    } else {
        best_k[i] = (int64_t)(0xFFFFFFFFu - (unsigned)(k & 0xFFFFFFFFull));
        best_p[i] = __uint_as_float((unsigned)(k >> 32));
    }
}

cudaError_t launch_best_finish(const unsigned long long *keys, int n, int64_t *best_k,
                               float *best_p, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_best_finish<<<(n + 255) / 256, 256, 0, s>>>(keys, n, best_k, best_p);
    return cudaGetLastError();
}

cudaError_t launch_plan_tables(float2 *dst, int G1, int G2, int B, cudaStream_t s) {
    const int n1 = fft_table_len(G1), n2 = fft_table_len(G2);
    const long long total = n1 + n2 + (long long)G1 * G2;
    const int blocks = (int)std::min<long long>((total + 255) / 256, 4096);
    k_plan_tables<<<blocks, 256, 0, s>>>(dst, G1, G2, B, n1, n2);
    return cudaGetLastError();
}

cudaError_t launch_es_deconv(float *dst, long long G, int m, double beta, cudaStream_t s) {
    if (G < 2 || m < 1) return cudaErrorInvalidValue;
    const int n = (int)(G / 2 + 1);
    k_es_deconv<<<(n + 255) / 256, 256, 0, s>>>(dst, n, (double)G, m, beta);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
cudaError_t launch_bin_count(const SegEntry *segs, int n_segs, const DevCurve *cv,
                             const double *t, int *binsAB, int *binsC, const Plan &p,
                             int ngrids, int fp32_positions, cudaStream_t s) {
    if (n_segs <= 0) return cudaSuccess;
    if (p.nb > kMaxBins) return cudaErrorInvalidValue;
    if (fp32_positions)
        k_bin_count<true><<<n_segs, kSegThreads, 0, s>>>(segs, cv, t, binsAB, binsC, p, ngrids);
    else
        k_bin_count<false><<<n_segs, kSegThreads, 0, s>>>(segs, cv, t, binsAB, binsC, p, ngrids);
    return cudaGetLastError();
}

cudaError_t launch_bin_scan(const DevCurve *cv, int n_curves, const double *t, int *binsAB,
                            int *binsC, int *curAB, int *curC, float4 *aux, const Plan &p,
                            int ngrids, cudaStream_t s) {
    if (n_curves <= 0) return cudaSuccess;
    k_bin_scan<<<(n_curves + 3) / 4, 128, 0, s>>>(cv, n_curves, t, binsAB, binsC, curAB, curC,
                                                  aux, p.nb, ngrids);
    return cudaGetLastError();
}

cudaError_t launch_bin_scatter(const SegEntry *segs, int n_segs, const DevCurve *cv,
                               const double *t, const float *ya, const float *wv,
                               RecAB *recAB, RecC *recC, int *binsAB, int *binsC, int *curAB,
                               int *curC, float4 *aux, const Plan &p, int ngrids,
                               int fp32_positions, unsigned *errflag, cudaStream_t s) {
    if (n_segs <= 0) return cudaSuccess;
    if (p.nb > kMaxBins) return cudaErrorInvalidValue;
    if (fp32_positions)
        k_bin_scatter<true><<<n_segs, kSegThreads, 0, s>>>(segs, cv, t, ya, wv, recAB, recC,
                                                           binsAB, binsC, curAB, curC, aux, p,
                                                           ngrids, errflag);
    else
        k_bin_scatter<false><<<n_segs, kSegThreads, 0, s>>>(segs, cv, t, ya, wv, recAB, recC,
                                                            binsAB, binsC, curAB, curC, aux, p,
                                                            ngrids, errflag);
    return cudaGetLastError();
}

#define CUVGLS_LEN_CASES(X) X(16) X(32) X(64) X(80) X(128) X(160) X(256) X(320) \
    X(400) X(512) X(640) X(800) X(1024) X(1280) X(1600) X(2048)
#define CUVGLS_ROW_LEN_CASES(X) CUVGLS_LEN_CASES(X) X(4096)

cudaError_t launch_pass1(const DevCurve *cv, int n_curves, const RecAB *recAB,
                         const RecC *recC, const int *binsAB, const int *binsC,
                         float2 *inter, const Plan &p, int ngrids, cudaStream_t s) {
    if (n_curves <= 0) return cudaSuccess;
#define CUVGLS_P1(L) \
    case L: return ngrids == 3 ? launch_pass1_t<3, L>(cv, n_curves, recAB, recC, binsAB, binsC, inter, p, s) \
                               : launch_pass1_t<1, L>(cv, n_curves, recAB, recC, binsAB, binsC, inter, p, s);
    switch (p.G1) {
        CUVGLS_LEN_CASES(CUVGLS_P1)
        default: return cudaErrorInvalidValue;
    }
#undef CUVGLS_P1
}

cudaError_t preload_pass_kernels(int G1, int G2, int ngrids) {
    cudaError_t e = cudaErrorInvalidValue;
#define CUVGLS_PL1(L) \
    case L: e = ngrids == 3 ? preload_pass1_t<3, L>() : preload_pass1_t<1, L>(); break;
    switch (G1) {
        CUVGLS_LEN_CASES(CUVGLS_PL1)
        default: return cudaErrorInvalidValue;
    }
#undef CUVGLS_PL1
    if (e != cudaSuccess) return e;
#define CUVGLS_PL2(L) case L: return preload_pass2_t<L>(ngrids);
    switch (G2) {
        CUVGLS_ROW_LEN_CASES(CUVGLS_PL2)
        default: return cudaErrorInvalidValue;
    }
#undef CUVGLS_PL2
}

cudaError_t launch_pass2_gls(const DevCurve *cv, int n_curves,
                             const float2 *inter, float *out, const Plan &p,
                             GlsParams g, cudaStream_t s) {
    if (n_curves <= 0) return cudaSuccess;
#define CUVGLS_P2(L) case L: return launch_pass2_gls_t<L>(cv, n_curves, inter, out, p, g, s);
    switch (p.G2) {
        CUVGLS_ROW_LEN_CASES(CUVGLS_P2)
        default: return cudaErrorInvalidValue;
    }
#undef CUVGLS_P2
}

cudaError_t launch_pass2_nfft(const DevCurve *cv, int n_curves,
                              const float2 *inter, float2 *out,
                              const float4 *aux, const Plan &p, cudaStream_t s) {
    if (n_curves <= 0) return cudaSuccess;
#define CUVGLS_P2N(L) case L: return launch_pass2_nfft_t<L>(cv, n_curves, inter, out, aux, p, s);
    switch (p.G2) {
        CUVGLS_ROW_LEN_CASES(CUVGLS_P2N)
        default: return cudaErrorInvalidValue;
    }
#undef CUVGLS_P2N
}

cudaError_t launch_spread_ref(const RefGridCurve *cv, int n_curves,
                              long long max_n, const double *t, const float *y,
                              float *grid, int m, float binv, float norm,
                              cudaStream_t s) {
    if (n_curves <= 0 || max_n <= 0) return cudaSuccess;
    dim3 g((unsigned)((max_n + 255) / 256), n_curves);
    k_spread_ref<<<g, 256, 0, s>>>(cv, t, y, grid, m, binv, norm);
    return cudaGetLastError();
}

cudaError_t launch_gls_direct(const DevCurve *cv, int n_curves, int max_nf,
                              const double *t, const float *yw, const float *w,
                              float *out, GlsParams g, cudaStream_t s) {
    if (n_curves <= 0 || max_nf <= 0) return cudaSuccess;
    dim3 grid((max_nf + 255) / 256, n_curves);
    k_gls_direct<<<grid, 256, 0, s>>>(cv, t, yw, w, out, g);
    return cudaGetLastError();
}

}  // namespace cuvgls
