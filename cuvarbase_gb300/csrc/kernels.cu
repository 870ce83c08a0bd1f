// cuvgls kernels for sm_103a.
//
// The path per size class (G = G1 * G2 grid cells):
//   k_prep_bin   one CTA per curve.  FP64 offsets t - t0, grid cell index and
//                band-centring phase per point; counting sort of the points by
//                the column block (cell mod G2) / B their Gaussian window
//                starts in.  Writes compact FP32 spreading records.
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

#include "fft.cuh"
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

// Exclusive scan of h[0..n) in place (warp 0 only); h[n] = total.
__device__ __forceinline__ void warp_exclusive_scan(int *h, int n) {
    const int lane = threadIdx.x & 31;
    int carry = 0;
    for (int base = 0; base < n; base += 32) {
        int i = base + lane;
        int x = (i < n) ? h[i] : 0;
        int inc = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (i < n) h[i] = carry + inc - x;
        carry += __shfl_sync(0xffffffffu, inc, 31);
    }
    if (lane == 0) h[n] = carry;
}

template <bool FP32POS>
__global__ void __launch_bounds__(512)
k_prep_bin(const DevCurve *__restrict__ cvs, const double *__restrict__ t,
           const float *__restrict__ ya, const float *__restrict__ wv,
           RecAB *__restrict__ recAB, RecC *__restrict__ recC,
           int *__restrict__ binsAB, int *__restrict__ binsC,
           float4 *__restrict__ aux, Plan p, int ngrids,
           unsigned *__restrict__ errflag) {
    __shared__ int hA[kMaxBins + 1];
    __shared__ int hC[kMaxBins + 1];
    const DevCurve cv = cvs[blockIdx.x];
    const int tid = threadIdx.x, nthr = blockDim.x;
    const int nb = p.nb, G2 = p.G2, B = p.B;
    const int G = (int)p.G;
    const double *tc = t + cv.pt_off;
    const double tref = tc[0];
    const double kc = cv.kc;

    for (int i = tid; i <= nb; i += nthr) { hA[i] = 0; hC[i] = 0; }
    __syncthreads();
    for (int j = tid; j < cv.n; j += nthr) {
        double tj = tc[j];
        if (!isfinite(tj)) tj = tref;
        Pos ps = position<FP32POS>(tj, tref, cv.df, G);
        atomicAdd(&hA[(ps.ca % G2) / B], 1);
        if (ngrids == 3) atomicAdd(&hC[(ps.cc % G2) / B], 1);
    }
    __syncthreads();
    if (tid < 32) {
        warp_exclusive_scan(hA, nb);
        if (ngrids == 3) warp_exclusive_scan(hC, nb);
    }
    __syncthreads();
    for (int i = tid; i <= nb; i += nthr) {
        binsAB[cv.bin_off + i] = hA[i];
        if (ngrids == 3) binsC[cv.bin_off + i] = hC[i];
    }
    __syncthreads();
    bool bad = false;
    for (int j = tid; j < cv.n; j += nthr) {
        double tj = tc[j];
        float a = ya[cv.pt_off + j];
        float w = (ngrids == 3) ? wv[cv.pt_off + j] : 0.f;
        bool ok = isfinite(tj) && isfinite(a) && isfinite(w);
        if (!ok) { bad = true; tj = isfinite(tj) ? tj : tref; a = 0.f; w = 0.f; }
        Pos ps = position<FP32POS>(tj, tref, cv.df, G);
        float2 ph = centre_phase<FP32POS>(tj, tref, cv.df, kc);
        RecAB r;
        r.cell = ps.ca;
        r.frac = ps.fa;
        r.a = cscale(ph, a);
        r.b = cscale(ph, w);
        int slot = atomicAdd(&hA[(ps.ca % G2) / B], 1);
        recAB[cv.rec_off + slot] = r;
        if (ngrids == 3) {
            float2 ph2 = make_float2(ph.x * ph.x - ph.y * ph.y, 2.f * ph.x * ph.y);
            RecC rc;
            rc.cell = ps.cc;
            rc.frac = ps.fc;
            rc.c = cscale(ph2, w);
            int s2 = atomicAdd(&hC[(ps.cc % G2) / B], 1);
            recC[cv.rec_off + s2] = rc;
        }
    }
    if (bad) atomicOr(errflag, 1u);
    if (aux != nullptr && tid == 0) {
        // out[k] needs exp(2 pi i (kc + k') df t0): base = exp(2 pi i kc df t0),
        // alpha = frac(df t0) split into hi + lo floats.
        double v = kc * cv.df * tref;
        v -= floor(v);
        double s, c;
        sincospi(2.0 * v, &s, &c);
        double al = cv.df * tref;
        al -= floor(al);
        float ah = (float)al;
        float alo = (float)(al - (double)ah);
        aux[cv.aux] = make_float4((float)c, (float)s, ah, alo);
    }
}

// ---------------------------------------------------------------------------
// pass 1: spreading + column FFTs
// ---------------------------------------------------------------------------
__device__ __forceinline__ void bin_ranges(const int *__restrict__ bins, int cb,
                                           int lo, int hi, int nb, int &a0,
                                           int &a1, int &b0, int &b1) {
    if (hi - lo + 1 >= nb) {
        a0 = bins[0]; a1 = bins[nb]; b0 = 0; b1 = 0;
        return;
    }
    const int s = cb + lo, e = cb + hi;
    if (s < 0) {
        a0 = bins[s + nb]; a1 = bins[nb]; b0 = bins[0]; b1 = bins[e + 1];
    } else if (e >= nb) {
        a0 = bins[s]; a1 = bins[nb]; b0 = bins[0]; b1 = bins[e - nb + 1];
    } else {
        a0 = bins[s]; a1 = bins[e + 1]; b0 = 0; b1 = 0;
    }
}

// Add the taps of one record that fall into columns [c0, c0 + B) of the tile.
// Taps cover cells cell + d, d = 1-m .. m, with weights exp(-(d - frac)^2 / b).
template <int NV>
__device__ __forceinline__ void add_taps(float2 *tile, int gstride, int cell,
                                         float frac, float2 v0, float2 v1,
                                         int c0, const Plan &p) {
    const int G2 = p.G2, G1 = p.G1, B = p.B, m = p.m;
    const int ck = cell % G2, rk = cell / G2;
    int dlo = c0 - ck, carry = 0;
    if (dlo + B - 1 < 1 - m) { dlo += G2; carry = 1; }
    else if (dlo > m) { dlo -= G2; carry = -1; }
    const int d0 = max(dlo, 1 - m), d1 = min(dlo + B - 1, m);
    int row = rk + carry;
    if (row < 0) row += G1;
    else if (row >= G1) row -= G1;
    for (int d = d0; d <= d1; ++d) {
        const float dd = (float)d - frac;
        const float wg = __expf(-dd * dd * p.binv);
        float2 *cp = tile + row * B + (d - dlo);
        atomicAdd(&cp->x, v0.x * wg);
        atomicAdd(&cp->y, v0.y * wg);
        if (NV == 2) {
            atomicAdd(&cp[gstride].x, v1.x * wg);
            atomicAdd(&cp[gstride].y, v1.y * wg);
        }
    }
}

template <int NG, int NT>
__global__ void __launch_bounds__(NT)
k_pass1(const DevCurve *__restrict__ cvs, const RecAB *__restrict__ recAB,
        const RecC *__restrict__ recC, const int *__restrict__ binsAB,
        const int *__restrict__ binsC, float2 *__restrict__ inter, Plan p) {
    extern __shared__ __align__(16) float2 sm[];
    const int G1 = p.G1, G2 = p.G2, B = p.B, m = p.m;
    const int gstride = G1 * B;
    const int tile_elems = NG * gstride;
    float2 *tile = sm;
    float2 *tw = tile + tile_elems;
    float2 *thi = tw + G1;
    float2 *tlo = thi + p.n_thi;
    const int tid = threadIdx.x;
    const int cb = blockIdx.x;
    const DevCurve cv = cvs[blockIdx.y];
    const int c0 = cb * B;

    for (int i = tid; i < tile_elems; i += NT) tile[i] = make_float2(0.f, 0.f);
    for (int i = tid; i < G1; i += NT) tw[i] = p.tw1[i];
    for (int i = tid; i < p.n_thi; i += NT) thi[i] = p.thi[i];
    for (int i = tid; i <= p.tw_mask; i += NT) tlo[i] = p.tlo[i];
    __syncthreads();

    const int lo = -((m + B - 1) / B), hi = (B + m - 2) / B;
    {
        int a0, a1, b0, b1;
        bin_ranges(binsAB + cv.bin_off, cb, lo, hi, p.nb, a0, a1, b0, b1);
        const int na = a1 - a0, tot = na + (b1 - b0);
        const RecAB *rb = recAB + cv.rec_off;
        for (int i = tid; i < tot; i += NT) {
            const RecAB r = rb[i < na ? a0 + i : b0 + (i - na)];
            if (NG == 3) add_taps<2>(tile, gstride, r.cell, r.frac, r.a, r.b, c0, p);
            else add_taps<1>(tile, gstride, r.cell, r.frac, r.a, r.a, c0, p);
        }
    }
    if (NG == 3) {
        int a0, a1, b0, b1;
        bin_ranges(binsC + cv.bin_off, cb, lo, hi, p.nb, a0, a1, b0, b1);
        const int na = a1 - a0, tot = na + (b1 - b0);
        const RecC *rc = recC + cv.rec_off;
        for (int i = tid; i < tot; i += NT) {
            const RecC r = rc[i < na ? a0 + i : b0 + (i - na)];
            add_taps<1>(tile + 2 * gstride, 0, r.cell, r.frac, r.c, r.c, c0, p);
        }
    }
    __syncthreads();

    TileLayout lay{NG * B, B, 1, gstride, B};
    smem_fft(tile, G1, p.fac1, p.nfac1, lay, tw, NT, tid);

    float2 *dst = inter + cv.inter_off;
    for (int e = tid; e < tile_elems; e += NT) {
        const int c = e % B;
        const int rest = e / B;
        const int q1 = rest % G1;
        const int g = rest / G1;
        const int n = q1 * (c0 + c);
        const float2 w = cmul(thi[n >> p.tw_shift], tlo[n & p.tw_mask]);
        dst[((long long)g * G1 + q1) * G2 + c0 + c] = cmul(tile[e], w);
    }
}

// ---------------------------------------------------------------------------
// pass 2: row FFTs + finishing epilogue
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T gls_from_sums(T YCh, T YSh, T C, T S, T C2, T S2,
                                           int mode, T reg, T wsum, T ywsum,
                                           T ybar, T pnorm) {
    // 2x2 normal equations of the sinusoid fit; P = b^T A^-1 b / norm.
    // mode 1 (floating mean): cuvarbase/lombscargle.py:337-536 (H=1) and
    // cuvarbase/kernels/lomb.cu:36-83; mode 0 (standard): lomb.cu:85-123;
    // mode 2 (window): lomb.cu:136-137.  The closed forms in lomb.cu rotate
    // to the frame where A is diagonal; the value is the same.
    T YC, YS, CC, SS, CS;
    const T half = (T)0.5;
    if (mode == 1) {
        YC = YCh - ywsum * C;
        YS = YSh - ywsum * S;
        CC = half * (wsum + C2) - C * C + reg;
        SS = half * (wsum - C2) - S * S + reg;
        CS = half * S2 - C * S;
    } else if (mode == 0) {
        YC = YCh + ybar * C;
        YS = YSh + ybar * S;
        CC = half * ((T)1 + C2) + reg;
        SS = half * ((T)1 - C2) + reg;
        CS = half * S2;
    } else {
        YC = C + C;
        YS = S + S;
        CC = half * ((T)1 + C2);
        SS = half * ((T)1 - C2);
        CS = half * S2;
    }
    const T det = CC * SS - CS * CS;
    T P = (YC * YC * SS - (T)2 * YC * YS * CS + YS * YS * CC) / det * pnorm;
    if (!(P >= (T)0) || isinf(P)) P = (T)-1;
    return P;
}

template <int NT>
__global__ void __launch_bounds__(NT)
k_pass2_gls(const DevCurve *__restrict__ cvs, const float2 *__restrict__ inter,
            float *__restrict__ out, Plan p, GlsParams gp) {
    extern __shared__ __align__(16) float2 sm[];
    const int G1 = p.G1, G2 = p.G2, R = p.R;
    const int LDS = G2 + 2;
    float2 *tile = sm;
    float2 *tw = tile + 3 * R * LDS;
    const int tid = threadIdx.x, rb = blockIdx.x;
    const DevCurve cv = cvs[blockIdx.y];
    const float2 *src = inter + cv.inter_off;
    const int half = G2 / 2;
    for (int e = tid; e < 3 * R * half; e += NT) {
        const int v = e / half, i2 = e - v * half;
        const int g = v / R, r = v - g * R;
        const float4 *row = reinterpret_cast<const float4 *>(
            src + ((long long)g * G1 + rb * R + r) * G2);
        reinterpret_cast<float4 *>(tile + v * LDS)[i2] = row[i2];
    }
    for (int i = tid; i < G2; i += NT) tw[i] = p.tw2[i];
    __syncthreads();
    TileLayout lay{3 * R, 1, 0, LDS, 1};
    smem_fft(tile, G2, p.fac2, p.nfac2, lay, tw, NT, tid);

    const long long G = p.G;
    const int nf = cv.nf, h = nf / 2;
    for (int e = tid; e < R * G2; e += NT) {
        const int r = e % R, q2 = e / R;
        const long long q = (long long)(rb * R + r) + (long long)G1 * q2;
        int kp;
        if (q < nf - h) kp = (int)q;
        else if (q >= G - h) kp = (int)(q - G);
        else continue;
        const float kf = (float)kp;
        const float D = __expf(kf * kf * p.dc1) * p.dc2;
        const float2 A = tile[r * LDS + q2];
        const float2 Bv = tile[(R + r) * LDS + q2];
        const float2 Cv = tile[(2 * R + r) * LDS + q2];
        out[cv.out_off + kp + h] = gls_from_sums<float>(
            A.x * D, A.y * D, Bv.x * D, Bv.y * D, Cv.x * D, Cv.y * D, gp.mode,
            gp.reg, cv.w_sum, cv.yw_sum, cv.ybar, cv.yy_inv);
    }
}

template <int NT>
__global__ void __launch_bounds__(NT)
k_pass2_nfft(const DevCurve *__restrict__ cvs, const float2 *__restrict__ inter,
             float2 *__restrict__ out, const float4 *__restrict__ aux, Plan p) {
    extern __shared__ __align__(16) float2 sm[];
    const int G1 = p.G1, G2 = p.G2, R = p.R;
    const int LDS = G2 + 2;
    float2 *tile = sm;
    float2 *tw = tile + R * LDS;
    const int tid = threadIdx.x, rb = blockIdx.x;
    const DevCurve cv = cvs[blockIdx.y];
    const float2 *src = inter + cv.inter_off;
    const int half = G2 / 2;
    for (int e = tid; e < R * half; e += NT) {
        const int r = e / half, i2 = e - r * half;
        const float4 *row = reinterpret_cast<const float4 *>(
            src + ((long long)rb * R + r) * G2);
        reinterpret_cast<float4 *>(tile + r * LDS)[i2] = row[i2];
    }
    for (int i = tid; i < G2; i += NT) tw[i] = p.tw2[i];
    __syncthreads();
    TileLayout lay{R, 1, 0, LDS, 1};
    smem_fft(tile, G2, p.fac2, p.nfac2, lay, tw, NT, tid);

    const float4 ax = aux[cv.aux];
    const float2 base = make_float2(ax.x, ax.y);
    const long long G = p.G;
    const int nf = cv.nf, h = nf / 2;
    for (int e = tid; e < R * G2; e += NT) {
        const int r = e % R, q2 = e / R;
        const long long q = (long long)(rb * R + r) + (long long)G1 * q2;
        int kp;
        if (q < nf - h) kp = (int)q;
        else if (q >= G - h) kp = (int)(q - G);
        else continue;
        const float kf = (float)kp;
        const float D = __expf(kf * kf * p.dc1) * p.dc2;
        // frac(k' alpha) with alpha = hi + lo, k' alpha_hi split exactly.
        const float pr = kf * ax.z;
        const float er = fmaf(kf, ax.z, -pr);
        const float th = (pr - rintf(pr)) + (er + kf * ax.w);
        float s, c;
        sincospif(2.0f * th, &s, &c);
        const float2 ph = cmul(base, make_float2(c, s));
        out[cv.out_off + kp + h] = cmul(cscale(tile[r * LDS + q2], D), ph);
    }
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
// launchers
// ---------------------------------------------------------------------------
int pick_threads(long long elems) {
    const int opts[4] = {128, 256, 512, 1024};
    for (int i = 0; i < 4; ++i)
        if (elems <= (long long)kEPT * opts[i]) return opts[i];
    return 0;
}

template <typename K>
static cudaError_t allow_smem(K kernel) {
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                227 * 1024);
}

cudaError_t configure_kernels(int) {
    cudaError_t e = cudaSuccess;
#define CUVGLS_ALLOW(...) if (e == cudaSuccess) e = allow_smem(__VA_ARGS__)
    CUVGLS_ALLOW(k_pass1<3, 128>); CUVGLS_ALLOW(k_pass1<3, 256>);
    CUVGLS_ALLOW(k_pass1<3, 512>); CUVGLS_ALLOW(k_pass1<3, 1024>);
    CUVGLS_ALLOW(k_pass1<1, 128>); CUVGLS_ALLOW(k_pass1<1, 256>);
    CUVGLS_ALLOW(k_pass1<1, 512>); CUVGLS_ALLOW(k_pass1<1, 1024>);
    CUVGLS_ALLOW(k_pass2_gls<128>); CUVGLS_ALLOW(k_pass2_gls<256>);
    CUVGLS_ALLOW(k_pass2_gls<512>); CUVGLS_ALLOW(k_pass2_gls<1024>);
    CUVGLS_ALLOW(k_pass2_nfft<128>); CUVGLS_ALLOW(k_pass2_nfft<256>);
    CUVGLS_ALLOW(k_pass2_nfft<512>); CUVGLS_ALLOW(k_pass2_nfft<1024>);
#undef CUVGLS_ALLOW
    return e;
}

cudaError_t launch_prep_bin(const DevCurve *cv, int n_curves, const double *t,
                            const float *ya, const float *wv, RecAB *recAB,
                            RecC *recC, int *binsAB, int *binsC, float4 *aux,
                            const Plan &p, int ngrids, int fp32_positions,
                            unsigned *errflag, cudaStream_t s) {
    if (n_curves <= 0) return cudaSuccess;
    if (fp32_positions)
        k_prep_bin<true><<<n_curves, 512, 0, s>>>(cv, t, ya, wv, recAB, recC, binsAB,
                                                  binsC, aux, p, ngrids, errflag);
    else
        k_prep_bin<false><<<n_curves, 512, 0, s>>>(cv, t, ya, wv, recAB, recC, binsAB,
                                                   binsC, aux, p, ngrids, errflag);
    return cudaGetLastError();
}

cudaError_t launch_pass1(const DevCurve *cv, int n_curves, const RecAB *recAB,
                         const RecC *recC, const int *binsAB, const int *binsC,
                         float2 *inter, const Plan &p, int ngrids, int nthreads,
                         size_t smem, cudaStream_t s) {
    if (n_curves <= 0) return cudaSuccess;
    dim3 grid(p.nb, n_curves);
#define CUVGLS_P1(NG, NT) k_pass1<NG, NT><<<grid, NT, smem, s>>>(cv, recAB, recC, binsAB, binsC, inter, p)
    if (ngrids == 3) {
        if (nthreads == 128) CUVGLS_P1(3, 128);
        else if (nthreads == 256) CUVGLS_P1(3, 256);
        else if (nthreads == 512) CUVGLS_P1(3, 512);
        else CUVGLS_P1(3, 1024);
    } else {
        if (nthreads == 128) CUVGLS_P1(1, 128);
        else if (nthreads == 256) CUVGLS_P1(1, 256);
        else if (nthreads == 512) CUVGLS_P1(1, 512);
        else CUVGLS_P1(1, 1024);
    }
#undef CUVGLS_P1
    return cudaGetLastError();
}

cudaError_t launch_pass2_gls(const DevCurve *cv, int n_curves,
                             const float2 *inter, float *out, const Plan &p,
                             GlsParams g, int nthreads, size_t smem,
                             cudaStream_t s) {
    if (n_curves <= 0) return cudaSuccess;
    dim3 grid(p.G1 / p.R, n_curves);
    if (nthreads == 128) k_pass2_gls<128><<<grid, 128, smem, s>>>(cv, inter, out, p, g);
    else if (nthreads == 256) k_pass2_gls<256><<<grid, 256, smem, s>>>(cv, inter, out, p, g);
    else if (nthreads == 512) k_pass2_gls<512><<<grid, 512, smem, s>>>(cv, inter, out, p, g);
    else k_pass2_gls<1024><<<grid, 1024, smem, s>>>(cv, inter, out, p, g);
    return cudaGetLastError();
}

cudaError_t launch_pass2_nfft(const DevCurve *cv, int n_curves,
                              const float2 *inter, float2 *out,
                              const float4 *aux, const Plan &p, int nthreads,
                              size_t smem, cudaStream_t s) {
    if (n_curves <= 0) return cudaSuccess;
    dim3 grid(p.G1 / p.R, n_curves);
    if (nthreads == 128) k_pass2_nfft<128><<<grid, 128, smem, s>>>(cv, inter, out, aux, p);
    else if (nthreads == 256) k_pass2_nfft<256><<<grid, 256, smem, s>>>(cv, inter, out, aux, p);
    else if (nthreads == 512) k_pass2_nfft<512><<<grid, 512, smem, s>>>(cv, inter, out, aux, p);
    else k_pass2_nfft<1024><<<grid, 1024, smem, s>>>(cv, inter, out, aux, p);
    return cudaGetLastError();
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
