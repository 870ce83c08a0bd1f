// cuvgls kernels for sm_103a.
//
// This file holds the per-point and auxiliary kernels and the length
// dispatch; the pass kernels are in pass_kernels.cuh.
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

__global__ void __launch_bounds__(256)
k_raw_prep(const DevCurve *__restrict__ cvs, const double *__restrict__ y,
           const double *__restrict__ dy, float *__restrict__ yw, float *__restrict__ w,
           RawStats *__restrict__ stats) {
    __shared__ double red[32];
    const DevCurve cv = cvs[blockIdx.x];
    if (cv.best_off != 0) return;  // one CTA per curve: its first band
    const long long o = cv.pt_off;
    const int n = cv.n;
    double sw = 0.0, swy = 0.0, sy = 0.0, cy = 0.0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const double yj = y[o + j], dj = dy[o + j];
        const double wj = 1.0 / (dj * dj);
        sw += wj;
        swy += wj * yj;
        if (!isnan(yj)) { sy += yj; cy += 1.0; }
    }
    sw = block_sum(sw, red);
    swy = block_sum(swy, red);
    sy = block_sum(sy, red);
    cy = block_sum(cy, red);
    const double ybar_w = swy / sw;  // weighted mean of y (weights sum to 1)
    double yy = 0.0, ys = 0.0, ws = 0.0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const double dj = dy[o + j];
        const double wj = 1.0 / (dj * dj) / sw;
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
    if (threadIdx.x == 0) {
        RawStats st;
        st.yy = yy;
        st.ybar = ybar_w - sy / cy;  // after the unweighted mean is removed
        st.yw_sum = ys;
        st.w_sum = ws;
        stats[cv.best_slot] = st;
    }
}

__global__ void k_fill_desc(DevCurve *__restrict__ cvs, int n, const RawStats *__restrict__ stats,
                            int mode) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    DevCurve &cv = cvs[i];
    const RawStats st = stats[cv.best_slot];
    double norm = 1.0;
    if (mode == 1) norm = 1.0 / st.yy;
    else if (mode == 0) norm = 1.0 / (st.yy + st.ybar * st.ybar);
    cv.yy_inv = (float)norm;
    cv.ybar = (float)st.ybar;
    cv.yw_sum = (float)st.yw_sum;
    cv.w_sum = (float)st.w_sum;
}

cudaError_t launch_raw_prep(const DevCurve *cv, int n_bands, const double *y,
                            const double *dy, float *yw, float *w, RawStats *stats,
                            cudaStream_t s) {
    if (n_bands <= 0) return cudaSuccess;
    k_raw_prep<<<n_bands, 256, 0, s>>>(cv, y, dy, yw, w, stats);
    return cudaGetLastError();
}

cudaError_t launch_fill_desc(DevCurve *cv, int n_bands, const RawStats *stats, int mode,
                             cudaStream_t s) {
    if (n_bands <= 0) return cudaSuccess;
    k_fill_desc<<<(n_bands + 255) / 256, 256, 0, s>>>(cv, n_bands, stats, mode);
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

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
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

#define CUVGLS_LEN_CASES(X) X(16) X(32) X(64) X(80) X(128) X(160) X(256) X(320) \
    X(400) X(512) X(640) X(800) X(1024) X(1280) X(1600) X(2048)

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

cudaError_t launch_pass2_gls(const DevCurve *cv, int n_curves,
                             const float2 *inter, float *out, const Plan &p,
                             GlsParams g, cudaStream_t s) {
    if (n_curves <= 0) return cudaSuccess;
#define CUVGLS_P2(L) case L: return launch_pass2_gls_t<L>(cv, n_curves, inter, out, p, g, s);
    switch (p.G2) {
        CUVGLS_LEN_CASES(CUVGLS_P2)
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
        CUVGLS_LEN_CASES(CUVGLS_P2N)
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
