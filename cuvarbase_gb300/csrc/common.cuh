// Device-side types shared by the cuvgls kernels and the host launcher.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "plan_rules.h"

namespace cuvgls {

// Largest column-block count of a plan (G2 / B) the binning kernel handles.
constexpr int kMaxBins = 2048;

// Preparation kernels take a curve in segments of kSegPoints points, one
// CTA of kSegThreads threads per segment, so a long curve (or a batch of a
// few curves) still spreads over the SMs.
constexpr int kSegThreads = 256;
constexpr int kSegPoints = 4 * kSegThreads;

__host__ __device__ inline int seg_count(int n) { return (n + kSegPoints - 1) / kSegPoints; }

// One segment of a curve: descriptor index and first point of the segment.
struct SegEntry {
    int desc;
    int start;
};

// Spreading windows.  The Gaussian is the reference's (its b from sigma and
// m); the exponential of semicircle (ES) reaches the same accuracy on a
// smaller grid with fewer taps, and its Fourier transform, which has no
// closed form, is tabulated per plan.
constexpr int kWinGauss = 0;
constexpr int kWinES = 1;

// Grid plan of one size class: G = G1 * G2 cells, window half-width m.
// Pass 1 transforms columns (length G1, B columns per CTA), pass 2 rows
// (length G2, R rows per CTA).
struct Plan {
    int G1, G2;
    long long G;
    int m;
    int B;          // columns per pass-1 CTA
    int R;          // rows per pass-2 CTA
    int nb;         // G2 / B column blocks
    int win;        // spreading window: kWinGauss or kWinES
    // Gaussian exp(-d^2 / b), b = 2 sigma m / ((2 sigma - 1) pi)
    float binv;     // 1 / b
    float dc1;      // b pi^2 / G^2   (deconvolution exponent per k'^2)
    float dc2;      // 1 / sqrt(pi b) (deconvolution scale)
    // "exponential of semicircle" exp(beta (sqrt(1 - d^2 / m^2) - 1)), |d| <= m
    float es_beta;
    float es_im2;   // 1 / m^2
    const float *dtab;   // ES deconvolution 1 / phihat(k'), |k'| <= G / 2
    const float2 *st1;   // FFT table of the length-G1 transform
    const float2 *st2;   // FFT table of the length-G2 transform
    const float2 *itw;   // [cb][q1][c]: exp(+2 pi i q1 (cb B + c) / G), G entries
};

// Per-curve device descriptor (offsets are chunk-local where noted).
struct DevCurve {
    long long pt_off;    // first point in t / y arrays (global)
    long long out_off;   // first output element (global)
    long long rec_off;   // first spreading record (chunk-local)
    long long inter_off; // first intermediate element, float2 units (chunk-local)
    double kc;           // band-centre frequency index k0 + nf/2 (+ fraction)
    int n;               // points
    int nf;              // frequencies
    int bin_off;         // first bin offset entry (chunk-local), nb + 1 entries
    int aux;             // index into the per-curve aux array
    double df;           // frequency spacing
    float yy_inv;        // 1 / YY
    float ybar;          // weighted mean (mode 0)
    float yw_sum;        // sum(yw) (mode 1)
    float w_sum;         // sum(w)
    int best_slot;       // curve of the caller's batch this band belongs to
    int best_off;        // first frequency of this (sub-)band within that curve
    int seg0;            // first binning segment of this descriptor
    int raw_seg;         // first raw-preparation segment of its curve (raw input)
    int flags;           // kDescFillHere
    int pad_;
};

// Raw input: the curve of this descriptor is one segment and one band, and
// k_raw_finish writes its statistics into the descriptor.
constexpr int kDescFillHere = 1;

// Spreading record of the x-position grids (A: yw or y, B: w).
// The cell is stored as row << 16 | column of the G1 x G2 grid
// (cell = row G2 + column), so pass 1 needs no division by G2.
struct __align__(8) RecAB {
    int rc;        // cell floor(G * frac(x)) as row << 16 | column
    float frac;    // G * frac(x) - cell
    float2 a;      // yw * exp(2 pi i kc x)
    float2 b;      // w  * exp(2 pi i kc x)
};

// Spreading record of the 2x-position grid (C: w at 2x).
struct __align__(8) RecC {
    int rc;
    float frac;
    float2 c;      // w * exp(2 pi i kc 2x)
};

// GLS finishing parameters.
struct GlsParams {
    int mode;      // 0 standard, 1 floating mean, 2 window
    float reg;     // isotropic amplitude-prior regulariser lambda
    // per-curve best power as (power bits << 32 | ~index), maximised with
    // atomicMax (ties: lowest index); nullptr when not wanted
    unsigned long long *best;
};

// Window value at offset dd (cells) from a point, |dd| <= m.  The ES
// exponent beta (sqrt(1 - z^2) - 1) is evaluated as -beta z^2 / (1 +
// sqrt(1 - z^2)): near the centre the direct form multiplies the rounding
// of the square root by beta (~19), a relative error of ~2e-6 in the
// largest taps; this form keeps the exponent's error relative to its size.
// Full-precision expf, sqrtf and division: with the approximate ones the
// benchmark batch's max |dP| was 2.1e-5 instead of 1.3e-5 (pass 1 0.15 ms
// faster per 10,000 curves).
__device__ __forceinline__ float win_tap(float dd, const Plan &p) {
    if (p.win == kWinES) {
        const float z2 = dd * dd * p.es_im2;
        const float s = 1.f - z2;
        return s > 0.f ? expf(-p.es_beta * z2 / (1.f + sqrtf(s))) : 0.f;
    }
    return __expf(-dd * dd * p.binv);
}

// Deconvolution factor 1 / phihat(k') of band index k' (|k'| <= G / 2):
// the plan's table (ES) or the Gaussian's exp(b (pi k' / G)^2) / sqrt(pi b).
template <bool ES>
__device__ __forceinline__ float win_deconv(int k, const Plan &p) {
    if constexpr (ES) {
        return __ldg(p.dtab + (k < 0 ? -k : k));
    } else {
        const float kf = (float)k;
        return __expf(kf * kf * p.dc1) * p.dc2;
    }
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// Complex add, subtract and real scale as packed FP32x2 instructions (one
// FADD2 / FMUL2 instead of two scalar ones; same IEEE rounding per lane).
// The complex product stays scalar: its packed form needs swapped operand
// pairs, whose moves cost more than they save.
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
    return __fadd2_rn(a, make_float2(-b.x, -b.y));
}
__device__ __forceinline__ float2 cscale(float2 a, float s) {
    return __fmul2_rn(a, make_float2(s, s));
}
// a * i
__device__ __forceinline__ float2 cmuli(float2 a) { return make_float2(-a.y, a.x); }

}  // namespace cuvgls
