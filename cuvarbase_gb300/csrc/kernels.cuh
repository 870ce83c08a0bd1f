// Host-side launch wrappers of the cuvgls kernels (implemented in kernels.cu).
#pragma once

#include <cstdint>

#include "common.cuh"

namespace cuvgls {

struct RefGridCurve {  // device copy of cuvgls_grid_curve
    long long pt_off, n, ng;
    double tmin, scale;  // x = (t - tmin) * scale
    long long out_off;
};

// Segment tables of a descriptor table: binning segments of every
// descriptor at its seg0 and, where raw_segs is given, the raw-preparation
// segments of every curve (its band with best_off == 0) at raw_seg.
cudaError_t launch_seg_fill(const DevCurve *cv, int n, SegEntry *bin_segs, SegEntry *raw_segs,
                            cudaStream_t s);

// Binning of a group (ngrids = 3, GLS: yw@x, w@x, w@2x; or 1, NFFT: y@x).
// For curves longer than one segment: the count per segment into binsAB /
// binsC (nb + 1 entries per descriptor at bin_off, zeroed by the caller),
// then the scan per descriptor (offsets, cursors curAB / curC, aux).  Then
// the scatter per segment, which also bins each curve of one segment
// completely (offsets, records, aux).  Segment entries index cv; the scan
// takes the group's own descriptors.  Count and scan skip single-segment
// curves.
cudaError_t launch_bin_count(const SegEntry *segs, int n_segs, const DevCurve *cv,
                             const double *t, int *binsAB, int *binsC, const Plan &p,
                             int ngrids, int fp32_positions, cudaStream_t s);
cudaError_t launch_bin_scan(const DevCurve *cv, int n_curves, const double *t, int *binsAB,
                            int *binsC, int *curAB, int *curC, float4 *aux, const Plan &p,
                            int ngrids, cudaStream_t s);
cudaError_t launch_bin_scatter(const SegEntry *segs, int n_segs, const DevCurve *cv,
                               const double *t, const float *ya, const float *wv,
                               RecAB *recAB, RecC *recC, int *binsAB, int *binsC, int *curAB,
                               int *curC, float4 *aux, const Plan &p, int ngrids,
                               int fp32_positions, unsigned *errflag, cudaStream_t s);

// Dispatch on (G1, G2) to the compiled length templates; cudaErrorInvalidValue
// if a length has no kernel.
cudaError_t launch_pass1(const DevCurve *cv, int n_curves, const RecAB *recAB,
                         const RecC *recC, const int *binsAB, const int *binsC,
                         float2 *inter, const Plan &p, int ngrids, cudaStream_t s);

cudaError_t launch_pass2_gls(const DevCurve *cv, int n_curves,
                             const float2 *inter, float *out, const Plan &p,
                             GlsParams g, cudaStream_t s);

cudaError_t launch_pass2_nfft(const DevCurve *cv, int n_curves,
                              const float2 *inter, float2 *out,
                              const float4 *aux, const Plan &p, cudaStream_t s);

// Length templates (pass_kernels.cuh, instantiated in inst_*.cu).
template <int NG, int L1>
cudaError_t launch_pass1_t(const DevCurve *, int, const RecAB *, const RecC *,
                           const int *, const int *, float2 *, const Plan &, cudaStream_t);
template <int L2>
cudaError_t launch_pass2_gls_t(const DevCurve *, int, const float2 *, float *,
                               const Plan &, GlsParams, cudaStream_t);
template <int L2>
cudaError_t launch_pass2_nfft_t(const DevCurve *, int, const float2 *, float2 *,
                                const float4 *, const Plan &, cudaStream_t);

template <int NG, int L1>
cudaError_t preload_pass1_t();
template <int L2>
cudaError_t preload_pass2_t(int ng);
// Load the pass-1 and pass-2 kernels of a (G1, G2) plan for ngrids grids.
cudaError_t preload_pass_kernels(int G1, int G2, int ngrids);

// Fill the deconvolution table of an ES-window plan: G / 2 + 1 floats
// 1 / phihat(k'), |k'| <= G / 2 (kernels.cu: k_es_deconv).
cudaError_t launch_es_deconv(float *dst, long long G, int m, double beta, cudaStream_t s);

// Fill the tables of a plan (FFT tables of G1 and G2, then the inter-pass
// twiddles), fft_table_len(G1) + fft_table_len(G2) + G1 G2 entries at dst.
cudaError_t launch_plan_tables(float2 *dst, int G1, int G2, int B, cudaStream_t s);

// Host preparation of LombScargleMemory.setdata on the device for raw
// (t, y, dy) input, over the raw-preparation segments (one double4 of
// partA and partB each): k_raw_sums sums the segments of curves longer than
// one segment; k_raw_finish does a curve of one segment completely
// (w = dy^-2 / sum dy^-2 and yw = w (y - ybar) as FP32, the sums of YY, yw
// and w, and the descriptor where flagged kDescFillHere) and writes w, yw
// and the partial sums of the longer curves' segments; k_fill_desc gives
// every unflagged descriptor its curve's statistics.
cudaError_t launch_raw_sums(const SegEntry *segs, int n_segs, const DevCurve *cv,
                            const double *y, const double *dy, double *ir, double4 *partA,
                            cudaStream_t s);
cudaError_t launch_raw_finish(const SegEntry *segs, int n_segs, DevCurve *cv, const double *y,
                              const double *dy, const double *ir, float *yw, float *w,
                              double4 *partA, double4 *partB, int mode, cudaStream_t s);
cudaError_t launch_fill_desc(DevCurve *cv, int n, const double4 *partA, const double4 *partB,
                             int mode, cudaStream_t s);

// Per-curve best keys of k_pass2_gls to (index, power); -1 / -1 where a
// curve had no valid power.
cudaError_t launch_best_finish(const unsigned long long *keys, int n, int64_t *best_k,
                               float *best_p, cudaStream_t s);

cudaError_t launch_spread_ref(const RefGridCurve *cv, int n_curves,
                              long long max_n, const double *t, const float *y,
                              float *grid, int m, float binv, float norm,
                              cudaStream_t s);

// Adjoint NFFT by FP64 direct summation: out[k] = sum_j y_j
// exp(+2 pi i (f0 + k df) t_j) for k < nf, complex128.
struct Direct64Curve {
    long long pt_off, n, nf, out_off;
    double f0, df;
};
cudaError_t launch_nfft_direct64(const Direct64Curve *cv, int n_curves, long long max_nf,
                                 const double *t, const double *y, double2 *out,
                                 cudaStream_t s);

// Finish of a caller-given reference-convention grid g of length ng (the
// reference's use_grid): shift by exp(2 pi i j ks / ng), inverse DFT, then
// for k < nf the phase exp(2 pi i n0 (k0 + k) / ng) and the Gaussian
// deconvolution exp(b (pi (k0 + k) / ng)^2); FP64, complex128.
struct GridFinishCurve {
    long long grid_off, ng, nf, out_off;
    double k0;   // f0 spp (tmax - tmin)
    double ks;   // k0 when the reference shifts (|f0| > 1e-9), else 0
    double n0;   // tmin / (spp (tmax - tmin)) ng
    double b;
};
cudaError_t launch_grid_finish(const GridFinishCurve *cv, int n_curves, long long max_nf,
                               const double2 *grid, double2 *out, cudaStream_t s);

// Multi-harmonic floating-mean GLS of one curve by FP64 direct sums, H
// harmonics (1..kMaxHarm): sums of w and yw against cos / sin of n phi, the
// regularised 2H x 2H normal equations solved per frequency (partial
// pivoting), P = (YX - sum XX) / YY; NaN where the system is singular.
constexpr int kMaxHarm = 8;
struct MhParams {
    double ybar, yy;
    double d[kMaxHarm];    // amplitude-prior regulariser per harmonic
    double cn0[kMaxHarm];  // prior centres of the cosine amplitudes
    double sn0[kMaxHarm];  // prior centres of the sine amplitudes
};
cudaError_t launch_mhgls_direct(int nharms, const double *t, const double *yw, const double *w,
                                long long n, const double *freqs, long long nf,
                                const MhParams &mp, double *out, cudaStream_t s);

cudaError_t launch_gls_direct(const DevCurve *cv, int n_curves, int max_nf,
                              const double *t, const float *yw, const float *w,
                              float *out, GlsParams g, cudaStream_t s);


}  // namespace cuvgls
