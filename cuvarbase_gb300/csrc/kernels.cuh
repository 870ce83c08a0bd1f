// Host-side launch wrappers of the cuvgls kernels (implemented in kernels.cu).
#pragma once

#include "common.cuh"

namespace cuvgls {

struct RefGridCurve {  // device copy of cuvgls_grid_curve
    long long pt_off, n, ng;
    double tmin, scale;  // x = (t - tmin) * scale
    long long out_off;
};

// ngrids = 3 (GLS: yw@x, w@x, w@2x) or 1 (NFFT: y@x).
cudaError_t launch_prep_bin(const DevCurve *cv, int n_curves, const double *t,
                            const float *ya, const float *wv, RecAB *recAB,
                            RecC *recC, int *binsAB, int *binsC, float4 *aux,
                            const Plan &p, int ngrids, int fp32_positions,
                            unsigned *errflag, cudaStream_t s);

cudaError_t launch_pass1(const DevCurve *cv, int n_curves, const RecAB *recAB,
                         const RecC *recC, const int *binsAB, const int *binsC,
                         float2 *inter, const Plan &p, int ngrids, int nthreads,
                         size_t smem, cudaStream_t s);

cudaError_t launch_pass2_gls(const DevCurve *cv, int n_curves,
                             const float2 *inter, float *out, const Plan &p,
                             GlsParams g, int nthreads, size_t smem,
                             cudaStream_t s);

cudaError_t launch_pass2_nfft(const DevCurve *cv, int n_curves,
                              const float2 *inter, float2 *out,
                              const float4 *aux, const Plan &p, int nthreads,
                              size_t smem, cudaStream_t s);

cudaError_t launch_spread_ref(const RefGridCurve *cv, int n_curves,
                              long long max_n, const double *t, const float *y,
                              float *grid, int m, float binv, float norm,
                              cudaStream_t s);

cudaError_t launch_gls_direct(const DevCurve *cv, int n_curves, int max_nf,
                              const double *t, const float *yw, const float *w,
                              float *out, GlsParams g, cudaStream_t s);

// Smallest supported threads-per-CTA for a tile of `elems` complex elements
// (0 if none); and the attribute set-up for large dynamic shared memory.
int pick_threads(long long elems);
cudaError_t configure_kernels(int device);

}  // namespace cuvgls
