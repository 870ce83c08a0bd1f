/*
 * cuvgls — GB300-native (sm_103a) generalized Lomb-Scargle periodograms and
 * adjoint NFFTs for batches of irregularly sampled light curves.
 *
 * Plain C ABI: no C++ types, no exceptions, plain pointers and sizes.  Every
 * entry point returns a status code (CUVGLS_OK = 0, negative on error) and
 * records a message retrievable with cuvgls_last_error().  A handle is not
 * thread-safe: use one handle per host thread.  The caller owns inputs and
 * outputs; the handle owns its device workspaces.
 *
 * Each entry point below names the cuvarbase interface it replaces
 * (paths relative to the cuvarbase source tree).
 */
#ifndef CUVGLS_H
#define CUVGLS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CUVGLS_VERSION 1000 /* major*1000 + minor */

/* ---- status codes ---- */
#define CUVGLS_OK 0
#define CUVGLS_EINVAL -1    /* invalid argument (size, pointer, mode, ...) */
#define CUVGLS_ENOMEM -2    /* device or pinned allocation failed */
#define CUVGLS_EBUDGET -3   /* request exceeds the handle's memory budget */
#define CUVGLS_ETIMEOUT -4  /* cuvgls_sync deadline passed */
#define CUVGLS_ECUDA -5     /* CUDA runtime error */
#define CUVGLS_ENOTSUP -6   /* size outside what the kernels support */
#define CUVGLS_EDEVICE -7   /* a kernel raised its device-side error flag */
#define CUVGLS_ECLOSED -8   /* server shut down and drained */

/* ---- flags ---- */
/* Host inputs that are page-locked (cuvgls_host_alloc, cudaHostAlloc) are
 * copied asynchronously and must stay valid until the call's work completes
 * (cuvgls_sync); pageable host inputs are staged by the CUDA runtime before
 * the call returns.  Host outputs are written asynchronously: read them
 * after cuvgls_sync.  Both overlap the work: a batch of several FFT chunks
 * copies the first chunk's points first and the rest while that chunk runs,
 * and copies its outputs back a quarter chunk at a time as they are done,
 * on the handle's own streams, which join the caller's stream before the
 * call's work completes. */
#define CUVGLS_HOST_INPUT 1  /* t / y arrays are host pointers */
#define CUVGLS_HOST_OUTPUT 2 /* output pointer is a host pointer */

/* ---- GLS modes (cuvarbase/kernels/lomb.cu:15-17, :126-141) ---- */
#define CUVGLS_MODE_STANDARD 0
#define CUVGLS_MODE_FLOATING_MEAN 1
#define CUVGLS_MODE_WINDOW 2

/* ---- precision (position / phase arithmetic of the spreading stage) ---- */
#define CUVGLS_PREC_MIXED 0   /* FP32 bulk; FP64 t - t0, grid index, phases */
#define CUVGLS_PREC_FP32 1    /* everything FP32 (comparison variant) */

/* device-side error flags, OR-ed into the handle's status word */
#define CUVGLS_DEVERR_NONFINITE 1 /* a non-finite input was skipped */
#define CUVGLS_DEVERR_TIMEOUT 2   /* a bounded device wait ran out */
#define CUVGLS_DEVERR_BINNING 4   /* binning count and scatter disagreed (records dropped) */

/* largest number of points of one curve (kernels index points of a curve in
 * 32 bits, in segments of 1024) */
#define CUVGLS_MAX_CURVE_POINTS 2147482623LL

typedef struct cuvgls_handle cuvgls_handle;

typedef struct {
    double sigma;            /* minimum oversampling G/nf (default 2); < 0 lets the
                                planner autotune (window, sigma, m) per nf
                                under a max |dP| <= 2e-5 budget */
    int32_t m;               /* Gaussian half-width in grid cells (default 8;
                                ignored when sigma < 0) */
    int32_t device;          /* CUDA device ordinal (default 0) */
    int64_t workspace_bytes; /* cap on the handle's device workspace (grown only
                                as batches need it); 0 = 16 GiB */
    int32_t precision;       /* CUVGLS_PREC_* (default MIXED) */
    int32_t chunk_mb;        /* device bytes (MiB) of one chunk's intermediate;
                                0 = 4096.  Larger chunks mean fewer, longer
                                launches (less tail per launch) */
} cuvgls_opts;

/* One light curve of a GLS batch.  Frequencies are f_k = (k0 + k) df,
 * k = 0 .. nf-1 (cuvarbase/lombscargle.py:25-33: freqs = df (k0 + arange)). */
typedef struct {
    int64_t pt_off;  /* first point of this curve in t / yw / w */
    int64_t n;       /* number of points (>= 1) */
    int64_t nf;      /* number of frequencies (>= 1) */
    int64_t k0;      /* index of the first frequency */
    double df;       /* frequency spacing (> 0) */
    double yy;       /* YY = sum w (y - ybar)^2  (lombscargle.py:254-257) */
    double ybar;     /* weighted mean of y (mode 0 uses it, lomb.cu:85-123) */
    double yw_sum;   /* sum(yw) as the reference forms it (lombscargle.py:384) */
    double w_sum;    /* sum(w) (1 up to float32 rounding) */
    int64_t out_off; /* first output element of this curve */
} cuvgls_curve;

typedef struct {
    int32_t n_curves;
    int32_t mode;                /* CUVGLS_MODE_* */
    const cuvgls_curve *curves;  /* HOST array of n_curves descriptors */
    const double *t;             /* observation times, FP64 */
    const float *yw;             /* w (y - ybar) */
    const float *w;              /* normalised weights */
    float reg[3];                /* amplitude-prior regulariser (lomb.cu:42-47) */
    int32_t flags;               /* CUVGLS_HOST_INPUT | CUVGLS_HOST_OUTPUT */
    int64_t n_points_total;      /* length of t / yw / w */
    int64_t n_out_total;         /* length of the output array */
} cuvgls_gls_input;

/* One light curve of raw (t, y, dy) input. */
typedef struct {
    int64_t pt_off;  /* first point in t / y / dy */
    int64_t n;       /* points */
    int64_t nf;      /* frequencies: f_k = (k0 + k) df, k < nf */
    int64_t k0;
    double df;
    int64_t out_off; /* first power in p_out (ignored for best-frequency output) */
} cuvgls_raw_curve;

/* A ragged batch of raw light curves: t, y, dy as given by the user (FP64).
 * The host preparation of cuvarbase (normalize_light_curves,
 * cuvarbase/utils.py:113-146; weights and LombScargleMemory.setdata,
 * cuvarbase/lombscargle.py:235-261) runs on the device. */
typedef struct {
    int32_t n_curves;
    int32_t mode;            /* CUVGLS_MODE_* */
    const cuvgls_raw_curve *curves;
    const double *t;
    const double *y;
    const double *dy;
    float reg[3];            /* (lambda, lambda, 0) */
    int32_t flags;           /* CUVGLS_HOST_INPUT / CUVGLS_HOST_OUTPUT */
    int64_t n_points_total;
    int64_t n_out_total;
} cuvgls_raw_input;

/* One curve of an adjoint-NFFT batch:
 * out[k] = sum_j y_j exp(+2 pi i (f0 + k df) t_j),  k = 0 .. nf-1.
 * f0 / df need not be an integer. */
typedef struct {
    int64_t pt_off;
    int64_t n;
    int64_t nf;
    double f0;       /* first frequency */
    double df;       /* frequency spacing (> 0) */
    int64_t out_off; /* in complex elements */
} cuvgls_nfft_curve;

typedef struct {
    int32_t n_curves;
    int32_t flags;
    const cuvgls_nfft_curve *curves; /* HOST array */
    const double *t;
    const float *y;
    int64_t n_points_total;
    int64_t n_out_total; /* complex elements (2 floats each) */
} cuvgls_nfft_input;

/* One curve of a reference-convention gridding call (just_return_gridded_data). */
typedef struct {
    int64_t pt_off;
    int64_t n;
    int64_t ng;      /* grid length (reference: int(sigma * nf)) */
    double tmin;     /* x = (t - tmin) / (spp (tmax - tmin)) */
    double tmax;
    double spp;      /* samples per peak */
    int64_t out_off; /* first grid element of this curve */
} cuvgls_grid_curve;

/* Library version (CUVGLS_VERSION). */
int cuvgls_version(void);

/* Create a handle bound to opts->device (opts may be NULL for defaults).
 * Replaces the state cuvarbase keeps in NFFTAsyncProcess.__init__ /
 * LombScargleAsyncProcess.__init__ (cuvarbase/cunfft.py:349-376,
 * cuvarbase/lombscargle.py:713-730). */
int cuvgls_create(cuvgls_handle **out, const cuvgls_opts *opts);

/* Release the handle and its workspaces. */
int cuvgls_destroy(cuvgls_handle *h);

/* Floating-mean / standard / window GLS for a ragged batch of curves.
 * p_out receives float32 powers at curves[i].out_off .. + nf; invalid powers
 * are -1 (cuvarbase/kernels/lomb.cu:79-80).  Enqueued on `stream`
 * (a cudaStream_t, NULL = legacy default stream); returns before completion.
 * A band wider than the largest grid (2048 x 4096 cells) is computed as
 * consecutive sub-bands of the same points, each centred on its own grid.
 * Replaces lomb_scargle_async with use_fft=True
 * (cuvarbase/lombscargle.py:579-689: two nfft_adjoint_async calls plus the
 * `lomb` kernel, cuvarbase/kernels/lomb.cu:189-220). */
int cuvgls_gls_batch(cuvgls_handle *h, const cuvgls_gls_input *batch,
                     float *p_out, void *stream);

/* GLS of raw light curves: per curve, on the device, w = dy^-2 / sum dy^-2,
 * ybar, yw = w (y - ybar) (FP32, as the reference casts them) and
 * YY = sum w (y - ybar)^2 in FP64, then the same path as cuvgls_gls_batch.
 * Output: the powers into p_out (best_k and best_p NULL), or, with p_out
 * NULL, the best frequency of each curve into best_k / best_p as
 * cuvgls_gls_best gives it.  sum(yw) is an FP64 sum of the FP32 values
 * (the reference sums them sequentially in FP32: powers differ by ~1e-7).
 * Replaces the per-curve host preparation of LombScargleAsyncProcess.run
 * (cuvarbase/lombscargle.py:923-1010 -> setdata, :235-293). */
int cuvgls_gls_raw(cuvgls_handle *h, const cuvgls_raw_input *batch, float *p_out,
                   int64_t *best_k, float *best_p, void *stream);

/* A GLS batch over fixed device buffers, captured once as a CUDA graph.
 * cuvgls_gls_plan_create runs the batch (t, y, dy device pointers, flags 0)
 * once on a private handle -- allocating its workspace, building its plan
 * tables, staging its descriptors -- and captures a second run; each
 * cuvgls_gls_plan_launch then replays every kernel of the batch on whatever
 * the buffers hold now (the per-curve weights and normalisation are
 * recomputed on the device each time), with one launch call and no host
 * planning.  For pipelines that process many batches of one shape.  No
 * reference counterpart (cuvarbase launches nine kernels per curve). */
typedef struct cuvgls_gls_plan cuvgls_gls_plan;
int cuvgls_gls_plan_create(cuvgls_handle *h, const cuvgls_raw_input *batch, float *p_out,
                           int64_t *best_k, float *best_p, cuvgls_gls_plan **plan);
int cuvgls_gls_plan_launch(cuvgls_gls_plan *plan, void *stream);
int cuvgls_gls_plan_destroy(cuvgls_gls_plan *plan);

/* Best frequency of each curve without writing the powers: best_k[i] is the
 * index k (within curve i's band) of its largest valid power, best_p[i] that
 * power (ties: lowest k; -1 and -1 when a curve has no valid power).  The
 * argmax is reduced on the device inside the GLS finish, so no periodogram
 * leaves the GPU.  With CUVGLS_HOST_OUTPUT, best_k / best_p are host arrays;
 * out_off and n_out_total are ignored.  Replaces the host argmax of
 * batched_run_const_nfreq(only_return_best_freqs=True)
 * (cuvarbase/lombscargle.py:1094-1105), whose FAP (fap_baluev, :1115-1184)
 * stays on the host. */
int cuvgls_gls_best(cuvgls_handle *h, const cuvgls_gls_input *batch, int64_t *best_k,
                    float *best_p, void *stream);

/* Same powers by direct summation on the GPU (FP64 phases and sums).
 * Replaces the use_fft=False branch of lomb_scargle_async
 * (cuvarbase/lombscargle.py:641-659, kernel lomb_dirsum at
 * cuvarbase/kernels/lomb.cu:144-165). */
int cuvgls_gls_direct_batch(cuvgls_handle *h, const cuvgls_gls_input *batch,
                            float *p_out, void *stream);

/* Adjoint NFFT of a ragged batch; out is interleaved complex64.  Bands wider
 * than the largest grid are split into sub-bands as in cuvgls_gls_batch.
 * Replaces nfft_adjoint_async (cuvarbase/cunfft.py:163-308). */
int cuvgls_nfft_adjoint_batch(cuvgls_handle *h, const cuvgls_nfft_input *batch,
                              float *out, void *stream);

/* Multi-harmonic floating-mean GLS of one curve by FP64 direct summation
 * (lomb_scargle_direct_sums with nharms harmonics, cuvarbase/lombscargle.py:
 * 337-400 mhdirect_sums, :403-447 add_regularization, :450-536
 * mhgls_from_sums): sums of w and yw against cos and sin of n phi
 * (phi = 2 pi frac(t f), n up to 2 nharms), the 2 nharms x 2 nharms normal
 * equations solved per frequency, P = (YX - sum XX) / YY.  t, yw, w (n
 * points) and freqs (nf, any values) are FP64; ybar = sum(yw) as the caller
 * forms it; amp_d (amplitude prior^-2 per harmonic), cn0, sn0 may be NULL
 * (zeros).  A singular system gives NaN at that frequency.  1 <= nharms <= 8.
 * out: nf doubles.  Flags: CUVGLS_HOST_INPUT / CUVGLS_HOST_OUTPUT. */
int cuvgls_mhgls_direct(cuvgls_handle *h, int32_t nharms, const double *t, const double *yw,
                        const double *w, int64_t n, const double *freqs, int64_t nf,
                        double yy, double ybar, const double *amp_d, const double *cn0,
                        const double *sn0, int32_t flags, double *out, void *stream);

/* Adjoint NFFT in FP64 by direct summation, for use_double: out[k] =
 * sum_j y_j exp(+2 pi i (f0 + k df) t_j), k < nf, as interleaved complex128
 * (exact up to FP64 rounding, cost N x nf per curve).  The batch is read as
 * for cuvgls_nfft_adjoint_batch except that y is given here in FP64
 * (batch->y is not read).  Replaces NFFTAsyncProcess / nfft_adjoint_async
 * with use_double=True (cuvarbase/cunfft.py:23-58, :163-308 in FP64). */
int cuvgls_nfft_adjoint_fp64(cuvgls_handle *h, const cuvgls_nfft_input *batch,
                             const double *y, double *out, void *stream);

/* One curve of a grid finish (the use_grid branch). */
typedef struct {
    int64_t grid_off;  /* first grid cell (complex) of this curve */
    int64_t ng;        /* grid length (reference: int(sigma * nf)) */
    int64_t nf;        /* output frequencies */
    double tmin, tmax; /* observation span of the curve */
    double spp;        /* samples per peak */
    double f0;         /* minimum frequency */
    double b;          /* Gaussian parameter 2 sigma m / ((2 sigma - 1) pi) */
    int64_t out_off;   /* first output element (complex) */
} cuvgls_gridfin_curve;

/* The steps of nfft_adjoint_async after gridding, applied to caller-given
 * grids (its use_grid debug branch, cuvarbase/cunfft.py:270-301): the shift
 * by exp(2 pi i j k0 / ng) when |f0| > 1e-9 (k0 = f0 spp (tmax - tmin);
 * kernel nfft_shift, cuvarbase/kernels/cunfft.cu:59-82), the unnormalised
 * inverse DFT of length ng, and for k < nf the phase and Gaussian
 * deconvolution of kernel normalize (cunfft.cu:214-248).  FP64 by direct
 * summation (cost ng x nf per curve); grid and out are interleaved
 * complex128. */
int cuvgls_nfft_from_grid(cuvgls_handle *h, int32_t n_curves,
                          const cuvgls_gridfin_curve *curves, const double *grid,
                          int64_t n_grid_total, int64_t n_out_total, int32_t flags,
                          double *out, void *stream);

/* Reference-convention real Gaussian grid (the just_return_gridded_data
 * branch of nfft_adjoint_async, cuvarbase/cunfft.py:266-268, kernels
 * precompute_psi + fast_gaussian_grid, cuvarbase/kernels/cunfft.cu:84-163).
 * Uses the handle's sigma and m; grid_out is float32. */
int cuvgls_spread_ref(cuvgls_handle *h, int32_t n_curves,
                      const cuvgls_grid_curve *curves, const double *t,
                      const float *y, int64_t n_points_total,
                      int64_t n_out_total, int32_t flags, float *grid_out,
                      void *stream);

/* Wait for all work the handle enqueued on `stream`, polling with a
 * deadline; returns CUVGLS_ETIMEOUT instead of blocking forever, and
 * CUVGLS_EDEVICE if a kernel raised a device-side error flag
 * (replaces GPUAsyncProcess.finish, cuvarbase/core.py:37-40). */
int cuvgls_sync(cuvgls_handle *h, void *stream, int32_t timeout_ms);

/* Device-side error flags accumulated since the last call (and cleared). */
int cuvgls_device_flags(cuvgls_handle *h, int32_t *flags);

/* Message of the last failing call on this handle ("" if none). */
const char *cuvgls_last_error(cuvgls_handle *h);

/* Grid plan chosen for nf frequencies: total length G = G1 * G2, window
 * half-width m.  (Replaces the sizing in NFFTMemory.allocate_grid and
 * LombScargleMemory.allocate_grids, cuvarbase/cunfft.py:82-92,
 * cuvarbase/lombscargle.py:154-181.) */
int cuvgls_plan(cuvgls_handle *h, int64_t nf, int64_t *G, int32_t *G1,
                int32_t *G2, int32_t *m);

/* Spreading window of the plan chosen for nf frequencies: CUVGLS_WIN_GAUSS
 * (the reference's Gaussian, exp(-d^2 / b), b = 2 sigma m / ((2 sigma - 1)
 * pi)) or CUVGLS_WIN_ES (exponential of semicircle, exp(beta (sqrt(1 - d^2 /
 * m^2) - 1)), chosen only by the autotuner, sigma < 0 at cuvgls_create), and
 * the nominal oversampling sigma it was designed for (G >= sigma nf).  No
 * reference counterpart: cuvarbase always spreads with the Gaussian
 * (cuvarbase/kernels/cunfft.cu:84-163). */
#define CUVGLS_WIN_GAUSS 0
#define CUVGLS_WIN_ES 1
int cuvgls_plan_window(cuvgls_handle *h, int64_t nf, int32_t *window, double *sigma);

/* Grid shapes the planner weighs for GLS bands of nf frequencies with this
 * handle's window, sigma and m: every G1 x G2 of compiled lengths that fits
 * and is at most 10 % above the smallest, cheapest first by the pass costs
 * measured on GB300 (the first is the default choice when it is within 5 %).
 * Writes up to max_shapes pairs to G1[], G2[] and the number available to
 * *n_shapes.  With cuvgls_plan_pin, the input of a run-time tuner that times
 * the shapes on the caller's own curves (cuvarbase_gb300/tune.py).  No
 * reference counterpart: cuvarbase sizes its grids as sigma * nf for cuFFT
 * (cuvarbase/lombscargle.py:154-181). */
int cuvgls_plan_shapes(cuvgls_handle *h, int64_t nf, int32_t max_shapes, int32_t *G1,
                       int32_t *G2, int32_t *n_shapes);

/* Pin the grid shape of GLS bands of exactly nf frequencies on this handle
 * (G1 = G2 = 0 removes the pin).  The shape must fit the handle's plan for
 * nf (CUVGLS_EINVAL otherwise); the window, sigma and m stay the planner's.
 * Pinned shapes are not built ahead by cuvgls_warm.  No reference
 * counterpart. */
int cuvgls_plan_pin(cuvgls_handle *h, int64_t nf, int32_t G1, int32_t G2);

/* The same plan without a handle or a GPU (for hosts planning work). */
int cuvgls_plan_nf(double sigma, int32_t m, int64_t nf, int64_t *G, int32_t *G1,
                   int32_t *G2);

/* Build the grid tables of every plan the handle would choose for GLS
 * bands of nf_min..nf_max frequencies (and for the sub-bands of wider ones)
 * and, with reserve != 0, allocate its whole workspace budget now, so that
 * later batches in that range allocate and build nothing.  No reference
 * counterpart (cuvarbase creates cuFFT plans per curve,
 * cuvarbase/cunfft.py:82-92). */
int cuvgls_warm(cuvgls_handle *h, int64_t nf_min, int64_t nf_max, int32_t reserve);

/* Device bytes a GLS batch of these curves needs, for admission control
 * (the corrected form of LombScargleAsyncProcess.memory_requirement,
 * cuvarbase/lombscargle.py:752-796). */
int cuvgls_batch_bytes(cuvgls_handle *h, int32_t n_curves, const int64_t *n,
                       const int64_t *nf, int32_t host_io, int64_t *bytes);

/* Stages of the profile counters. */
#define CUVGLS_STAGE_PREP 0     /* binning and raw-input preparation */
#define CUVGLS_STAGE_PASS1 1    /* spreading + column FFTs */
#define CUVGLS_STAGE_PASS2 2    /* row FFTs + finish */
#define CUVGLS_STAGE_DIRECT 3   /* direct sums */
#define CUVGLS_STAGE_SPREAD 4   /* reference-convention gridding */
#define CUVGLS_NSTAGES 5

/* Turn per-launch CUDA-event timing on (1, clearing earlier records) or off
 * (0).  Launch counters are always kept.  No reference counterpart: the
 * reference only wraps cuda.start_profiler / stop_profiler
 * (docs/source/plots/benchmarks.py:44-51). */
int cuvgls_profile(cuvgls_handle *h, int32_t enable);

/* Synchronise and read, per stage, the kernel launches since the last
 * cuvgls_profile(h, 1) and the summed launch durations in ms (0 when timing
 * was off).  launches and ms point to CUVGLS_NSTAGES elements. */
int cuvgls_profile_read(cuvgls_handle *h, int64_t *launches, double *ms);

/* A non-blocking CUDA stream for the caller to pass to the batch calls
 * (replaces the pycuda streams of GPUAsyncProcess._create_streams,
 * cuvarbase/core.py:27-29). */
int cuvgls_stream_create(void **stream);
int cuvgls_stream_destroy(void *stream);

/* Page-locked host memory for asynchronous result copies (replaces the
 * aligned host buffers of NFFTMemory.allocate_pinned_cpu and
 * LombScargleMemory.allocate_pinned_cpu, cuvarbase/cunfft.py:94-103,
 * cuvarbase/lombscargle.py:183-191). */
int cuvgls_host_alloc(void **ptr, int64_t bytes);
int cuvgls_host_free(void *ptr);

/* Size of the fixed device scratch array of cuvgls_gls_noalloc (32 MiB) and
 * the most light curves it takes per call. */
#define CUVGLS_NOALLOC_SCRATCH_BYTES (32LL << 20)
#define CUVGLS_NOALLOC_MAX_CURVES 256

/* The GLS batch for callers that cannot allocate memory: code inside a host
 * framework that owns every device allocation (its pool accounts for all of
 * the GPU's memory, so a private cudaMalloc would bypass or starve it), or a
 * real-time loop that may not touch the allocator, which can block or fail,
 * once it runs.  No counterpart in the reference (cuvarbase allocates per
 * curve).  Same arithmetic as cuvgls_gls_batch, with no handle and no
 * allocation of any kind: inputs (t, yw, w) and p_out are device pointers
 * (flags must be 0), and every temporary lives in one static device array of
 * CUVGLS_NOALLOC_SCRATCH_BYTES that each GPU loading the library holds until
 * exit.
 *
 * Limits: at most CUVGLS_NOALLOC_MAX_CURVES curves and only as many as fit in
 * the array (e.g. six curves of nf = 100,000 at sigma 2; one curve up to about
 * nf = 500,000), else CUVGLS_EBUDGET with a message in err (err_len bytes, may
 * be NULL).  One grid plan, that of the largest nf, serves all curves of a
 * call, and bands are not split into sub-bands: an nf beyond the largest
 * single grid (about 4.2e6 at sigma 2) is CUVGLS_ENOTSUP.
 *
 * device_flags (may be NULL): one int32 in device or page-locked host memory
 * that receives this call's device error word (CUVGLS_DEVERR_*) once the
 * call's work on `stream` is done; read it after synchronising the stream.
 * NONFINITE means non-finite inputs were skipped; BINNING means records were
 * lost and the powers are wrong.
 *
 * The first call on a device looks up the array's device address; make that
 * first call before any stream capture.  Calls share the array and each
 * overwrites it, so calls that overlap on the GPU race: serialise them. */
int cuvgls_gls_noalloc(double sigma, int32_t m, const cuvgls_gls_input *batch,
                       float *p_out, int32_t *device_flags, void *stream, char *err,
                       int32_t err_len);

/* ---- continuous-batching server ------------------------------------------
 * No counterpart in the reference (cuvarbase runs one synchronous batch per
 * call); the arithmetic is that of cuvgls_gls_batch.  Requests (one light
 * curve each) are prepared on the submitting thread as
 * LombScargleMemory.setdata does (cuvarbase/lombscargle.py:235-293: nan-means
 * of t and y removed, w = dy^-2 / sum, ybar, yw, YY) and queued; a loop thread
 * admits queued requests under hbm_budget into the next free slot (one handle,
 * stream and hbm_budget / inflight workspace each) and runs them as one batch.
 * A completed request's powers stay in its slot's page-locked result buffer
 * until released; a slot is reused once all of its results are released. */
typedef struct cuvgls_server cuvgls_server;

typedef struct {
    double sigma;        /* as cuvgls_opts (negative: autotune) */
    int32_t m;
    int32_t device;
    int64_t hbm_budget;  /* bytes the batches in flight may use together */
    int32_t max_batch;   /* most requests in one batch */
    int32_t inflight;    /* batches in flight, 1..16 */
    int32_t precision;   /* CUVGLS_PREC_* */
    int32_t mode;        /* CUVGLS_MODE_* */
    float reg;           /* amplitude-prior regulariser lambda (0: none) */
    int32_t reserved;
    int64_t warm_nf_min; /* plan tables built at creation for nf in */
    int64_t warm_nf_max; /*   [warm_nf_min, warm_nf_max] (0: none)  */
    int64_t stage_points;  /* page-locked input staging per slot (0: 1 Mi points) */
    int64_t stage_results; /* page-locked results per slot (0: 16 Mi powers) */
} cuvgls_server_opts;

int cuvgls_server_create(cuvgls_server **out, const cuvgls_server_opts *opts);

/* Queue one light curve (t, y, dy of n points, FP64 host arrays, copied) for
 * the grid f_k = (k0 + k) df, k < nf.  `id` is the caller's tag, unique among
 * requests not yet released.  CUVGLS_EBUDGET if the request alone exceeds a
 * slot's share of the budget. */
int cuvgls_server_submit(cuvgls_server *srv, int64_t id, const double *t, const double *y,
                         const double *dy, int64_t n, int64_t nf, double df, int64_t k0);

/* Wait up to timeout_ms for completed requests and return how many (<= max)
 * were written: tag, status (CUVGLS_OK or the batch's error), pointer to the
 * nf float32 powers (valid until cuvgls_server_release of that tag; NULL on
 * error) and latency in ms (submit to completion).  CUVGLS_ECLOSED once the
 * server has shut down and every completion was returned. */
int cuvgls_server_poll(cuvgls_server *srv, int32_t max, int32_t timeout_ms, int64_t *ids,
                       int32_t *status, const float **results, int64_t *nf,
                       double *latency_ms);

/* Hand a polled request's result buffer back to the server (one, or n at
 * once). */
int cuvgls_server_release(cuvgls_server *srv, int64_t id);
int cuvgls_server_release_many(cuvgls_server *srv, const int64_t *ids, int32_t n);

/* Base and length (powers) of slot k's page-locked result buffer, where
 * polled results point; the buffer moves only when a batch outgrows it. */
int cuvgls_server_slot_buffer(cuvgls_server *srv, int32_t k, const float **ptr, int64_t *len);

/* Device bytes a request of n points and nf frequencies occupies in flight. */
int cuvgls_server_request_bytes(cuvgls_server *srv, int64_t n, int64_t nf, int64_t *bytes);

/* counts[8]: submitted, completed, rejected, batches, requests in batches,
 * bytes per slot, queued, bytes in flight. */
int cuvgls_server_stats(cuvgls_server *srv, int64_t *counts);

/* Stop accepting requests; queued ones still run.  cuvgls_server_destroy
 * shuts down, waits for the queue to drain and frees everything. */
int cuvgls_server_shutdown(cuvgls_server *srv);
int cuvgls_server_destroy(cuvgls_server *srv);

#ifdef __cplusplus
}
#endif

#endif /* CUVGLS_H */
