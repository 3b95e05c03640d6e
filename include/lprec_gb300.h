/*
 * lprec_gb300 -- C ABI of the GB300 log-polar Radon transform library.
 *
 * Drop-in for the native operator class of lprec (src/cuda/lpRgpu.cuh:6-81,
 * exposed to Python through SWIG in src/cuda/lpRgpu.i:10-41) and for the
 * parameter precompute that lprec runs in Python (src/lprec/initsgl.py,
 * initsfwd.py, initsadj.py).  Plain pointers and sizes only; every entry
 * point returns LP_OK or an error code and never resets the device (the
 * reference's callErr, src/cuda/callerr.cu:3-8, calls cudaDeviceReset()).
 * The message of the last error on the calling thread is lp_last_error().
 *
 * Device pointers are float32, C-contiguous:
 *   image    f[S0][N0][N0]
 *   sinogram R[S0][Nproj][N0]
 * with S0 <= Nslices (the batch capacity given at precompute time).
 */
#ifndef LPREC_GB300_H
#define LPREC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LP_OK 0
#define LP_ERR_ARG 1         /* bad argument or malformed parameter arrays */
#define LP_ERR_CUDA 2        /* a CUDA runtime call or kernel launch failed */
#define LP_ERR_OOM 3         /* device or host allocation failed */
#define LP_ERR_STATE 4       /* e.g. lp_fwd before lp_init_fwd */
#define LP_ERR_UNSUPPORTED 5 /* geometry outside what the kernels handle */

#define LP_PRECISION_REFERENCE 0 /* tables evaluated with the reference's float32 steps */
#define LP_PRECISION_FP64 1      /* same index sets, every value in float64, rounded once */

typedef struct lp_handle lp_handle;

/* Message of the last failed call on this thread ("" if none). */
const char* lp_last_error(void);

/* Library version, e.g. 100 for 0.1.0. */
int lp_version(void);

/*
 * Sizes of the five packed parameter arrays for a geometry:
 *   sizes[0] glpars (float32)      initsgl.py:55-56
 *   sizes[1] fwdparsi (int32)      initsfwd.py:96-126 (savePfwdpars)
 *   sizes[2] fwdparamsf (float32)
 *   sizes[3] adjparsi (int32)      initsadj.py:205-244 (savePadjpars)
 *   sizes[4] adjparamsf (float32)
 * filter is one of "none", "ramp", "shepp-logan", "cosine", "cosine2",
 * "hamming", "hann", "parzen" (initsadj.py:107,146-173).  Host only.
 */
int lp_precompute_sizes(int N0, int Nproj, int Nslices, double cor, int cubic, const char* filter,
                        int64_t sizes[5]);

/*
 * Compute the packed parameter arrays (replaces create_gl/create_fwd/
 * create_adj, lpTransform.py:19-31).  fwdparsi/fwdparamsf may be NULL when
 * with_fwd is 0.  precision: LP_PRECISION_REFERENCE or LP_PRECISION_FP64.
 * nthreads: host threads (0 = all).  Host only.
 */
int lp_precompute(int N0, int Nproj, int Nslices, double cor, int cubic, const char* filter, int precision,
                  int with_fwd, int nthreads, float* glpars, int32_t* fwdparsi, float* fwdparamsf,
                  int32_t* adjparsi, float* adjparamsf);

/*
 * The same with the float arrays (fwdparamsf, adjparamsf) in float64: every
 * value rounded once from the float64 computation to double instead of to
 * float32 (no reference counterpart; the reference's format is float32).
 * Feed them to lp_init_fwd_f64 / lp_init_adj_f64.
 */
int lp_precompute_f64(int N0, int Nproj, int Nslices, double cor, int cubic, const char* filter, int precision,
                      int with_fwd, int nthreads, float* glpars, int32_t* fwdparsi, double* fwdparamsf,
                      int32_t* adjparsi, double* adjparamsf);

/*
 * Create a handle on `device` from glpars (replaces lpRgpu::lpRgpu(size_t
 * params, int gpu), src/cuda/lpRgpu.cu:7-39).  n = number of floats.  Besides
 * the spectrum of Nslices slices, a handle whose slices are too few to hold three
 * spectra of a small call (at most 8 * 2048^2 image samples) takes two more spectrum
 * regions of up to that many slices, if they fit in 1 GiB, so that its small calls
 * run their three spans concurrently.
 */
int lp_create(const float* glpars, int64_t n, int device, lp_handle** out);

/* Upload forward tables (replaces lpRgpu::initFwd, src/cuda/lpRgpu.cu:61-85). */
int lp_init_fwd(lp_handle* h, const int32_t* parsi, int64_t ni, const float* parsf, int64_t nf);

/* Upload adjoint tables and filter (replaces lpRgpu::initAdj, src/cuda/lpRgpu.cu:98-133). */
int lp_init_adj(lp_handle* h, const int32_t* parsi, int64_t ni, const float* parsf, int64_t nf);

/*
 * lp_init_fwd / lp_init_adj with the float arrays in float64 (same layout as
 * the packed float32 arrays; no reference counterpart).  Interpolation
 * coordinates are kept on the device as 32-bit fixed point with F fraction
 * bits (F = 17 at N = 2048, steps of 7.6e-6 texel), so float64 tables carry
 * about 60 times less coordinate rounding than float32 ones near 4096.
 */
int lp_init_fwd_f64(lp_handle* h, const int32_t* parsi, int64_t ni, const double* parsf, int64_t nf);
int lp_init_adj_f64(lp_handle* h, const int32_t* parsi, int64_t ni, const double* parsf, int64_t nf);

/* Free everything the handle owns (replaces lpRgpu::~lpRgpu, src/cuda/lpRgpu.cu:41-58). */
int lp_destroy(lp_handle* h);

/*
 * Forward transform R = Radon(f) on device pointers, enqueued on `stream`
 * (a cudaStream_t; NULL = legacy default stream).  Replaces
 * lpRgpu::execFwdManyPtr(size_t Rptr, size_t fptr, int Nslices0, int gpu),
 * src/cuda/lpRgpu.cu:184-193.  Calls of few slices (S0 * N^2 <= 8 * 2048^2 and
 * 3 * S0 <= Nslices, run as one chunk) fork their three spans onto two streams
 * owned by the handle and join them back into `stream` with events before
 * returning work to it, so ordering on `stream` is preserved (a captured graph
 * gets three branches).
 */
int lp_fwd(lp_handle* h, float* R, const float* f, int S0, void* stream);

/*
 * Adjoint / filtered back-projection f = R*(filter(R)) on device pointers.
 * Replaces lpRgpu::execAdjManyPtr(size_t fptr, size_t Rptr, int Nslices0,
 * int gpu), src/cuda/lpRgpu.cu:196-207.  R is read only.  Small calls run their
 * spans concurrently as lp_fwd does (joined before the final sum).
 */
int lp_adj(lp_handle* h, float* f, const float* R, int S0, void* stream);

/*
 * Exact transpose of lp_fwd: f = Radon^T(R), the gradient of <lp_fwd(f), R>
 * with respect to f (used as the autograd backward).  No counterpart in the
 * reference, whose adjoint execAdjManyPtr is a different discretisation
 * (its own kernel fZadj and grids, src/lprec/initsadj.py) and only
 * approximately the transpose.  R is read only.  No atomics: repeated calls give
 * the same bits.  The first call on a handle builds the gather tables and
 * allocates their buffers (make it outside stream capture); when the row spectra
 * and spectra of the three spans fit in 1 GiB more, it allocates them per span
 * and calls of at most 8 * 2048^2 image samples run the spans on the handle's
 * span streams (joined on the caller's stream before the Cartesian gather).
 */
int lp_fwd_transpose(lp_handle* h, float* f, const float* R, int S0, void* stream);

/*
 * Geometry of a handle: out[0..9] = N, N0, Ntheta, Nrho, Nproj (internal),
 * Nproj (caller), Nslices, cor, osangles, cubic.
 */
int lp_get_geometry(const lp_handle* h, int32_t out[10]);

/* Bytes of device memory the handle holds. */
int lp_device_bytes(const lp_handle* h, int64_t* bytes);

/*
 * Instrumentation (no counterpart in the reference, whose only timing is
 * wall-clock tic/toc in tests/timing.py:2-11).
 *   lp_launch_count   kernels this library has launched in the process
 *   lp_kernel_count   number of kernel kinds; lp_kernel_name(id) their names
 *   lp_set_profiling  bracket every launch of the handle with CUDA events on
 *                     the launch stream
 *   lp_profile_collect  wait for the recorded events and return, per kernel
 *                     kind, total milliseconds and launches (arrays of
 *                     lp_kernel_count() entries); clears the record
 */
/*
 * Forward transform without device allocation (no counterpart in the
 * reference).  Same result as lp_fwd, but its scratch -- the prefiltered
 * image and the log-polar spectrum -- lives in one device array of
 * LP_NOALLOC_SCRATCH_BYTES that the library declares at file scope, so the
 * call allocates and frees nothing.  Meant for callers whose device memory is
 * owned by another allocator or a fixed pool and that may not call cudaMalloc
 * or cudaFree while processing.  Calls needing more scratch than the fixed
 * size (lp_noalloc_scratch_bytes) fail with LP_ERR_UNSUPPORTED.  The first
 * call on a device loads the array (with lazy module loading, the CUDA
 * default, its 64 MiB of device memory are reserved then) and looks up its
 * address: make that first call -- S0 = 0 does only this -- before reserving
 * a fixed pool and before any stream capture.  The address is looked up again
 * if the device's context is recreated.  All calls share the array, so calls
 * that overlap on the GPU race.
 */
#define LP_NOALLOC_SCRATCH_BYTES (64LL * 1024 * 1024)
int lp_fwd_noalloc(lp_handle* h, float* R, const float* f, int S0, void* stream);
int lp_noalloc_scratch_bytes(const lp_handle* h, int S0, int64_t* bytes);
/* Test hook: fill the allocation-free scratch array of `device` with `value`. */
int lp_debug_fill_noalloc_scratch(int device, float value, void* stream);

/*
 * Helpers for device arrays handed over through __cuda_array_interface__
 * (no reference counterpart; lprec's lpTransform.fwdp/adjp pass raw CuPy
 * pointers unchecked, src/lprec/lpTransform.py:42-50).
 *   lp_pointer_device  the device a pointer's memory belongs to (LP_ERR_ARG if
 *                      it is not device or managed memory)
 *   lp_stream_wait     make `waiter` wait for the work enqueued on `producer`
 *                      so far (an event recorded on `producer`); the special
 *                      handles 1 (legacy default stream) and 2 (per-thread
 *                      default stream) are accepted as CUDA defines them
 */
int lp_pointer_device(const void* p, int* device);
int lp_stream_wait(int device, void* waiter, void* producer);

long long lp_launch_count(void);
int lp_kernel_count(void);
const char* lp_kernel_name(int id);
int lp_set_profiling(lp_handle* h, int enable);
int lp_profile_collect(lp_handle* h, double* ms, int64_t* launches);

/*
 * Batch schedule and kernel shapes (no reference counterpart; the reference
 * runs every kernel once over the whole batch on the legacy stream).
 * sched[LP_SCHEDULE_LEN] = {fwd_chunk, fwd_streams, fwd_theta_block,
 *                           adj_chunk, adj_streams, adj_theta_block}:
 * lp_fwd / lp_adj split a call's S0 slices into chunks of `chunk` slices
 * (0: one chunk) processed in turn, alternating between the caller's stream
 * and a second stream owned by the handle when `streams` is 2 (forked from
 * and joined back into the caller's stream with events); `theta_block` is the
 * thread count (256 or 512) of the theta-convolution blocks.  Results do not
 * depend on the schedule.  lp_set_schedule takes the first n entries (the
 * rest get the defaults {0, 1, 256, 0, 1, 256}); lp_get_schedule writes n.
 */
#define LP_SCHEDULE_LEN 6
int lp_set_schedule(lp_handle* h, const int32_t* sched, int n);
int lp_get_schedule(const lp_handle* h, int32_t* out, int n);

/*
 * Autotuner (no reference counterpart): time every candidate schedule (chunks
 * of 64, 32, 16, 8 slices or none; one or two streams; theta-convolution
 * blocks of 256 or 512 threads) of lp_fwd and lp_adj on
 * S0 slices, using the caller's device buffers R[S0][Nproj][N0] and
 * f[S0][N0][N0] as scratch input/output (their contents are overwritten), and
 * keep the fastest for this handle.  Synchronises `stream`; do not call it
 * during graph capture.  out_ms (may be NULL): best fwd and adj ms per call.
 */
int lp_autotune(lp_handle* h, float* R, float* f, int S0, void* stream, float out_ms[2]);

/*
 * Test hook (no reference counterpart): fill the handle's intermediate device
 * buffers (log-polar spectrum, prefiltered image and sinogram, log-polar
 * columns) with `value`, enqueued on `stream`.  Results of later calls must
 * not depend on it: every buffer element a kernel reads was written earlier
 * in the same call.
 */
int lp_debug_fill_scratch(lp_handle* h, float value, void* stream);

/*
 * Fused vector kernels of the iterative solvers (no single reference
 * counterpart: they replace the CuPy elementwise updates and float32 sums of
 * src/lprec/lpmethods.py:62-128).  Device pointers; float32 vectors, float64
 * accumulation; scalars (num, den, results) are device float64 values, so an
 * iteration needs no host round trip.  Reductions are deterministic (fixed
 * grid and summation order).  `work` is caller-provided device scratch of
 * lp_vec_work_doubles(S) doubles (lp_vec_work_doubles(1) for lp_cg_step);
 * these calls allocate nothing.
 *
 *   lp_vec_dot:  out[s] = sum_i a[s*m + i] * b[s*m + i], s < S
 *   lp_cg_step:  alpha = (float)(*num / *den); x += alpha p; r -= alpha q;
 *                *rr = r.r (after the update)
 *   lp_cg_dir:   p = r + (float)(*num / *den) * p
 *   lp_em_ratio: g = tomo / (g + eps)
 *   lp_em_step:  x *= upd / xi
 */
int64_t lp_vec_work_doubles(int S);
int lp_vec_dot(const float* a, const float* b, int64_t m, int S, double* work, double* out, void* stream);
int lp_cg_step(float* x, float* r, const float* p, const float* q, int64_t n, const double* num, const double* den,
               double* work, double* rr, void* stream);
int lp_cg_dir(float* p, const float* r, int64_t n, const double* num, const double* den, void* stream);
int lp_em_ratio(float* g, const float* tomo, float eps, int64_t n, void* stream);
int lp_em_step(float* x, const float* upd, const float* xi, int64_t n, void* stream);

/*
 * Fused updates of the total-variation solvers tv, tve and tvl1 (one
 * Chambolle-Pock iteration = lp_tv_prox0, lp_fwd, lp_tv_prox1, lp_adj,
 * lp_tv_recon).  Each replaces a group of the reference's CuPy statements
 * (src/lprec/lpmethods.py:158-178 for tv, :209-232 tve, :264-286 tvl1) by one
 * pass, computed in the statements' float32 operation order without fused
 * multiply-adds, so results equal the statement sequence's bit for bit.  Images
 * are [S][ny][nx] float32, sinograms n floats; c and lam are the reference's
 * Python scalars, rounded to float32 where they meet an array (1 + c and 4*c
 * rounded once).  Device pointers; nothing is allocated.
 *
 *   lp_tv_prox0: prox0x[.., :-1] += c*(recon[.., 1:] - recon[.., :-1]) along x,
 *                prox0y likewise along y; both divided by
 *                maximum(1, sqrt(prox0x^2 + prox0y^2)/lam)       (:158-163)
 *   lp_tv_prox1: prox1 <- the data term's proximal step (mode):
 *                LP_TV_L2      (prox1 + c g - c tomo)/(1 + c)     (:166)
 *                LP_TV_ENTROPY u = prox1 + c g; t = 0.5(u - 1 + sqrt((u-1)^2 + 4c tomo));
 *                              u - max(t, 0)                      (:218-220)
 *                LP_TV_L1      t = prox1 + c g - c tomo; t - max(|t| - 1, 0) sign(t) (:272-275)
 *   lp_tv_recon: div0 from backward differences of prox0x (x) and prox0y (y);
 *                recon0 <- recon0 - c p + c div0; recon <- 2 recon0(new) - recon0(old)
 *                                                                 (:169-178)
 */
#define LP_TV_L2 0
#define LP_TV_ENTROPY 1
#define LP_TV_L1 2
int lp_tv_prox0(float* prox0x, float* prox0y, const float* recon, int S, int ny, int nx, double c, double lam,
                void* stream);
int lp_tv_prox1(float* prox1, const float* g, const float* tomo, int64_t n, double c, int mode, void* stream);
int lp_tv_recon(float* recon0, float* recon, const float* p, const float* prox0x, const float* prox0y, int S, int ny,
                int nx, double c, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* LPREC_GB300_H */
