// Host side of the library: the C ABI, the handle, conversion of the packed
// parameter arrays (src/cuda/params.cu:40-145 layout) into the column-major
// device tables the kernels read, and the fwd/adj pipelines.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <string>
#include <vector>

#include "../../include/lprec_gb300.h"
#include "host_fft.h"
#include "lp_kernels.cuh"

using namespace lpgb;

// ---------------------------------------------------------------------------
// errors: status codes plus a thread-local message; the device is never reset
// ---------------------------------------------------------------------------
static thread_local std::string g_err;

static int set_err(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

// shared with precompute.cpp
int lp_internal_set_err(int code, const char* msg) { return set_err(code, "%s", msg); }

#define CUDA_TRY(call)                                                                                   \
  do {                                                                                                   \
    cudaError_t e_ = (call);                                                                             \
    if (e_ != cudaSuccess)                                                                               \
      return set_err(e_ == cudaErrorMemoryAllocation ? LP_ERR_OOM : LP_ERR_CUDA, "%s: %s (%s:%d)", #call, \
                     cudaGetErrorString(e_), __FILE__, __LINE__);                                        \
  } while (0)

namespace {

// Makes `dev` current for the scope of a call (only switching when needed, so
// calls made while a stream on that device is being captured stay free of
// device changes).
struct DeviceGuard {
  int prev = -1;
  bool switched = false;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) {
      cudaSetDevice(dev);
      switched = true;
    }
  }
  ~DeviceGuard() {
    if (switched && prev >= 0) cudaSetDevice(prev);
  }
};

template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  void free_() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

template <typename T>
static cudaError_t dev_alloc(DevBuf<T>& b, size_t n) {
  b.free_();
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc((void**)&b.p, n * sizeof(T));
  if (e == cudaSuccess) b.n = n;
  else b.p = nullptr;
  return e;
}

template <typename T>
static cudaError_t dev_upload(DevBuf<T>& b, const std::vector<T>& v) {
  cudaError_t e = dev_alloc(b, v.size());
  if (e != cudaSuccess) return e;
  if (v.empty()) return cudaSuccess;
  return cudaMemcpy(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
}


}  // namespace

struct FwdDev {
  int F = 16;              // fixed-point fraction bits of every coordinate table below
  float fsc = 1.f / 65536.f;
  DevBuf<int2> c2lp[3];    // [Nth][Nrho]
  DevBuf<int> thc;         // [Nproj]
  DevBuf<int> rhoc;        // [Nproj][N]
  DevBuf<int> rows[3];     // internal rows per span (multiples of os only)
  int nrows[3] = {0, 0, 0};
  DevBuf<float2> fz;       // Hermitian-extended kernel, tiled spectrum layout
  int lo = 0, hi = 0;      // theta columns the polar gather reads
  DevBuf<float> fbuf;      // [Nslices][N][N]
  // cubic mode: the prefiltered image of each slice as a 2-D CUDA array that
  // the Cartesian -> log-polar gather reads with texture gathers
  std::vector<cudaArray_t> arr;
  std::vector<cudaTextureObject_t> tex_h;
  std::vector<cudaSurfaceObject_t> surf_h;
  DevBuf<cudaTextureObject_t> tex;
  DevBuf<cudaSurfaceObject_t> surf;
  // exact transpose: per span, column blocks of kTransposeCW columns with the
  // range of sinogram rows whose theta taps touch them; columns holding disk points
  DevBuf<int2> blk[3];
  int nblk[3] = {0, 0, 0};
  int dlo = 0, dhi = -1;
  DevBuf<int2> ival;       // [Nth] rho interval of each column's disk points (same for every span)
  int rho_mono = 1;        // every row's first rho tap strictly monotone over the row (see FwdTRowsArgs)
  DevBuf<int> rbase;       // [Nproj] per internal row: its smallest first rho tap
  // exact transpose, built by its first call: the image cells' lists of log-polar
  // points of all spans (CSR), the points' real values in list order (FwdTColsArgs)
  // and the row spectra [Nslices][rows of a span][rowspec_stride(Nk)]
  bool gather_ready = false;
  DevBuf<int> cell_off;
  DevBuf<int2> cell_pts;
  DevBuf<int> lppos[3];    // per span [W][Nrho]: a log-polar point's index in cell_pts, -1 for none
  size_t npts = 0;
  DevBuf<float> lpg;
  DevBuf<float2> rowspec;
  // per span, the theta columns' lists of (row, tap weight), rows ascending (CSR over
  // the Nth columns): the theta convolution gathers its input from the row spectra
  DevBuf<int> coff[3];
  DevBuf<int2> cent[3];
  // small handles run the three spans on their own streams: the row spectra then hold
  // one region per span and spans 1 and 2 take their spectra from tspec
  bool tspread = false;
  DevBuf<float2> tspec;
};
static const int kTransposeCW = 8;
// extra device memory the exact transpose may take to run its spans concurrently
static const size_t kTransposeSpreadBytes = (size_t)1 << 30;

struct AdjDev {
  int F = 16;              // fixed-point fraction bits of every coordinate table below
  float fsc = 1.f / 65536.f;
  DevBuf<int> ta[3];       // [Nth]
  DevBuf<int> sx[3];       // [Nth][Nrho]
  DevBuf<int> woff[3];     // [Nth+1]
  DevBuf<int4> wpt[3];
  DevBuf<int2> c2lp[3];    // [N0][N0]
  int clo[3], chi[3];
  int lo2 = 0, hi2 = 0, W2 = 1;
  DevBuf<float2> fz;       // Hermitian-extended kernel, tiled spectrum layout
  DevBuf<float> H;         // [4N] or empty
  bool filter = false;
  DevBuf<float> rbuf;      // [Nslices][Nproj][N]
  DevBuf<float> rin;       // [Nslices][Nproj][N] ingest output before the column prefilter (cubic)
  DevBuf<float> G[3];      // [Nslices][W2][Nrho] (linear mode)
  // cubic mode: the real log-polar columns of each span and slice as 2-D CUDA
  // arrays (x = rho, y = theta - lo2), written through surfaces, read by gathers
  std::vector<cudaArray_t> arr;
  std::vector<cudaTextureObject_t> tex_h[3];
  std::vector<cudaSurfaceObject_t> surf_h[3];
  DevBuf<cudaTextureObject_t> tex[3];
  DevBuf<cudaSurfaceObject_t> surf[3];
};

enum KernelId {
  K_FWD_INGEST = 0,
  K_COL_PREFILTER,
  K_FWD_C2LP,
  K_THETA_CONV,
  K_FWD_LP2POLAR,
  K_ADJ_INGEST,
  K_ADJ_POLAR2LP,
  K_ADJ_LPCOLS,
  K_ADJ_LP2CART,
  K_FWDT_ROWS,
  K_FWDT_COLSUM,
  K_FWDT_COLS,
  K_FWDT_GATHER,
  K_PREFILTER_T,
  K_CROP,
  K_COUNT
};
static const char* kKernelNames[K_COUNT] = {"fwd_ingest",   "col_prefilter", "fwd_c2lp",   "theta_conv",
                                             "fwd_lp2polar", "adj_ingest",    "adj_polar2lp", "adj_lpcols",
                                             "adj_lp2cart",  "fwdT_rows",     "fwdT_colsum", "fwdT_cols",  "fwdT_gather",
                                             "prefilter_T", "crop"};

static std::atomic<long long> g_launches(0);

struct ProfRec {
  int kid;
  cudaEvent_t a, b;
};

struct lp_handle {
  int device = 0;
  bool profiling = false;
  std::vector<ProfRec> prof;        // recorded launches not yet collected
  std::vector<cudaEvent_t> evpool;  // reusable events
  int N = 0, N0 = 0, Nth = 0, Nrho = 0, Nk = 0, Nproj = 0, Nproj0 = 0, Nslices = 0, cor = 0, os = 1, cubic = 1;
  float cor_f = 0.f;
  std::vector<float> erho_h;
  DevBuf<float> erho;
  DevBuf<float2> spec;     // [Nslices][Nk][Nth]
  // spans 1 and 2 of a concurrent-span call that the handle's own spectrum slots do not
  // hold 3 times over (a handle of few slices): [2][sspec_slices][Nk][Nth]
  DevBuf<float2> sspec;
  int sspec_slices = 0;
  DevBuf<float2> tw_rho;   // FFT twiddles for length Nrho (also the FBP filter's 2N)
  DevBuf<float2> tw_th;    // FFT twiddles for length Nth
  FwdDev* fwd = nullptr;
  AdjDev* adj = nullptr;
  FFTPlan plan_rho, plan_th, plan_filt;
  // batch schedule of lp_fwd / lp_adj: slices per chunk (0: the whole call in
  // one chunk) and streams the chunks alternate on (1 or 2); set by
  // lp_set_schedule or lp_autotune
  int fwd_chunk = 0, fwd_streams = 1, adj_chunk = 0, adj_streams = 1;
  int fwd_tblock = 256, adj_tblock = 256;  // threads per block of the theta convolution
  cudaStream_t side = nullptr;        // second stream of a 2-stream schedule
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // spans 1 and 2 of a call of few slices run on their own streams (spread_spans)
  cudaStream_t span_st[2] = {nullptr, nullptr};
  cudaEvent_t ev_sfork = nullptr, ev_sjoin[2] = {nullptr, nullptr};
};

static void free_fwd(FwdDev* f) {
  if (!f) return;
  for (int k = 0; k < 3; ++k) {
    f->c2lp[k].free_();
    f->rows[k].free_();
    f->blk[k].free_();
    f->coff[k].free_();
    f->cent[k].free_();
  }
  f->tspec.free_();
  f->rbase.free_();
  f->cell_off.free_();
  f->cell_pts.free_();
  for (int k = 0; k < 3; ++k) f->lppos[k].free_();
  f->lpg.free_();
  f->rowspec.free_();
  f->thc.free_();
  f->rhoc.free_();
  f->fz.free_();
  f->fbuf.free_();
  f->ival.free_();
  for (cudaTextureObject_t t : f->tex_h) cudaDestroyTextureObject(t);
  for (cudaSurfaceObject_t t : f->surf_h) cudaDestroySurfaceObject(t);
  for (cudaArray_t a : f->arr) cudaFreeArray(a);
  f->tex.free_();
  f->surf.free_();
  delete f;
}

static void free_adj(AdjDev* a) {
  if (!a) return;
  for (int k = 0; k < 3; ++k) {
    a->ta[k].free_();
    a->sx[k].free_();
    a->woff[k].free_();
    a->wpt[k].free_();
    a->c2lp[k].free_();
    a->G[k].free_();
  }
  a->fz.free_();
  a->H.free_();
  a->rbuf.free_();
  a->rin.free_();
  for (int k = 0; k < 3; ++k) {
    for (cudaTextureObject_t t : a->tex_h[k]) cudaDestroyTextureObject(t);
    for (cudaSurfaceObject_t t : a->surf_h[k]) cudaDestroySurfaceObject(t);
    a->tex[k].free_();
    a->surf[k].free_();
  }
  for (cudaArray_t x : a->arr) cudaFreeArray(x);
  delete a;
}

// Hermitian extension of the half kernel fZ[Nrho][Nth/2+1] (cuFFT R2C layout,
// lpRgpu.cu:28-34) to the rho-half / theta-full layout [Nrho/2+1][Nth], times the
// 1/(Nrho*Nth) that the reference applies in its kernel multiply (lpRgpu.cu:274,
// 318; a power of two at power-of-two sizes, so the products are unchanged).  Only the Hermitian part of the kernel affects C2R output, so the
// kt = 0 and kt = Nth/2 columns are symmetrised.
template <typename Real>
static std::vector<float2> extend_kernel(const Real* v, int Nrho, int Nth) {
  const int nh = Nth / 2 + 1;
  const int Nk = Nrho / 2 + 1;
  auto at = [&](int kr, int kt) {
    const size_t i = 2 * ((size_t)kr * nh + kt);
    return std::make_pair((double)v[i], (double)v[i + 1]);
  };
  const double scale = 1.0 / ((double)Nrho * (double)Nth);
  std::vector<float2> out(spec_slice(Nk, Nth), make_float2(0.f, 0.f));
  for (int kr = 0; kr < Nk; ++kr) {
    const int mr = (Nrho - kr) % Nrho;
    for (int kt = 0; kt < Nth; ++kt) {
      double re, im;
      if (kt == 0 || kt == Nth / 2) {
        auto a = at(kr, kt);
        auto b = at(mr, kt);
        re = 0.5 * (a.first + b.first);
        im = 0.5 * (a.second - b.second);
      } else if (kt < Nth / 2) {
        auto a = at(kr, kt);
        re = a.first;
        im = a.second;
      } else {
        auto b = at(mr, Nth - kt);
        re = b.first;
        im = -b.second;
      }
      out[sidx(kr, kt, Nth)] = make_float2((float)(re * scale), (float)(im * scale));
    }
  }
  return out;
}

static bool finite_coord(double v, double lim) { return std::isfinite(v) && std::fabs(v) < lim; }

// A W x H float array with a gather texture (normalised, wrap) and a surface.
static cudaError_t make_gather_array(int W, int H, std::vector<cudaArray_t>& arrs, cudaTextureObject_t* tex,
                                     cudaSurfaceObject_t* surf) {
  cudaChannelFormatDesc fd = cudaCreateChannelDesc<float>();
  cudaArray_t a = nullptr;
  cudaError_t e = cudaMallocArray(&a, &fd, W, H, cudaArrayTextureGather | cudaArraySurfaceLoadStore);
  if (e != cudaSuccess) return e;
  arrs.push_back(a);
  cudaResourceDesc rd;
  memset(&rd, 0, sizeof(rd));
  rd.resType = cudaResourceTypeArray;
  rd.res.array.array = a;
  cudaTextureDesc td;
  memset(&td, 0, sizeof(td));
  td.addressMode[0] = cudaAddressModeWrap;
  td.addressMode[1] = cudaAddressModeWrap;
  td.filterMode = cudaFilterModePoint;
  td.readMode = cudaReadModeElementType;
  td.normalizedCoords = 1;
  e = cudaCreateTextureObject(tex, &rd, &td, nullptr);
  if (e != cudaSuccess) return e;
  return cudaCreateSurfaceObject(surf, &rd);
}

// One N x N float array per slice, written through a surface by the column
// prefilter and read through a gather texture (normalised, wrap on both axes)
// by the Cartesian -> log-polar gather.  Skipped (left empty) when the device
// cannot gather from textures that large.
static cudaError_t make_slice_textures(FwdDev* F, int S, int N, int device) {
  int gw = 0, gh = 0;
  cudaDeviceGetAttribute(&gw, cudaDevAttrMaxTexture2DGatherWidth, device);
  cudaDeviceGetAttribute(&gh, cudaDevAttrMaxTexture2DGatherHeight, device);
  if (N > gw || N > gh) return cudaSuccess;
  cudaChannelFormatDesc fd = cudaCreateChannelDesc<float>();
  for (int s = 0; s < S; ++s) {
    cudaArray_t a = nullptr;
    cudaError_t e = cudaMallocArray(&a, &fd, N, N, cudaArrayTextureGather | cudaArraySurfaceLoadStore);
    if (e != cudaSuccess) return e;
    F->arr.push_back(a);
    cudaResourceDesc rd;
    memset(&rd, 0, sizeof(rd));
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = a;
    cudaTextureDesc td;
    memset(&td, 0, sizeof(td));
    td.addressMode[0] = cudaAddressModeWrap;
    td.addressMode[1] = cudaAddressModeWrap;
    td.filterMode = cudaFilterModePoint;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 1;
    cudaTextureObject_t t = 0;
    e = cudaCreateTextureObject(&t, &rd, &td, nullptr);
    if (e != cudaSuccess) return e;
    F->tex_h.push_back(t);
    cudaSurfaceObject_t so = 0;
    e = cudaCreateSurfaceObject(&so, &rd);
    if (e != cudaSuccess) return e;
    F->surf_h.push_back(so);
  }
  cudaError_t e = dev_upload(F->tex, F->tex_h);
  if (e == cudaSuccess) e = dev_upload(F->surf, F->surf_h);
  return e;
}

// W[t] = exp(-2 pi i t / L), evaluated in float64
static std::vector<float2> twiddles(int L) {
  std::vector<float2> w(L);
  for (int t = 0; t < L; ++t) {
    const double a = -2.0 * lpgb_host::kPi * (double)t / (double)L;
    w[t] = make_float2((float)cos(a), (float)sin(a));
  }
  return w;
}

// The FBP filter of applyFilter (src/cuda/lpRgpu.cu:333-382) is a circular
// convolution of length 4N of a zero-padded row with h = IFFT(filter shifted
// by 2N).  Outputs and inputs both lie in one N-sample window, so only
// h[d] for |d| < N matters and a circular convolution of length 2N with the
// folded kernel gives the same result.  Returns its spectrum divided by 2N
// (real: the filter is symmetric), or an empty vector if it is not symmetric.
template <typename Real>
static std::vector<float> fbp_kernel_2n(const Real* filt, int N) {
  using lpgb_host::cd;
  const int M = 4 * N, L2 = 2 * N;
  std::vector<cd> H(M), tmp(M);
  for (int k = 0; k < M; ++k) H[k] = cd((double)filt[(k + 2 * N) % M], 0.0);
  for (int k = 1; k < M; ++k)
    if (H[k].real() != H[M - k].real()) return {};
  // h = IFFT(H) / M; H is real and symmetric, so IFFT = FFT
  lpgb_host::HostFFT fM(M);
  fM.run(H.data(), tmp.data());
  std::vector<cd> h2(L2, cd(0, 0)), t2(L2);
  for (int d = 0; d < N; ++d) h2[d] = cd(H[d].real() / M, 0.0);
  for (int e = 1; e < N; ++e) h2[L2 - e] = cd(H[M - e].real() / M, 0.0);
  lpgb_host::HostFFT f2(L2);
  f2.run(h2.data(), t2.data());
  std::vector<float> out(L2);
  for (int k = 0; k < L2; ++k) out[k] = (float)(h2[k].real() / L2);
  return out;
}

// taps of one axis for coordinate t: first index and count
// Fixed-point coordinates (value = v * 2^-F): F is the largest number of fraction
// bits that keeps (max |coordinate| + 2) * 2^F below 2^30, so sums of a
// coordinate and a table offset stay inside int32.
static int fixed_bits(double maxabs) {
  int F = 0;
  while (F < 24 && std::ldexp(maxabs + 2.0, F + 1) < 1073741824.0) ++F;
  return F;
}
static inline int to_fixed(double x, int F) { return std::isnan(x) ? LP_FX_NONE : (int)std::llrint(std::ldexp(x, F)); }
// first interpolation tap of a fixed-point coordinate (the kernels' v >> F)
static inline int first_tap(int v, int F, int cubic) { return (v >> F) - (cubic ? 1 : 0); }

static void destroy_span_streams(lp_handle* h) {
  for (int i = 0; i < 2; ++i) {
    if (h->span_st[i]) cudaStreamDestroy(h->span_st[i]);
    if (h->ev_sjoin[i]) cudaEventDestroy(h->ev_sjoin[i]);
  }
  if (h->ev_sfork) cudaEventDestroy(h->ev_sfork);
}

// A call of at most kSpreadSamples image samples (n slices of N x N), run as one
// chunk, runs its three spans concurrently: span k on its own stream (span 0 on
// the caller's) in spectrum slots slot + k*n.  Small grids leave most SMs idle,
// and the spans are independent from the prefiltered input until the forward's
// output rows (disjoint per span) or the adjoint's final sum (after the join).
// Measured: up to 8 slices at N=2048 and 32 at N=1024 gain; larger calls fill
// the GPU already and their concurrent spans compete.
constexpr double kSpreadSamples = 8.0 * 2048 * 2048;
// the extra spectrum regions of a handle of few slices may take at most this much
static const size_t kSpreadSpecBytes = (size_t)1 << 30;
static bool spread_spans(const lp_handle* h, int slot, int n, bool one_chunk) {
  return one_chunk && (double)n * h->N * h->N <= kSpreadSamples &&
         (slot + 3 * n <= h->Nslices || n <= h->sspec_slices);
}
// the spectrum of span k of a call of n slices from slot (spread: its own region)
static float2* span_spec(lp_handle* h, int slot, int n, int k, bool spread) {
  const size_t sl = spec_slice(h->Nk, h->Nth);
  float2* spec = h->spec.p + (size_t)slot * sl;
  if (!spread || k == 0) return spec;
  if (slot + 3 * n <= h->Nslices) return spec + (size_t)k * n * sl;
  return h->sspec.p + (size_t)(k - 1) * h->sspec_slices * sl;
}
static cudaError_t span_fork(lp_handle* h, cudaStream_t st) {
  cudaError_t e = cudaEventRecord(h->ev_sfork, st);
  for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaStreamWaitEvent(h->span_st[i], h->ev_sfork, 0);
  return e;
}
static cudaError_t span_join(lp_handle* h, cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
    e = cudaEventRecord(h->ev_sjoin[i], h->span_st[i]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, h->ev_sjoin[i], 0);
  }
  return e;
}

static cudaEvent_t take_event(lp_handle* h) {
  if (!h->evpool.empty()) {
    cudaEvent_t e = h->evpool.back();
    h->evpool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// Launch one kernel; with profiling on, bracket it with events on its stream.
template <typename F>
static cudaError_t launch(lp_handle* h, int kid, cudaStream_t st, F fn) {
  ProfRec r{kid, nullptr, nullptr};
  if (h->profiling) {
    r.a = take_event(h);
    r.b = take_event(h);
    cudaEventRecord(r.a, st);
  }
  cudaError_t e = fn();
  if (e == cudaSuccess) g_launches.fetch_add(1, std::memory_order_relaxed);
  if (h->profiling) {
    cudaEventRecord(r.b, st);
    h->prof.push_back(r);
  }
  return e;
}

extern "C" {

const char* lp_last_error(void) { return g_err.c_str(); }

long long lp_launch_count(void) { return g_launches.load(); }

int lp_kernel_count(void) { return K_COUNT; }

const char* lp_kernel_name(int id) { return (id >= 0 && id < K_COUNT) ? kKernelNames[id] : ""; }

int lp_set_profiling(lp_handle* h, int enable) {
  if (!h) return set_err(LP_ERR_ARG, "lp_set_profiling: null handle");
  h->profiling = enable != 0;
  return LP_OK;
}

int lp_profile_collect(lp_handle* h, double* ms, int64_t* launches) {
  if (!h || !ms || !launches) return set_err(LP_ERR_ARG, "lp_profile_collect: null pointer");
  DeviceGuard g(h->device);
  for (int k = 0; k < K_COUNT; ++k) {
    ms[k] = 0.0;
    launches[k] = 0;
  }
  for (const ProfRec& r : h->prof) {
    float t = 0.f;
    CUDA_TRY(cudaEventSynchronize(r.b));
    CUDA_TRY(cudaEventElapsedTime(&t, r.a, r.b));
    ms[r.kid] += t;
    launches[r.kid] += 1;
    h->evpool.push_back(r.a);
    h->evpool.push_back(r.b);
  }
  h->prof.clear();
  return LP_OK;
}

int lp_version(void) { return 100; }

int lp_create(const float* glpars, int64_t n, int device, lp_handle** out) {
  if (!glpars || !out) return set_err(LP_ERR_ARG, "lp_create: null pointer");
  *out = nullptr;
  if (n < 10) return set_err(LP_ERR_ARG, "lp_create: glpars too short (%lld)", (long long)n);
  lp_handle h0;
  h0.device = device;
  h0.N = (int)glpars[0];
  h0.N0 = (int)glpars[1];
  h0.Nth = (int)glpars[2];
  h0.Nrho = (int)glpars[3];
  const int nspan = (int)glpars[4];
  h0.Nproj = (int)glpars[5];
  h0.Nslices = (int)glpars[6];
  h0.cor_f = glpars[7];
  h0.cor = (int)glpars[7];
  h0.os = (int)glpars[8];
  h0.cubic = (int)glpars[9];
  if (nspan != 3) return set_err(LP_ERR_UNSUPPORTED, "lp_create: Nspan=%d (only 3 is supported)", nspan);
  if (h0.N < 16 || h0.N % 16 != 0 || h0.N > 8192)
    return set_err(LP_ERR_UNSUPPORTED, "lp_create: N=%d must be a multiple of 16 in [16, 8192]", h0.N);
  if (h0.Nth != h0.N || h0.Nrho != 2 * h0.N) return set_err(LP_ERR_ARG, "lp_create: Ntheta/Nrho inconsistent");
  if (h0.Nslices > 65535) return set_err(LP_ERR_UNSUPPORTED, "lp_create: Nslices=%d above 65535", h0.Nslices);
  if (h0.N0 < 1 || h0.N0 > h0.N || h0.os < 1 || h0.Nproj < 1 || h0.Nproj % h0.os != 0 || h0.Nslices < 1)
    return set_err(LP_ERR_ARG, "lp_create: inconsistent geometry");
  if (h0.N / 2 - h0.cor < 0 || h0.N / 2 - h0.cor + h0.N0 > h0.N)
    return set_err(LP_ERR_ARG, "lp_create: cor=%d out of range", h0.cor);
  if ((int64_t)n < 10 + (int64_t)h0.Nrho * h0.Nth)
    return set_err(LP_ERR_ARG, "lp_create: glpars too short for erho");
  h0.Nproj0 = h0.Nproj / h0.os;
  h0.Nk = h0.Nrho / 2 + 1;
  lp_handle* h = new lp_handle(h0);
  h->erho_h.resize(h->Nrho);
  for (int r = 0; r < h->Nrho; ++r) h->erho_h[r] = glpars[10 + (size_t)r * h->Nth];
  DeviceGuard g(device);
  cudaError_t e = configure_kernels(h->N);
  if (e == cudaSuccess) e = dev_upload(h->erho, h->erho_h);
  if (e == cudaSuccess) e = dev_upload(h->tw_rho, twiddles(h->Nrho));
  if (e == cudaSuccess) e = dev_upload(h->tw_th, twiddles(h->Nth));
  if (e == cudaSuccess) e = dev_alloc(h->spec, (size_t)h->Nslices * spec_slice(h->Nk, h->Nth));
  {
    // concurrent spans for the calls that qualify (spread_spans) but would not fit 3
    // times in the handle's own slots
    const int nmax = (int)std::min<double>(h->Nslices, std::floor(kSpreadSamples / ((double)h->N * h->N)));
    const size_t need = 2 * (size_t)std::max(nmax, 0) * spec_slice(h->Nk, h->Nth);
    if (e == cudaSuccess && nmax > 0 && 3 * nmax > h->Nslices && need * sizeof(float2) <= kSpreadSpecBytes) {
      // optional: without the regions the spans run in sequence
      if (dev_alloc(h->sspec, need) == cudaSuccess) h->sspec_slices = nmax;
      else (void)cudaGetLastError();
    }
  }
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming);
  for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
    e = cudaStreamCreateWithFlags(&h->span_st[i], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_sjoin[i], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_sfork, cudaEventDisableTiming);
  h->plan_rho = make_fft_plan(h->Nrho, h->tw_rho.p);
  h->plan_th = make_fft_plan(h->Nth, h->tw_th.p);
  h->plan_filt = h->plan_rho;
  if (e != cudaSuccess) {
    h->erho.free_();
    h->tw_rho.free_();
    h->tw_th.free_();
    h->spec.free_();
    h->sspec.free_();
    if (h->side) cudaStreamDestroy(h->side);
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    destroy_span_streams(h);
    delete h;
    return set_err(e == cudaErrorMemoryAllocation ? LP_ERR_OOM : LP_ERR_CUDA, "lp_create: %s",
                   cudaGetErrorString(e));
  }
  *out = h;
  return LP_OK;
}

}  // extern "C"

template <typename Real>
static int init_fwd_impl(lp_handle* h, const int32_t* pi, int64_t ni, const Real* pf, int64_t nf) {
  if (!h || !pi || !pf) return set_err(LP_ERR_ARG, "lp_init_fwd: null pointer");
  const int N = h->N, Nth = h->Nth, Nrho = h->Nrho, Nproj = h->Nproj;
  // layout: Npids[3], pids[k]..., Ncids, cids  |  lp2C1[3], lp2C2[3], p2lp1[3], p2lp2[3], fZ
  if (ni < 4) return set_err(LP_ERR_ARG, "lp_init_fwd: parsi too short");
  int64_t npids[3];
  int64_t sum_p = 0;
  for (int k = 0; k < 3; ++k) {
    npids[k] = pi[k];
    if (npids[k] < 0 || npids[k] > (int64_t)Nproj * N) return set_err(LP_ERR_ARG, "lp_init_fwd: bad Npids");
    sum_p += npids[k];
  }
  if (ni < 3 + sum_p + 1) return set_err(LP_ERR_ARG, "lp_init_fwd: parsi too short");
  const int32_t* pids[3];
  int64_t o = 3;
  for (int k = 0; k < 3; ++k) {
    pids[k] = pi + o;
    o += npids[k];
  }
  const int64_t ncids = pi[o];
  const int32_t* cids = pi + o + 1;
  if (ncids < 0 || ncids > (int64_t)Nrho * Nth || ni != o + 1 + ncids)
    return set_err(LP_ERR_ARG, "lp_init_fwd: parsi size %lld inconsistent", (long long)ni);
  const int64_t nh = Nth / 2 + 1;
  if (nf != 6 * ncids + 2 * sum_p + 2 * (int64_t)Nrho * nh)
    return set_err(LP_ERR_ARG, "lp_init_fwd: parsf size %lld inconsistent", (long long)nf);
  const Real* lp2C1 = pf;
  const Real* lp2C2 = pf + 3 * ncids;
  const Real* p2lp1 = pf + 6 * ncids;
  const Real* p2lp2 = p2lp1 + sum_p;
  const Real* fzv = p2lp2 + sum_p;

  FwdDev* F = new FwdDev();
  const double lim = 8.0 * Nrho;
  // fixed-point format from the largest coordinate
  double maxabs = 0.0;
  for (int64_t i = 0; i < 6 * ncids + 2 * sum_p; ++i) {
    const double v = (double)pf[i];
    if (!finite_coord(v, lim)) {
      free_fwd(F);
      return set_err(LP_ERR_ARG, "lp_init_fwd: coordinate %lld not finite or out of range", (long long)i);
    }
    maxabs = std::max(maxabs, std::fabs(v));
  }
  F->F = fixed_bits(maxabs);
  F->fsc = (float)std::ldexp(1.0, -F->F);
  const int FB = F->F;
  std::vector<int2> ival(Nth, make_int2(1, 0));
  // dense column-major Cartesian coordinates of every log-polar point
  std::vector<int2> c2lp((size_t)Nth * Nrho);
  for (int k = 0; k < 3; ++k) {
    std::fill(c2lp.begin(), c2lp.end(), make_int2(LP_FX_NONE, LP_FX_NONE));
    for (int64_t i = 0; i < ncids; ++i) {
      const int idx = cids[i];
      if (idx < 0 || idx >= Nrho * Nth) {
        free_fwd(F);
        return set_err(LP_ERR_ARG, "lp_init_fwd: bad cids entry %lld", (long long)i);
      }
      const int r = idx / Nth, t = idx % Nth;
      c2lp[(size_t)t * Nrho + r] = make_int2(to_fixed((double)lp2C1[k * ncids + i], FB),
                                             to_fixed((double)lp2C2[k * ncids + i], FB));
      int2& iv = ival[t];
      if (iv.y < iv.x) iv = make_int2(r, r);
      else iv = make_int2(std::min(iv.x, r), std::max(iv.y, r));
      if (F->dhi < F->dlo) {
        F->dlo = t;
        F->dhi = t;
      } else {
        F->dlo = std::min(F->dlo, t);
        F->dhi = std::max(F->dhi, t);
      }
    }
    DeviceGuard g(h->device);
    cudaError_t e = dev_upload(F->c2lp[k], c2lp);
    if (e == cudaSuccess && k == 0) e = dev_upload(F->ival, ival);
    if (e != cudaSuccess) {
      free_fwd(F);
      return set_err(LP_ERR_OOM, "lp_init_fwd: %s", cudaGetErrorString(e));
    }
  }
  // polar points: every span must own whole sinogram rows with one theta coordinate
  std::vector<int> thc(Nproj, LP_FX_NONE);
  std::vector<int> rhoc((size_t)Nproj * N, 0);
  std::vector<int> owner(Nproj, -1);
  std::vector<int> cnt(Nproj, 0);
  int64_t off = 0;
  int lo = Nth, hi = -1;
  bool wraps = false;
  for (int k = 0; k < 3; ++k) {
    for (int64_t i = 0; i < npids[k]; ++i) {
      const int idx = pids[k][i];
      const int t = to_fixed((double)p2lp1[off + i], FB), rr = to_fixed((double)p2lp2[off + i], FB);
      if (idx < 0 || idx >= Nproj * N) {
        free_fwd(F);
        return set_err(LP_ERR_ARG, "lp_init_fwd: bad pids/p2lp entry");
      }
      const int row = idx / N, x = idx % N;
      if (owner[row] == -1) {
        owner[row] = k;
        thc[row] = t;
      } else if (owner[row] != k || thc[row] != t) {
        free_fwd(F);
        return set_err(LP_ERR_UNSUPPORTED,
                       "lp_init_fwd: sinogram row %d is not one span with one log-polar angle", row);
      }
      cnt[row]++;
      rhoc[(size_t)row * N + x] = rr;
    }
    off += npids[k];
  }
  std::vector<int> rows[3];
  for (int row = 0; row < Nproj; ++row) {
    if (owner[row] < 0 || cnt[row] != N) {
      free_fwd(F);
      return set_err(LP_ERR_UNSUPPORTED, "lp_init_fwd: sinogram row %d not covered exactly once", row);
    }
    if (row % h->os == 0) rows[owner[row]].push_back(row);
    const int c = first_tap(thc[row], FB, h->cubic);
    const int n = h->cubic ? 4 : 2;
    if (c < 0 || c + n - 1 >= Nth) wraps = true;
    lo = std::min(lo, c);
    hi = std::max(hi, c + n - 1);
  }
  if (wraps) {
    lo = 0;
    hi = Nth - 1;
  }
  F->lo = lo;
  F->hi = hi;
  // the transposed rho interpolation adds all taps of the points of one residue class
  // of x per pass, in two windows of first taps (below and from rbase + Nrho - ntap + 1):
  // that needs the rows' first taps strictly monotone in x (the log-polar rho of a
  // polar point is the log of an affine function of s, and it steps by more than one
  // texel per detector sample) spanning at most 2 (Nrho - ntap) + 1 bins -- a row's
  // points at the low end of the rho range wrap onto its high end
  std::vector<int> rbase(Nproj, 0);
  {
    const int coff = N / 2 - h->cor;
    for (int k = 0; k < 3 && F->rho_mono; ++k)
      for (int row : rows[k]) {
        int prev = 0, dir = 0, cmin = INT32_MAX, cmax = INT32_MIN, npt = 0;
        for (int x = std::max(0, coff); x < std::min(N, coff + h->N0); ++x) {
          const int c = first_tap(rhoc[(size_t)row * N + x], FB, h->cubic);
          if (npt > 0) {
            const int d = c > prev ? 1 : (c < prev ? -1 : 0);
            if (d == 0 || (dir != 0 && d != dir)) F->rho_mono = 0;
            dir = d;
          }
          prev = c;
          cmin = std::min(cmin, c);
          cmax = std::max(cmax, c);
          ++npt;
        }
        // two windows of first taps spanning at most Nrho - ntap each (rho_scatter_T)
        const int ntap = h->cubic ? 4 : 2;
        if (npt > 0 && cmax - cmin > 2 * (Nrho - ntap) + 1) F->rho_mono = 0;
        // rows whose first taps span at most Nrho - ntap bins need only the first window
        rbase[row] = (npt > 0 && cmax - cmin > Nrho - ntap) ? cmin : kNoWrap;
        if (!F->rho_mono) break;
      }
  }
  // column blocks for the transpose
  std::vector<int2> blk[3];
  {
    const int ntap = h->cubic ? 4 : 2;
    const int nb = (hi - lo + kTransposeCW) / kTransposeCW;
    for (int k = 0; k < 3; ++k) {
      for (int b = 0; b < nb; ++b) {
        const int c0 = lo + b * kTransposeCW, c1 = std::min(c0 + kTransposeCW, hi + 1);
        int first = -1, last = -1;
        for (int i = 0; i < (int)rows[k].size(); ++i) {
          const int c = first_tap(thc[rows[k][i]], FB, h->cubic);
          bool touch = false;
          for (int j = 0; j < ntap && !touch; ++j) {
            int cc = (c + j) % Nth;
            if (cc < 0) cc += Nth;
            touch = cc >= c0 && cc < c1;
          }
          if (touch) {
            if (first < 0) first = i;
            last = i;
          }
        }
        blk[k].push_back(first < 0 ? make_int2(0, 0) : make_int2(first, last + 1));
      }
    }
  }
  {
    DeviceGuard g(h->device);
    cudaError_t e = dev_upload(F->thc, thc);
    if (e == cudaSuccess) e = dev_upload(F->rhoc, rhoc);
    for (int k = 0; k < 3 && e == cudaSuccess; ++k) {
      F->nrows[k] = (int)rows[k].size();
      e = dev_upload(F->rows[k], rows[k]);
      if (e == cudaSuccess && k == 0) e = dev_upload(F->rbase, rbase);
      if (e == cudaSuccess) e = dev_upload(F->blk[k], blk[k]);
      F->nblk[k] = (int)blk[k].size();
    }
    if (e == cudaSuccess) e = dev_upload(F->fz, extend_kernel(fzv, Nrho, Nth));
    if (e == cudaSuccess) e = dev_alloc(F->fbuf, (size_t)h->Nslices * N * N);
    if (e == cudaSuccess && h->cubic) e = make_slice_textures(F, h->Nslices, N, h->device);
    if (e != cudaSuccess) {
      free_fwd(F);
      return set_err(e == cudaErrorMemoryAllocation ? LP_ERR_OOM : LP_ERR_CUDA, "lp_init_fwd: %s",
                     cudaGetErrorString(e));
    }
  }
  free_fwd(h->fwd);
  h->fwd = F;
  return LP_OK;
}

extern "C" {

int lp_init_fwd(lp_handle* h, const int32_t* pi, int64_t ni, const float* pf, int64_t nf) {
  return init_fwd_impl(h, pi, ni, pf, nf);
}

int lp_init_fwd_f64(lp_handle* h, const int32_t* pi, int64_t ni, const double* pf, int64_t nf) {
  return init_fwd_impl(h, pi, ni, pf, nf);
}

}  // extern "C"

template <typename Real>
static int init_adj_impl(lp_handle* h, const int32_t* pi, int64_t ni, const Real* pf, int64_t nf) {
  if (!h || !pi || !pf) return set_err(LP_ERR_ARG, "lp_init_adj: null pointer");
  const int N = h->N, N0 = h->N0, Nth = h->Nth, Nrho = h->Nrho, Nproj = h->Nproj;
  // layout: Ncids, Nlpids, Nwids, cids, lpids, wids, flag |
  //         C2lp1[3], C2lp2[3], lp2p1[3], lp2p2[3], lp2p1w[3], lp2p2w[3], fZ, filter[4N]?
  if (ni < 4) return set_err(LP_ERR_ARG, "lp_init_adj: parsi too short");
  const int64_t nc = pi[0], nl = pi[1], nw = pi[2];
  if (nc < 0 || nl < 0 || nw < 0 || nc > (int64_t)N * N || nl > (int64_t)Nrho * Nth || nw > (int64_t)Nrho * Nth ||
      ni != 3 + nc + nl + nw + 1)
    return set_err(LP_ERR_ARG, "lp_init_adj: parsi size %lld inconsistent", (long long)ni);
  const int32_t* cids = pi + 3;
  const int32_t* lpids = cids + nc;
  const int32_t* wids = lpids + nl;
  const int flag = wids[nw];
  const int64_t nh = Nth / 2 + 1;
  const int64_t nbase = 6 * nc + 6 * nl + 6 * nw + 2 * (int64_t)Nrho * nh;
  if (nf != nbase + (flag == 1 ? 4 * (int64_t)N : 0))
    return set_err(LP_ERR_ARG, "lp_init_adj: parsf size %lld inconsistent", (long long)nf);
  const Real* C2lp1 = pf;
  const Real* C2lp2 = C2lp1 + 3 * nc;
  const Real* lp2p1 = C2lp2 + 3 * nc;
  const Real* lp2p2 = lp2p1 + 3 * nl;
  const Real* lp2p1w = lp2p2 + 3 * nl;
  const Real* lp2p2w = lp2p1w + 3 * nw;
  const Real* fzv = lp2p2w + 3 * nw;
  const Real* filt = fzv + 2 * (size_t)Nrho * nh;
  const double lim = 8.0 * std::max(Nrho, Nproj);

  AdjDev* A = new AdjDev();
  auto fail = [&](int code, const char* msg) {
    free_adj(A);
    return set_err(code, "lp_init_adj: %s", msg);
  };
  // fixed-point format from the largest coordinate
  double maxabs = 0.0;
  for (int64_t i = 0; i < 6 * (nc + nl + nw); ++i) {
    const double v = (double)pf[i];
    if (!finite_coord(v, lim)) return fail(LP_ERR_ARG, "coordinate not finite or out of range");
    maxabs = std::max(maxabs, std::fabs(v));
  }
  A->F = fixed_bits(maxabs);
  A->fsc = (float)std::ldexp(1.0, -A->F);
  const int FB = A->F;
  DeviceGuard g(h->device);
  const int off = N / 2 - N0 / 2;
  int lo2 = Nth, hi2 = -1;
  bool wraps = false;
  for (int k = 0; k < 3; ++k) {
    std::vector<int> ta(Nth, LP_FX_NONE);
    std::vector<int> sx((size_t)Nth * Nrho, LP_FX_NONE);
    for (int64_t i = 0; i < nl; ++i) {
      const int idx = lpids[i];
      const int s = to_fixed((double)lp2p2[k * nl + i], FB), a = to_fixed((double)lp2p1[k * nl + i], FB);
      if (idx < 0 || idx >= Nrho * Nth) return fail(LP_ERR_ARG, "bad lpids entry");
      const int r = idx / Nth, t = idx % Nth;
      if (ta[t] == LP_FX_NONE) ta[t] = a;
      else if (ta[t] != a) return fail(LP_ERR_UNSUPPORTED, "log-polar column with more than one angle coordinate");
      sx[(size_t)t * Nrho + r] = s;
    }
    // wrap points grouped by column
    std::vector<int> woff(Nth + 1, 0);
    for (int64_t i = 0; i < nw; ++i) {
      const int idx = wids[i];
      if (idx < 0 || idx >= Nrho * Nth) return fail(LP_ERR_ARG, "bad wids entry");
      woff[idx % Nth + 1]++;
    }
    for (int t = 0; t < Nth; ++t) woff[t + 1] += woff[t];
    std::vector<int4> wpt(std::max<int64_t>(nw, 1), make_int4(0, 0, 0, 0));
    std::vector<int> fillp(woff.begin(), woff.end() - 1);
    for (int64_t i = 0; i < nw; ++i) {
      const int idx = wids[i];
      const int r = idx / Nth, t = idx % Nth;
      wpt[fillp[t]++] = make_int4(r, to_fixed((double)lp2p2w[k * nw + i], FB), to_fixed((double)lp2p1w[k * nw + i], FB), 0);
    }
    int clo = Nth, chi = -1;
    for (int t = 0; t < Nth; ++t) {
      if (ta[t] != LP_FX_NONE || woff[t + 1] > woff[t]) {
        clo = std::min(clo, t);
        chi = std::max(chi, t);
      }
    }
    A->clo[k] = clo;
    A->chi[k] = chi;
    // Cartesian pixels of the output window
    std::vector<int2> c2((size_t)N0 * N0, make_int2(LP_FX_NONE, LP_FX_NONE));
    for (int64_t i = 0; i < nc; ++i) {
      const int idx = cids[i];
      const int tt = to_fixed((double)C2lp1[k * nc + i], FB), tr = to_fixed((double)C2lp2[k * nc + i], FB);
      if (idx < 0 || idx >= N * N) return fail(LP_ERR_ARG, "bad cids entry");
      const int Y = idx / N - off, X = idx % N - off;
      if (Y < 0 || Y >= N0 || X < 0 || X >= N0) continue;
      c2[(size_t)Y * N0 + X] = make_int2(tt, tr);
      const int c = first_tap(tt, FB, h->cubic);
      const int n = h->cubic ? 4 : 2;
      if (c < 0 || c + n - 1 >= Nth) wraps = true;
      lo2 = std::min(lo2, c);
      hi2 = std::max(hi2, c + n - 1);
    }
    cudaError_t e = dev_upload(A->ta[k], ta);
    if (e == cudaSuccess) e = dev_upload(A->sx[k], sx);
    if (e == cudaSuccess) e = dev_upload(A->woff[k], woff);
    if (e == cudaSuccess) e = dev_upload(A->wpt[k], wpt);
    if (e == cudaSuccess) e = dev_upload(A->c2lp[k], c2);
    if (e != cudaSuccess) return fail(LP_ERR_OOM, cudaGetErrorString(e));
  }
  if (hi2 < lo2) {
    lo2 = 0;
    hi2 = 0;
  }
  if (wraps) {
    lo2 = 0;
    hi2 = Nth - 1;
  }
  A->lo2 = lo2;
  A->hi2 = hi2;
  A->W2 = hi2 - lo2 + 1;
  cudaError_t e = dev_upload(A->fz, extend_kernel(fzv, Nrho, Nth));
  if (e == cudaSuccess && flag == 1) {
    std::vector<float> Hh = fbp_kernel_2n(filt, N);
    if (Hh.empty()) return fail(LP_ERR_UNSUPPORTED, "FBP filter is not symmetric");
    e = dev_upload(A->H, Hh);
    A->filter = true;
  }
  if (e == cudaSuccess) e = dev_alloc(A->rbuf, (size_t)h->Nslices * Nproj * N);
  if (e == cudaSuccess && h->cubic) e = dev_alloc(A->rin, (size_t)h->Nslices * Nproj * N);
  int gw = 0, gh = 0;
  cudaDeviceGetAttribute(&gw, cudaDevAttrMaxTexture2DGatherWidth, h->device);
  cudaDeviceGetAttribute(&gh, cudaDevAttrMaxTexture2DGatherHeight, h->device);
  const bool use_tex = h->cubic && Nrho <= gw && A->W2 <= gh;
  for (int k = 0; k < 3 && e == cudaSuccess; ++k) {
    if (use_tex) {
      for (int s = 0; s < h->Nslices && e == cudaSuccess; ++s) {
        cudaTextureObject_t t = 0;
        cudaSurfaceObject_t so = 0;
        e = make_gather_array(Nrho, A->W2, A->arr, &t, &so);
        A->tex_h[k].push_back(t);
        A->surf_h[k].push_back(so);
      }
      if (e == cudaSuccess) e = dev_upload(A->tex[k], A->tex_h[k]);
      if (e == cudaSuccess) e = dev_upload(A->surf[k], A->surf_h[k]);
    } else {
      e = dev_alloc(A->G[k], (size_t)h->Nslices * A->W2 * Nrho);
    }
  }
  if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? LP_ERR_OOM : LP_ERR_CUDA, cudaGetErrorString(e));
  free_adj(h->adj);
  h->adj = A;
  return LP_OK;
}

extern "C" {

int lp_init_adj(lp_handle* h, const int32_t* pi, int64_t ni, const float* pf, int64_t nf) {
  return init_adj_impl(h, pi, ni, pf, nf);
}

int lp_init_adj_f64(lp_handle* h, const int32_t* pi, int64_t ni, const double* pf, int64_t nf) {
  return init_adj_impl(h, pi, ni, pf, nf);
}

int lp_destroy(lp_handle* h) {
  if (!h) return LP_OK;
  DeviceGuard g(h->device);
  free_fwd(h->fwd);
  free_adj(h->adj);
  h->erho.free_();
  h->spec.free_();
  h->sspec.free_();
  h->tw_rho.free_();
  h->tw_th.free_();
  for (const ProfRec& r : h->prof) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  for (cudaEvent_t e : h->evpool) cudaEventDestroy(e);
  if (h->side) cudaStreamDestroy(h->side);
  if (h->ev_fork) cudaEventDestroy(h->ev_fork);
  if (h->ev_join) cudaEventDestroy(h->ev_join);
  destroy_span_streams(h);
  delete h;
  return LP_OK;
}

int lp_get_geometry(const lp_handle* h, int32_t out[10]) {
  if (!h || !out) return set_err(LP_ERR_ARG, "lp_get_geometry: null pointer");
  const int32_t v[10] = {h->N, h->N0, h->Nth, h->Nrho, h->Nproj, h->Nproj0, h->Nslices, h->cor, h->os, h->cubic};
  memcpy(out, v, sizeof(v));
  return LP_OK;
}

namespace {
__global__ void k_fill(float* p, size_t n, float v) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    p[i] = v;
}
cudaError_t fill_async(float* p, size_t n, float v, cudaStream_t st) {
  if (!p || n == 0) return cudaSuccess;
  k_fill<<<1024, 256, 0, st>>>(p, n, v);
  return cudaGetLastError();
}
}  // namespace

int lp_debug_fill_scratch(lp_handle* h, float value, void* stream) {
  if (!h) return set_err(LP_ERR_ARG, "lp_debug_fill_scratch: null handle");
  DeviceGuard g(h->device);
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = fill_async((float*)h->spec.p, h->spec.n * 2, value, st);
  if (e == cudaSuccess && h->sspec.p) e = fill_async((float*)h->sspec.p, h->sspec.n * 2, value, st);
  if (e == cudaSuccess && h->fwd) e = fill_async(h->fwd->fbuf.p, h->fwd->fbuf.n, value, st);
  if (e == cudaSuccess && h->fwd && h->fwd->lpg.p) e = fill_async(h->fwd->lpg.p, h->fwd->lpg.n, value, st);
  if (e == cudaSuccess && h->fwd && h->fwd->rowspec.p)
    e = fill_async((float*)h->fwd->rowspec.p, 2 * h->fwd->rowspec.n, value, st);
  if (e == cudaSuccess && h->fwd && h->fwd->tspec.p)
    e = fill_async((float*)h->fwd->tspec.p, 2 * h->fwd->tspec.n, value, st);
  if (e == cudaSuccess && h->adj) {
    e = fill_async(h->adj->rbuf.p, h->adj->rbuf.n, value, st);
    if (e == cudaSuccess && h->adj->rin.p) e = fill_async(h->adj->rin.p, h->adj->rin.n, value, st);
    for (int k = 0; k < 3 && e == cudaSuccess; ++k) e = fill_async(h->adj->G[k].p, h->adj->G[k].n, value, st);
  }
  if (e != cudaSuccess) return set_err(LP_ERR_CUDA, "lp_debug_fill_scratch: %s", cudaGetErrorString(e));
  return LP_OK;
}

int lp_device_bytes(const lp_handle* h, int64_t* bytes) {
  if (!h || !bytes) return set_err(LP_ERR_ARG, "lp_device_bytes: null pointer");
  int64_t b = h->erho.n * 4 + h->spec.n * 8 + h->sspec.n * 8 + h->tw_rho.n * 8 + h->tw_th.n * 8;
  if (h->fwd) {
    for (int k = 0; k < 3; ++k) b += h->fwd->c2lp[k].n * 8 + h->fwd->rows[k].n * 4;
    b += h->fwd->thc.n * 4 + h->fwd->rhoc.n * 4 + h->fwd->fz.n * 8 + h->fwd->fbuf.n * 4;
    b += (int64_t)h->fwd->arr.size() * h->N * h->N * 4;
  }
  if (h->adj) {
    for (int k = 0; k < 3; ++k)
      b += h->adj->ta[k].n * 4 + h->adj->sx[k].n * 4 + h->adj->woff[k].n * 4 + h->adj->wpt[k].n * 16 +
           h->adj->c2lp[k].n * 8 + h->adj->G[k].n * 4;
    b += h->adj->fz.n * 8 + h->adj->H.n * 4 + h->adj->rbuf.n * 4 + h->adj->rin.n * 4;
    b += (int64_t)h->adj->arr.size() * h->Nrho * h->adj->W2 * 4;
  }
  *bytes = b;
  return LP_OK;
}

}  // extern "C"

// Run `body(s0, n, stream)` over the slices [0, S0) in chunks of `chunk`
// (0: one chunk), alternating between the caller's stream and the handle's
// second stream when `streams` is 2.  Chunks use disjoint slices of every
// scratch buffer, so chunks on the two streams never share memory; the
// second stream is forked from and joined back into the caller's stream with
// events (graph capture turns them into parallel branches).
template <typename Body>
static int run_chunks(lp_handle* h, cudaStream_t st, int S0, int chunk, int streams, Body body) {
  const int c = chunk > 0 ? std::min(chunk, S0) : S0;
  const int nch = (S0 + c - 1) / c;
  const bool two = streams == 2 && nch >= 2;
  if (two) {
    CUDA_TRY(cudaEventRecord(h->ev_fork, st));
    CUDA_TRY(cudaStreamWaitEvent(h->side, h->ev_fork, 0));
  }
  for (int i = 0; i < nch; ++i) {
    const int rc = body(i * c, std::min(c, S0 - i * c), (two && (i & 1)) ? h->side : st);
    if (rc != LP_OK) return rc;
  }
  if (two) {
    CUDA_TRY(cudaEventRecord(h->ev_join, h->side));
    CUDA_TRY(cudaStreamWaitEvent(st, h->ev_join, 0));
  }
  return LP_OK;
}

// forward transform of slices [s0, s0 + n) of the call (scratch slots s0..; with
// spread spans also the spectrum slots up to s0 + 3n)
static int fwd_slices(lp_handle* h, float* R, const float* f, int s0, int n, cudaStream_t st, bool one_chunk) {
  FwdDev* F = h->fwd;
  const bool tex = !F->tex_h.empty();
  f += (size_t)s0 * h->N0 * h->N0;
  R += (size_t)s0 * h->Nproj0 * h->N0;
  float* fbuf = F->fbuf.p + (size_t)s0 * h->N * h->N;
  const cudaTextureObject_t* tx = tex ? F->tex.p + s0 : nullptr;
  const cudaSurfaceObject_t* sf = tex ? F->surf.p + s0 : nullptr;
  FwdIngestArgs ia{f, fbuf, h->N, h->N0, h->N / 2 - h->N0 / 2, h->cubic};
  CUDA_TRY(launch(h, K_FWD_INGEST, st, [&] { return launch_fwd_ingest(ia, n, st); }));
  if (h->cubic) {
    ColPrefilterArgs ca{fbuf, h->N, h->N, sf};
    CUDA_TRY(launch(h, K_COL_PREFILTER, st, [&] { return launch_col_prefilter(ca, n, st); }));
  }
  const bool spread = spread_spans(h, s0, n, one_chunk);
  if (spread) CUDA_TRY(span_fork(h, st));
  for (int k = 0; k < 3; ++k) {
    const cudaStream_t sk = spread && k > 0 ? h->span_st[k - 1] : st;
    float2* spk = span_spec(h, s0, n, k, spread);
    FwdC2LPArgs a1{fbuf, spk, F->c2lp[k].p, h->erho.p, h->N, h->Nth, h->Nrho, h->Nk, h->cubic,
                   h->plan_rho, tx, F->ival.p, F->dlo, F->dhi, F->F, F->fsc};
    CUDA_TRY(launch(h, K_FWD_C2LP, sk, [&] { return launch_fwd_c2lp(a1, n, sk); }));
    ThetaConvArgs a2{spk, F->fz.p, h->Nth, h->Nk, F->dlo, F->dhi,
                     F->lo & ~1, std::min(F->hi | 1, h->Nth - 1), 0, h->plan_th, h->fwd_tblock};
    CUDA_TRY(launch(h, K_THETA_CONV, sk, [&] { return launch_theta_conv(a2, n, sk); }));
    FwdLP2PolarArgs a3{spk, R, F->thc.p, F->rhoc.p, F->rows[k].p, F->nrows[k], h->N, h->N0, h->Nth,
                       h->Nrho, h->Nk, h->Nproj0, h->os, h->N / 2 - h->cor, h->cubic, h->plan_rho, F->F, F->fsc};
    CUDA_TRY(launch(h, K_FWD_LP2POLAR, sk, [&] { return launch_fwd_lp2polar(a3, n, sk); }));
  }
  if (spread) CUDA_TRY(span_join(h, st));
  return LP_OK;
}

// adjoint of slices [s0, s0 + n) of the call (scratch slots s0..; with spread spans
// also the spectrum slots up to s0 + 3n)
static int adj_slices(lp_handle* h, float* f, const float* R, int s0, int n, cudaStream_t st, bool one_chunk) {
  AdjDev* A = h->adj;
  R += (size_t)s0 * h->Nproj0 * h->N0;
  f += (size_t)s0 * h->N0 * h->N0;
  float* rbuf = A->rbuf.p + (size_t)s0 * h->Nproj * h->N;
  // cubic: the ingest writes rin and the column prefilter rin -> rbuf (out of place)
  float* rin = h->cubic ? A->rin.p + (size_t)s0 * h->Nproj * h->N : rbuf;
  const size_t gstride = (size_t)A->W2 * h->Nrho;
  AdjIngestArgs ia{R, rin, A->filter ? A->H.p : nullptr, h->N, h->N0, h->Nproj, h->Nproj0, h->os,
                   h->N / 2 - h->cor, h->cubic, h->plan_filt};
  CUDA_TRY(launch(h, K_ADJ_INGEST, st, [&] { return launch_adj_ingest(ia, n, st); }));
  if (h->cubic) {
    ColPrefilterArgs ca{rin, h->Nproj, h->N, nullptr, rbuf};
    CUDA_TRY(launch(h, K_COL_PREFILTER, st, [&] { return launch_col_prefilter(ca, n, st); }));
  }
  float* G[3];
  for (int k = 0; k < 3; ++k) G[k] = A->G[k].p ? A->G[k].p + s0 * gstride : nullptr;
  const bool spread = spread_spans(h, s0, n, one_chunk);
  if (spread) CUDA_TRY(span_fork(h, st));
  for (int k = 0; k < 3; ++k) {
    const cudaStream_t sk = spread && k > 0 ? h->span_st[k - 1] : st;
    float2* spk = span_spec(h, s0, n, k, spread);
    const bool tex = !A->tex_h[k].empty();
    if (A->chi[k] < A->clo[k]) {
      if (tex) return set_err(LP_ERR_UNSUPPORTED, "lp_adj: span %d has no log-polar points", k);
      CUDA_TRY(cudaMemsetAsync(G[k], 0, n * gstride * sizeof(float), sk));
      continue;
    }
    AdjPolar2LPArgs a1{rbuf, spk, A->ta[k].p, A->sx[k].p, A->woff[k].p, A->wpt[k].p, h->N, h->Nth,
                       h->Nrho, h->Nk, h->Nproj, h->cubic, A->clo[k], A->chi[k], h->plan_rho, A->F, A->fsc};
    CUDA_TRY(launch(h, K_ADJ_POLAR2LP, sk, [&] { return launch_adj_polar2lp(a1, n, sk); }));
    ThetaConvArgs a2{spk, A->fz.p, h->Nth, h->Nk, A->clo[k],
                     A->chi[k], A->lo2, A->hi2, 0, h->plan_th, h->adj_tblock};
    CUDA_TRY(launch(h, K_THETA_CONV, sk, [&] { return launch_theta_conv(a2, n, sk); }));
    AdjLPColsArgs a3{spk, G[k], h->Nth, h->Nrho, h->Nk, A->lo2, A->hi2, A->W2, h->plan_rho,
                     tex ? A->surf[k].p + s0 : nullptr};
    CUDA_TRY(launch(h, K_ADJ_LPCOLS, sk, [&] { return launch_adj_lpcols(a3, n, sk); }));
  }
  if (spread) CUDA_TRY(span_join(h, st));
  const bool tex = !A->tex_h[0].empty();
  AdjLP2CartArgs a4{G[0], G[1], G[2], A->c2lp[0].p, A->c2lp[1].p, A->c2lp[2].p, f,
                    h->N0, h->Nth, h->Nrho, A->lo2, A->W2, h->cubic, h->N0 * h->N0,
                    tex ? A->tex[0].p + s0 : nullptr, tex ? A->tex[1].p + s0 : nullptr,
                    tex ? A->tex[2].p + s0 : nullptr, A->F, A->fsc};
  CUDA_TRY(launch(h, K_ADJ_LP2CART, st, [&] { return launch_adj_lp2cart(a4, n, st); }));
  return LP_OK;
}

extern "C" {

int lp_fwd(lp_handle* h, float* R, const float* f, int S0, void* stream) {
  if (!h) return set_err(LP_ERR_ARG, "lp_fwd: null handle");
  if (!h->fwd) return set_err(LP_ERR_STATE, "lp_fwd: forward tables not initialised (lp_init_fwd)");
  if (S0 < 0 || S0 > h->Nslices) return set_err(LP_ERR_ARG, "lp_fwd: S0=%d outside [0, %d]", S0, h->Nslices);
  if (S0 == 0) return LP_OK;
  if (!R || !f) return set_err(LP_ERR_ARG, "lp_fwd: null data pointer");
  DeviceGuard g(h->device);
  return run_chunks(h, (cudaStream_t)stream, S0, h->fwd_chunk, h->fwd_streams,
                    [&](int s0, int n, cudaStream_t st) { return fwd_slices(h, R, f, s0, n, st, n == S0); });
}

// Tables of the exact transpose's gather (built on its first call, from the
// forward's device tables): the log-polar points of all spans with coordinates,
// grouped by image cell (the integer part of the coordinates, wrapped onto the
// grid) in (span, theta, rho) order; the buffers of real log-polar values and of
// row spectra.  Allocates device memory, so make the first call outside stream
// capture.
static int build_transpose_tables(lp_handle* h) {
  FwdDev* F = h->fwd;
  const int N = h->N, Nth = h->Nth, Nrho = h->Nrho;
  const int W = F->dhi - F->dlo + 1;
  if (W > 0) {
    std::vector<int2> c2[3];
    for (int k = 0; k < 3; ++k) {
      c2[k].resize((size_t)Nth * Nrho);
      CUDA_TRY(cudaMemcpy(c2[k].data(), F->c2lp[k].p, c2[k].size() * sizeof(int2), cudaMemcpyDeviceToHost));
    }
    std::vector<int> off((size_t)N * N + 1, 0);
    auto cell = [&](int2 p) {
      const int ix = p.x >> F->F, iy = p.y >> F->F;
      return (size_t)(((iy % N) + N) % N) * N + (((ix % N) + N) % N);
    };
    for (int k = 0; k < 3; ++k)
      for (int t = F->dlo; t <= F->dhi; ++t)
        for (int r = 0; r < Nrho; ++r) {
          const int2 p = c2[k][(size_t)t * Nrho + r];
          if (p.x != LP_FX_NONE) off[cell(p) + 1]++;
        }
    for (size_t c = 0; c < (size_t)N * N; ++c) off[c + 1] += off[c];
    const size_t npts = off[(size_t)N * N];
    std::vector<int2> pts(std::max<size_t>(npts, 1), make_int2(0, 0));
    std::vector<int> fill(off.begin(), off.end() - 1);
    for (int k = 0; k < 3; ++k) {
      std::vector<int> pos((size_t)W * Nrho, -1);
      for (int t = F->dlo; t <= F->dhi; ++t)
        for (int r = 0; r < Nrho; ++r) {
          const int2 p = c2[k][(size_t)t * Nrho + r];
          if (p.x == LP_FX_NONE) continue;
          const int e = fill[cell(p)]++;
          pts[e] = p;
          pos[(size_t)(t - F->dlo) * Nrho + r] = e;
        }
      CUDA_TRY(dev_upload(F->lppos[k], pos));
    }
    CUDA_TRY(dev_upload(F->cell_off, off));
    CUDA_TRY(dev_upload(F->cell_pts, pts));
    F->npts = npts;
    const size_t groups = (h->Nslices + kGatherSlices - 1) / kGatherSlices;
    CUDA_TRY(dev_alloc(F->lpg, groups * kGatherSlices * std::max<size_t>(npts, 1)));
  }
  const int nr = std::max(F->nrows[0], std::max(F->nrows[1], F->nrows[2]));
  const size_t rs_slots = (size_t)h->Nslices * std::max(nr, 1) * rowspec_stride(h->Nk);
  const size_t spec_slots = (size_t)h->Nslices * spec_slice(h->Nk, h->Nth);
  F->tspread = (2 * rs_slots + 2 * spec_slots) * sizeof(float2) <= kTransposeSpreadBytes;
  if (F->tspread && (dev_alloc(F->rowspec, 3 * rs_slots) != cudaSuccess ||
                     dev_alloc(F->tspec, 2 * spec_slots) != cudaSuccess)) {
    // optional: without the per-span regions the spans run in sequence
    (void)cudaGetLastError();
    F->rowspec.free_();
    F->tspec.free_();
    F->tspread = false;
  }
  if (!F->tspread) CUDA_TRY(dev_alloc(F->rowspec, rs_slots));
  // the theta columns' (row, tap) lists: a row's taps reach columns first_tap + j (mod
  // Nth); entries of a column in ascending row order; the weights come from the same
  // device function as the forward's theta interpolation (k_fwdT_tapw)
  {
    std::vector<int> thc(F->thc.n);
    CUDA_TRY(cudaMemcpy(thc.data(), F->thc.p, thc.size() * sizeof(int), cudaMemcpyDeviceToHost));
    const int ntap = h->cubic ? 4 : 2;
    for (int k = 0; k < 3; ++k) {
      std::vector<int> rows(F->nrows[k]);
      if (!rows.empty())
        CUDA_TRY(cudaMemcpy(rows.data(), F->rows[k].p, rows.size() * sizeof(int), cudaMemcpyDeviceToHost));
      std::vector<int> off(Nth + 1, 0);
      auto col = [&](int i, int j) {
        const int c = (first_tap(thc[rows[i]], F->F, h->cubic) + j) % Nth;
        return c < 0 ? c + Nth : c;
      };
      for (int i = 0; i < (int)rows.size(); ++i)
        for (int j = 0; j < ntap; ++j) off[col(i, j) + 1]++;
      for (int c = 0; c < Nth; ++c) off[c + 1] += off[c];
      std::vector<int2> ent(std::max(off[Nth], 1), make_int2(0, 0));
      std::vector<int> fill(off.begin(), off.end() - 1);
      for (int i = 0; i < (int)rows.size(); ++i)
        for (int j = 0; j < ntap; ++j) ent[fill[col(i, j)]++] = make_int2(i, j);
      CUDA_TRY(dev_upload(F->coff[k], off));
      CUDA_TRY(dev_upload(F->cent[k], ent));
      if (off[Nth] > 0)
        CUDA_TRY(launch_fwdT_tapw(F->cent[k].p, off[Nth], F->rows[k].p, F->thc.p, F->F, F->fsc, h->cubic, 0));
    }
    CUDA_TRY(cudaStreamSynchronize(0));
  }
  F->gather_ready = true;
  return LP_OK;
}

int lp_fwd_transpose(lp_handle* h, float* f, const float* R, int S0, void* stream) {
  if (!h) return set_err(LP_ERR_ARG, "lp_fwd_transpose: null handle");
  if (!h->fwd) return set_err(LP_ERR_STATE, "lp_fwd_transpose: forward tables not initialised (lp_init_fwd)");
  if (S0 < 0 || S0 > h->Nslices)
    return set_err(LP_ERR_ARG, "lp_fwd_transpose: S0=%d outside [0, %d]", S0, h->Nslices);
  if (S0 == 0) return LP_OK;
  if (!R || !f) return set_err(LP_ERR_ARG, "lp_fwd_transpose: null data pointer");
  DeviceGuard g(h->device);
  cudaStream_t st = (cudaStream_t)stream;
  FwdDev* F = h->fwd;
  if (!F->gather_ready) {
    int rc = build_transpose_tables(h);
    if (rc != LP_OK) return rc;
  }
  float* acc = F->fbuf.p;
  const int W = F->dhi - F->dlo + 1;
  if (W <= 0) CUDA_TRY(cudaMemsetAsync(acc, 0, (size_t)S0 * h->N * h->N * sizeof(float), st));
  // register-FFT theta lengths gather the theta convolution's input from the row
  // spectra; the generic FFT sums them into the spectrum first (k_fwdT_colsum)
  const int nr = std::max(F->nrows[0], std::max(F->nrows[1], F->nrows[2]));
  const bool gathered = theta_conv_gathers(h->Nth, nr);
  // spans on their own streams for calls of at most kSpreadSamples image samples
  const bool spread = F->tspread && (double)S0 * h->N * h->N <= kSpreadSamples;
  if (spread && W > 0) CUDA_TRY(span_fork(h, st));
  for (int k = 0; k < 3 && W > 0; ++k) {
    const cudaStream_t sk = spread && k > 0 ? h->span_st[k - 1] : st;
    float2* rsk = F->rowspec.p + (spread ? (size_t)k * h->Nslices * std::max(nr, 1) * rowspec_stride(h->Nk) : 0);
    float2* spk = spread && k > 0 ? F->tspec.p + (size_t)(k - 1) * h->Nslices * spec_slice(h->Nk, h->Nth) : h->spec.p;
    FwdTRowsArgs a0{R, rsk, F->rhoc.p, F->rows[k].p, F->rbase.p, F->nrows[k], h->N, h->N0, h->Nrho,
                    h->Nk, h->Nproj0, h->os, h->N / 2 - h->cor, h->cubic, h->plan_rho, F->F, F->fsc, F->rho_mono};
    CUDA_TRY(launch(h, K_FWDT_ROWS, sk, [&] { return launch_fwdT_rows(a0, S0, sk); }));
    if (!gathered) {
      FwdTColSumArgs a1{rsk, spk, F->thc.p, F->rows[k].p, F->blk[k].p, F->nrows[k], h->Nth, h->Nk,
                        F->lo, F->hi, kTransposeCW, h->cubic, F->F, F->fsc};
      CUDA_TRY(launch(h, K_FWDT_COLSUM, sk, [&] { return launch_fwdT_colsum(a1, S0, F->nblk[k], sk); }));
    }
    ThetaConvArgs a2{spk, F->fz.p, h->Nth, h->Nk, F->lo, F->hi,
                     F->dlo, F->dhi, 1, h->plan_th, h->fwd_tblock};
    if (gathered) {
      a2.rowspec = rsk;
      a2.coff = F->coff[k].p;
      a2.cent = F->cent[k].p;
      a2.nrows = F->nrows[k];
    }
    CUDA_TRY(launch(h, K_THETA_CONV, sk, [&] { return launch_theta_conv(a2, S0, sk); }));
    FwdTColsArgs a3{spk, F->lpg.p, F->lppos[k].p, F->npts, h->erho.p, h->Nth, h->Nrho, h->Nk, F->dlo, F->dhi,
                    h->plan_rho};
    CUDA_TRY(launch(h, K_FWDT_COLS, sk, [&] { return launch_fwdT_cols(a3, S0, sk); }));
  }
  if (spread && W > 0) CUDA_TRY(span_join(h, st));
  if (W > 0) {
    FwdTGatherArgs a4{F->lpg.p, F->npts, acc, F->cell_off.p, F->cell_pts.p, h->N, h->cubic, F->F, F->fsc};
    CUDA_TRY(launch(h, K_FWDT_GATHER, st, [&] { return launch_fwdT_gather(a4, S0, st); }));
  }
  if (h->cubic) {
    // transposed column prefilter acc -> the spectrum buffer (free now; it holds S0 N x N
    // float images), then the transposed row prefilter into the caller's cropped image
    float* tmp = reinterpret_cast<float*>(h->spec.p);
    PrefilterTColsArgs pc{acc, tmp, h->N, h->N};
    CUDA_TRY(launch(h, K_PREFILTER_T, st, [&] { return launch_prefilter_T_cols(pc, S0, st); }));
    PrefilterTRowsCropArgs pr{tmp, f, h->N, h->N0, h->N / 2 - h->N0 / 2};
    CUDA_TRY(launch(h, K_PREFILTER_T, st, [&] { return launch_prefilter_T_rows_crop(pr, S0, st); }));
    return LP_OK;
  }
  CropArgs cr{acc, f, h->N, h->N0, h->N / 2 - h->N0 / 2};
  CUDA_TRY(launch(h, K_CROP, st, [&] { return launch_crop(cr, S0, st); }));
  return LP_OK;
}

int lp_adj(lp_handle* h, float* f, const float* R, int S0, void* stream) {
  if (!h) return set_err(LP_ERR_ARG, "lp_adj: null handle");
  if (!h->adj) return set_err(LP_ERR_STATE, "lp_adj: adjoint tables not initialised (lp_init_adj)");
  if (S0 < 0 || S0 > h->Nslices) return set_err(LP_ERR_ARG, "lp_adj: S0=%d outside [0, %d]", S0, h->Nslices);
  if (S0 == 0) return LP_OK;
  if (!R || !f) return set_err(LP_ERR_ARG, "lp_adj: null data pointer");
  DeviceGuard g(h->device);
  return run_chunks(h, (cudaStream_t)stream, S0, h->adj_chunk, h->adj_streams,
                    [&](int s0, int n, cudaStream_t st) { return adj_slices(h, f, R, s0, n, st, n == S0); });
}

int lp_set_schedule(lp_handle* h, const int32_t* sched, int n) {
  if (!h || (!sched && n > 0)) return set_err(LP_ERR_ARG, "lp_set_schedule: null pointer");
  if (n < 0 || n > LP_SCHEDULE_LEN) return set_err(LP_ERR_ARG, "lp_set_schedule: n=%d outside [0, %d]", n, LP_SCHEDULE_LEN);
  int v[LP_SCHEDULE_LEN] = {0, 1, 256, 0, 1, 256};
  for (int i = 0; i < n; ++i) v[i] = sched[i];
  for (int d = 0; d < 2; ++d) {
    const int* q = v + 3 * d;
    if (q[0] < 0 || q[1] < 1 || q[1] > 2 || (q[2] != 256 && q[2] != 512))
      return set_err(LP_ERR_ARG, "lp_set_schedule: chunk >= 0, streams in {1, 2}, theta block in {256, 512}");
  }
  h->fwd_chunk = v[0];
  h->fwd_streams = v[1];
  h->fwd_tblock = v[2];
  h->adj_chunk = v[3];
  h->adj_streams = v[4];
  h->adj_tblock = v[5];
  return LP_OK;
}

int lp_get_schedule(const lp_handle* h, int32_t* out, int n) {
  if (!h || (!out && n > 0)) return set_err(LP_ERR_ARG, "lp_get_schedule: null pointer");
  const int v[LP_SCHEDULE_LEN] = {h->fwd_chunk, h->fwd_streams, h->fwd_tblock,
                                  h->adj_chunk, h->adj_streams, h->adj_tblock};
  for (int i = 0; i < n && i < LP_SCHEDULE_LEN; ++i) out[i] = v[i];
  return LP_OK;
}

// Time every candidate schedule of one direction on the caller's buffers and
// keep the fastest (ties go to the earlier, simpler candidate).
static int tune_one(lp_handle* h, bool fwd, float* R, float* f, int S0, cudaStream_t st, int reps,
                    int* best_chunk, int* best_streams, int* best_tblock, float* best_ms) {
  const int chunks[] = {0, 64, 32, 16, 8};
  cudaEvent_t a = nullptr, b = nullptr;
  CUDA_TRY(cudaEventCreate(&a));
  CUDA_TRY(cudaEventCreate(&b));
  const bool prof = h->profiling;
  h->profiling = false;
  float best = 1e30f;
  int rc = LP_OK;
  int* tblock = fwd ? &h->fwd_tblock : &h->adj_tblock;
  for (int tb = 256; tb <= 512 && rc == LP_OK; tb += 256)
  for (int ci = 0; ci < 5 && rc == LP_OK; ++ci) {
    const int c = chunks[ci];
    if (c != 0 && c >= S0) continue;
    *tblock = tb;
    for (int ns = 1; ns <= 2 && rc == LP_OK; ++ns) {
      if (ns == 2 && (c == 0 || (S0 + c - 1) / c < 2)) continue;
      auto one = [&] {
        return run_chunks(h, st, S0, c, ns, [&](int s0, int n, cudaStream_t s2) {
          return fwd ? fwd_slices(h, R, f, s0, n, s2, n == S0) : adj_slices(h, f, R, s0, n, s2, n == S0);
        });
      };
      rc = one();  // warm-up
      if (rc != LP_OK) break;
      cudaEventRecord(a, st);
      for (int r = 0; r < reps && rc == LP_OK; ++r) rc = one();
      cudaEventRecord(b, st);
      if (cudaEventSynchronize(b) != cudaSuccess) rc = set_err(LP_ERR_CUDA, "lp_autotune: timing failed");
      float ms = 0.f;
      if (rc == LP_OK) cudaEventElapsedTime(&ms, a, b);
      if (rc == LP_OK && ms / reps < 0.98f * best) {
        best = ms / reps;
        *best_chunk = c;
        *best_streams = ns;
        *best_tblock = tb;
      }
    }
  }
  h->profiling = prof;
  *tblock = *best_tblock;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *best_ms = best;
  return rc;
}

int lp_autotune(lp_handle* h, float* R, float* f, int S0, void* stream, float out_ms[2]) {
  if (!h) return set_err(LP_ERR_ARG, "lp_autotune: null handle");
  if (S0 < 1 || S0 > h->Nslices) return set_err(LP_ERR_ARG, "lp_autotune: S0=%d outside [1, %d]", S0, h->Nslices);
  if (!R || !f) return set_err(LP_ERR_ARG, "lp_autotune: null data pointer");
  DeviceGuard g(h->device);
  cudaStream_t st = (cudaStream_t)stream;
  float ms[2] = {0.f, 0.f};
  if (h->fwd) {
    int c = 0, ns = 1, tb = 256;
    int rc = tune_one(h, true, R, f, S0, st, 2, &c, &ns, &tb, &ms[0]);
    h->fwd_chunk = c;
    h->fwd_streams = ns;
    h->fwd_tblock = tb;
    if (rc != LP_OK) return rc;
  }
  if (h->adj) {
    int c = 0, ns = 1, tb = 256;
    int rc = tune_one(h, false, R, f, S0, st, 2, &c, &ns, &tb, &ms[1]);
    h->adj_chunk = c;
    h->adj_streams = ns;
    h->adj_tblock = tb;
    if (rc != LP_OK) return rc;
  }
  if (out_ms) {
    out_ms[0] = ms[0];
    out_ms[1] = ms[1];
  }
  return LP_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Forward transform without device allocation.
//
// For callers that must not allocate or free device memory while they run:
// applications whose device memory belongs to another allocator (a
// framework's caching allocator or a fixed pool reserved at start-up), where
// cudaMalloc can fail although the pool has room and where cudaMalloc and
// cudaFree would synchronise the device in the middle of their pipeline.
// lp_fwd_noalloc takes its scratch (the prefiltered image and the log-polar
// spectrum) from one file-scope device array of LP_NOALLOC_SCRATCH_BYTES
// instead of the handle's buffers; it calls no allocating routine.
//
// Every GPU that loads this library holds the array until the process exits.
// The array lives in this file's device module; with lazy module loading (the
// CUDA default) the module, and with it the array's device memory, is loaded
// by the first lp_fwd_noalloc call on a device.  So a caller that reserves a
// fixed pool at start-up makes one call first (it may process zero slices of
// a real handle: S0 = 0 still resolves the array), and a caller that captures
// streams into graphs makes that first call before any capture.  The array's
// device address is looked up with cudaGetSymbolAddress once per device and
// context (with that device current): if the process's context on a device
// is destroyed and recreated (cudaDeviceReset), the next call looks it up
// again.  All calls share the array and it keeps the last call's contents:
// calls whose work overlaps on the GPU (other streams, other host threads)
// race on it and must be serialised by the caller.  Nothing in it has to start
// at zero: every scratch word this path reads was written earlier in the same
// call.
// ---------------------------------------------------------------------------
#include <cuda.h>  // CUcontext / CUresult types only; the driver calls are resolved at run time

#include <mutex>

static __device__ __align__(256) unsigned char g_noalloc_scratch[LP_NOALLOC_SCRATCH_BYTES];

#define LP_NOALLOC_MAX_DEVICES 64
struct NoallocSlot {
  unsigned long long ctx = 0;  // driver id of the context the address belongs to (0: none yet)
  void* ptr = nullptr;
};
static NoallocSlot g_noalloc[LP_NOALLOC_MAX_DEVICES];
static std::mutex g_noalloc_mu;

typedef CUresult (*PfnCtxGetCurrent)(CUcontext*);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long*);

// Process-unique id of the calling thread's current context (ids are never
// reused, unlike context handles).  Returns false when no context is current.
// Called with g_noalloc_mu held.
static bool current_ctx_id(unsigned long long* id) {
  static PfnCtxGetCurrent get_cur = nullptr;
  static PfnCtxGetId get_id = nullptr;
  if (!get_cur || !get_id) {
    void* a = nullptr;
    void* b = nullptr;
    cudaDriverEntryPointQueryResult qa, qb;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) != cudaSuccess ||
        qa != cudaDriverEntryPointSuccess || qb != cudaDriverEntryPointSuccess || !a || !b)
      return false;
    get_cur = (PfnCtxGetCurrent)a;
    get_id = (PfnCtxGetId)b;
  }
  CUcontext c = nullptr;
  if (get_cur(&c) != CUDA_SUCCESS || !c) return false;
  return get_id(c, id) == CUDA_SUCCESS;
}

// Device address of the scratch array for `device` (which must be current).
static int noalloc_scratch(int device, void** out) {
  if (device < 0 || device >= LP_NOALLOC_MAX_DEVICES)
    return set_err(LP_ERR_UNSUPPORTED, "lp_fwd_noalloc: device id %d too large", device);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  NoallocSlot& slot = g_noalloc[device];
  unsigned long long id = 0;
  const bool have = current_ctx_id(&id);
  if (!have || !slot.ptr || slot.ctx != id) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);  // loads the module if needed
    if (e != cudaSuccess)
      return set_err(LP_ERR_CUDA, "lp_fwd_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    if (!current_ctx_id(&id))
      return set_err(LP_ERR_CUDA, "lp_fwd_noalloc: no current CUDA context on device %d", device);
    slot.ctx = id;
    slot.ptr = p;
  }
  *out = slot.ptr;
  return LP_OK;
}

static inline size_t round256(size_t b) { return (b + 255) / 256 * 256; }

extern "C" int lp_noalloc_scratch_bytes(const lp_handle* h, int S0, int64_t* bytes) {
  if (!h || !bytes) return set_err(LP_ERR_ARG, "lp_noalloc_scratch_bytes: null pointer");
  if (S0 < 0 || S0 > h->Nslices)
    return set_err(LP_ERR_ARG, "lp_noalloc_scratch_bytes: S0=%d outside [0, %d]", S0, h->Nslices);
  *bytes = (int64_t)(round256((size_t)S0 * h->N * h->N * sizeof(float)) +
                     round256((size_t)S0 * spec_slice(h->Nk, h->Nth) * sizeof(float2)));
  return LP_OK;
}

extern "C" int lp_fwd_noalloc(lp_handle* h, float* R, const float* f, int S0, void* stream) {
  if (!h) return set_err(LP_ERR_ARG, "lp_fwd_noalloc: null handle");
  if (!h->fwd) return set_err(LP_ERR_STATE, "lp_fwd_noalloc: forward tables not initialised (lp_init_fwd)");
  if (S0 < 0 || S0 > h->Nslices)
    return set_err(LP_ERR_ARG, "lp_fwd_noalloc: S0=%d outside [0, %d]", S0, h->Nslices);
  if (S0 > 0 && (!R || !f)) return set_err(LP_ERR_ARG, "lp_fwd_noalloc: null data pointer");
  const size_t fbytes = round256((size_t)S0 * h->N * h->N * sizeof(float));
  const size_t sbytes = round256((size_t)S0 * spec_slice(h->Nk, h->Nth) * sizeof(float2));
  if (fbytes + sbytes > (size_t)LP_NOALLOC_SCRATCH_BYTES)
    return set_err(LP_ERR_UNSUPPORTED,
                   "lp_fwd_noalloc: %d slices of N=%d need %zu bytes of scratch, more than the fixed %lld; "
                   "use fewer slices per call or lp_fwd",
                   S0, h->N, fbytes + sbytes, (long long)LP_NOALLOC_SCRATCH_BYTES);
  DeviceGuard g(h->device);
  void* base = nullptr;
  int rc = noalloc_scratch(h->device, &base);
  if (rc != LP_OK) return rc;
  if (S0 == 0) return LP_OK;  // set-up only: the array is resolved (and its module loaded)
  float* fbuf = (float*)base;
  float2* spec = (float2*)((unsigned char*)base + fbytes);
  cudaStream_t st = (cudaStream_t)stream;
  FwdDev* F = h->fwd;
  FwdIngestArgs ia{f, fbuf, h->N, h->N0, h->N / 2 - h->N0 / 2, h->cubic};
  CUDA_TRY(launch(h, K_FWD_INGEST, st, [&] { return launch_fwd_ingest(ia, S0, st); }));
  if (h->cubic) {
    ColPrefilterArgs ca{fbuf, h->N, h->N};
    CUDA_TRY(launch(h, K_COL_PREFILTER, st, [&] { return launch_col_prefilter(ca, S0, st); }));
  }
  for (int k = 0; k < 3; ++k) {
    FwdC2LPArgs a1{fbuf, spec, F->c2lp[k].p, h->erho.p, h->N, h->Nth, h->Nrho, h->Nk, h->cubic, h->plan_rho,
                   nullptr, F->ival.p, F->dlo, F->dhi, F->F, F->fsc};
    CUDA_TRY(launch(h, K_FWD_C2LP, st, [&] { return launch_fwd_c2lp(a1, S0, st); }));
    ThetaConvArgs a2{spec, F->fz.p, h->Nth, h->Nk, F->dlo, F->dhi,
                     F->lo & ~1, std::min(F->hi | 1, h->Nth - 1), 0, h->plan_th, h->fwd_tblock};
    CUDA_TRY(launch(h, K_THETA_CONV, st, [&] { return launch_theta_conv(a2, S0, st); }));
    FwdLP2PolarArgs a3{spec, R, F->thc.p, F->rhoc.p, F->rows[k].p, F->nrows[k], h->N, h->N0, h->Nth,
                       h->Nrho, h->Nk, h->Nproj0, h->os, h->N / 2 - h->cor, h->cubic, h->plan_rho, F->F, F->fsc};
    CUDA_TRY(launch(h, K_FWD_LP2POLAR, st, [&] { return launch_fwd_lp2polar(a3, S0, st); }));
  }
  return LP_OK;
}

// Test hook: fill the whole allocation-free scratch array of `device` with
// `value` (enqueued on `stream`), so a test can show that no later call reads
// a word it did not write first.
extern "C" int lp_debug_fill_noalloc_scratch(int device, float value, void* stream) {
  DeviceGuard g(device);
  void* base = nullptr;
  int rc = noalloc_scratch(device, &base);
  if (rc != LP_OK) return rc;
  cudaError_t e = fill_async((float*)base, (size_t)LP_NOALLOC_SCRATCH_BYTES / sizeof(float), value,
                             (cudaStream_t)stream);
  if (e != cudaSuccess) return set_err(LP_ERR_CUDA, "lp_debug_fill_noalloc_scratch: %s", cudaGetErrorString(e));
  return LP_OK;
}

// ---------------------------------------------------------------------------
// Helpers for arrays that arrive through __cuda_array_interface__ (CuPy and
// others): the device a pointer belongs to, and ordering against the stream
// the array's producer named.
// ---------------------------------------------------------------------------
extern "C" int lp_pointer_device(const void* p, int* device) {
  if (!p || !device) return set_err(LP_ERR_ARG, "lp_pointer_device: null pointer");
  cudaPointerAttributes at;
  cudaError_t e = cudaPointerGetAttributes(&at, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_err(LP_ERR_ARG, "lp_pointer_device: %s", cudaGetErrorString(e));
  }
  if (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)
    return set_err(LP_ERR_ARG, "lp_pointer_device: %p is not device memory", p);
  *device = at.device;
  return LP_OK;
}

extern "C" int lp_stream_wait(int device, void* waiter, void* producer) {
  DeviceGuard g(device);
  cudaEvent_t ev = nullptr;
  CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  cudaError_t e = cudaEventRecord(ev, (cudaStream_t)producer);
  if (e == cudaSuccess) e = cudaStreamWaitEvent((cudaStream_t)waiter, ev, 0);
  cudaEventDestroy(ev);  // released once the wait has been satisfied
  if (e != cudaSuccess) return set_err(LP_ERR_CUDA, "lp_stream_wait: %s", cudaGetErrorString(e));
  return LP_OK;
}
