// Kernel argument blocks and launch helpers shared by lp_kernels.cu and lp_handle.cu.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fft_device.cuh"

namespace lpgb {

// Interpolation coordinates are 32-bit fixed point, value = v * 2^-F (F per
// handle direction); LP_FX_NONE marks a table entry without a point.
#define LP_FX_NONE ((int)0x80000000)

// ---- spectrum layout ------------------------------------------------------
// The log-polar spectrum of one slice (Nk rho frequencies x Ntheta columns,
// complex) is stored in tiles of kSpecTile consecutive rho frequencies:
// element (kk, th) sits at ((kk / 4) * Ntheta + th) * 4 + kk % 4.  A theta
// column is then contiguous in runs of 4 frequencies (32 bytes) and a tile
// row of 4 frequencies is contiguous across theta, so the column kernels
// (one column per signal, frequencies across lanes) and the theta
// convolution (4 frequencies per block, theta across lanes) both touch few
// lines per warp access.  fZ uses the same layout.
constexpr int kSpecTile = 4;
__host__ __device__ inline int spec_rows(int Nk) { return (Nk + kSpecTile - 1) / kSpecTile * kSpecTile; }
__host__ __device__ inline size_t spec_slice(int Nk, int Nth) { return (size_t)spec_rows(Nk) * Nth; }
__host__ __device__ __forceinline__ size_t sidx(int kk, int th, int Nth) {
  return ((size_t)(kk >> 2) * Nth + th) * 4 + (kk & 3);
}

// ---- forward ----------------------------------------------------------------
struct FwdIngestArgs {        // centre f into the padded grid, prefilter rows
  const float* fin;           // [S][N0][N0] caller's image
  float* fbuf;                // [S][N][N]
  int N, N0, off, cubic;
};

struct ColPrefilterArgs {     // prefilter along the slow axis, in place
  float* img;                 // [S][H][W]
  int H, W;
  const cudaSurfaceObject_t* surf;  // if set: final coefficients go to these per-slice 2-D arrays instead
                                    // (img is then only read)
  float* out;                 // else if set: final coefficients go to out [S][H][W] (img only read)
};

struct FwdC2LPArgs {          // Cartesian -> log-polar gather, e^rho, FFT along rho
  const float* fbuf;          // [S][N][N] prefiltered image
  float2* spec;               // [S] spectra (Nk = N+1 rho frequencies), tiled layout (sidx)
  const int2* c2lp;           // [Nth][Nrho] fixed-point texel coordinates (x, y); x = LP_FX_NONE outside the disk
  const float* erho;          // [Nrho]
  int N, Nth, Nrho, Nk, cubic;
  FFTPlan plan;               // length Nrho
  const cudaTextureObject_t* tex;  // if set: the prefiltered image per slice as a gather texture (cubic)
  const int2* ival;           // [Nth] rho interval [x, y] of a column's disk points (y < x: none); if set,
  int col_lo, col_hi;         //   only column pairs meeting [col_lo, col_hi] are launched (others untouched)
  int F;                      // fixed-point fraction bits of the coordinates
  float fsc;                  // 2^-F
};

struct ThetaConvArgs {        // FFT along theta, multiply by the kernel, inverse
  float2* spec;               // [S] spectra, tiled layout
  const float2* fz;           // Hermitian-extended kernel / (Nrho*Nth), tiled layout
  int Nth, Nk;
  int in_lo, in_hi;           // columns outside [in_lo, in_hi] are read as 0
  int out_lo, out_hi;         // only these columns are written back
  int conj_fz;
  FFTPlan plan;               // length Nth
  int block;                  // power-of-two kernels: threads per block (256 or 512; 0 = 256)
  // exact transpose (register-FFT lengths only): with rowspec set, input column c of
  // frequency k is the sum over cent[coff[c] .. coff[c+1]) in that order (rows ascending) of
  // weight * rowspec[s][row][k] -- the transposed theta taps, gathered instead of summed
  // into the spectrum by a separate pass
  const float2* rowspec;      // [S][nrows][rowspec_stride(Nk)]
  const int* coff;            // [Nth + 1]
  const int2* cent;           // (row within the span, float bits of the tap weight)
  int nrows;
};

// row stride of the transpose's row spectra: Nk rounded up to a multiple of 4, so that
// frequencies k, k+1 (k even) of a row are one aligned 16-byte access
__host__ __device__ inline int rowspec_stride(int Nk) { return spec_rows(Nk); }

struct FwdLP2PolarArgs {      // inverse FFT along rho of theta-combined columns, polar gather
  const float2* spec;         // [S] spectra, tiled layout
  float* Rout;                // [S][Nproj0][N0] caller's sinogram
  const int* thc;             // [Nproj] theta texel coordinate per internal angle row (fixed point)
  const int* rhoc;            // [Nproj][N] rho texel coordinate per polar point (fixed point)
  const int* rows;            // internal rows handled by this launch
  int nrows;
  int N, N0, Nth, Nrho, Nk, Nproj0, os, cor_off, cubic;
  FFTPlan plan;               // length Nrho
  int F;
  float fsc;
};

// ---- adjoint ----------------------------------------------------------------
struct AdjIngestArgs {        // cor shift, angle step, edge padding, FBP filter, row prefilter
  const float* Rin;           // [S][Nproj0][N0]
  float* rbuf;                // [S][Nproj][N]
  const float* H;             // [2N] real filter spectrum for a 2N circular convolution, / 2N; or null
  int N, N0, Nproj, Nproj0, os, cor_off, cubic;
  FFTPlan plan;               // length 2N (filter)
};

struct AdjPolar2LPArgs {      // polar -> log-polar gather (+ wrap points), FFT along rho
  const float* rbuf;          // [S][Nproj][N] prefiltered sinogram
  float2* spec;               // [S][Nk][Nth]
  const int* ta;              // [Nth] angle texel coordinate per column, fixed point (LP_FX_NONE: no points)
  const int* sx;              // [Nth][Nrho] s texel coordinate, fixed point (LP_FX_NONE: not a point)
  const int* woff;            // [Nth+1] wrap-point offsets per column
  const int4* wpt;            // wrap points: (rho index, s coordinate, angle coordinate, 0), fixed point
  int N, Nth, Nrho, Nk, Nproj, cubic;
  int clo, chi;
  FFTPlan plan;               // length Nrho
  int F;
  float fsc;
};

struct AdjLPColsArgs {        // inverse FFT along rho, write real log-polar columns
  const float2* spec;         // [S][Nk][Nth]
  float* G;                   // [S][W2][Nrho]
  int Nth, Nrho, Nk, lo2, hi2, W2;
  FFTPlan plan;
  const cudaSurfaceObject_t* surf;  // if set: columns go to per-slice 2-D arrays (x = rho, y = theta - lo2)
};

struct AdjLP2CartArgs {       // log-polar -> Cartesian gather summed over spans, crop
  const float* G0;
  const float* G1;
  const float* G2;            // [S][W2][Nrho] per span
  const int2* c2lp0;
  const int2* c2lp1;
  const int2* c2lp2;          // [N0][N0] (theta, rho) texel coordinates per span, fixed point; LP_FX_NONE outside
  float* fout;                // [S][N0][N0]
  int N0, Nth, Nrho, lo2, W2, cubic;
  int npix;
  const cudaTextureObject_t* tex0;  // if set (cubic): the columns of each span and slice as gather textures
  const cudaTextureObject_t* tex1;
  const cudaTextureObject_t* tex2;
  int F;
  float fsc;
};

// launches (defined in lp_kernels.cu); return the launch error
cudaError_t launch_fwd_ingest(const FwdIngestArgs& a, int S, cudaStream_t st);
cudaError_t launch_col_prefilter(const ColPrefilterArgs& a, int S, cudaStream_t st);
cudaError_t launch_fwd_c2lp(const FwdC2LPArgs& a, int S, cudaStream_t st);
cudaError_t launch_theta_conv(const ThetaConvArgs& a, int S, cudaStream_t st);
// launch_theta_conv takes ThetaConvArgs::rowspec at this length and row count
bool theta_conv_gathers(int Nth, int nrows);
cudaError_t launch_fwd_lp2polar(const FwdLP2PolarArgs& a, int S, cudaStream_t st);
cudaError_t launch_adj_ingest(const AdjIngestArgs& a, int S, cudaStream_t st);
cudaError_t launch_adj_polar2lp(const AdjPolar2LPArgs& a, int S, cudaStream_t st);
cudaError_t launch_adj_lpcols(const AdjLPColsArgs& a, int S, cudaStream_t st);
cudaError_t launch_adj_lp2cart(const AdjLP2CartArgs& a, int S, cudaStream_t st);
cudaError_t configure_kernels(int N);
// false: always use the generic (any-size) FFT kernels
void set_use_p2(bool on);

}  // namespace lpgb

namespace lpgb {
// ---- exact transpose of the forward (autograd backward) --------------------
constexpr int kNoWrap = 1 << 28;  // FwdTRowsArgs::rbase of a row whose taps do not wrap onto themselves

struct FwdTRowsArgs {         // sinogram rows -> their log-polar rho half spectra (transposed lp2polar, part 1)
  const float* Rin;           // [S][Nproj0][N0] caller's gradient
  float2* rowspec;            // [S][nrows][rowspec_stride(Nk)] per row of the span: a_k x R2C of the
                              // transposed rho interpolation
  const int* rhoc;            // [Nproj][N] rho coordinate per polar point (fixed point)
  const int* rows;            // rows of the span (multiples of os), sorted
  const int* rbase;           // [Nproj] smallest first rho tap of each row whose first taps span more
                              // than Nrho - ntap bins; kNoWrap for the others
  int nrows;
  int N, N0, Nrho, Nk, Nproj0, os, cor_off, cubic;
  FFTPlan plan;               // length Nrho
  int F;
  float fsc;
  int mono;                   // every row's first rho tap strictly monotone in x, spanning at most
                              // 2 (Nrho - ntap) + 1 bins: the transposed interpolation runs as two
                              // windows per residue class of x modulo ntap (taps below and from
                              // rbase + Nrho - ntap + 1) without conflicts; else one thread per row
                              // adds in order
};

struct FwdTColSumArgs {       // row spectra -> spectrum columns (transposed theta taps, part 2)
  const float2* rowspec;      // [S][nrows][rowspec_stride(Nk)]
  float2* spec;               // [S] spectra, tiled layout; columns [lo, hi] written
  const int* thc;             // [Nproj] theta coordinate per internal row (fixed point)
  const int* rows;            // rows of the span, sorted
  const int2* blk;            // per column block of CW columns from lo: [first, last) into rows
  int nrows, Nth, Nk, lo, hi, CW, cubic;
  int F;
  float fsc;
};

// the exact transpose's real log-polar values are stored slice-interleaved in groups
// of kGatherSlices slices and in the order of the cell-sorted point list the gather
// walks, [S / kGatherSlices][npts][kGatherSlices]: a point's values for all slices of
// a group are two 16-byte loads, and the points of consecutive cells are consecutive
constexpr int kGatherSlices = 8;

struct FwdTColsArgs {         // spectrum columns -> real log-polar columns x e^rho
  const float2* spec;         // [S][Nk][Nth]
  float* G;                   // [S / kGatherSlices][npts][kGatherSlices]
  const int* pos;             // [dhi - dlo + 1][Nrho] of this span: the point's index in the cell-sorted
                              // list, -1 for no point
  size_t npts;
  const float* erho;          // [Nrho]
  int Nth, Nrho, Nk, dlo, dhi;
  FFTPlan plan;
};

struct FwdTGatherArgs {       // transposed Cartesian interpolation as a per-pixel gather, all spans
  const float* G;             // [groups][npts][kGatherSlices] the points' values (FwdTColsArgs)
  size_t npts;
  float* acc;                 // [S][N][N], written
  const int* cell_off;        // [N*N + 1] CSR over image cells (floor of the point's coordinates)
  const int2* pts;            // per cell: (x, y) fixed point, in (span, theta, rho) order within a cell
  int N, cubic;
  int F;
  float fsc;
};

struct PrefilterTColsArgs {   // transposed prefilter along columns, out of place
  const float* in;            // [S][H][W]
  float* out;                 // [S][H][W]
  int H, W;
};

struct PrefilterTRowsCropArgs {  // transposed prefilter along rows, cropped into the caller's image
  const float* in;            // [S][N][N]
  float* out;                 // [S][N0][N0]
  int N, N0, off;
};

struct CropArgs {
  const float* src;           // [S][N][N]
  float* dst;                 // [S][N0][N0]
  int N, N0, off;
};

cudaError_t launch_fwdT_rows(const FwdTRowsArgs& a, int S, cudaStream_t st);
cudaError_t launch_fwdT_colsum(const FwdTColSumArgs& a, int S, int nblk, cudaStream_t st);
cudaError_t launch_fwdT_cols(const FwdTColsArgs& a, int S, cudaStream_t st);
cudaError_t launch_fwdT_tapw(int2* cent, int n, const int* rows, const int* thc, int F, float fsc, int cubic,
                             cudaStream_t st);
cudaError_t launch_fwdT_gather(const FwdTGatherArgs& a, int S, cudaStream_t st);
cudaError_t launch_prefilter_T_cols(const PrefilterTColsArgs& a, int S, cudaStream_t st);
cudaError_t launch_prefilter_T_rows_crop(const PrefilterTRowsCropArgs& a, int S, cudaStream_t st);
cudaError_t launch_crop(const CropArgs& a, int S, cudaStream_t st);
}  // namespace lpgb
