// Device-side data structures and profile arithmetic for the render path.
//
// Reference behaviour restated here (AstroPhot 0.x):
//   brightness  : models/_shared_methods.py:286-339 (inclined transform, radius metric,
//                 sersic_radial_model / exponential_radial_model),
//                 utils/parametric_profiles.py:7-18,63-74, utils/conversions/functions.py:7-22
//   quadrature  : utils/operations.py:94-147 (displacement_grid, quad_table,
//                 single_quad_integrate)
//
// Samples are evaluated in FP32 with analytic partial derivatives.  Each data-dependent
// branch of the reference's adaptive integration (refine a pixel when a float64
// comparison says so) is decided in FP32 when an error bound on the FP32 operands keeps
// the comparison clear of its threshold, and otherwise re-decided from a float64
// re-evaluation of the same samples, so the integration masks follow the float64 path.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/astrophot_gb300.h"

namespace apgb {

constexpr int kMaxQuad = 5;   // quad levels <= 5  (quad_level^2 <= 32 lanes)
constexpr int kMaxGrid = 5;   // gridding <= 5     (gridding^2 <= 32 lanes)
constexpr int kMaxDepth = 3;  // integrate_max_depth <= 3
constexpr int kMaxLanczos = 8; // psf_subpixel_shift "lanczos:k", k <= 8
constexpr int kTile = 16;     // 16 x 16 working-pixel tiles (sampling / selection)
constexpr int kOutTileX = 32; // output tiles of the convolve/accumulate pass: 32 x 32 pixels,
constexpr int kOutTileY = 32; // 128 threads, each thread 8 consecutive rows of one column
constexpr int kConvRows = 8;
// Batches with a kernel the register-blocked sizes do not cover (k_conv's large flavour) use
// 32 x 16 tiles with 4 rows per thread: their kernels and input tiles fill most of an SM's shared
// memory, and shorter tiles keep each block's share of it and of the work small.
constexpr int kOutTileYL = 16;
constexpr int kConvRowsL = 4;
constexpr int kConvThreads = kOutTileX * kOutTileY / kConvRows;
static_assert(kOutTileX * kOutTileYL / kConvRowsL == kConvThreads, "both flavours use 128 threads");
__host__ __device__ constexpr int conv_tile_y(bool large) { return large ? kOutTileYL : kOutTileY; }
__host__ __device__ constexpr int conv_rows(bool large) { return large ? kConvRowsL : kConvRows; }
constexpr int kConvMaxKP = 29; // square kernels up to this size use the register-blocked path
constexpr int kNumPlanes = 7; // deep + 6 partial planes
constexpr int kNacc = 56;     // per (stamp, slot) accumulator doubles
constexpr float kLn10f = 2.302585092994046f;
constexpr double kLn10 = 2.302585092994046;
constexpr double kPi = 3.141592653589793;
constexpr float kEps = 5.9604645e-08f;  // 2^-24

// full parameter vector slots (value space)
enum ParamSlot { PX = 0, PY = 1, PQ = 2, PPA = 3, PN = 4, PRE = 5, PIE = 6, PF = 7, NPARAM = 8 };
// partial planes stored after the deep plane: d/dX, d/dY (X = x - cx), q, PA, n, Re
enum GradSlot { GX = 0, GY = 1, GQ = 2, GPA = 3, GN = 4, GRE = 5, NGRAD = 6 };

// accumulator layout inside one (stamp, slot) block of kNacc doubles
enum AccSlot { ACC_CHI2 = 0, ACC_G = 1, ACC_RPP = 9, ACC_H = 17, ACC_N = 17 + 36 };

// operations requested from the convolve/accumulate pass for one (stamp, slot)
enum EvalOps : int32_t {
  OP_NONE = 0,
  OP_FWD = 1,          // render the model
  OP_JAC = 2,          // also the partial planes / Jacobian columns
  OP_WRITE_MODEL = 4,  // write model to the caller's buffer (or the LM's Y0 buffer)
  OP_WRITE_JAC = 8,    // write Jacobian columns (caller's buffer or the LM's J buffer)
  OP_CHI2 = 16,        // accumulate sum W (y - m)^2 over unmasked pixels
  OP_HG = 32,          // accumulate J^T W J and J^T W (y - m)
  OP_RPP = 64,         // accumulate J^T [(2/d)(W (m - Y0)/d - W J h)]
  OP_REP = 128,        // chain Jacobian columns to representation space
  OP_VJP = 256,        // accumulate sum_pixels g * d model / d theta (adjoint of the render)
  OP_VJP_COORD = 512,  // VJP in shift mode: add the sampling-coordinate path to the center
  OP_BASE = 1024,      // keep this evaluation (constants, kernel, deep image, integration
                       // pattern) as the base of later OP_DIFF evaluations of the stamp
  OP_DIFF = 2048,      // render the difference to the stamp's base evaluation: the deep
                       // difference (plane 1), convolved as K1 * dS + dK * S0; OP_CHI2 then
                       // accumulates sum W dm (dm - 2 (y - y0)) and OP_RPP uses dm
};

struct QuadTables {
  int32_t quad_level;  // integrate_quad_level
  int32_t gridding;    // integrate_gridding
  int32_t nsub;        // sub-samples of the sampling mode (1 midpoint, 4 trapezoid, 9 simpsons, k^2 quad)
  int32_t sub_center;  // index of the reference sub-sample (simpsons: midpoint, quad: middle)
  // integration quadrature offsets (unit pixel, before the pixel-scale matrix) and weights
  double qx[kMaxQuad * kMaxQuad], qy[kMaxQuad * kMaxQuad], qw[kMaxQuad * kMaxQuad];
  // displacement grid (unit pixel)
  double gx[kMaxGrid * kMaxGrid], gy[kMaxGrid * kMaxGrid];
  // sampling-mode sub-sample offsets (unit pixel) and weights
  double sx[kMaxQuad * kMaxQuad], sy[kMaxQuad * kMaxQuad], sw[kMaxQuad * kMaxQuad];
  // FP32 copies for the per-sample paths (a double -> float conversion runs on the FP64
  // pipe, which is narrow on this GPU)
  float qxf[kMaxQuad * kMaxQuad], qyf[kMaxQuad * kMaxQuad], qwf[kMaxQuad * kMaxQuad];
  float gxf[kMaxGrid * kMaxGrid], gyf[kMaxGrid * kMaxGrid];
  float sxf[kMaxQuad * kMaxQuad], syf[kMaxQuad * kMaxQuad], swf[kMaxQuad * kMaxQuad];
};

// fill the FP32 copies of a table (host side)
inline void quad_tables_fill_f32(QuadTables& T) {
  for (int k = 0; k < kMaxQuad * kMaxQuad; ++k) {
    T.qxf[k] = (float)T.qx[k];
    T.qyf[k] = (float)T.qy[k];
    T.qwf[k] = (float)T.qw[k];
    T.sxf[k] = (float)T.sx[k];
    T.syf[k] = (float)T.sy[k];
    T.swf[k] = (float)T.sw[k];
  }
  for (int k = 0; k < kMaxGrid * kMaxGrid; ++k) {
    T.gxf[k] = (float)T.gx[k];
    T.gyf[k] = (float)T.gy[k];
  }
}

struct StampDev {
  int32_t nx, ny;    // output window
  int32_t wnx, wny;  // working window
  int32_t kx, ky;    // raw PSF shape (0 = none)
  int32_t kpx, kpy;  // convolution kernel shape (kx + 2 with the bilinear shift, else kx)
  int32_t bx, by;    // psf_border_int (0 without PSF)
  int32_t tile_w0, ntw_x, ntw;  // working tiles: first index, tiles per row, count
  int32_t tile_o0, nto_x, nto;  // output tiles
  int32_t pad0;
  int64_t out_off;   // packed output pixels
  int64_t work_off;  // packed working pixels (per plane)
  int64_t psf_off;   // packed raw PSF pixels
  int64_t spsf_off;  // packed kernels: [2 slots][3 kernels][kpy * kpx]
  double P[4], Pinv[4];
  double ref_ij[2], ref_xy[2];
  double pixel_area;
  float Pf[4], Pinvf[4];  // FP32 copies for the per-pixel paths
  double thr_numel;       // pixel count of the integration threshold (default: working window)
  // PSF convolution by FFT (large kernels): transform sides (powers of two, 0 = direct
  // convolution), offset of the stamp's complex buffers [2 slots][6][fft_ny][fft_nx] and of its
  // convolved planes [2 slots][3 + NGRAD][ny][nx]
  int32_t fft_nx, fft_ny;
  int64_t fft_off;
  int64_t pre_off;
  // window whose samples the exponential / PSF-profile integration threshold sums, in this
  // stamp's working-pixel indices (x0, y0, nx, ny; nx = 0: the stamp's own working window)
  int32_t gw_x0, gw_y0, gw_nx, gw_ny;
};

struct EvalDev {
  int32_t ops;        // EvalOps bitmask; 0 = idle
  int32_t cix, cjy;   // centre pixel (working grid): integer part
  int32_t pad0;
  float fx, fy;       // fractional part (0 with the bilinear shift)
  double fx64, fy64;
  float c, s, invq, Re, invRe, invn, bn, dbn, amp;
  float sky, soft2, thresh;
  double thresh64, soft2_64;
  double shift[2];
  double v[NPARAM];   // value-space parameters
  double amp64, bn64, c64, s64;
  double invq64, invRe64, invn64;  // reciprocals for the float64 re-decisions
  float drep[NPARAM]; // d value / d representation
  // OP_DIFF: differences of this evaluation's constants to the stamp's base evaluation,
  // computed in float64 without cancellation, stored FP32 (see eval_profile_delta)
  float d_c, d_s, d_invq, d_lnire, d_invn, d_bn, d_lnamp, d_X, d_Y, d_sky;
};

// The OP_DIFF constants in registers.
struct DeltaF {
  float c, s, invq, lnire, invn, bn, lnamp, X, Y;
};

// The FP32 constants of one evaluation, held in registers by the pixel kernels (read once
// per tile or queue entry instead of through a reference the compiler must re-load after
// every store).
struct EvalF {
  float c, s, invq, invRe, invn, bn, dbn, amp, soft2, fx, fy;
  float P0, P1, P2, P3;
  int cix, cjy;
};

// everything the kernels need, passed by value
// persistent-grid sizes of the render pass, in blocks per SM (set by the in-project
// autotuner, ap_batch_autotune)
enum GridKnob { GK_SAMPLE = 0, GK_INTEGRATE = 1, GK_CONV = 2, GK_PSF = 3, GK_COUNT = 4 };

// rows of an FFT side-nx transform taken by one CTA of the row passes (1024 complex values)
__host__ __device__ inline int fft_rows_per_block(int nx) { return nx >= 1024 ? 1 : 1024 / nx; }

struct BatchArgs {
  int32_t grid_mult[GK_COUNT];  // blocks per SM of sample/select, level 1-3, convolve, PSF shift
  int32_t n_stamps;
  int32_t kind;         // AP_PROFILE_*
  int32_t sampling;     // AP_SAMPLING_*
  int32_t integrate;    // AP_INTEGRATE_*
  int32_t psf_mode;     // AP_PSF_*
  int32_t lanczos;      // psf_mode AP_PSF_FULL: 0 bilinear shift, k > 0 Lanczos of order k
  int32_t max_depth;
  int32_t free_mask;
  int32_t n_free;
  int32_t has_sky;
  int32_t n_work_tiles, n_out_tiles;
  int32_t max_kp2;      // largest kpy * kpx
  int32_t conv_large;   // some stamp's kernel is not a square of side 3..29 (k_conv's chunked flavour)
  int32_t thr_window;   // some stamp sums its integration threshold over its gw_* window
  float tolerance;
  float center_r2;      // AP_SAMPLING_MIDPOINT_CENTER: squared radius (+ 1e-6) in pixels
  double tolerance64, softening64;
  int64_t work_pixels, out_pixels;
  const StampDev* stamps;
  EvalDev* evals;             // [n_stamps][2]
  const int32_t* work_tiles;  // stamp of each working tile
  const int32_t* out_tiles;   // stamp of each output tile
  const QuadTables* tables;
  float* work;                // [2][kNumPlanes][work_pixels]
  float* aux;                 // [2][2][work_pixels]: reference sub-sample, FP32 error bound of deep
  float* spsf;                // kernels
  int64_t* queue;             // [2 * work_pixels] pixels to integrate
  int64_t* recheck;           // [2 * work_pixels] pixels whose selection needs float64
  int64_t* amb;               // [amb_cap] level-1 pixels whose split decision needs float64
  int64_t amb_cap;            // 0: decided inline
  uint32_t* counters;         // [0] queue len, [1] queue head, [2] fp64 re-decisions (select),
                              // [3] errors, [4] active, [5] recheck len, [6] fp64 (integrate),
                              // [7] active working tiles, [8] active output tiles,
                              // [9] active (stamp, slot) pairs, [10] level-2 integration queue,
                              // [11] convolve-pass tile head, [12] level-1 float64 decisions
  int64_t* wlist;             // [2 * n_work_tiles] active working tiles: slot<<62 | stamp<<32 | tile
  int64_t* olist;             // [2 * n_out_tiles]  active output tiles, same packing
  int32_t* slist;             // [2 * n_stamps]     active (stamp * 2 + slot)
  unsigned long long* work_ctr;  // [0] convolution FLOPs, [1] integration samples, [2] sampling
                                 // samples, [3] / [4] integration samples of difference / Jacobian
                                 // evaluations (of [1]); [8]
  double* mean_acc;           // [n_stamps][2]
  double* tile_acc;           // [n_out_tiles][2][kNacc]
  double* acc;                // [n_stamps][2][kNacc]
  // stamps convolved by FFT (ap_fft.cu): their list and prefix sums of transform rows, column
  // groups and output rows; complex buffers and the convolved planes read by the convolve pass
  int32_t n_fft;
  int32_t fft_rows, fft_cols, fft_outs;  // totals of the three prefix lists (row blocks of
                                         // fft_rows_per_block rows, 8-column groups, row blocks)
  int32_t fft_max_nx, fft_max_ny;
  const int32_t* fft_stamp;   // [n_fft]
  const int32_t* fft_row_pre; // [n_fft + 1] transform row blocks
  const int32_t* fft_col_pre; // [n_fft + 1]
  const int32_t* fft_out_pre; // [n_fft + 1] output row blocks
  float2* fft_buf;
  float* preconv;
  // base of OP_DIFF evaluations (the LM's current point; null outside the LM): its
  // evaluation constants, shifted kernel, deep image and integration pattern per working pixel
  EvalDev* base_eval;         // [n_stamps]
  float* base_psf;            // [n_stamps][max_kp2]
  float* base_deep;           // [work_pixels]
  uint32_t* base_code;        // [work_pixels]
};

// Stamps whose trials the LM renders as differences to the base point: the Sersic and
// exponential profiles (direct, FFT or no convolution).
// (a Lanczos shift has no kernel-difference form: its trials render in full)
__host__ __device__ inline bool diff_capable(const BatchArgs& b, const StampDev&) {
  return (b.kind == AP_PROFILE_SERSIC || b.kind == AP_PROFILE_EXPONENTIAL) && b.lanczos == 0;
}

// Integration pattern of a working pixel: 0 midpoint only, 1 level 1 (one Q x Q quadrature),
// 2 | (sub-pixels refined to level 3) << 2 for a pixel split at level 2.  Two evaluations of a
// pixel with the same pattern use the same sample positions.
constexpr uint32_t kCodeLevel1 = 1u;
__device__ __forceinline__ uint32_t code_split(unsigned level3_mask) { return 2u | (level3_mask << 2); }

// buffers of the convolve/accumulate pass
struct ConvIO {
  const float* psf;       // packed raw PSFs
  const float* psf_base;  // non-null: psf is a perturbation of these raw PSFs and the render
                          // convolves with the derivative of the renormalised shifted kernel
  const float* data;      // packed output pixels (may be null)
  const float* weight;    // (null = 1)
  const uint8_t* mask;    // (null = none)
  float* model_out;       // OP_WRITE_MODEL target
  float* jac_out;         // OP_WRITE_JAC target [n_free][out_pixels]
  const float* y0;        // OP_RPP: model at the base point
  const float* jbase;     // OP_RPP: Jacobian at the base point [n_free][out_pixels]
  const double* hvec;     // OP_RPP: h per stamp [n_stamps][8]
  double rpp_d;           // OP_RPP: d (0.1)
  const float* vjp_in;    // OP_VJP: upstream gradient d loss / d model, output layout
};

// dynamic shared memory of the convolve pass for a kpx x kpy kernel: 3 kernels stored
// transposed with columns padded to a multiple of 4 floats, and two input tiles (the next
// plane's is filled while this one is convolved)
__host__ __device__ inline int conv_col_stride(int kpy) { return (kpy + 3) & ~3; }
// Row pitch of the column-major input tile: at least its kOutTileY + kpy - 1 rows plus the
// 2 rows that the last float4 of a column may overrun, and 4 mod 8 so that the 8 lanes of a
// quarter-warp read 16-byte slots in 8 different bank groups
__host__ __device__ inline int conv_tile_pitch(int kpy, bool large) {
  const int th = conv_tile_y(large) + kpy - 1 + 2;
  return th + ((4 - th % 8) + 8) % 8;
}

// floats after the second tile: the chunked convolution of large kernels reads up to 3 past it
constexpr int kConvSmemPad = 16;
__host__ __device__ inline size_t conv_smem_bytes(int kpx, int kpy, bool large) {
  return sizeof(float) * (3 * (size_t)kpx * conv_col_stride(kpy) +
                          2 * (size_t)(kOutTileX + kpx - 1) * conv_tile_pitch(kpy, large) + kConvSmemPad);
}
// k_conv's large flavour: a kernel that is not a square of side 3..kConvMaxKP
__host__ __device__ inline bool conv_kernel_large(int kpx, int kpy) { return kpx != kpy || kpx > kConvMaxKP; }

__host__ __device__ inline int64_t work_plane(const BatchArgs& b, int slot, int plane) {
  return ((int64_t)slot * kNumPlanes + plane) * b.work_pixels;
}

// profiles with an index n (slot PN) and its Jacobian plane
__host__ __device__ inline bool profile_has_n(int kind) {
  return kind == AP_PROFILE_SERSIC || kind == AP_PROFILE_MOFFAT;
}

// ---------------------------------------------------------------------------
// sample evaluation
// ---------------------------------------------------------------------------

struct Sample {
  float v;
  float arg;  // |exponent argument| for the FP32 error bound
  float g[NGRAD];
};

// Relative error bound of one FP32 sample.  u = R/Re carries a few ulp (<= 2e-7); the MUFU
// log2 adds <= 2.4e-7 absolute, so t = 2^(log2(u)/n) has relative error <= 4e-7 + 5e-7/n;
// the exponent b (t - 1) inherits b t times that, and the MUFU exp adds <= 3e-7 plus
// 1.2e-7 per unit of exponent.  Hence |dI/I| <= 4e-7 + (|b (t - 1)| + b) (5e-7 + 5e-7/n).
// Moffat (e.bn = n, e.invn = 1): ln(1 + u^2) carries <= 2.4e-7 absolute from the log2, 6e-8
// from rounding 1 + u^2 and 3e-7 from u's own error, n times that in the exponent n ln(1 + u^2),
// plus 2.4e-7 relative from its rounding and the exp's 1.4e-7 per unit: the same formula with
// invn = 1 gives 4e-7 + (|arg| + n) 1e-6, above that bound.
// Gaussian (arg = u^2 / 2, e.bn = e.invn = 1): u^2 carries ~5 ulp (6e-7 relative of arg) and
// the exp adds 2.4e-7 plus 1.4e-7 per unit: below 4e-7 + (|arg| + 1) 1e-6.
__device__ __forceinline__ float sample_rel_err(const EvalF& e, float arg) {
  return 4e-7f + (fabsf(arg) + e.bn) * (5e-7f + 5e-7f * e.invn);
}

// EXT: the PSF-model profiles (Moffat, Gaussian) are compiled in; galaxy batches use EXT = false
// and get the Sersic / exponential code alone
template <bool GRAD, bool EXT>
__device__ __forceinline__ Sample eval_profile(const EvalF& e, int kind, float X, float Y,
                                               float area_scale) {
  Sample out;
  const float Xr = e.c * X - e.s * Y;
  const float Yr0 = e.s * X + e.c * Y;
  const float Yr = Yr0 * e.invq;
  const float R = sqrtf(fmaf(Xr, Xr, fmaf(Yr, Yr, e.soft2)));
  const float u = R * e.invRe;
  const float amp = e.amp * area_scale;
  float t = u, lu2 = 0.f, w = 1.f, arg;
  if (EXT && kind == AP_PROFILE_MOFFAT) {
    // I0 / (1 + u^2)^n = I0 exp(-n ln(1 + u^2)); e.bn holds n
    w = fmaf(u, u, 1.f);
    lu2 = __log2f(w);
    arg = e.bn * (lu2 * 0.6931471805599453f);
  } else if (EXT && kind == AP_PROFILE_GAUSSIAN) {
    // I0 / sqrt(2 pi sigma^2) exp(-u^2 / 2), u = R / sigma: the prefactor is in amp
    arg = 0.5f * u * u;
  } else {
    if (kind == AP_PROFILE_SERSIC) {
      lu2 = __log2f(u);
      t = exp2f(lu2 * e.invn);
    }
    arg = e.bn * (t - 1.f);
  }
  const float I = amp * __expf(-arg);
  out.v = I;
  out.arg = arg;
  if (GRAD) {
    const float invR = 1.f / R;
    float dIdR;
    if (kind == AP_PROFILE_SERSIC) {
      const float bt = e.bn * t * e.invn;
      dIdR = -I * bt * invR;
      out.g[GRE] = I * bt * e.invRe;
      out.g[GN] = I * (-e.dbn * (t - 1.f) + bt * (lu2 * 0.6931471805599453f) * e.invn);
    } else if (EXT && kind == AP_PROFILE_MOFFAT) {
      const float nu = 2.f * e.bn * u / w;  // -d ln I / d u
      dIdR = -I * nu * e.invRe;
      out.g[GRE] = I * nu * u * e.invRe;
      out.g[GN] = -I * (lu2 * 0.6931471805599453f);
    } else if (EXT && kind == AP_PROFILE_GAUSSIAN) {
      dIdR = -I * u * e.invRe;
      out.g[GRE] = I * (u * u - 1.f) * e.invRe;  // the prefactor's 1/sigma included
      out.g[GN] = 0.f;
    } else {
      dIdR = -I * e.bn * e.invRe;
      out.g[GRE] = I * e.bn * u * e.invRe;
      out.g[GN] = 0.f;
    }
    out.g[GQ] = dIdR * (-(Yr * Yr) * e.invq * invR);
    out.g[GPA] = dIdR * (Xr * Yr0 * (1.f - e.invq * e.invq) * invR);
    out.g[GX] = dIdR * ((Xr * e.c + Yr * e.s * e.invq) * invR);
    out.g[GY] = dIdR * ((-Xr * e.s + Yr * e.c * e.invq) * invR);
  }
  return out;
}

// Value of one Sersic / exponential sample (the same FP32 operations as eval_profile, so the
// integration decisions do not change) and its difference to the base evaluation,
// dI = I1 - I0, formed without cancellation: every difference below is built from the
// float64 parameter differences of k_eval_setup (DeltaF) and the p1 intermediates, never by
// subtracting two rounded values, so dI keeps a relative error of a few 1e-7 however small
// the step.  With X, Y the sample's plane offsets at p1 and X0 = X - dX:
//   Xr = c X - s Y,  Yr = (s X + c Y) / q,  R^2 = Xr^2 + Yr^2 + eps^2,  u = R / Re,
//   t = u^(1/n),  ln I = ln amp - b (t - 1)   (exponential: t = u, b fixed)
//   d(R^2) = dXr (Xr1 + Xr0) + dYr (Yr1 + Yr0),  d ln u = log1p(d(R^2) / R0^2) / 2 + d ln(1/Re)
//   d ln t = d ln u / n1 + ln u0 d(1/n),  dt = -t1 expm1(-d ln t),  d arg = db (t1 - 1) + b0 dt
//   dI = -I1 expm1(-(d ln amp - d arg))
// log1p / expm1 of the difference arithmetic, from their series: below |x| = 1/2,
// log1p(x) = 2 atanh(u) = 2 (u + u^3/3 + ... + u^11/11) with u = x / (2 + x) (|u| <= 1/3: the
// truncation, about u^13/13, stays below 2e-7 relative there and below 1e-15 for |x| < 1/32), and
// expm1 by its Taylor series to x^9 (truncation below 3e-10); beyond, the MUFU log / exp,
// whose absolute error of ~2e-7 is below 5e-7 of log1p and expm1 there.
__device__ __forceinline__ float d_log1p(float x) {
  // near convergence the arguments are tiny: three terms (truncation x^4/4 < 1e-12 relative)
  if (fabsf(x) < 9.765625e-4f) return x * (1.f + x * (-0.5f + x * 0.33333334f));
  if (fabsf(x) < 0.5f) {
    const float u = __fdividef(x, 2.f + x), u2 = u * u;
    return 2.f * u * (1.f + u2 * (0.33333334f + u2 * (0.2f + u2 * (0.14285715f + u2 * (0.11111111f + u2 * 0.09090909f)))));
  }
  return __logf(1.f + x);
}

__device__ __forceinline__ float d_expm1(float x) {
  if (fabsf(x) < 9.765625e-4f) return x * (1.f + x * (0.5f + x * 0.16666667f));  // (x^4/24: < 1e-13)
  if (fabsf(x) < 0.5f)
    return x * (1.f + x * (0.5f + x * (0.16666667f + x * (0.041666668f + x * (0.008333334f + x * (1.3888889e-3f +
               x * (1.984127e-4f + x * (2.4801588e-5f + x * 2.7557319e-6f))))))));
  return __expf(x) - 1.f;
}

__device__ __forceinline__ Sample eval_profile_delta(const EvalF& e, const DeltaF& d, int kind, float X,
                                                     float Y, float area_scale, float& dI) {
  Sample out;
  const float Xr = e.c * X - e.s * Y;
  const float Yr0 = e.s * X + e.c * Y;
  const float Yr = Yr0 * e.invq;
  const float R2 = fmaf(Xr, Xr, fmaf(Yr, Yr, e.soft2));
  const float R = sqrtf(R2);
  const float u = R * e.invRe;
  const float amp = e.amp * area_scale;
  float t = u, lu2 = 0.f;
  if (kind == AP_PROFILE_SERSIC) {
    lu2 = __log2f(u);
    t = exp2f(lu2 * e.invn);
  }
  const float arg = e.bn * (t - 1.f);
  const float I = amp * __expf(-arg);
  out.v = I;
  out.arg = arg;
  const float c0 = e.c - d.c, s0 = e.s - d.s;
  const float dXr = d.c * X + c0 * d.X - (d.s * Y + s0 * d.Y);
  const float dYr0 = d.s * X + s0 * d.X + (d.c * Y + c0 * d.Y);
  const float dYr = dYr0 * e.invq + (Yr0 - dYr0) * d.invq;
  const float dR2 = dXr * (2.f * Xr - dXr) + dYr * (2.f * Yr - dYr);
  const float dlnu = 0.5f * d_log1p(__fdividef(dR2, R2 - dR2)) + d.lnire;
  float darg;
  if (kind == AP_PROFILE_SERSIC) {
    const float lnu1 = lu2 * 0.6931471805599453f;
    const float dlnt = dlnu * e.invn + (lnu1 - dlnu) * d.invn;
    const float dt = -t * d_expm1(-dlnt);
    darg = d.bn * (t - 1.f) + (e.bn - d.bn) * dt;
  } else {
    darg = e.bn * (-u * d_expm1(-dlnu));
  }
  dI = -I * d_expm1(darg - d.lnamp);
  return out;
}

__device__ __forceinline__ DeltaF load_deltaf(const EvalDev& e) {
  DeltaF d;
  d.c = __ldg(&e.d_c);
  d.s = __ldg(&e.d_s);
  d.invq = __ldg(&e.d_invq);
  d.lnire = __ldg(&e.d_lnire);
  d.invn = __ldg(&e.d_invn);
  d.bn = __ldg(&e.d_bn);
  d.lnamp = __ldg(&e.d_lnamp);
  d.X = __ldg(&e.d_X);
  d.Y = __ldg(&e.d_Y);
  return d;
}

// float64 value, same operation order as the reference.
template <bool EXT>
__device__ __forceinline__ double eval_profile64(const EvalDev& e, int kind, double X, double Y,
                                                 double area_scale) {
  const double Xr = e.c64 * X - e.s64 * Y;
  const double Yr = (e.s64 * X + e.c64 * Y) * e.invq64;
  const double R = sqrt(Xr * Xr + Yr * Yr + e.soft2_64);
  const double amp = e.amp64 * area_scale;
  if (kind == AP_PROFILE_SERSIC) {
    return amp * exp(-e.bn64 * (exp(log(R * e.invRe64) * e.invn64) - 1.0));
  }
  if (EXT && kind == AP_PROFILE_MOFFAT) {
    const double u = R * e.invRe64;
    return amp / pow(1.0 + u * u, e.bn64);
  }
  if (EXT && kind == AP_PROFILE_GAUSSIAN) {
    const double u = R * e.invRe64;
    return amp * exp(-0.5 * (u * u));
  }
  return amp * exp(-e.bn64 * ((R * e.invRe64) - 1.0));
}

// Plane offset (X, Y) of a point given in working-pixel units relative to the
// integer centre pixel, FP32 and FP64.
__device__ __forceinline__ void pix_to_offset(const EvalF& e, float di, float dj, float& X,
                                              float& Y) {
  const float a = di - e.fx, b = dj - e.fy;
  X = e.P0 * a + e.P1 * b;
  Y = e.P2 * a + e.P3 * b;
}

__device__ __forceinline__ EvalF load_evalf(const StampDev& st, const EvalDev& e) {
  EvalF f;
  f.c = __ldg(&e.c);
  f.s = __ldg(&e.s);
  f.invq = __ldg(&e.invq);
  f.invRe = __ldg(&e.invRe);
  f.invn = __ldg(&e.invn);
  f.bn = __ldg(&e.bn);
  f.dbn = __ldg(&e.dbn);
  f.amp = __ldg(&e.amp);
  f.soft2 = __ldg(&e.soft2);
  f.fx = __ldg(&e.fx);
  f.fy = __ldg(&e.fy);
  f.P0 = __ldg(&st.Pf[0]);
  f.P1 = __ldg(&st.Pf[1]);
  f.P2 = __ldg(&st.Pf[2]);
  f.P3 = __ldg(&st.Pf[3]);
  f.cix = __ldg(&e.cix);
  f.cjy = __ldg(&e.cjy);
  return f;
}

__device__ __forceinline__ void pix_to_offset64(const StampDev& st, const EvalDev& e, double di,
                                                double dj, double& X, double& Y) {
  const double a = di - e.fx64, b = dj - e.fy64;
  X = st.P[0] * a + st.P[1] * b;
  Y = st.P[2] * a + st.P[3] * b;
}

// ---------------------------------------------------------------------------
// batched damped solve (LM._h): Cholesky, LU with partial pivoting if not SPD
// ---------------------------------------------------------------------------
__device__ inline bool damped_solve_dev(int p, const double* H, const double* g, double L, double* h) {
  double A[NPARAM * NPARAM];
  double bvec[NPARAM];
  for (int i = 0; i < p; ++i) {
    for (int j = 0; j < p; ++j) {
      const double hij = H[i * p + j];
      A[i * p + j] = (i == j) ? hij * 1.0 + L * (1.0 + H[i * p + i]) : hij * (0.0 + 1.0 / (1.0 + L));
    }
    bvec[i] = g[i];
  }
  // Cholesky
  double C[NPARAM * NPARAM];
  bool spd = true;
  for (int j = 0; j < p && spd; ++j) {
    double d = A[j * p + j];
    for (int k = 0; k < j; ++k) d -= C[j * p + k] * C[j * p + k];
    if (!(d > 0.0)) {
      spd = false;
      break;
    }
    const double ljj = sqrt(d);
    C[j * p + j] = ljj;
    for (int i = j + 1; i < p; ++i) {
      double v = A[i * p + j];
      for (int k = 0; k < j; ++k) v -= C[i * p + k] * C[j * p + k];
      C[i * p + j] = v / ljj;
    }
  }
  if (spd) {
    double z[NPARAM];
    for (int i = 0; i < p; ++i) {
      double v = bvec[i];
      for (int k = 0; k < i; ++k) v -= C[i * p + k] * z[k];
      z[i] = v / C[i * p + i];
    }
    for (int i = p - 1; i >= 0; --i) {
      double v = z[i];
      for (int k = i + 1; k < p; ++k) v -= C[k * p + i] * h[k];
      h[i] = v / C[i * p + i];
    }
    return true;
  }
  // LU with partial pivoting (what torch.linalg.solve does)
  for (int k = 0; k < p; ++k) {
    int best = k;
    double bv = fabs(A[k * p + k]);
    for (int i = k + 1; i < p; ++i)
      if (fabs(A[i * p + k]) > bv) {
        bv = fabs(A[i * p + k]);
        best = i;
      }
    if (best != k) {
      for (int j = 0; j < p; ++j) {
        const double t = A[k * p + j];
        A[k * p + j] = A[best * p + j];
        A[best * p + j] = t;
      }
      const double t = bvec[k];
      bvec[k] = bvec[best];
      bvec[best] = t;
    }
    const double d = A[k * p + k];
    for (int i = k + 1; i < p; ++i) {
      const double f = A[i * p + k] / d;
      for (int j = k; j < p; ++j) A[i * p + j] -= f * A[k * p + j];
      bvec[i] -= f * bvec[k];
    }
  }
  for (int i = p - 1; i >= 0; --i) {
    double v = bvec[i];
    for (int k = i + 1; k < p; ++k) v -= A[i * p + k] * h[k];
    h[i] = v / A[i * p + i];
  }
  return false;
}


}  // namespace apgb
