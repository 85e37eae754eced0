// Render-pass kernels: evaluation setup, PSF shift, sampling, integration-mask selection,
// adaptive sub-pixel integration, PSF convolution with fused Jacobian / chi^2 / J^T W J /
// J^T W r accumulation, and the per-stamp reduction of the tile partials.
//
// One render pass handles every stamp of a batch and two evaluation slots per stamp
// (the LM evaluates two parameter vectors per damping trial).  Reference stages:
//   _sample_init          astrophot/models/_model_methods.py:82-148
//   _sample_integrate     astrophot/models/_model_methods.py:155-184
//   grid_integrate        astrophot/utils/operations.py:150-247
//   _shift_psf, renorm    astrophot/models/_model_methods.py:187-243
//   fft/direct convolve   astrophot/models/_model_methods.py:245-257, utils/operations.py:9-36
//   crop                  astrophot/models/model_object.py:345-349
//   chi2, hess, grad, rpp astrophot/fit/lm.py:374-406
#include <algorithm>
#include <cmath>
#include <mutex>

#include "ap_internal.h"

namespace apgb {

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double sersic_b64(double n) {
  return 2 * n - 1.0 / 3.0 + 4.0 / (405.0 * n) + 46.0 / (25515.0 * n * n) +
         131.0 / (1148175.0 * n * n * n) - 2194697.0 / (30690717750.0 * n * n * n * n);
}

__device__ __forceinline__ double sersic_db64(double n) {
  return 2.0 - 4.0 / (405.0 * n * n) - 2.0 * 46.0 / (25515.0 * n * n * n) -
         3.0 * 131.0 / (1148175.0 * n * n * n * n) +
         4.0 * 2194697.0 / (30690717750.0 * n * n * n * n * n);
}

// d value / d representation (utils/conversions/optimization.py:40-47), from the value.
__device__ __forceinline__ double drep_from_value(int kind, int slot, double v) {
  switch (slot) {
    case PQ: {  // limits (0, 1)
      const double r = tan((v - 0.0) * kPi / 1.0 - kPi / 2);
      return 1.0 / (kPi * (r * r + 1));
    }
    case PN: {
      if (kind == AP_PROFILE_MOFFAT) {  // limits (0.1, 10), models/moffat_model.py:89
        const double r = tan((v - 0.1) * kPi / (10.0 - 0.1) - kPi / 2);
        return (10.0 - 0.1) / (kPi * (r * r + 1));
      }
      // limits (0.36, 8)
      const double r = tan((v - 0.36) * kPi / (8.0 - 0.36) - kPi / 2);
      return (8.0 - 0.36) / (kPi * (r * r + 1));
    }
    case PRE: {  // limits (0, None)
      const double r = v - 1.0 / (v - 0.0);
      return 0.5 + 0.5 * (r - 0.0) / sqrt((r - 0.0) * (r - 0.0) + 4);
    }
    default:
      return 1.0;
  }
}

// ---------------------------------------------------------------------------
// evaluation setup: FP64 parameters -> per (stamp, slot) constants
// ---------------------------------------------------------------------------
__global__ void k_eval_setup(BatchArgs b, const double* params, int64_t stamp_stride,
                             int64_t slot_stride, const int32_t* ops, int32_t ops_uniform) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t == 0) {
    b.counters[0] = 0;  // queue length
    b.counters[1] = 0;  // queue head
    b.counters[5] = 0;  // recheck length
    b.counters[7] = 0;  // active working tiles
    b.counters[8] = 0;  // active output tiles
    b.counters[9] = 0;  // active (stamp, slot) pairs
    b.counters[10] = 0; // level-2 integration list of Jacobian evaluations (front of recheck)
    b.counters[13] = 0; // level-2 integration list of forward evaluations (back of recheck)
    b.counters[14] = 0; // its head
    b.counters[11] = 0; // convolve-pass tile head
    b.counters[12] = 0; // level-1 float64 decisions
  }
  if (t >= b.n_stamps * 2) return;
  const int s = t >> 1, slot = t & 1;
  EvalDev& e = b.evals[t];
  b.mean_acc[t] = 0.0;
  int32_t op = ops ? ops[t] : (slot == 0 ? ops_uniform : 0);
  const StampDev& st = b.stamps[s];
  // (OP_BASE and OP_DIFF need the LM's base buffers; OP_DIFF also a direct-convolution stamp)
  if ((op & OP_BASE) && !b.base_eval) op &= ~OP_BASE;
  if ((op & OP_DIFF) && !(b.base_eval && diff_capable(b, st))) op &= ~OP_DIFF;
  e.ops = op;
  if (!op) return;
  const double* v = params + s * stamp_stride + slot * slot_stride;
  for (int i = 0; i < NPARAM; ++i) e.v[i] = v[i];
  // centre in the working grid: plane_to_pixel (image/wcs.py:587-610) of the padded window
  const double dx = v[PX] - st.ref_xy[0], dy = v[PY] - st.ref_xy[1];
  const double pcx = st.Pinv[0] * dx + st.Pinv[1] * dy + st.ref_ij[0] + st.bx;
  const double pcy = st.Pinv[2] * dx + st.Pinv[3] * dy + st.ref_ij[1] + st.by;
  if (b.psf_mode == AP_PSF_FULL) {
    // sub-pixel shift onto a pixel centre (models/model_object.py:320-323)
    const double rx = rint(pcx), ry = rint(pcy);
    e.shift[0] = pcx - rx;
    e.shift[1] = pcy - ry;
    e.cix = (int32_t)rx;
    e.cjy = (int32_t)ry;
    e.fx64 = e.fy64 = 0.0;
  } else {
    const double fxx = floor(pcx), fyy = floor(pcy);
    e.shift[0] = e.shift[1] = 0.0;
    e.cix = (int32_t)fxx;
    e.cjy = (int32_t)fyy;
    e.fx64 = pcx - fxx;
    e.fy64 = pcy - fyy;
  }
  e.fx = (float)e.fx64;
  e.fy = (float)e.fy64;
  // inclined transform (models/_shared_methods.py:301-307): rotate by -(PA - north)
  const double theta = -(v[PPA] - kPi / 2);
  e.c64 = cos(theta);
  e.s64 = sin(theta);
  e.c = (float)e.c64;
  e.s = (float)e.s64;
  e.invq64 = 1.0 / v[PQ];
  e.invq = (float)e.invq64;
  e.Re = (float)v[PRE];
  e.invRe64 = 1.0 / v[PRE];
  e.invRe = (float)e.invRe64;
  const double n = profile_has_n(b.kind) ? v[PN] : 1.0;
  if (b.kind == AP_PROFILE_GAUSSIAN) {  // (FP32 error bound of eval_profile: bn = invn = 1)
    e.invn64 = 1.0;
    e.invn = 1.f;
    e.bn64 = 1.0;
    e.bn = 1.f;
    e.dbn = 0.f;
  } else if (b.kind == AP_PROFILE_MOFFAT) {  // I0 / (1 + (R/Rd)^2)^n: the power in bn, Rd in Re
    e.invn64 = 1.0 / n;
    e.invn = 1.f;  // (FP32 error bound of eval_profile)
    e.bn64 = n;
    e.bn = (float)n;
    e.dbn = 0.f;
  } else {
    e.invn64 = 1.0 / n;
    e.invn = (float)e.invn64;
    e.bn64 = sersic_b64(n);
    e.bn = (float)e.bn64;
    e.dbn = (float)sersic_db64(n);
  }
  e.amp64 = st.pixel_area * pow(10.0, v[PIE]);
  // gaussian_torch (utils/parametric_profiles.py:39-48): I0 / sqrt(2 pi sigma^2), sigma in slot Re
  if (b.kind == AP_PROFILE_GAUSSIAN) e.amp64 = e.amp64 / sqrt(2 * kPi * v[PRE] * v[PRE]);
  e.amp = (float)e.amp64;
  e.sky = b.has_sky ? (float)(st.pixel_area * pow(10.0, v[PF])) : 0.f;
  e.soft2_64 = b.softening64 * b.softening64;
  e.soft2 = (float)e.soft2_64;
  // integration reference: Sersic total flux / numel (models/sersic_model.py:78-89,
  // utils/conversions/functions.py:168-190); exponential and Moffat use sum(deep) / numel
  // later (the default _integrate_reference, models/_model_methods.py:151-152)
  if (b.kind == AP_PROFILE_SERSIC) {
    const double Ie = pow(10.0, v[PIE]);
    const double bn = e.bn64;
    const double flux = 2 * kPi * Ie * v[PRE] * v[PRE] * v[PQ] * n * (exp(bn) * pow(bn, -2 * n)) *
                        exp(lgamma(2 * n));
    e.thresh64 = b.tolerance64 * (flux / st.thr_numel);
  } else {
    e.thresh64 = 0.0;
  }
  e.thresh = (float)e.thresh64;
  for (int i = 0; i < NPARAM; ++i) e.drep[i] = (float)drep_from_value(b.kind, i, v[i]);
  if (op & OP_DIFF) {
    // differences to the base evaluation, each formed without subtracting rounded values
    const EvalDev& e0 = b.base_eval[s];
    const double* v0 = e0.v;
    // sample plane offsets X = P (ij - centre pixel - f): the centre moved by (dpx, dpy) pixels
    const double dpx = (double)(e.cix - e0.cix) + (e.fx64 - e0.fx64);
    const double dpy = (double)(e.cjy - e0.cjy) + (e.fy64 - e0.fy64);
    e.d_X = (float)(-(st.P[0] * dpx + st.P[1] * dpy));
    e.d_Y = (float)(-(st.P[2] * dpx + st.P[3] * dpy));
    // cos / sin of theta = -(PA - pi/2) by the sum-to-product identities
    const double th1 = -(v[PPA] - kPi / 2), th0 = -(v0[PPA] - kPi / 2);
    const double hm = 0.5 * (th1 + th0), hd = sin(0.5 * (th1 - th0));
    e.d_c = (float)(-2.0 * sin(hm) * hd);
    e.d_s = (float)(2.0 * cos(hm) * hd);
    e.d_invq = (float)((v0[PQ] - v[PQ]) / (v0[PQ] * v[PQ]));
    e.d_lnire = (float)(-log1p((v[PRE] - v0[PRE]) / v0[PRE]));
    if (b.kind == AP_PROFILE_SERSIC) {
      // b(n) = 2n - 1/3 + sum_k a_k n^-k: powers of 1/n differenced as dy sum y1^j y0^(k-1-j)
      const double n1 = v[PN], n0 = v0[PN];
      const double y1 = 1.0 / n1, y0 = 1.0 / n0, dy = (n0 - n1) / (n0 * n1);
      const double dy2 = dy * (y1 + y0), dy3 = dy * (y1 * y1 + y1 * y0 + y0 * y0);
      const double dy4 = dy * (y1 * y1 * y1 + y1 * y1 * y0 + y1 * y0 * y0 + y0 * y0 * y0);
      e.d_invn = (float)dy;
      e.d_bn = (float)(2 * (n1 - n0) + 4.0 / 405.0 * dy + 46.0 / 25515.0 * dy2 + 131.0 / 1148175.0 * dy3 -
                       2194697.0 / 30690717750.0 * dy4);
    } else {
      e.d_invn = 0.f;
      e.d_bn = 0.f;
    }
    e.d_lnamp = (float)(kLn10 * (v[PIE] - v0[PIE]));
    e.d_sky = b.has_sky ? (float)(st.pixel_area * pow(10.0, v0[PF]) * expm1(kLn10 * (v[PF] - v0[PF]))) : 0.f;
  }
  if (op & OP_BASE) b.base_eval[s] = e;
}

// Compacted work lists of this pass: the tiles of active (stamp, slot) pairs only, so the
// pixel kernels (persistent grid-stride loops) never visit idle stamps.
__global__ void k_build_lists(BatchArgs b) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= b.n_stamps * 2) return;
  if (!b.evals[t].ops) return;
  const int s = t >> 1, slot = t & 1;
  const StampDev& st = b.stamps[s];
  const int64_t key = ((int64_t)slot << 62) | ((int64_t)s << 32);
  const uint32_t w0 = atomicAdd(&b.counters[7], (unsigned)st.ntw);
  for (int k = 0; k < st.ntw; ++k) b.wlist[w0 + k] = key | k;
  const uint32_t o0 = atomicAdd(&b.counters[8], (unsigned)st.nto);
  for (int k = 0; k < st.nto; ++k) b.olist[o0 + k] = key | k;
  b.slist[atomicAdd(&b.counters[9], 1u)] = t;
  // algorithmic work of this evaluation (counted here, once, not per warp in the kernels):
  // convolution = 2 FLOP per kernel tap per convolved plane per output pixel
  const int ops = b.evals[t].ops;
  if (b.psf_mode != AP_PSF_NONE && st.fft_nx == 0) {  // (FFT-convolved stamps: not k_conv's work)
    const bool jac = (ops & OP_JAC) != 0, shiftmode = (b.psf_mode == AP_PSF_FULL);
    // (a difference evaluation convolves dS with K1 and, with the shift, S0 with dK)
    const int nconv = jac ? ((shiftmode ? 3 : 1) + (profile_has_n(b.kind) ? 4 : 3) +
                             ((shiftmode && !(ops & OP_VJP_COORD)) ? 0 : 2))
                          : ((ops & OP_DIFF) && shiftmode ? 2 : 1);
    atomicAdd(b.work_ctr, (unsigned long long)st.nx * st.ny * 2ull *
                              (unsigned long long)(st.kpx * st.kpy) * (unsigned long long)nconv);
  }
  atomicAdd(b.work_ctr + 2, (unsigned long long)st.wnx * st.wny * (unsigned long long)b.tables->nsub);
}

__device__ __forceinline__ void unpack_entry(int64_t ent, int& slot, int& s, int& local) {
  slot = (int)(ent >> 62);
  s = (int)((ent >> 32) & 0x3fffffff);
  local = (int)(ent & 0xffffffffll);
}

// ---------------------------------------------------------------------------
// PSF shift (bilinear interp2d of the 1-padded PSF) and renormalisation, with d/d shift
// ---------------------------------------------------------------------------
// Bilinear interp2d of the 1-padded PSF at (ix - sx, iy - sy) (indices clamped, weights not:
// the reference extrapolates at the edge) and its derivatives with respect to the shift.
// FP32: the shifted values are stored as floats and the weights of a shift |s| <= 1/2 need no
// more (relative error ~1e-7)
struct ShiftValF {
  float v, dx, dy;
};

__device__ __forceinline__ ShiftValF shifted_psf_at_f(const float* psf, int kx, int ky, int ix, int iy,
                                                      float sx, float sy) {
  const int w = kx + 2, h = ky + 2;
  auto pad = [&](int r, int c) -> float {
    const int rr = r - 1, cc = c - 1;
    return (rr >= 0 && rr < ky && cc >= 0 && cc < kx) ? psf[rr * kx + cc] : 0.f;
  };
  const float x = (float)ix - sx, y = (float)iy - sy;
  int x0 = (int)floorf(x), y0 = (int)floorf(y);
  int x1 = x0 + 1, y1 = y0 + 1;
  x0 = min(max(x0, 0), w - 2);
  x1 = min(max(x1, 1), w - 1);
  y0 = min(max(y0, 0), h - 2);
  y1 = min(max(y1, 1), h - 1);
  const float fa = pad(y0, x0), fb = pad(y1, x0), fc = pad(y0, x1), fd = pad(y1, x1);
  const float ax = (float)x1 - x, bx = x - (float)x0, ay = (float)y1 - y, by = y - (float)y0;
  ShiftValF r;
  r.v = fa * (ax * ay) + fb * (ax * by) + fc * (bx * ay) + fd * (bx * by);
  r.dx = -(-fa * ay - fb * by + fc * ay + fd * by);
  r.dy = -(-fa * ax + fb * ax - fc * bx + fd * bx);
  return r;
}

// ---- Lanczos sub-pixel shift (psf_subpixel_shift "lanczos:k", models/_model_methods.py:209-227):
// the PSF zero-padded by k and cross-correlated ("same") with the (2k+1)^2 kernel
// LL[b][a] = Lx[a] Ly[b], Lx[a] = f(a - k + shift_x), f(t) = sinc(t) sinc(t / k)
// (utils/interpolate.py:145-163), then renormalised.  LL's own normalisation cancels in the
// renormalisation, so the weights here are unnormalised.
__device__ __forceinline__ void sinc_and_slope(double t, double& v, double& dv) {
  constexpr double kPi = 3.14159265358979323846;
  const double x = kPi * t;
  if (fabs(x) < 1e-4) {  // series: sinc = 1 - x^2/6 + x^4/120, d/dt = pi (-x/3 + x^3/30)
    const double x2 = x * x;
    v = 1.0 - x2 / 6.0 + x2 * x2 / 120.0;
    dv = kPi * x * (-1.0 / 3.0 + x2 / 30.0);
  } else {
    double sn, cs;
    sincos(x, &sn, &cs);
    v = sn / x;
    dv = kPi * (cs - v) / x;
  }
}

// w[a] = f(a - k + shift), dw[a] = d w[a] / d shift, a = 0 .. 2k
__device__ __forceinline__ void lanczos_weights(double shift, int k, float* w, float* dw) {
  for (int a = 0; a <= 2 * k; ++a) {
    const double t = (double)(a - k) + shift;
    double s1, d1, s2, d2;
    sinc_and_slope(t, s1, d1);
    sinc_and_slope(t / k, s2, d2);
    w[a] = (float)(s1 * s2);
    dw[a] = (float)(d1 * s2 + s1 * d2 / k);
  }
}

// The shifted kernel (size (kx + 2k) x (ky + 2k)) at (ix, iy) and its shift derivatives:
// sum over a, b of Lx[a] Ly[b] psf[iy + b - 2k][ix + a - 2k] (zero outside the PSF)
__device__ __forceinline__ ShiftValF lanczos_psf_at_f(const float* psf, int kx, int ky, int ix, int iy, int k,
                                                      const float* wx, const float* dwx, const float* wy,
                                                      const float* dwy) {
  ShiftValF r{0.f, 0.f, 0.f};
  for (int b = 0; b <= 2 * k; ++b) {
    const int rr = iy + b - 2 * k;
    if (rr < 0 || rr >= ky) continue;
    float sv = 0.f, sdx = 0.f;
    for (int a = 0; a <= 2 * k; ++a) {
      const int cc = ix + a - 2 * k;
      if (cc < 0 || cc >= kx) continue;
      const float p = psf[rr * kx + cc];
      sv = fmaf(wx[a], p, sv);
      sdx = fmaf(dwx[a], p, sdx);
    }
    r.v = fmaf(wy[b], sv, r.v);
    r.dx = fmaf(wy[b], sdx, r.dx);
    r.dy = fmaf(dwy[b], sv, r.dy);
  }
  return r;
}

// Shifted value at shift s1 and its difference to the value at shift s0 (ds = s1 - s0 exact).
// Inside one bilinear cell the value is bilinear in the shift, so the difference of each
// weight product is expanded in ds; a tap whose cell differs between the shifts takes B1 - B0.
__device__ __forceinline__ float2 shifted_psf_delta(const float* psf, int kx, int ky, int ix, int iy, float sx1,
                                                    float sy1, float sx0, float sy0, float dsx, float dsy) {
  const int w = kx + 2, h = ky + 2;
  auto pad = [&](int r, int c) -> float {
    const int rr = r - 1, cc = c - 1;
    return (rr >= 0 && rr < ky && cc >= 0 && cc < kx) ? psf[rr * kx + cc] : 0.f;
  };
  auto cell = [](float x, int lim, int& c0, int& c1) {
    c0 = (int)floorf(x);
    c1 = c0 + 1;
    c0 = min(max(c0, 0), lim - 2);
    c1 = min(max(c1, 1), lim - 1);
  };
  const float x = (float)ix - sx1, y = (float)iy - sy1;
  const float xb = (float)ix - sx0, yb = (float)iy - sy0;
  int x0, x1, y0, y1, bx0, bx1, by0, by1;
  cell(x, w, x0, x1);
  cell(y, h, y0, y1);
  cell(xb, w, bx0, bx1);
  cell(yb, h, by0, by1);
  const float fa = pad(y0, x0), fb = pad(y1, x0), fc = pad(y0, x1), fd = pad(y1, x1);
  const float ax = (float)x1 - x, bx = x - (float)x0, ay = (float)y1 - y, by = y - (float)y0;
  float2 r;
  r.x = fa * (ax * ay) + fb * (ax * by) + fc * (bx * ay) + fd * (bx * by);
  if (x0 == bx0 && y0 == by0) {
    // base weights: ax - dsx, bx + dsx, ay - dsy, by + dsy
    const float pxy = dsx * dsy;
    const float d00 = ax * dsy + dsx * ay - pxy, d01 = -ax * dsy + dsx * by + pxy;
    const float d10 = bx * dsy - dsx * ay + pxy, d11 = -bx * dsy - dsx * by - pxy;
    r.y = fa * d00 + fb * d01 + fc * d10 + fd * d11;
  } else {
    r.y = r.x - shifted_psf_at_f(psf, kx, ky, ix, iy, sx0, sy0).v;
  }
  return r;
}

__device__ __forceinline__ double warp_sum_d(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Derivative of the shifted, renormalised kernel N(K) = S(K) / sum S(K) (S: the shift, linear)
// along a perturbation D of the raw kernel K:
//   dN = (S(D) - N(K) sum S(D)) / sum S(K),
// so that a render with dN in place of N(K) is d model / d (PSF parameter) when D = dK/dtheta.
__device__ void psf_derivative_warp(const BatchArgs& b, const float* D, const float* K, int s, int slot,
                                    int lane) {
  const EvalDev& e = b.evals[s * 2 + slot];
  const StampDev& st = b.stamps[s];
  const int kp2 = st.kpx * st.kpy;
  const float* Pd = D + st.psf_off;
  const float* Pk = K + st.psf_off;
  float* out = b.spsf + st.spsf_off + (int64_t)slot * 3 * kp2;
  const bool shift = (b.psf_mode == AP_PSF_FULL);
  const float sx = (float)e.shift[0], sy = (float)e.shift[1];
  auto val = [&](const float* P, int idx) -> float {
    return shift ? shifted_psf_at_f(P, st.kx, st.ky, idx % st.kpx, idx / st.kpx, sx, sy).v : P[idx];
  };
  double SK = 0, SD = 0;
  for (int idx = lane; idx < kp2; idx += 32) {
    SK += val(Pk, idx);
    SD += val(Pd, idx);
  }
  SK = warp_sum_d(SK);
  SD = warp_sum_d(SD);
  const float inv = (float)(1.0 / SK), c = (float)(SD / (SK * SK));
  for (int idx = lane; idx < kp2; idx += 32) out[idx] = val(Pd, idx) * inv - val(Pk, idx) * c;
}

// one warp per (stamp, evaluation slot): sums in FP64 across the warp, values in FP32
__device__ void psf_shift_warp(const BatchArgs& b, const float* psf, int s, int slot, int lane) {
  const EvalDev& e = b.evals[s * 2 + slot];
  const StampDev& st = b.stamps[s];
  const int kp2 = st.kpx * st.kpy;
  const float* P = psf + st.psf_off;
  float* out = b.spsf + st.spsf_off + (int64_t)slot * 3 * kp2;
  const bool jac = (e.ops & OP_JAC) != 0;
  if (b.psf_mode == AP_PSF_FULL && (e.ops & OP_DIFF)) {
    // K1 (kernel 0) and dK = K1 - K0 = (dB - K0 sum dB) / sum B1 (kernel 1), B the shifted
    // unnormalised kernel and K0 the base's normalised one
    const EvalDev& e0 = b.base_eval[s];
    const float* K0 = b.base_psf + (int64_t)s * b.max_kp2;
    const float sx1 = (float)e.shift[0], sy1 = (float)e.shift[1];
    const float sx0 = (float)e0.shift[0], sy0 = (float)e0.shift[1];
    const float dsx = (float)(e.shift[0] - e0.shift[0]), dsy = (float)(e.shift[1] - e0.shift[1]);
    double S = 0, SD = 0;
    for (int idx = lane; idx < kp2; idx += 32) {
      const float2 r = shifted_psf_delta(P, st.kx, st.ky, idx % st.kpx, idx / st.kpx, sx1, sy1, sx0, sy0, dsx, dsy);
      S += r.x;
      SD += r.y;
    }
    S = warp_sum_d(S);
    SD = warp_sum_d(SD);
    const float inv = (float)(1.0 / S), c = (float)SD;
    for (int idx = lane; idx < kp2; idx += 32) {
      const float2 r = shifted_psf_delta(P, st.kx, st.ky, idx % st.kpx, idx / st.kpx, sx1, sy1, sx0, sy0, dsx, dsy);
      out[idx] = r.x * inv;
      out[kp2 + idx] = (r.y - K0[idx] * c) * inv;
    }
  } else if (b.psf_mode == AP_PSF_FULL && b.lanczos > 0) {
    // Lanczos shift: the same renormalisation and derivative rule as the bilinear one below
    const int k = b.lanczos;
    float wx[2 * kMaxLanczos + 1], dwx[2 * kMaxLanczos + 1], wy[2 * kMaxLanczos + 1], dwy[2 * kMaxLanczos + 1];
    lanczos_weights(e.shift[0], k, wx, dwx);
    lanczos_weights(e.shift[1], k, wy, dwy);
    double S = 0, Sx = 0, Sy = 0;
    for (int idx = lane; idx < kp2; idx += 32) {
      const ShiftValF r = lanczos_psf_at_f(P, st.kx, st.ky, idx % st.kpx, idx / st.kpx, k, wx, dwx, wy, dwy);
      S += r.v;
      Sx += r.dx;
      Sy += r.dy;
    }
    S = warp_sum_d(S);
    Sx = warp_sum_d(Sx);
    Sy = warp_sum_d(Sy);
    const float inv = (float)(1.0 / S), cx = (float)(Sx / (S * S)), cy = (float)(Sy / (S * S));
    for (int idx = lane; idx < kp2; idx += 32) {
      const ShiftValF r = lanczos_psf_at_f(P, st.kx, st.ky, idx % st.kpx, idx / st.kpx, k, wx, dwx, wy, dwy);
      out[idx] = r.v * inv;
      if (jac) {
        out[kp2 + idx] = r.dx * inv - r.v * cx;
        out[2 * kp2 + idx] = r.dy * inv - r.v * cy;
      }
    }
  } else if (b.psf_mode == AP_PSF_FULL) {
    const float sx = (float)e.shift[0], sy = (float)e.shift[1];
    double S = 0, Sx = 0, Sy = 0;
    for (int idx = lane; idx < kp2; idx += 32) {
      const ShiftValF r = shifted_psf_at_f(P, st.kx, st.ky, idx % st.kpx, idx / st.kpx, sx, sy);
      S += r.v;
      Sx += r.dx;
      Sy += r.dy;
    }
    S = warp_sum_d(S);
    Sx = warp_sum_d(Sx);
    Sy = warp_sum_d(Sy);
    const float inv = (float)(1.0 / S), cx = (float)(Sx / (S * S)), cy = (float)(Sy / (S * S));
    for (int idx = lane; idx < kp2; idx += 32) {
      const ShiftValF r = shifted_psf_at_f(P, st.kx, st.ky, idx % st.kpx, idx / st.kpx, sx, sy);
      out[idx] = r.v * inv;
      if (jac) {
        out[kp2 + idx] = r.dx * inv - r.v * cx;
        out[2 * kp2 + idx] = r.dy * inv - r.v * cy;
      }
      if (e.ops & OP_BASE) b.base_psf[(int64_t)s * b.max_kp2 + idx] = r.v * inv;
    }
  } else {
    double S = 0;
    for (int idx = lane; idx < kp2; idx += 32) S += (double)P[idx];
    S = warp_sum_d(S);
    const float inv = (float)(1.0 / S);
    for (int idx = lane; idx < kp2; idx += 32) out[idx] = P[idx] * inv;
  }
}

// psf_base == nullptr: the shifted, renormalised kernels of psf; otherwise psf is a
// perturbation of psf_base and the kernels are the derivatives of psf_derivative_warp
__global__ void k_psf_shift(BatchArgs b, const float* psf, const float* psf_base) {
  const uint32_t n = b.counters[9];
  const int wpb = blockDim.x >> 5, lane = threadIdx.x & 31;
  for (uint32_t it = blockIdx.x * wpb + (threadIdx.x >> 5); it < n; it += gridDim.x * wpb) {
    const int t = b.slist[it];
    if (psf_base)
      psf_derivative_warp(b, psf, psf_base, t >> 1, t & 1, lane);
    else
      psf_shift_warp(b, psf, t >> 1, t & 1, lane);
  }
}

// ---------------------------------------------------------------------------
// sampling (_sample_init): deep value, partials, reference sub-sample, FP32 error bound
// ---------------------------------------------------------------------------
// DIFF (forward only): also ddeep = the difference of deep to the base evaluation
// mid_only: one sample at the pixel centre (sampling mode midpoint_center outside its radius)
template <bool JAC, bool EXT, bool DIFF>
__device__ __forceinline__ void sample_pixel(const BatchArgs& b, const EvalF& e, const DeltaF& d, int i, int j,
                                             bool mid_only, float& deep, float* g, float& refsub, float& errb,
                                             float& ddeep) {
  const QuadTables& T = *b.tables;
  const float di = (float)(i - e.cix), dj = (float)(j - e.cjy);
  const int nsub = mid_only ? 1 : T.nsub, sub_center = mid_only ? 0 : T.sub_center;
  deep = 0.f;
  ddeep = 0.f;
#pragma unroll
  for (int k = 0; k < NGRAD; ++k) g[k] = 0.f;
  float absb = 0.f, mag = 0.f;
  refsub = 0.f;
  float referr = 0.f;
  for (int k = 0; k < nsub; ++k) {
    float X, Y;
    pix_to_offset(e, di + (mid_only ? 0.f : T.sxf[k]), dj + (mid_only ? 0.f : T.syf[k]), X, Y);
    float dI = 0.f;
    const Sample sm = DIFF ? eval_profile_delta(e, d, b.kind, X, Y, 1.f, dI) : eval_profile<JAC, EXT>(e, b.kind, X, Y, 1.f);
    const float w = mid_only ? 1.f : T.swf[k];
    deep = fmaf(w, sm.v, deep);
    if (DIFF) ddeep = fmaf(w, dI, ddeep);
    if (JAC) {
#pragma unroll
      for (int q = 0; q < NGRAD; ++q) g[q] = fmaf(w, sm.g[q], g[q]);
    }
    const float a = fabsf(w * sm.v);
    mag += a;
    absb += a * sample_rel_err(e, sm.arg);
    if (k == sub_center) {
      refsub = sm.v;
      referr = fabsf(sm.v) * sample_rel_err(e, sm.arg);
    }
  }
  // bound on |deep_fp32 - deep_fp64| (+ the reference sub-sample's for simpsons / quad)
  errb = absb + 2.f * (float)nsub * kEps * mag + referr;
}

// Deep value of a working pixel that is final (not refined further): the base evaluation
// keeps it with its integration pattern; a difference evaluation stores its difference to the
// base, from the sample differences when the base integrated the pixel with the same pattern
// (same sample positions), else as the plain difference of the two values.
__device__ __forceinline__ void write_diff_base(const BatchArgs& b, int ops, int slot, int64_t wp, float v,
                                                float dv, uint32_t code) {
  if (ops & OP_DIFF) b.work[work_plane(b, slot, 1) + wp] = (b.base_code[wp] == code) ? dv : v - b.base_deep[wp];
  if (ops & OP_BASE) {
    b.base_deep[wp] = v;
    b.base_code[wp] = code;
  }
}

template <bool EXT>
__device__ double sample_pixel64(const BatchArgs& b, const StampDev& st, const EvalDev& e, int i,
                                 int j, double* refsub) {
  const QuadTables& T = *b.tables;
  const double di = (double)(i - e.cix), dj = (double)(j - e.cjy);
  double deep = 0.0;
  for (int k = 0; k < T.nsub; ++k) {
    double X, Y;
    pix_to_offset64(st, e, di + T.sx[k], dj + T.sy[k], X, Y);
    const double f = eval_profile64<EXT>(e, b.kind, X, Y, 1.0);
    deep += T.sw[k] * f;
    if (k == T.sub_center && refsub) *refsub = f;
  }
  return deep;
}

template <bool JAC, bool EXT, bool DIFF>
__device__ void sample_tile(const BatchArgs& b, const EvalF& e, const DeltaF& d, int ops, int s, int slot,
                            int tile_local) {
  const StampDev& st = b.stamps[s];
  const int tx = threadIdx.x & (kTile - 1), ty = threadIdx.x / kTile;
  const int i = (tile_local % st.ntw_x) * kTile + tx;
  const int j = (tile_local / st.ntw_x) * kTile + ty;
  const bool valid = (i < st.wnx) && (j < st.wny);
  float deep = 0.f;
  if (valid) {
    // midpoint_center: the quadrature table only for pixel centres within the radius
    bool mid_only = false;
    if (b.sampling == AP_SAMPLING_MIDPOINT_CENTER) {
      const float ax = (float)(i - e.cix) - e.fx, ay = (float)(j - e.cjy) - e.fy;
      mid_only = ax * ax + ay * ay > b.center_r2;
    }
    float g[NGRAD], refsub, errb, ddeep;
    sample_pixel<JAC, EXT, DIFF>(b, e, d, i, j, mid_only, deep, g, refsub, errb, ddeep);
    const int64_t p = st.work_off + (int64_t)j * st.wnx + i;
    b.work[work_plane(b, slot, 0) + p] = deep;
    if (JAC) {
#pragma unroll
      for (int q = 0; q < NGRAD; ++q) b.work[work_plane(b, slot, 1 + q) + p] = g[q];
    }
    float* aux = b.aux + (int64_t)slot * 2 * b.work_pixels;
    aux[p] = refsub;
    aux[b.work_pixels + p] = errb;
    // (pixels the integration refines are written again there; midpoint_center marks its
    // quadrature pixels, which a moved centre may change)
    if (ops & (OP_DIFF | OP_BASE))
      write_diff_base(b, ops, slot, p, deep, ddeep,
                      (b.sampling == AP_SAMPLING_MIDPOINT_CENTER && !mid_only) ? kCodeLevel1 : 0u);
  }
  if (b.kind != AP_PROFILE_SERSIC && b.integrate == AP_INTEGRATE_THRESHOLD && st.gw_nx == 0) {
    // sum(deep) for the default _integrate_reference (models/_model_methods.py:151-152)
    float v = warp_sum(valid ? deep : 0.f);
    __shared__ float sh[kTile * kTile / 32];
    __syncthreads();  // sh reuse across the persistent loop
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0;
      for (int w = 0; w < kTile * kTile / 32; ++w) t += (double)sh[w];
      atomicAdd(&b.mean_acc[s * 2 + slot], t);
    }
  }
}

// Each block takes a contiguous chunk of the working-tile list: a stamp's tiles are
// consecutive there, so its evaluation constants are loaded once per run of tiles instead of
// once per tile, and the next list entry is fetched while a tile is sampled.
__device__ __forceinline__ void tile_chunk(uint32_t n, uint32_t& c0, uint32_t& c1) {
  const uint32_t per = (n + gridDim.x - 1) / gridDim.x;
  c0 = min(n, blockIdx.x * per);
  c1 = min(n, c0 + per);
}

template <bool EXT>
__global__ void __launch_bounds__(256) k_sample(BatchArgs b) {
  const uint32_t n = b.counters[7];
  uint32_t c0, c1;
  tile_chunk(n, c0, c1);
  int cur = -1, ops = 0;
  EvalF e{};
  DeltaF d{};
  int64_t next = (c0 < c1) ? b.wlist[c0] : 0;
  for (uint32_t it = c0; it < c1; ++it) {
    const int64_t ent = next;
    if (it + 1 < c1) next = b.wlist[it + 1];
    int slot, s, local;
    unpack_entry(ent, slot, s, local);
    if (s * 2 + slot != cur) {
      cur = s * 2 + slot;
      const EvalDev& ed = b.evals[cur];
      e = load_evalf(b.stamps[s], ed);
      ops = ed.ops;
      if (!EXT && (ops & OP_DIFF)) d = load_deltaf(ed);
    }
    if (ops & OP_JAC)
      sample_tile<true, EXT, false>(b, e, d, ops, s, slot, local);
    else if (!EXT && (ops & OP_DIFF))
      sample_tile<false, false, true>(b, e, d, ops, s, slot, local);
    else
      sample_tile<false, EXT, false>(b, e, d, ops, s, slot, local);
  }
}

// Column i and row j of working pixel p (the low 32-bit word of a queue entry) of a window
// wnx wide, by 32-bit unsigned division (the 64-bit one costs several times the instructions)
__device__ __forceinline__ void pix_ij(int64_t p, int wnx, int& i, int& j) {
  const uint32_t q = (uint32_t)p, w = (uint32_t)wnx;
  const uint32_t jj = q / w;
  j = (int)jj;
  i = (int)(q - jj * w);
}

// ---------------------------------------------------------------------------
// threshold selection (_sample_integrate) + enqueue
// ---------------------------------------------------------------------------
__device__ __forceinline__ void stamp_threshold(const BatchArgs& b, const StampDev& st,
                                                const EvalDev& e, int s, int slot, float& thr,
                                                double& thr64, float& thr_err) {
  // Sersic: closed-form flux (k_eval_setup); exponential: sum(deep) (k_exp_threshold).
  thr = e.thresh;
  thr64 = e.thresh64;
  // the exponential's mean comes from FP32 samples: uncertain at the 1e-6 level
  thr_err = (b.kind == AP_PROFILE_SERSIC) ? 2.f * kEps * thr : 2e-6f * thr;
}

// sum(deep) over a stamp's threshold window (gw_*) instead of its own working window: a source
// of a group is evaluated by the reference on the group's working window, whose samples its
// default _integrate_reference sums (models/_model_methods.py:151-152, model_object.py:290-296),
// while the render keeps to the source's own window.  Grid (2 n_stamps, row blocks); each
// thread sums a row's samples in FP32 (a handful) and the rows in FP64.
template <bool EXT>
__global__ void __launch_bounds__(256) k_window_msum(BatchArgs b) {
  const int t = blockIdx.x;
  if (t >= 2 * b.n_stamps) return;
  const EvalDev& ed = b.evals[t];
  if (!ed.ops) return;
  const int s = t >> 1;
  const StampDev& st = b.stamps[s];
  if (st.gw_nx <= 0) return;
  const EvalF e = load_evalf(st, ed);
  const DeltaF d{};
  double acc = 0.0;
  for (int r = blockIdx.y; r < st.gw_ny; r += gridDim.y) {
    float row = 0.f;
    for (int c = threadIdx.x; c < st.gw_nx; c += blockDim.x) {
      float deep, g[NGRAD], refsub, errb, dd;
      sample_pixel<false, EXT, false>(b, e, d, st.gw_x0 + c, st.gw_y0 + r, false, deep, g, refsub, errb, dd);
      row += deep;
    }
    acc += (double)row;
  }
  acc = warp_sum_d(acc);
  __shared__ double sh[8];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += sh[w];
    atomicAdd(&b.mean_acc[t], tot);
  }
}

// Exponential threshold: sampling_tolerance * sum(deep) / numel, once per (stamp, slot).
__global__ void k_exp_threshold(BatchArgs b) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= b.n_stamps * 2) return;
  EvalDev& e = b.evals[t];
  if (!e.ops) return;
  const StampDev& st = b.stamps[t >> 1];
  e.thresh64 = b.tolerance64 * (b.mean_acc[t] / st.thr_numel);
  e.thresh = (float)e.thresh64;
}

__device__ __forceinline__ void select_tile(const BatchArgs& b, int slot, int s, int local) {
  const EvalDev& e = b.evals[s * 2 + slot];
  const StampDev& st = b.stamps[s];
  const int i = (local % st.ntw_x) * kTile + (threadIdx.x & (kTile - 1));
  const int j = (local / st.ntw_x) * kTile + threadIdx.x / kTile;
  const bool valid = (i < st.wnx) && (j < st.wny);
  bool sel = false, redecided = false;
  int64_t p = 0;
  if (valid) {
    float thr, thr_err;
    double thr64;
    stamp_threshold(b, st, e, s, slot, thr, thr64, thr_err);
    const float* d = b.work + work_plane(b, slot, 0) + st.work_off;
    const float* aux = b.aux + (int64_t)slot * 2 * b.work_pixels + st.work_off;
    const float* eb = aux + b.work_pixels;
    p = (int64_t)j * st.wnx + i;
    const float deep = d[p];
    float err, bound;
    const bool stencil =
        (b.sampling == AP_SAMPLING_MIDPOINT || b.sampling == AP_SAMPLING_TRAPEZOID);
    int ic = 0, jc = 0;
    if (stencil) {
      // Laplacian 3x3 'valid' then replicate pad (models/_model_methods.py:87-98)
      ic = min(max(i, 1), st.wnx - 2);
      jc = min(max(j, 1), st.wny - 2);
      const int64_t c = (int64_t)jc * st.wnx + ic;
      const float u = d[c - st.wnx], l = d[c - 1], m = d[c], r = d[c + 1], dn = d[c + st.wnx];
      const float lap = u + l + (-4.f) * m + r + dn;
      const float refimg = deep + lap;
      err = fabsf(deep - refimg);
      const float mag = fabsf(u) + fabsf(l) + 4.f * fabsf(m) + fabsf(r) + fabsf(dn);
      bound = eb[c - st.wnx] + eb[c - 1] + 4.f * eb[c] + eb[c + 1] + eb[c + st.wnx] + eb[p] +
              8.f * kEps * mag + 4.f * kEps * (fabsf(deep) + fabsf(refimg));
    } else {
      const float ref = aux[p];
      err = fabsf(deep - ref);
      bound = eb[p] + 4.f * kEps * (fabsf(deep) + fabsf(ref));
    }
    bound = 1.5f * bound + thr_err;
    if (err > thr + bound) {
      sel = true;
    } else if (err >= thr - bound) {
      redecided = true;  // too close to call in FP32: k_recheck decides from float64 samples
    }
  }
  // warp-aggregated enqueue: one atomic per warp instead of one per pixel
  const int lane = threadIdx.x & 31;
  const int64_t entry = ((int64_t)slot << 62) | ((int64_t)s << 32) | (int64_t)p;
  const unsigned mask = __ballot_sync(0xffffffffu, sel);
  if (mask) {
    const int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(&b.counters[0], (unsigned)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (sel) {
      const uint32_t q = base + __popc(mask & ((1u << lane) - 1u));
      if ((int64_t)q < 2 * b.work_pixels)
        b.queue[q] = entry;
      else
        atomicOr(&b.counters[3], 1u);
    }
  }
  const unsigned rmask = __ballot_sync(0xffffffffu, redecided);
  if (rmask) {
    const int leader = __ffs(rmask) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(&b.counters[5], (unsigned)__popc(rmask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (redecided) {
      const uint32_t q = base + __popc(rmask & ((1u << lane) - 1u));
      if ((int64_t)q < 2 * b.work_pixels)
        b.recheck[q] = entry;
      else
        atomicOr(&b.counters[3], 2u);
    }
  }
}

__global__ void __launch_bounds__(256) k_select(BatchArgs b) {
  const uint32_t n = b.counters[7];
  uint32_t c0, c1;
  tile_chunk(n, c0, c1);
  int64_t next = (c0 < c1) ? b.wlist[c0] : 0;
  for (uint32_t it = c0; it < c1; ++it) {
    const int64_t ent = next;
    if (it + 1 < c1) next = b.wlist[it + 1];
    int slot, s, local;
    unpack_entry(ent, slot, s, local);
    select_tile(b, slot, s, local);
  }
}

// Selection of the pixels the FP32 bound could not settle, one pixel per thread in float64
// (the FP64 pipe retires whole-warp instructions, so the work is packed densely here).
template <bool EXT>
__global__ void __launch_bounds__(256) k_recheck(BatchArgs b) {
  const uint32_t n = min((uint32_t)b.counters[5], (uint32_t)(2 * b.work_pixels));
  const int lane = threadIdx.x & 31;
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
    const uint32_t idx = base + threadIdx.x;
    bool sel = false;
    int64_t ent = 0;
    if (idx < n) {
      ent = b.recheck[idx];
      const int slot = (int)(ent >> 62);
      const int s = (int)((ent >> 32) & 0x3fffffff);
      const int64_t p = ent & 0xffffffffll;
      const StampDev& st = b.stamps[s];
      const EvalDev& e = b.evals[s * 2 + slot];
      float thr, thr_err;
      double thr64;
      stamp_threshold(b, st, e, s, slot, thr, thr64, thr_err);
      int i, j;
      pix_ij(p, st.wnx, i, j);
      double err64;
      if (b.sampling == AP_SAMPLING_MIDPOINT || b.sampling == AP_SAMPLING_TRAPEZOID) {
        const int ic = min(max(i, 1), st.wnx - 2), jc = min(max(j, 1), st.wny - 2);
        const double m0 = sample_pixel64<EXT>(b, st, e, i, j, nullptr);
        const double u = sample_pixel64<EXT>(b, st, e, ic, jc - 1, nullptr);
        const double l = sample_pixel64<EXT>(b, st, e, ic - 1, jc, nullptr);
        const double m = (ic == i && jc == j) ? m0 : sample_pixel64<EXT>(b, st, e, ic, jc, nullptr);
        const double r = sample_pixel64<EXT>(b, st, e, ic + 1, jc, nullptr);
        const double dn = sample_pixel64<EXT>(b, st, e, ic, jc + 1, nullptr);
        const double lap = u + l + (-4.0) * m + r + dn;
        err64 = fabs(m0 - (m0 + lap));
      } else {
        double ref64 = 0;
        const double deep64 = sample_pixel64<EXT>(b, st, e, i, j, &ref64);
        err64 = fabs(deep64 - ref64);
      }
      sel = err64 > thr64;
    }
    const unsigned mask = __ballot_sync(0xffffffffu, sel);
    if (mask) {
      const int leader = __ffs(mask) - 1;
      uint32_t qb = 0;
      if (lane == leader) qb = atomicAdd(&b.counters[0], (unsigned)__popc(mask));
      qb = __shfl_sync(0xffffffffu, qb, leader);
      if (sel) {
        const uint32_t q = qb + __popc(mask & ((1u << lane) - 1u));
        if ((int64_t)q < 2 * b.work_pixels)
          b.queue[q] = ent;
        else
          atomicOr(&b.counters[3], 1u);
      }
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&b.counters[2], n);
}

// Sampling and threshold selection in one pass, for Sersic batches with a stencil sampling mode
// (midpoint / trapezoid), whose integration threshold (the closed-form flux) is known before
// sampling.  A 16 x 16 working tile samples its pixels as k_sample does (value, partials, the
// base / difference planes; not the reference sub-sample and error-bound planes, which only the
// selection reads) and, for the Laplacian stencil, the ring of pixels around it (value and FP32
// error bound only), into shared memory; it then decides its own pixels from there with
// select_tile's arithmetic and enqueue.  Every ring value is computed by the same sample
// functions as the pixel's own tile computes it, within the same FP32 error bound, and the
// decisions inside that bound are taken in float64 by k_recheck as before.
__device__ __forceinline__ void enqueue_selection(const BatchArgs& b, bool sel, bool redecided, int64_t entry) {
  const int lane = threadIdx.x & 31;
  const unsigned mask = __ballot_sync(0xffffffffu, sel);
  if (mask) {
    const int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(&b.counters[0], (unsigned)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (sel) {
      const uint32_t q = base + __popc(mask & ((1u << lane) - 1u));
      if ((int64_t)q < 2 * b.work_pixels)
        b.queue[q] = entry;
      else
        atomicOr(&b.counters[3], 1u);
    }
  }
  const unsigned rmask = __ballot_sync(0xffffffffu, redecided);
  if (rmask) {
    const int leader = __ffs(rmask) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(&b.counters[5], (unsigned)__popc(rmask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (redecided) {
      const uint32_t q = base + __popc(rmask & ((1u << lane) - 1u));
      if ((int64_t)q < 2 * b.work_pixels)
        b.recheck[q] = entry;
      else
        atomicOr(&b.counters[3], 2u);
    }
  }
}

template <bool JAC, bool DIFF>
__device__ __forceinline__ void sample_select_tile(const BatchArgs& b, const EvalF& e, const DeltaF& d, int ops,
                                                   int s, int slot, int tile_local, float (*sd)[kTile + 2],
                                                   float (*se)[kTile + 2]) {
  const StampDev& st = b.stamps[s];
  const int tx = threadIdx.x & (kTile - 1), ty = threadIdx.x / kTile;
  const int i0 = (tile_local % st.ntw_x) * kTile, j0 = (tile_local / st.ntw_x) * kTile;
  const int i = i0 + tx, j = j0 + ty;
  const bool valid = (i < st.wnx) && (j < st.wny);
  if (valid) {
    float deep, g[NGRAD], refsub, errb, ddeep;
    sample_pixel<JAC, false, DIFF>(b, e, d, i, j, false, deep, g, refsub, errb, ddeep);
    const int64_t p = st.work_off + (int64_t)j * st.wnx + i;
    b.work[work_plane(b, slot, 0) + p] = deep;
    if (JAC) {
#pragma unroll
      for (int q = 0; q < NGRAD; ++q) b.work[work_plane(b, slot, 1 + q) + p] = g[q];
    }
    if (ops & (OP_DIFF | OP_BASE)) write_diff_base(b, ops, slot, p, deep, ddeep, 0u);
    sd[ty + 1][tx + 1] = deep;
    se[ty + 1][tx + 1] = errb;
  }
  // the ring around the tile: rows lj = 0 and kTile + 1 (li = 0 .. kTile + 1), then columns
  // li = 0 and kTile + 1 (lj = 1 .. kTile); one point per thread
  if (threadIdx.x < 4 * kTile + 4) {
    const int r = threadIdx.x;
    int li, lj;
    if (r < kTile + 2) {
      li = r;
      lj = 0;
    } else if (r < 2 * (kTile + 2)) {
      li = r - (kTile + 2);
      lj = kTile + 1;
    } else if (r < 2 * (kTile + 2) + kTile) {
      li = 0;
      lj = 1 + r - 2 * (kTile + 2);
    } else {
      li = kTile + 1;
      lj = 1 + r - 2 * (kTile + 2) - kTile;
    }
    const int gi = i0 - 1 + li, gj = j0 - 1 + lj;
    if (gi >= 0 && gi < st.wnx && gj >= 0 && gj < st.wny) {
      float deep, g[NGRAD], refsub, errb, ddeep;
      sample_pixel<false, false, DIFF>(b, e, d, gi, gj, false, deep, g, refsub, errb, ddeep);
      sd[lj][li] = deep;
      se[lj][li] = errb;
    }
  }
  __syncthreads();
  bool sel = false, redecided = false;
  int64_t pp = 0;
  if (valid) {
    const EvalDev& ed = b.evals[s * 2 + slot];
    float thr, thr_err;
    double thr64;
    stamp_threshold(b, st, ed, s, slot, thr, thr64, thr_err);
    pp = (int64_t)j * st.wnx + i;
    const float deep = sd[ty + 1][tx + 1];
    // Laplacian 3x3 'valid' then replicate pad (models/_model_methods.py:87-98)
    const int ic = min(max(i, 1), st.wnx - 2), jc = min(max(j, 1), st.wny - 2);
    const int lc = ic - i0 + 1, lr = jc - j0 + 1;
    const float u = sd[lr - 1][lc], l = sd[lr][lc - 1], m = sd[lr][lc], r = sd[lr][lc + 1], dn = sd[lr + 1][lc];
    const float lap = u + l + (-4.f) * m + r + dn;
    const float refimg = deep + lap;
    const float err = fabsf(deep - refimg);
    const float mag = fabsf(u) + fabsf(l) + 4.f * fabsf(m) + fabsf(r) + fabsf(dn);
    float bound = se[lr - 1][lc] + se[lr][lc - 1] + 4.f * se[lr][lc] + se[lr][lc + 1] + se[lr + 1][lc] +
                  se[ty + 1][tx + 1] + 8.f * kEps * mag + 4.f * kEps * (fabsf(deep) + fabsf(refimg));
    bound = 1.5f * bound + thr_err;
    if (err > thr + bound) {
      sel = true;
    } else if (err >= thr - bound) {
      redecided = true;  // too close to call in FP32: k_recheck decides from float64 samples
    }
  }
  enqueue_selection(b, sel, redecided, ((int64_t)slot << 62) | ((int64_t)s << 32) | pp);
  // no barrier here: the caller alternates two sd / se buffers, and the next tile's barrier
  // (which every thread reaches only after its reads of this tile) orders them before the
  // writes of the tile after it into this buffer
}

__global__ void __launch_bounds__(256) k_sample_select(BatchArgs b) {
  __shared__ float sdb[2][kTile + 2][kTile + 2], seb[2][kTile + 2][kTile + 2];
  const uint32_t n = b.counters[7];
  uint32_t c0, c1;
  tile_chunk(n, c0, c1);
  int cur = -1, ops = 0;
  EvalF e{};
  DeltaF d{};
  int64_t next = (c0 < c1) ? b.wlist[c0] : 0;
  for (uint32_t it = c0; it < c1; ++it) {
    const int64_t ent = next;
    if (it + 1 < c1) next = b.wlist[it + 1];
    int slot, s, local;
    unpack_entry(ent, slot, s, local);
    if (s * 2 + slot != cur) {
      cur = s * 2 + slot;
      const EvalDev& ed = b.evals[cur];
      e = load_evalf(b.stamps[s], ed);
      ops = ed.ops;
      if (ops & OP_DIFF) d = load_deltaf(ed);
    }
    float(*sd)[kTile + 2] = sdb[(it - c0) & 1];
    float(*se)[kTile + 2] = seb[(it - c0) & 1];
    if (ops & OP_JAC)
      sample_select_tile<true, false>(b, e, d, ops, s, slot, local, sd, se);
    else if (ops & OP_DIFF)
      sample_select_tile<false, true>(b, e, d, ops, s, slot, local, sd, se);
    else
      sample_select_tile<false, false>(b, e, d, ops, s, slot, local, sd, se);
  }
}

// ---------------------------------------------------------------------------
// adaptive integration of the queued pixels (grid_integrate, max depth <= 3)
// ---------------------------------------------------------------------------
struct QuadResult {
  float res, ref, errb, mag;
  float dres;  // DIFF: difference of res to the base evaluation
  float g[NGRAD];
};

// One (sub-)pixel integrated by this lane alone: Q^2 samples at unit offsets
// (ci + qx / scale, cj + qy / scale) with amplitude scale area.  QC > 0 fixes the quadrature
// level at compile time (the sample loop unrolls into independent evaluations).
template <bool JAC, int QC, bool EXT, bool DIFF>
__device__ __forceinline__ QuadResult quad_lane(const BatchArgs& b, const EvalF& e, const DeltaF& d, float ci,
                                                float cj, float inv_g, float area) {
  const QuadTables& T = *b.tables;
  const int n = QC > 0 ? QC * QC : T.quad_level * T.quad_level;
  const int mid = n / 2;
  QuadResult r;
  r.res = 0.f;
  r.dres = 0.f;
  r.ref = 0.f;
  r.errb = 0.f;
  r.mag = 0.f;
#pragma unroll
  for (int q = 0; q < NGRAD; ++q) r.g[q] = 0.f;
  float referr = 0.f;
#pragma unroll
  for (int k = 0; k < (QC > 0 ? QC * QC : kMaxQuad * kMaxQuad); ++k) {
    if (QC == 0 && k >= n) break;
    float X, Y;
    pix_to_offset(e, ci + T.qxf[k] * inv_g, cj + T.qyf[k] * inv_g, X, Y);
    float dI = 0.f;
    const Sample sm = DIFF ? eval_profile_delta(e, d, b.kind, X, Y, area, dI) : eval_profile<JAC, EXT>(e, b.kind, X, Y, area);
    const float w = T.qwf[k];
    r.res = fmaf(w, sm.v, r.res);
    if (DIFF) r.dres = fmaf(w, dI, r.dres);
    if (JAC) {
#pragma unroll
      for (int q = 0; q < NGRAD; ++q) r.g[q] = fmaf(w, sm.g[q], r.g[q]);
    }
    const float a = fabsf(w * sm.v);
    r.mag += a;
    r.errb += a * sample_rel_err(e, sm.arg);
    if (k == mid) {
      r.ref = sm.v;
      referr = fabsf(sm.v) * sample_rel_err(e, sm.arg);
    }
  }
  r.errb += referr + 2.f * n * kEps * (r.mag + fabsf(r.ref));
  return r;
}

// float64 re-evaluation of one (sub-)pixel's quadrature: pixel (i, j) of the working grid,
// sub-pixel m of the displacement grid (m < 0: the pixel itself).
template <bool EXT>
__device__ bool refine64(const BatchArgs& b, const StampDev& st, const EvalDev& e, int i, int j,
                         int m, double thr64) {
  const QuadTables& T = *b.tables;
  const int n = T.quad_level * T.quad_level;
  double ci = (double)(i - e.cix), cj = (double)(j - e.cjy);
  double inv_g = 1.0, area = 1.0;
  if (m >= 0) {
    ci += T.gx[m];
    cj += T.gy[m];
    inv_g = 1.0 / (double)T.gridding;
    area = inv_g * inv_g;
  }
  double res = 0, ref = 0;
  for (int k = 0; k < n; ++k) {
    double X, Y;
    pix_to_offset64(st, e, ci + T.qx[k] * inv_g, cj + T.qy[k] * inv_g, X, Y);
    const double f = eval_profile64<EXT>(e, b.kind, X, Y, area);
    res += f * T.qw[k];
    if (k == n / 2) ref = f;
  }
  return fabs(res - ref) > thr64;
}

// Level-2 refinement decision of sub-pixel m: FP32 when clear of the error band, else
// float64 (threshold scaled by gridding^2 as the reference passes it down).
template <bool EXT>
__device__ __forceinline__ bool decide(const BatchArgs& b, const StampDev& st, const EvalDev& e,
                                       const QuadResult& r, float thr, int i, int j, int m,
                                       int& n64) {
  const float diff = fabsf(r.res - r.ref);
  const float band = 1.5f * r.errb + 4.f * kEps * thr;
  if (diff > thr + band) return true;
  if (diff < thr - band) return false;
  ++n64;
  const int g = b.tables->gridding;
  return refine64<EXT>(b, st, e, i, j, m, e.thresh64 * (double)(g * g));
}

__device__ __forceinline__ void write_deep(const BatchArgs& b, const StampDev& st, int slot,
                                           int64_t p, float v, const float* g, bool jac) {
  const int64_t wp = st.work_off + p;
  b.work[work_plane(b, slot, 0) + wp] = v;
  if (jac) {
#pragma unroll
    for (int q = 0; q < NGRAD; ++q) b.work[work_plane(b, slot, 1 + q) + wp] = g[q];
  }
}

// Level 1 of grid_integrate, one queued pixel per thread: the Q x Q Gauss-Legendre
// integral and its refinement decision.  Pixels that stop here are written; the others go
// to the level-2 queue (b.recheck, emptied by k_recheck before this kernel runs).
template <int QC, bool EXT>
__device__ __forceinline__ void level1_pixel(const BatchArgs& b, int64_t ent, bool& push, bool& amb,
                                             int& n64) {
  const int slot = (int)(ent >> 62);
  const int s = (int)((ent >> 32) & 0x3fffffff);
  const int64_t p = ent & 0xffffffffll;
  const StampDev& st = b.stamps[s];
  const EvalDev& e = b.evals[s * 2 + slot];
  const EvalF f = load_evalf(st, e);
  int i, j;
  pix_ij(p, st.wnx, i, j);
  const float di = (float)(i - f.cix), dj = (float)(j - f.cjy);
  const int ops = e.ops;
  const bool jac = (ops & OP_JAC) != 0;
  DeltaF d{};
  QuadResult r;
  if (jac) {
    r = quad_lane<true, QC, EXT, false>(b, f, d, di, dj, 1.f, 1.f);
  } else if (!EXT && (ops & OP_DIFF)) {
    d = load_deltaf(e);
    r = quad_lane<false, QC, false, true>(b, f, d, di, dj, 1.f, 1.f);
  } else {
    r = quad_lane<false, QC, EXT, false>(b, f, d, di, dj, 1.f, 1.f);
  }
  bool split = false;
  if (b.max_depth > 1) {
    const float thr = e.thresh;
    const float diff = fabsf(r.res - r.ref);
    const float band = 1.5f * r.errb + 4.f * kEps * thr;
    split = diff > thr + band;
    // inside the FP32 error band: the float64 decision is taken by k_level1_amb, densely
    // (one pixel per lane), after this pixel's FP32 value is written; a split there
    // overwrites it
    if (!split && diff >= thr - band) amb = true;
  }
  if (split) {
    push = true;
  } else {
    write_deep(b, st, slot, p, r.res, r.g, jac);
    if (ops & (OP_DIFF | OP_BASE)) write_diff_base(b, ops, slot, st.work_off + p, r.res, r.dres, kCodeLevel1);
  }
}

// warp-aggregated append of flagged entries to a list (counter, capacity); returns false for
// the lanes whose entry did not fit
__device__ __forceinline__ bool warp_append(bool flag, int64_t ent, int64_t* list, uint32_t* counter,
                                            int64_t cap) {
  const int lane = threadIdx.x & 31;
  const unsigned mask = __ballot_sync(0xffffffffu, flag);
  if (!mask) return true;
  const int leader = __ffs(mask) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(counter, (unsigned)__popc(mask));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (!flag) return true;
  const int64_t k = (int64_t)base + __popc(mask & ((1u << lane) - 1u));
  if (k >= cap) return false;
  list[k] = ent;
  return true;
}

// Level-2 lists: pixels of Jacobian evaluations fill the recheck buffer from the front,
// pixels of forward (plain or difference) evaluations from the back, so each kind gets its
// own integration kernel (compiled, and given registers, for that kind alone).  Together they
// hold at most one entry per working pixel of each slot: the buffer's 2 * work_pixels.
__device__ __forceinline__ void level2_append(const BatchArgs& b, bool push, int64_t ent) {
  bool jac = false;
  if (push) {
    const int slot = (int)(ent >> 62);
    const int s = (int)((ent >> 32) & 0x3fffffff);
    jac = (b.evals[s * 2 + slot].ops & OP_JAC) != 0;
  }
  const int64_t cap = (int64_t)2 * b.work_pixels;
  const int lane = threadIdx.x & 31;
  const unsigned mj = __ballot_sync(0xffffffffu, push && jac);
  const unsigned mf = __ballot_sync(0xffffffffu, push && !jac);
  uint32_t bj = 0, bf = 0;
  if (lane == 0) {
    if (mj) bj = atomicAdd(&b.counters[10], (unsigned)__popc(mj));
    if (mf) bf = atomicAdd(&b.counters[13], (unsigned)__popc(mf));
  }
  bj = __shfl_sync(0xffffffffu, bj, 0);
  bf = __shfl_sync(0xffffffffu, bf, 0);
  if (!push) return;
  const unsigned below = (1u << lane) - 1u;
  if (jac) {
    const int64_t k = (int64_t)bj + __popc(mj & below);
    if (k < cap) b.recheck[k] = ent;
    else atomicOr(&b.counters[3], 4u);
  } else {
    const int64_t k = (int64_t)bf + __popc(mf & below);
    if (k < cap) b.recheck[cap - 1 - k] = ent;
    else atomicOr(&b.counters[3], 4u);
  }
}

template <bool EXT>
__global__ void __launch_bounds__(256, 3) k_level1(BatchArgs b) {
  const uint32_t n = min((uint32_t)b.counters[0], (uint32_t)(2 * b.work_pixels));
  const int Q = b.tables->quad_level;
  int n64 = 0;
  unsigned long long n_all = 0, n_diff = 0, n_jac = 0;  // samples by kind of evaluation
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
    const uint32_t idx = base + threadIdx.x;
    bool push = false, amb = false;
    int64_t ent = 0;
    if (idx < n) {
      ent = b.queue[idx];
      const int ops = b.evals[((ent >> 32) & 0x3fffffff) * 2 + (int)(ent >> 62)].ops;
      n_all += Q * Q;
      if (ops & OP_JAC) n_jac += Q * Q;
      else if (ops & OP_DIFF) n_diff += Q * Q;
      if (Q == 3)
        level1_pixel<3, EXT>(b, ent, push, amb, n64);
      else
        level1_pixel<0, EXT>(b, ent, push, amb, n64);
    }
    if (!warp_append(amb, ent, b.amb, &b.counters[12], b.amb_cap)) {
      // the dense list is full: decide here
      const int slot = (int)(ent >> 62);
      const int s = (int)((ent >> 32) & 0x3fffffff);
      const int64_t p = ent & 0xffffffffll;
      const StampDev& st = b.stamps[s];
      ++n64;
      int pi, pj;
      pix_ij(p, st.wnx, pi, pj);
      push = refine64<EXT>(b, st, b.evals[s * 2 + slot], pi, pj, -1,
                      b.evals[s * 2 + slot].thresh64);
    }
    level2_append(b, push, ent);
  }
  n64 = __reduce_add_sync(0xffffffffu, n64);
  if ((threadIdx.x & 31) == 0 && n64) atomicAdd(&b.counters[6], (unsigned)n64);
  for (int o = 16; o > 0; o >>= 1) {
    n_all += __shfl_xor_sync(0xffffffffu, n_all, o);
    n_diff += __shfl_xor_sync(0xffffffffu, n_diff, o);
    n_jac += __shfl_xor_sync(0xffffffffu, n_jac, o);
  }
  if ((threadIdx.x & 31) == 0 && n_all) {
    atomicAdd(b.work_ctr + 1, n_all);
    if (n_diff) atomicAdd(b.work_ctr + 3, n_diff);
    if (n_jac) atomicAdd(b.work_ctr + 4, n_jac);
  }
}

// float64 split decisions of the level-1 pixels inside the FP32 error band, one per lane
// (all lanes of a warp busy: the FP64 pipe is narrow); splits join the level-2 queue.
template <bool EXT>
__global__ void __launch_bounds__(256) k_level1_amb(BatchArgs b) {
  const int64_t n = min((int64_t)b.counters[12], b.amb_cap);
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t idx = base + threadIdx.x;
    bool push = false;
    int64_t ent = 0;
    if (idx < n) {
      ent = b.amb[idx];
      const int slot = (int)(ent >> 62);
      const int s = (int)((ent >> 32) & 0x3fffffff);
      const int64_t p = ent & 0xffffffffll;
      const StampDev& st = b.stamps[s];
      const EvalDev& e = b.evals[s * 2 + slot];
      int pi, pj;
      pix_ij(p, st.wnx, pi, pj);
      push = refine64<EXT>(b, st, e, pi, pj, -1, e.thresh64);
    }
    level2_append(b, push, ent);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && n > 0) atomicAdd(&b.counters[6], (unsigned)n);
}

// Levels 2 and 3 of grid_integrate for a pixel that level 1 split: one warp per pixel,
// one sub-pixel per lane; each level-2 sub-pixel flagged for refinement is split again and
// integrated by the whole warp.
template <bool JAC, int QC, bool EXT, bool DIFF>
__device__ void level23_pixel(const BatchArgs& b, int slot, int s, int64_t p, int lane,
                              unsigned long long& samples, int& n64) {
  const StampDev& st = b.stamps[s];
  const EvalDev& e = b.evals[s * 2 + slot];
  const QuadTables& T = *b.tables;
  const int Q2 = QC > 0 ? QC * QC : T.quad_level * T.quad_level;
  const int g = T.gridding, G2 = g * g;
  const EvalF f = load_evalf(st, e);
  DeltaF d{};
  if (DIFF) d = load_deltaf(e);
  int i, j;
  pix_ij(p, st.wnx, i, j);
  const float di = (float)(i - f.cix), dj = (float)(j - f.cjy);
  const float thr = e.thresh;
  const float ginv = 1.f / (float)g;
  const float area2 = ginv * ginv;
  int n_samples = G2 * Q2;
  QuadResult r2;
  r2.res = 0.f;
  r2.dres = 0.f;
#pragma unroll
  for (int q = 0; q < NGRAD; ++q) r2.g[q] = 0.f;
  float ci2 = 0.f, cj2 = 0.f;
  bool split2 = false;
  if (lane < G2) {
    ci2 = di + T.gxf[lane];
    cj2 = dj + T.gyf[lane];
    r2 = quad_lane<JAC, QC, EXT, DIFF>(b, f, d, ci2, cj2, ginv, area2);
    if (b.max_depth > 2) split2 = decide<EXT>(b, st, e, r2, thr * (float)G2, i, j, lane, n64);
  }
  // level 3: refine each flagged sub-pixel with the whole warp
  unsigned todo = __ballot_sync(0xffffffffu, split2);
  const uint32_t code = code_split(todo);
  n_samples += __popc(todo) * G2 * Q2;
  const float area3 = area2 * area2;
  while (todo) {
    const int m = __ffs(todo) - 1;
    todo &= todo - 1;
    const float cim = __shfl_sync(0xffffffffu, ci2, m);
    const float cjm = __shfl_sync(0xffffffffu, cj2, m);
    QuadResult r3;
    r3.res = 0.f;
    r3.dres = 0.f;
#pragma unroll
    for (int q = 0; q < NGRAD; ++q) r3.g[q] = 0.f;
    if (lane < G2) {
      r3 = quad_lane<JAC, QC, EXT, DIFF>(b, f, d, cim + T.gxf[lane] * ginv, cjm + T.gyf[lane] * ginv,
                                         ginv * ginv, area3);
    }
    const float s3 = warp_sum(r3.res);
    const float ds3 = DIFF ? warp_sum(r3.dres) : 0.f;
    float gs3[NGRAD];
    if (JAC) {
#pragma unroll
      for (int q = 0; q < NGRAD; ++q) gs3[q] = warp_sum(r3.g[q]);
    }
    if (lane == m) {
      r2.res = s3;
      r2.dres = ds3;
      if (JAC) {
#pragma unroll
        for (int q = 0; q < NGRAD; ++q) r2.g[q] = gs3[q];
      }
    }
  }
  const float out_v = warp_sum(lane < G2 ? r2.res : 0.f);
  float out_g[NGRAD];
#pragma unroll
  for (int q = 0; q < NGRAD; ++q) out_g[q] = JAC ? warp_sum(lane < G2 ? r2.g[q] : 0.f) : 0.f;
  const float out_d = DIFF ? warp_sum(lane < G2 ? r2.dres : 0.f) : 0.f;
  samples += (unsigned long long)n_samples;
  if (lane == 0) {
    write_deep(b, st, slot, p, out_v, out_g, JAC);
    if (e.ops & (OP_DIFF | OP_BASE)) write_diff_base(b, e.ops, slot, st.work_off + p, out_v, out_d, code);
  }
}

// Levels 2 and 3 of grid_integrate for forward evaluations (plain or difference to the base),
// packed: a warp takes kPack queued pixels and spreads their G2 = gridding^2 level-2 sub-pixels
// (and then the G2 level-3 sub-pixels of every sub-pixel flagged for refinement) over all 32
// lanes, one sub-pixel's quadrature per lane, instead of one pixel per warp with G2 of 32 lanes
// busy.  Each sub-pixel's result goes to shared memory and is summed per pixel in sub-pixel
// order by one lane, so a pixel's value does not depend on which pixels share its warp.
constexpr int kPack = 16;
constexpr int kPackWarps = 4;  // 128-thread blocks

struct PackSmem {
  int64_t ent[kPack];
  uint32_t mask[kPack];   // level-3 flags of each pixel's sub-pixels
  int32_t pre[kPack + 1]; // exclusive prefix of the flag counts
  // per pixel, loaded once by its lane: evaluation constants, differences to the base, working
  // pixel (i, j) relative to the centre pixel, threshold, difference evaluation or not
  EvalF ef[kPack];
  DeltaF df[kPack];
  float di[kPack], dj[kPack], thr[kPack];
  int32_t pi[kPack], pj[kPack], isdiff[kPack];
  float res[kPack * kMaxGrid * kMaxGrid], dres[kPack * kMaxGrid * kMaxGrid];
  float res3[kPack * kMaxGrid * kMaxGrid], dres3[kPack * kMaxGrid * kMaxGrid];
};

// one level-2 or level-3 sub-pixel of queued pixel P of the warp's batch (sub-pixel m, and
// sub-sub-pixel k >= 0 at level 3): its quadrature, plain or as a difference, from the pixel's
// constants staged in shared memory
template <int QC>
__device__ __forceinline__ QuadResult packed_quad(const BatchArgs& b, const PackSmem& S, int P, int m, int k) {
  const QuadTables& T = *b.tables;
  const EvalF f = S.ef[P];
  const float ginv = 1.f / (float)T.gridding;
  float ci = S.di[P] + T.gxf[m], cj = S.dj[P] + T.gyf[m];
  float ig = ginv, area = ginv * ginv;
  if (k >= 0) {
    ci += T.gxf[k] * ginv;
    cj += T.gyf[k] * ginv;
    ig = ginv * ginv;
    area = area * area;
  }
  if (S.isdiff[P]) {
    const DeltaF d = S.df[P];
    return quad_lane<false, QC, false, true>(b, f, d, ci, cj, ig, area);
  }
  const DeltaF d{};
  return quad_lane<false, QC, false, false>(b, f, d, ci, cj, ig, area);
}

// the batch's pixels: each lane P < np stages its pixel's constants
__device__ __forceinline__ void packed_stage(const BatchArgs& b, PackSmem& S, int np, int lane) {
  if (lane < np) {
    const int64_t ent = S.ent[lane];
    const int slot = (int)(ent >> 62);
    const int s = (int)((ent >> 32) & 0x3fffffff);
    const StampDev& st = b.stamps[s];
    const EvalDev& e = b.evals[s * 2 + slot];
    const EvalF f = load_evalf(st, e);
    S.ef[lane] = f;
    const bool diff = (e.ops & OP_DIFF) != 0;
    S.isdiff[lane] = diff ? 1 : 0;
    if (diff) S.df[lane] = load_deltaf(e);
    int i, j;
    pix_ij(ent & 0xffffffffll, st.wnx, i, j);
    S.pi[lane] = i;
    S.pj[lane] = j;
    S.di[lane] = (float)(i - f.cix);
    S.dj[lane] = (float)(j - f.cjy);
    S.thr[lane] = e.thresh;
  }
  __syncwarp();
}

template <int QC>
__device__ void level23_packed(const BatchArgs& b, PackSmem& S, int np, int lane, unsigned long long& samples,
                               unsigned long long& diff_samples, int& n64) {
  const QuadTables& T = *b.tables;
  const int G2 = T.gridding * T.gridding;
  const int Q2 = QC > 0 ? QC * QC : T.quad_level * T.quad_level;
  if (lane < kPack) S.mask[lane] = 0u;
  packed_stage(b, S, np, lane);
  // level 2: np * G2 sub-pixels over the lanes
  const int items = np * G2;
  for (int base = 0; base < items; base += 32) {
    const int it = base + lane;
    if (it < items) {
      const int P = it / G2, m = it - P * G2;
      const QuadResult r = packed_quad<QC>(b, S, P, m, -1);
      if (S.isdiff[P]) diff_samples += Q2;
      S.res[it] = r.res;
      S.dres[it] = r.dres;
      if (b.max_depth > 2) {
        const int64_t ent = S.ent[P];
        const int slot = (int)(ent >> 62), s = (int)((ent >> 32) & 0x3fffffff);
        if (decide<false>(b, b.stamps[s], b.evals[s * 2 + slot], r, S.thr[P] * (float)G2, S.pi[P], S.pj[P], m, n64))
          atomicOr(&S.mask[P], 1u << m);
      }
    }
  }
  __syncwarp();
  // flagged sub-pixels, enumerated pixel by pixel in sub-pixel order
  const int cnt = lane < np ? __popc(S.mask[lane]) : 0;
  int pre = cnt;
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, pre, o);
    if (lane >= o) pre += v;
  }
  const int total = __shfl_sync(0xffffffffu, pre, 31);
  if (lane < np) S.pre[lane] = pre - cnt;
  if (lane == 0) S.pre[np] = total;
  __syncwarp();
  samples += (unsigned long long)(items + total * G2) * (unsigned long long)Q2;
  auto flagged = [&](int fi, int& P, int& m) {
    P = 0;
    while (P + 1 < np && S.pre[P + 1] <= fi) ++P;
    unsigned msk = S.mask[P];
    for (int r = fi - S.pre[P]; r > 0; --r) msk &= msk - 1u;
    m = __ffs(msk) - 1;
  };
  // level 3 in batches of kPack flagged sub-pixels, G2 sub-sub-pixels each over the lanes
  for (int f0 = 0; f0 < total; f0 += kPack) {
    const int nf = min(kPack, total - f0);
    const int tasks = nf * G2;
    for (int base = 0; base < tasks; base += 32) {
      const int it = base + lane;
      if (it < tasks) {
        const int q = it / G2, k = it - q * G2;
        int P, m;
        flagged(f0 + q, P, m);
        const QuadResult r = packed_quad<QC>(b, S, P, m, k);
        if (S.isdiff[P]) diff_samples += Q2;
        S.res3[it] = r.res;
        S.dres3[it] = r.dres;
      }
    }
    __syncwarp();
    if (lane < nf) {
      int P, m;
      flagged(f0 + lane, P, m);
      float v = 0.f, dv = 0.f;
      for (int k = 0; k < G2; ++k) {
        v += S.res3[lane * G2 + k];
        dv += S.dres3[lane * G2 + k];
      }
      S.res[P * G2 + m] = v;
      S.dres[P * G2 + m] = dv;
    }
    __syncwarp();
  }
  // each pixel: its sub-pixels summed in order
  if (lane < np) {
    float v = 0.f, dv = 0.f;
    for (int m = 0; m < G2; ++m) {
      v += S.res[lane * G2 + m];
      dv += S.dres[lane * G2 + m];
    }
    const int64_t ent = S.ent[lane];
    const int slot = (int)(ent >> 62);
    const int s = (int)((ent >> 32) & 0x3fffffff);
    const int64_t p = ent & 0xffffffffll;
    const StampDev& st = b.stamps[s];
    const int ops = b.evals[s * 2 + slot].ops;
    write_deep(b, st, slot, p, v, nullptr, false);
    if (ops & (OP_DIFF | OP_BASE)) write_diff_base(b, ops, slot, st.work_off + p, v, dv, code_split(S.mask[lane]));
  }
  __syncwarp();
}

__global__ void __launch_bounds__(kPackWarps * 32, 6) k_integrate_packed(BatchArgs b) {
  __shared__ PackSmem smem[kPackWarps];
  const int lane = threadIdx.x & 31;
  PackSmem& S = smem[threadIdx.x >> 5];
  const int64_t cap = (int64_t)2 * b.work_pixels;
  const uint32_t n = min((uint32_t)b.counters[13], (uint32_t)cap);
  unsigned long long samples = 0, diff_samples = 0;
  int n64 = 0;
  while (true) {
    uint32_t idx0 = 0;
    if (lane == 0) idx0 = atomicAdd(&b.counters[14], (unsigned)kPack);
    idx0 = __shfl_sync(0xffffffffu, idx0, 0);
    if (idx0 >= n) break;
    const int np = (int)min((uint32_t)kPack, n - idx0);
    if (lane < np) S.ent[lane] = b.recheck[cap - 1 - (idx0 + lane)];
    __syncwarp();
    if (b.tables->quad_level == 3)
      level23_packed<3>(b, S, np, lane, samples, diff_samples, n64);
    else
      level23_packed<0>(b, S, np, lane, samples, diff_samples, n64);
  }
  n64 = __reduce_add_sync(0xffffffffu, n64);
  samples = __shfl_sync(0xffffffffu, samples, 0);
  for (int o = 16; o > 0; o >>= 1) diff_samples += __shfl_xor_sync(0xffffffffu, diff_samples, o);
  if (lane == 0) {
    if (samples) atomicAdd(b.work_ctr + 1, samples);
    if (diff_samples) atomicAdd(b.work_ctr + 3, diff_samples);
    if (n64) atomicAdd(&b.counters[6], (unsigned)n64);
  }
}

// FWD = false: the Jacobian evaluations' pixels (front of the recheck buffer); FWD = true: the
// forward evaluations' pixels (back of the buffer), plain or as differences to the base
template <bool EXT, bool FWD>
__global__ void __launch_bounds__(256, 3) k_integrate(BatchArgs b) {
  const int lane = threadIdx.x & 31;
  constexpr uint32_t kChunk = 2;  // queue entries grabbed per atomic
  const int64_t cap = (int64_t)2 * b.work_pixels;
  const uint32_t n = min((uint32_t)b.counters[FWD ? 13 : 10], (uint32_t)cap);
  const int Q = b.tables->quad_level;
  unsigned long long samples = 0;
  int n64 = 0;
  while (true) {
    uint32_t idx0 = 0;
    if (lane == 0) idx0 = atomicAdd(&b.counters[FWD ? 14 : 1], kChunk);
    idx0 = __shfl_sync(0xffffffffu, idx0, 0);
    if (idx0 >= n) break;
    const uint32_t idx1 = min(idx0 + kChunk, n);
    for (uint32_t idx = idx0; idx < idx1; ++idx) {
      const int64_t ent = FWD ? b.recheck[cap - 1 - idx] : b.recheck[idx];
      const int slot = (int)(ent >> 62);
      const int s = (int)((ent >> 32) & 0x3fffffff);
      const int64_t p = ent & 0xffffffffll;
      if (!FWD) {
        if (Q == 3)
          level23_pixel<true, 3, EXT, false>(b, slot, s, p, lane, samples, n64);
        else
          level23_pixel<true, 0, EXT, false>(b, slot, s, p, lane, samples, n64);
      } else {
        const bool diff = !EXT && (b.evals[s * 2 + slot].ops & OP_DIFF);
        if (Q == 3) {
          if (diff)
            level23_pixel<false, 3, false, true>(b, slot, s, p, lane, samples, n64);
          else
            level23_pixel<false, 3, EXT, false>(b, slot, s, p, lane, samples, n64);
        } else {
          if (diff)
            level23_pixel<false, 0, false, true>(b, slot, s, p, lane, samples, n64);
          else
            level23_pixel<false, 0, EXT, false>(b, slot, s, p, lane, samples, n64);
        }
      }
    }
  }
  // per-warp totals: the sample count is warp-uniform, the FP64 re-decisions are per lane
  n64 = __reduce_add_sync(0xffffffffu, n64);
  if (lane == 0) {
    if (samples) atomicAdd(b.work_ctr + 1, samples);
    if (samples && !FWD) atomicAdd(b.work_ctr + 4, samples);
    if (n64) atomicAdd(&b.counters[6], (unsigned)n64);
  }
}

// ---------------------------------------------------------------------------
// convolution + crop + fused accumulation
// ---------------------------------------------------------------------------
constexpr int kConvWarps = kConvThreads / 32;

// Block sums of nvals per-thread values (FP32 within a warp, FP64 across warps) -> dst.
__device__ __forceinline__ void conv_tile_reduce(const float* vals, int nvals, double* dst,
                                                 float* sh) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int k = 0; k < nvals; ++k) {
    const float v = warp_sum(vals[k]);
    if (lane == 0) sh[warp * kNacc + k] = v;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < nvals; k += blockDim.x) {
    double t = 0;
#pragma unroll
    for (int w = 0; w < kConvWarps; ++w) t += (double)sh[w * kNacc + k];
    dst[k] = t;
  }
}

// One column x R rows of a KP x KP convolution, register blocked: for each kernel
// column u the kernel column (float4 loads of the transposed kernel) and the input column
// window live in registers.  out[o] = sum_{v,u} K[v][u] T[ty0 + o + KP-1 - v][tx + KP-1 - u],
// with KT[u * stride + v] = K[v][u].
template <int KP, int R>
__device__ __forceinline__ void conv_col_fixed(const float* __restrict__ Tt, int TP,
                                               const float* __restrict__ KT, int tx, int ty0,
                                               float* out) {
  constexpr int C2 = KP - 1;
  constexpr int NT = R + KP - 1;
  constexpr int KS = (KP + 3) & ~3;
  constexpr int NT4 = (NT + 3) / 4;
  float acc[R];
#pragma unroll
  for (int o = 0; o < R; ++o) acc[o] = 0.f;
  // column-major tile (pitch TP): a thread's input column is contiguous, read as float4
  const float* base = Tt + (tx + C2) * TP + ty0;
#pragma unroll 1
  for (int u = 0; u < KP; ++u) {
    float kc[KS];
    const float4* kcol = reinterpret_cast<const float4*>(KT + u * KS);
#pragma unroll
    for (int q = 0; q < KS / 4; ++q) {
      const float4 k4 = kcol[q];
      kc[4 * q + 0] = k4.x;
      kc[4 * q + 1] = k4.y;
      kc[4 * q + 2] = k4.z;
      kc[4 * q + 3] = k4.w;
    }
    float t[4 * NT4];
    const float4* col = reinterpret_cast<const float4*>(base - u * TP);
#pragma unroll
    for (int q = 0; q < NT4; ++q) {
      const float4 c4 = col[q];
      t[4 * q + 0] = c4.x;
      t[4 * q + 1] = c4.y;
      t[4 * q + 2] = c4.z;
      t[4 * q + 3] = c4.w;
    }
#pragma unroll
    for (int v = 0; v < KP; ++v)
#pragma unroll
      for (int o = 0; o < R; ++o) acc[o] = fmaf(kc[v], t[o + C2 - v], acc[o]);
  }
#pragma unroll
  for (int o = 0; o < R; ++o) out[o] = acc[o];
}

template <int R>
__device__ __forceinline__ void conv_col_generic(const float* __restrict__ Tt, int TP,
                                                 const float* __restrict__ KT, int kpx, int kpy,
                                                 int tx, int ty0, float* out) {
  float acc[R];
#pragma unroll
  for (int o = 0; o < R; ++o) acc[o] = 0.f;
  const int ks = conv_col_stride(kpy);
  for (int u = 0; u < kpx; ++u) {
    const float* kcol = KT + u * ks;
    const float* tcol = Tt + (tx + kpx - 1 - u) * TP + ty0;
    for (int v = 0; v < kpy; ++v) {
      const float k = kcol[v];
      const float* tp = tcol + (kpy - 1 - v);
#pragma unroll
      for (int o = 0; o < R; ++o) acc[o] = fmaf(k, tp[o], acc[o]);
    }
  }
#pragma unroll
  for (int o = 0; o < R; ++o) out[o] = acc[o];
}

// Kernels the fixed instances do not cover (kpy >= 8): each kernel column in chunks of 8 rows,
// the chunk (two float4 loads) and the input window it meets (four float4 loads) in registers,
// 32 FMAs per chunk.  With lo = kpy - 1 - v0 - 7 the first input row of chunk v0, lo mod 4 =
// kpy mod 4 = SH, so the window (kWin floats) is read from the 16-byte aligned row lo - SH
// (the tile pitch and ty0 are multiples of 4).  It may reach up to 10 floats before the column
// (inside the kernels stored ahead of the tile: 3 kpx ks >= 24 floats) and 3 past the last
// column (the allocation is padded by kConvSmemPad floats); rows of the chunk at or beyond kpy
// are skipped.
template <int SH, int R>
__device__ __forceinline__ void conv_col_chunked(const float* __restrict__ Tt, int TP, const float* __restrict__ KT,
                                                 int kpx, int kpy, int tx, int ty0, float* out) {
  float acc[R];
#pragma unroll
  for (int o = 0; o < R; ++o) acc[o] = 0.f;
  const int ks = conv_col_stride(kpy);
  for (int u = 0; u < kpx; ++u) {
    const float* kcol = KT + u * ks;
    const float* tcol = Tt + (tx + kpx - 1 - u) * TP + ty0;
    for (int v0 = 0; v0 < kpy; v0 += 8) {
      float kc[8];
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const float4 k4 = *reinterpret_cast<const float4*>(kcol + v0 + 4 * q);
        kc[4 * q + 0] = k4.x;
        kc[4 * q + 1] = k4.y;
        kc[4 * q + 2] = k4.z;
        kc[4 * q + 3] = k4.w;
      }
      const float4* w4 = reinterpret_cast<const float4*>(tcol + (kpy - 8 - v0) - SH);
      constexpr int kWin = (R + 10 + 3) / 4 * 4;  // window rows SH .. SH + 7 + R - 1
      float t[kWin];
#pragma unroll
      for (int q = 0; q < kWin / 4; ++q) {
        const float4 c4 = w4[q];
        t[4 * q + 0] = c4.x;
        t[4 * q + 1] = c4.y;
        t[4 * q + 2] = c4.z;
        t[4 * q + 3] = c4.w;
      }
      const int nv = min(8, kpy - v0);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        if (j < nv) {
#pragma unroll
          for (int o = 0; o < R; ++o) acc[o] = fmaf(kc[j], t[SH + 7 - j + o], acc[o]);
        }
      }
    }
  }
#pragma unroll
  for (int o = 0; o < R; ++o) out[o] = acc[o];
}

// One copy of the kernel-size instances per k_conv flavour, shared by its k_conv<NF, LARGE>
// instantiations.  LARGE = false: the register-blocked square sizes 3..29 (and the plain loop
// for anything else); LARGE = true (a batch with a kernel the fixed sizes do not cover): the
// chunked columns for kpy >= 8.  Separate flavours keep the chunked code's registers out of the
// kernels that run the fixed sizes.
template <bool LARGE>
__device__ __noinline__ void conv_col(const float* Tt, int TP, const float* KT, int kpx, int kpy,
                                      int tx, int ty0, float* out) {
  if (LARGE) {
    if (kpy >= 8) {
      switch (kpy & 3) {
        case 0:
          conv_col_chunked<0, kConvRowsL>(Tt, TP, KT, kpx, kpy, tx, ty0, out);
          return;
        case 1:
          conv_col_chunked<1, kConvRowsL>(Tt, TP, KT, kpx, kpy, tx, ty0, out);
          return;
        case 2:
          conv_col_chunked<2, kConvRowsL>(Tt, TP, KT, kpx, kpy, tx, ty0, out);
          return;
        default:
          conv_col_chunked<3, kConvRowsL>(Tt, TP, KT, kpx, kpy, tx, ty0, out);
          return;
      }
    }
    conv_col_generic<kConvRowsL>(Tt, TP, KT, kpx, kpy, tx, ty0, out);
    return;
  }
  if (kpx == kpy) {
    switch (kpx) {
#define AP_CONV_CASE(K) \
  case K:               \
    conv_col_fixed<K, kConvRows>(Tt, TP, KT, tx, ty0, out); \
    return;
      AP_CONV_CASE(3) AP_CONV_CASE(5) AP_CONV_CASE(7) AP_CONV_CASE(9) AP_CONV_CASE(11)
      AP_CONV_CASE(13) AP_CONV_CASE(15) AP_CONV_CASE(17) AP_CONV_CASE(19) AP_CONV_CASE(21)
      AP_CONV_CASE(23) AP_CONV_CASE(25) AP_CONV_CASE(27) AP_CONV_CASE(29)
#undef AP_CONV_CASE
      default:
        break;
    }
  }
  conv_col_generic<kConvRows>(Tt, TP, KT, kpx, kpy, tx, ty0, out);
}

// Convolve/accumulate pass.  NF = number of fitted parameters (compile time, so the
// per-pixel J^T W J accumulators stay in registers).
template <int NF, bool LARGE>
__device__ __forceinline__ void conv_tile(const BatchArgs& b, const ConvIO& io, float* smem,
                                          float* shred, int slot, int s, int local) {
  const EvalDev& e = b.evals[s * 2 + slot];
  const int ops = e.ops;
  const StampDev& st = b.stamps[s];
  double* tacc = b.tile_acc + ((int64_t)(st.tile_o0 + local) * 2 + slot) * kNacc;
  const int tx = threadIdx.x & 31, tg = threadIdx.x >> 5;
  constexpr int kRows = conv_rows(LARGE), kTileY = conv_tile_y(LARGE);
  const int x0 = (local % st.nto_x) * kOutTileX, y0 = (local / st.nto_x) * kTileY;
  const int x = x0 + tx, yb = y0 + tg * kRows;
  const bool jac = (ops & OP_JAC) != 0;
  const bool diff = (ops & OP_DIFF) != 0;  // (forward only: no Jacobian planes)
  const bool shiftmode = (b.psf_mode == AP_PSF_FULL);
  const int nplanes = jac ? 1 + NGRAD : 1;

  // the epilogue's per-pixel operands (data, weight, the base model and, for the curvature
  // term, the base Jacobian) are requested into L2 now, so that their loads after the
  // convolution do not wait on DRAM: one thread per (tile row, plane) row segment, both ends
  {
    const bool fit = (ops & (OP_CHI2 | OP_HG | OP_RPP)) != 0 && !(ops & OP_VJP);
    const int npf = fit ? 2 + ((diff || (ops & OP_RPP)) ? 1 : 0) + ((ops & OP_RPP) ? NF : 0) : 0;
    const int rows = min(kTileY, st.ny - y0), w = min(kOutTileX, st.nx - x0);
    for (int k = threadIdx.x; k < npf * rows; k += blockDim.x) {
      const int pl = k / rows, r = k - pl * rows;
      const int64_t op = st.out_off + (int64_t)(y0 + r) * st.nx + x0;
      const float* base = pl == 0 ? io.data
                        : pl == 1 ? io.weight
                        : (pl == 2 && (diff || (ops & OP_RPP))) ? io.y0
                        : io.jbase + (int64_t)(pl - 3) * b.out_pixels;
      if (base) {
        asm volatile("prefetch.global.L2 [%0];" ::"l"(base + op));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(base + op + w - 1));
      }
    }
  }

  // conv results per row: [0] model, [1] d/dshift_x, [2] d/dshift_y, [3 + q] partial plane q
  float cv[3 + NGRAD][kRows];
#pragma unroll
  for (int k = 0; k < 3 + NGRAD; ++k)
#pragma unroll
    for (int o = 0; o < kRows; ++o) cv[k][o] = 0.f;

  if (b.psf_mode == AP_PSF_NONE) {
#pragma unroll
    for (int o = 0; o < kRows; ++o) {
      const int y = yb + o;
      if (x < st.nx && y < st.ny) {
        const int64_t wp = st.work_off + (int64_t)y * st.wnx + x;
        cv[0][o] = b.work[work_plane(b, slot, diff ? 1 : 0) + wp];
        if (jac) {
#pragma unroll
          for (int q = 0; q < NGRAD; ++q) cv[3 + q][o] = b.work[work_plane(b, slot, 1 + q) + wp];
        }
      }
    }
  } else if (st.fft_nx > 0) {
    // planes convolved by the FFT pass (ap_fft.cu), same indices as below
    const int64_t npix = (int64_t)st.nx * st.ny;
    const float* pre = b.preconv + st.pre_off + (int64_t)slot * (3 + NGRAD) * npix;
#pragma unroll
    for (int o = 0; o < kRows; ++o) {
      const int y = yb + o;
      if (!(x < st.nx && y < st.ny)) continue;
      const int64_t i = (int64_t)y * st.nx + x;
      cv[0][o] = pre[i];
      if (jac) {
        if (shiftmode) {
          cv[1][o] = pre[npix + i];
          cv[2][o] = pre[2 * npix + i];
        }
#pragma unroll
        for (int q = 0; q < NGRAD; ++q) {
          if (shiftmode && !(ops & OP_VJP_COORD) && (q == GX || q == GY)) continue;
          if (!profile_has_n(b.kind) && q == GN) continue;
          cv[3 + q][o] = pre[(int64_t)(3 + q) * npix + i];
        }
      }
    }
  } else {
    const int kpx = st.kpx, kpy = st.kpy, ks = conv_col_stride(kpy), kstride = kpx * ks;
    const int cx = (kpx - 1) / 2, cy = (kpy - 1) / 2;
    const int TW = kOutTileX + kpx - 1, TH = kTileY + kpy - 1, TP = conv_tile_pitch(kpy, LARGE);
    float* KT = smem;                // up to 3 kernels, transposed
    float* Tt = smem + 3 * kstride;  // input tile
    const int kp2 = kpx * kpy;
    const float* ksrc = b.spsf + st.spsf_off + (int64_t)slot * 3 * kp2;
    // kernels: K, dK/dshift_x, dK/dshift_y (Jacobian) or K1, dK (difference to the base)
    const int nk = (jac && shiftmode) ? 3 : ((diff && shiftmode) ? 2 : 1);
    for (int idx = threadIdx.x; idx < nk * kstride; idx += blockDim.x) {
      const int kk = idx / kstride, rem = idx - kk * kstride, u = rem / ks, v = rem - u * ks;
      KT[idx] = (v < kpy) ? ksrc[kk * kp2 + v * kpx + u] : 0.f;
    }
    const int row0 = y0 + st.by - cy, col0 = x0 + st.bx - cx;
    // difference: dm = K1 * dS (plane 1) + dK * S0 (the base's deep image)
    const int nsrc = diff ? nk : nplanes;
    // the planes this evaluation convolves, in order (the others are skipped)
    auto next_plane = [&](int pl) {
      for (; pl < nsrc; ++pl) {
        if (!diff && pl > 0 && shiftmode && !(ops & OP_VJP_COORD) && (pl - 1 == GX || pl - 1 == GY)) continue;
        if (!diff && pl > 0 && !profile_has_n(b.kind) && pl - 1 == GN) continue;
        break;
      }
      return pl;
    };
    // input tile of plane pl into buffer Tb by asynchronous copies (one commit group): rows over
    // warps, columns over lanes, coalesced reads; stored column-major (pitch TP), out-of-range
    // cells and rows TH..TP-1 zero-filled by the copies themselves
    auto fill = [&](float* Tb, int pl) {
      const float* src = diff ? (pl == 0 ? b.work + work_plane(b, slot, 1) : b.base_deep) + st.work_off
                              : b.work + work_plane(b, slot, pl) + st.work_off;
      for (int r = tg; r < TP; r += kConvThreads / 32) {
        const int wr = row0 + r;
        const bool rok = (r < TH && wr >= 0 && wr < st.wny);
        const float* srow = src + (int64_t)(rok ? wr : 0) * st.wnx;
        for (int c = tx; c < TW; c += 32) {
          const int wc = col0 + c;
          const bool ok = rok && wc >= 0 && wc < st.wnx;
          const uint32_t dst = (uint32_t)__cvta_generic_to_shared(Tb + c * TP + r);
          asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(dst), "l"(ok ? srow + wc : src),
                       "r"(ok ? 4 : 0)
                       : "memory");
        }
      }
      asm volatile("cp.async.commit_group;\n" ::: "memory");
    };
    // two tile buffers: the next plane's copies run while this plane is convolved
    const int tsz = TW * TP;
    int cur = next_plane(0), bi = 0;
    if (cur < nsrc) fill(Tt, cur);
    while (cur < nsrc) {
      const int nxt = next_plane(cur + 1);
      if (nxt < nsrc) {
        fill(Tt + (bi ? 0 : tsz), nxt);
        asm volatile("cp.async.wait_group 1;\n" ::: "memory");
      } else {
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
      }
      __syncthreads();
      const int pl = cur;
      const int nkp = (diff || pl > 0) ? 1 : nk;
      for (int kk = 0; kk < nkp; ++kk) {
        float outv[kRows];
        const int kidx = diff ? pl : kk;
        conv_col<LARGE>(Tt + (bi ? tsz : 0), TP, KT + kidx * kstride, kpx, kpy, tx, tg * kRows, outv);
        const int dst = diff ? pl : ((pl == 0) ? kk : 3 + (pl - 1));
#pragma unroll
        for (int o = 0; o < kRows; ++o) cv[dst][o] = outv[o];
      }
      __syncthreads();  // buffer bi is refilled by the next iteration's prefetch
      cur = nxt;
      bi ^= 1;
    }
  }

  const bool acc_any = (ops & (OP_CHI2 | OP_HG | OP_RPP | OP_VJP)) != 0;
  const bool do_hg = (ops & OP_HG) != 0, do_rpp = (ops & OP_RPP) != 0, do_vjp = (ops & OP_VJP) != 0;
  constexpr int NH = NF * (NF + 1) / 2;
  float a_chi2 = 0.f, a_g[NF > 0 ? NF : 1], a_h[NH > 0 ? NH : 1], a_rpp[NF > 0 ? NF : 1];
#pragma unroll
  for (int k = 0; k < NF; ++k) {
    a_g[k] = 0.f;
    a_rpp[k] = 0.f;
  }
#pragma unroll
  for (int k = 0; k < NH; ++k) a_h[k] = 0.f;
  const float d = (float)io.rpp_d;
  float hf[NF > 0 ? NF : 1];
  if (do_rpp) {
#pragma unroll
    for (int k = 0; k < NF; ++k) hf[k] = (float)io.hvec[s * NPARAM + k];
  }

#pragma unroll
  for (int o = 0; o < kRows; ++o) {
    const int y = yb + o;
    if (!(x < st.nx && y < st.ny)) continue;
    // (difference evaluations: mgal is the galaxy's difference, m the model's)
    const float mgal = diff ? cv[0][o] + cv[1][o] : cv[0][o];
    const float m = mgal + (diff ? e.d_sky : e.sky);
    // value-space Jacobian in full-vector order, compacted to the fitted slots
    float Jc[NF > 0 ? NF : 1];
    if (jac) {
      float J[NPARAM];
      if (shiftmode) {
        J[PX] = cv[1][o] * st.Pinvf[0] + cv[2][o] * st.Pinvf[2];
        J[PY] = cv[1][o] * st.Pinvf[1] + cv[2][o] * st.Pinvf[3];
        if (ops & OP_VJP_COORD) {
          J[PX] -= cv[3 + GX][o];
          J[PY] -= cv[3 + GY][o];
        }
      } else {
        J[PX] = -cv[3 + GX][o];
        J[PY] = -cv[3 + GY][o];
      }
      J[PQ] = cv[3 + GQ][o];
      J[PPA] = cv[3 + GPA][o];
      J[PN] = cv[3 + GN][o];
      J[PRE] = cv[3 + GRE][o];
      J[PIE] = kLn10f * mgal;
      J[PF] = kLn10f * e.sky;
      int nf = 0;
#pragma unroll
      for (int k = 0; k < NPARAM; ++k) {
        const float v = (ops & OP_REP) ? J[k] * e.drep[k] : J[k];
        if (b.free_mask & (1 << k)) {
#pragma unroll
          for (int c = 0; c < NF; ++c)
            if (c == nf) Jc[c] = v;
          ++nf;
        }
      }
    }
    const int64_t op = st.out_off + (int64_t)y * st.nx + x;
    if (ops & OP_WRITE_MODEL) io.model_out[op] = m;
    if (jac && (ops & OP_WRITE_JAC)) {
#pragma unroll
      for (int k = 0; k < NF; ++k) io.jac_out[(int64_t)k * b.out_pixels + op] = Jc[k];
    }
    if (!acc_any) continue;
    if (do_vjp) {
      // adjoint: the upstream gradient already carries weights and masks
      const float gin = io.vjp_in[op];
#pragma unroll
      for (int k = 0; k < NF; ++k) a_g[k] += Jc[k] * gin;
      continue;
    }
    // fused reductions (fit/lm.py:374-406); masked pixels are left out entirely
    if (io.mask && io.mask[op]) continue;
    const float w = io.weight ? io.weight[op] : 1.f;
    const float r = diff ? io.data[op] - io.y0[op] : io.data[op] - m;
    // chi^2 or, for a difference dm, its change W [(r - dm)^2 - r^2] = W dm (dm - 2 r)
    a_chi2 += diff ? w * m * (m - 2.f * r) : w * r * r;
    if (do_hg) {
      int h = 0;
#pragma unroll
      for (int a = 0; a < NF; ++a) {
        const float wja = w * Jc[a];
        a_g[a] += wja * r;
#pragma unroll
        for (int c = a; c < NF; ++c) a_h[h++] += wja * Jc[c];
      }
    }
    if (do_rpp) {
      float Jb[NF > 0 ? NF : 1];
      float jh = 0.f;
#pragma unroll
      for (int k = 0; k < NF; ++k) {
        Jb[k] = io.jbase[(int64_t)k * b.out_pixels + op];
        jh = fmaf(Jb[k], hf[k], jh);
      }
      // (2/d) * ((rh - r)/d - W (J h)),  rh - r = W (Y1 - Y0)
      const float ebase = (2.f / d) * ((w * (diff ? m : m - io.y0[op])) / d - w * jh);
#pragma unroll
      for (int k = 0; k < NF; ++k) a_rpp[k] += Jb[k] * ebase;
    }
  }
  if (!acc_any) return;
  // accumulator order: chi2, [g (NF), H upper (NH)], [rpp (NF)]
  float vals[1 + 2 * NF + NH];
  int nv = 0;
  vals[nv++] = a_chi2;
  if (do_hg || do_vjp) {
#pragma unroll
    for (int k = 0; k < NF; ++k) vals[nv++] = a_g[k];
  }
  if (do_hg) {
#pragma unroll
    for (int k = 0; k < NH; ++k) vals[nv++] = a_h[k];
  }
  if (do_rpp) {
#pragma unroll
    for (int k = 0; k < NF; ++k) vals[nv++] = a_rpp[k];
  }
  conv_tile_reduce(vals, nv, tacc, shred);
}

// fixed sizes: 6 blocks per SM (80 registers).  The large flavour is held to 1-2 blocks per SM
// by its shared memory, yet its register bound of 5 blocks (94 registers) measured 15 % faster on
// 67 x 67 kernels than no bound (114 registers)
template <int NF, bool LARGE>
__global__ void __launch_bounds__(kConvThreads, LARGE ? 5 : 6) k_conv(BatchArgs b, ConvIO io) {
  extern __shared__ __align__(16) float smem[];
  __shared__ float shred[kConvWarps * kNacc];
  __shared__ uint32_t next;
  const uint32_t n = b.counters[8];
  // tiles are fetched dynamically: their cost varies with the PSF size of their stamp
  while (true) {
    if (threadIdx.x == 0) next = atomicAdd(&b.counters[11], 1u);
    __syncthreads();
    const uint32_t it = next;
    if (it >= n) break;
    int slot, s, local;
    unpack_entry(b.olist[it], slot, s, local);
    conv_tile<NF, LARGE>(b, io, smem, shred, slot, s, local);
    __syncthreads();  // smem / shred / next reuse by the next tile
  }
}

// per-stamp sums of the tile partials (fixed order: deterministic)
__global__ void k_reduce_acc(BatchArgs b) {
  const uint32_t n = b.counters[9];
  for (uint32_t it = blockIdx.x; it < n; it += gridDim.x) {
    const int t = b.slist[it];
    const int s = t >> 1, slot = t & 1;
    const EvalDev& e = b.evals[t];
    if (!(e.ops & (OP_CHI2 | OP_HG | OP_RPP | OP_VJP))) continue;
    const StampDev& st = b.stamps[s];
    int nv = 1;
    if (e.ops & OP_HG) nv += b.n_free + b.n_free * (b.n_free + 1) / 2;
    if (e.ops & OP_VJP) nv += b.n_free;
    if (e.ops & OP_RPP) nv += b.n_free;
    for (int k = threadIdx.x; k < nv; k += blockDim.x) {
      double acc = 0;
      for (int tt = 0; tt < st.nto; ++tt)
        acc += b.tile_acc[((int64_t)(st.tile_o0 + tt) * 2 + slot) * kNacc + k];
      b.acc[((int64_t)s * 2 + slot) * kNacc + k] = acc;
    }
  }
}

// ---------------------------------------------------------------------------
// stand-alone chi^2 of a given model (LM._chi2 numerator)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kConvThreads) k_chi2(BatchArgs b, ConvIO io, const float* model) {
  const int tile = blockIdx.x;
  const int s = b.out_tiles[tile];
  const StampDev& st = b.stamps[s];
  const int local = tile - st.tile_o0;
  const int rows = conv_rows(b.conv_large != 0);
  const int x = (local % st.nto_x) * kOutTileX + (threadIdx.x & 31);
  const int yb = (local / st.nto_x) * conv_tile_y(b.conv_large != 0) + (threadIdx.x >> 5) * rows;
  float v = 0.f;
  for (int o = 0; o < rows; ++o) {
    const int y = yb + o;
    if (x < st.nx && y < st.ny) {
      const int64_t op = st.out_off + (int64_t)y * st.nx + x;
      if (!(io.mask && io.mask[op])) {
        const float w = io.weight ? io.weight[op] : 1.f;
        const float r = io.data[op] - model[op];
        v += w * r * r;
      }
    }
  }
  __shared__ float shred[kConvWarps * kNacc];
  conv_tile_reduce(&v, 1, b.tile_acc + (int64_t)tile * 2 * kNacc, shred);
}

__global__ void k_chi2_reduce(BatchArgs b, double* out) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= b.n_stamps) return;
  const StampDev& st = b.stamps[s];
  double t = 0;
  for (int tt = 0; tt < st.nto; ++tt) t += b.tile_acc[(int64_t)(st.tile_o0 + tt) * 2 * kNacc];
  out[s] = t;
}

// batched damped solve (LM._h): see damped_solve_dev in ap_device.cuh
__global__ void k_damped_solve(int m, int p, const double* hess, const double* grad,
                               const double* L, double* h) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  damped_solve_dev(p, hess + (int64_t)i * p * p, grad + (int64_t)i * p, L[i], h + (int64_t)i * p);
}

__global__ void k_psf_export(BatchArgs b, float* out, float* d_out, int64_t stride) {
  const int s = blockIdx.x;
  const StampDev& st = b.stamps[s];
  const int kp2 = st.kpx * st.kpy;
  const float* src = b.spsf + st.spsf_off;  // slot 0
  for (int idx = threadIdx.x; idx < kp2; idx += blockDim.x) {
    out[(int64_t)s * stride + idx] = src[idx];
    if (d_out) {
      d_out[((int64_t)s * 2 + 0) * stride + idx] = src[kp2 + idx];
      d_out[((int64_t)s * 2 + 1) * stride + idx] = src[2 * kp2 + idx];
    }
  }
}

// ---------------------------------------------------------------------------
// host launch wrappers
// ---------------------------------------------------------------------------
cudaError_t launch_eval_setup(const BatchArgs& b, const double* params, int64_t stamp_stride,
                              int64_t slot_stride, const int32_t* ops, int32_t ops_uniform,
                              cudaStream_t s) {
  const int n = b.n_stamps * 2;
  k_eval_setup<<<(n + 127) / 128, 128, 0, s>>>(b, params, stamp_stride, slot_stride, ops,
                                                ops_uniform);
  return cudaGetLastError();
}

// The limit on the convolve pass's dynamic shared memory is a property of the kernel on the
// current device, shared by every batch: it is only ever raised (per device), so a batch bound
// later with smaller kernels never lowers it below what an earlier batch launches with.
cudaError_t set_conv_smem(size_t bytes) {
  static std::mutex mu;
  static size_t raised[64] = {0};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  if (dev >= 0 && dev < 64 && bytes <= raised[dev]) return cudaSuccess;
  const int nb = (int)bytes;
  auto set = [&](const void* f) {
    const cudaError_t r = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, nb);
    if (r != cudaSuccess) e = r;
  };
  set((const void*)k_conv<0, false>); set((const void*)k_conv<1, false>); set((const void*)k_conv<2, false>);
  set((const void*)k_conv<3, false>); set((const void*)k_conv<4, false>); set((const void*)k_conv<5, false>);
  set((const void*)k_conv<6, false>); set((const void*)k_conv<7, false>); set((const void*)k_conv<8, false>);
  set((const void*)k_conv<0, true>); set((const void*)k_conv<1, true>); set((const void*)k_conv<2, true>);
  set((const void*)k_conv<3, true>); set((const void*)k_conv<4, true>); set((const void*)k_conv<5, true>);
  set((const void*)k_conv<6, true>); set((const void*)k_conv<7, true>); set((const void*)k_conv<8, true>);
  if (e == cudaSuccess && dev >= 0 && dev < 64) raised[dev] = bytes;
  return e;
}

cudaError_t launch_render_pass(const BatchArgs& b, const ConvIO& io, size_t conv_smem,
                               bool accumulate, cudaStream_t s, Profiler* prof) {
  auto B = [&](int k) { return (prof && prof->on) ? prof->begin(k, s) : -1; };
  auto E = [&](int i) {
    if (i >= 0) prof->end(i, s);
  };
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  // persistent grids over the compacted lists (fixed sizes: graph capturable)
  auto grid = [&](int64_t upper, int per_sm) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(upper, (int64_t)nsm * per_sm));
  };
  auto knob = [&](int k, int dflt) { return b.grid_mult[k] > 0 ? b.grid_mult[k] : dflt; };
  int t = B(KC_SETUP);
  k_build_lists<<<(b.n_stamps * 2 + 127) / 128, 128, 0, s>>>(b);
  E(t);
  if (b.psf_mode != AP_PSF_NONE) {
    t = B(KC_PSF);
    k_psf_shift<<<grid(2 * (int64_t)b.n_stamps, knob(GK_PSF, 8)), 256, 0, s>>>(b, io.psf, io.psf_base);
    E(t);
  }
  t = B(KC_SAMPLE);
  // PSF-model profiles take the kernels compiled with them; galaxies the Sersic/exponential ones
  const bool ext = b.kind == AP_PROFILE_MOFFAT || b.kind == AP_PROFILE_GAUSSIAN;
  const unsigned sgrid = grid(2 * (int64_t)b.n_work_tiles, knob(GK_SAMPLE, 8));
  // Sersic with a stencil sampling mode and threshold integration: sampling and selection fused
  const bool fused = b.kind == AP_PROFILE_SERSIC && b.integrate == AP_INTEGRATE_THRESHOLD &&
                     (b.sampling == AP_SAMPLING_MIDPOINT || b.sampling == AP_SAMPLING_TRAPEZOID);
  if (fused)
    k_sample_select<<<sgrid, kTile * kTile, 0, s>>>(b);
  else if (ext)
    k_sample<true><<<sgrid, kTile * kTile, 0, s>>>(b);
  else
    k_sample<false><<<sgrid, kTile * kTile, 0, s>>>(b);
  if (b.kind != AP_PROFILE_SERSIC && b.integrate == AP_INTEGRATE_THRESHOLD) {
    if (b.thr_window) {
      const dim3 wg(2 * b.n_stamps, 16);
      if (ext)
        k_window_msum<true><<<wg, 256, 0, s>>>(b);
      else
        k_window_msum<false><<<wg, 256, 0, s>>>(b);
    }
    k_exp_threshold<<<(b.n_stamps * 2 + 127) / 128, 128, 0, s>>>(b);
  }
  E(t);
  if (b.integrate == AP_INTEGRATE_THRESHOLD) {
    t = B(KC_SELECT);
    if (!fused) k_select<<<grid(2 * (int64_t)b.n_work_tiles, knob(GK_SAMPLE, 8)), kTile * kTile, 0, s>>>(b);
    if (ext)
      k_recheck<true><<<nsm * 4, 256, 0, s>>>(b);
    else
      k_recheck<false><<<nsm * 4, 256, 0, s>>>(b);
    E(t);
    t = B(KC_INTEGRATE);
    const int gi = nsm * knob(GK_INTEGRATE, 8);
    // (the two level-2 kernels share the persistent-grid size of the Jacobian one, scaled by
    // their resident blocks per SM)
    const int gf = gi;
    if (ext) {
      k_level1<true><<<gi, 256, 0, s>>>(b);
      if (b.amb_cap > 0) k_level1_amb<true><<<nsm * 4, 256, 0, s>>>(b);
      k_integrate<true, false><<<gi, 256, 0, s>>>(b);
      k_integrate<true, true><<<gf, 256, 0, s>>>(b);
    } else {
      k_level1<false><<<gi, 256, 0, s>>>(b);
      if (b.amb_cap > 0) k_level1_amb<false><<<nsm * 4, 256, 0, s>>>(b);
      k_integrate<false, false><<<gi, 256, 0, s>>>(b);
      // forward (plain or difference) pixels: sub-pixels packed over the lanes
      k_integrate_packed<<<(unsigned)nsm * 6, kPackWarps * 32, 0, s>>>(b);
    }
    E(t);
  }
  t = B(KC_CONV);
  if (b.n_fft > 0) {
    const cudaError_t fe = launch_fft_conv(b, b.fft_rows, b.fft_cols, b.fft_outs, b.fft_max_nx, b.fft_max_ny, s);
    if (fe != cudaSuccess) return fe;
  }
  const dim3 cgrid(grid(2 * (int64_t)b.n_out_tiles, knob(GK_CONV, 16)));
  if (b.conv_large) {
    switch (b.n_free) {
      case 0: k_conv<0, true><<<cgrid, kConvThreads, conv_smem, s>>>(b, io); break;
      case 1: k_conv<1, true><<<cgrid, kConvThreads, conv_smem, s>>>(b, io); break;
      case 2: k_conv<2, true><<<cgrid, kConvThreads, conv_smem, s>>>(b, io); break;
      case 3: k_conv<3, true><<<cgrid, kConvThreads, conv_smem, s>>>(b, io); break;
      case 4: k_conv<4, true><<<cgrid, kConvThreads, conv_smem, s>>>(b, io); break;
      case 5: k_conv<5, true><<<cgrid, kConvThreads, conv_smem, s>>>(b, io); break;
      case 6: k_conv<6, true><<<cgrid, kConvThreads, conv_smem, s>>>(b, io); break;
      case 7: k_conv<7, true><<<cgrid, kConvThreads, conv_smem, s>>>(b, io); break;
      default: k_conv<8, true><<<cgrid, kConvThreads, conv_smem, s>>>(b, io); break;
    }
  } else {
    switch (b.n_free) {
      case 0: k_conv<0, false><<<cgrid, kConvThreads, conv_smem, s>>>(b, io); break;
      case 1: k_conv<1, false><<<cgrid, kConvThreads, conv_smem, s>>>(b, io); break;
      case 2: k_conv<2, false><<<cgrid, kConvThreads, conv_smem, s>>>(b, io); break;
      case 3: k_conv<3, false><<<cgrid, kConvThreads, conv_smem, s>>>(b, io); break;
      case 4: k_conv<4, false><<<cgrid, kConvThreads, conv_smem, s>>>(b, io); break;
      case 5: k_conv<5, false><<<cgrid, kConvThreads, conv_smem, s>>>(b, io); break;
      case 6: k_conv<6, false><<<cgrid, kConvThreads, conv_smem, s>>>(b, io); break;
      case 7: k_conv<7, false><<<cgrid, kConvThreads, conv_smem, s>>>(b, io); break;
      default: k_conv<8, false><<<cgrid, kConvThreads, conv_smem, s>>>(b, io); break;
    }
  }
  E(t);
  if (accumulate) {
    t = B(KC_REDUCE);
    k_reduce_acc<<<grid(2 * (int64_t)b.n_stamps, 16), 64, 0, s>>>(b);
    E(t);
  }
  return cudaGetLastError();
}

// FP32 FMA throughput probe: 8 independent FMA chains per thread.
__global__ void k_fma_probe(float* out, int iters) {
  float a0 = threadIdx.x * 1e-7f, a1 = a0 + 1e-7f, a2 = a0 + 2e-7f, a3 = a0 + 3e-7f;
  float a4 = a0 + 4e-7f, a5 = a0 + 5e-7f, a6 = a0 + 6e-7f, a7 = a0 + 7e-7f;
  const float m = 0.999999f, c = 1e-7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      a0 = fmaf(a0, m, c); a1 = fmaf(a1, m, c); a2 = fmaf(a2, m, c); a3 = fmaf(a3, m, c);
      a4 = fmaf(a4, m, c); a5 = fmaf(a5, m, c); a6 = fmaf(a6, m, c); a7 = fmaf(a7, m, c);
    }
  }
  const float r = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (r == 123.456f) out[blockIdx.x * blockDim.x + threadIdx.x] = r;
}

// Sample-evaluation probe: the integration's per-sample arithmetic (a Sersic sample: plain,
// with its six partials, or as a difference to a base evaluation) at full occupancy with no
// memory traffic, four independent samples per step: the rate these device functions reach
// on this GPU, the compute roofline of the integration kernels.
template <int KIND>
__global__ void __launch_bounds__(256) k_sample_probe(float* out, int iters) {
  EvalF e{};
  e.c = 0.8f;
  e.s = 0.6f;
  e.invq = 1.6f;
  e.invRe = 0.125f;
  e.invn = 0.4f;
  e.bn = 4.67f;
  e.dbn = 2.0f;
  e.amp = 15.8f;
  e.soft2 = 1e-6f;
  DeltaF d{};
  d.c = 1e-5f;
  d.s = -2e-5f;
  d.invq = 3e-5f;
  d.lnire = -1e-5f;
  d.invn = 2e-5f;
  d.bn = -4e-5f;
  d.lnamp = 1e-5f;
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  const float x0 = 0.01f * (threadIdx.x & 31), y0 = 0.013f * (threadIdx.x >> 5);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float X = x0 + 0.37f * k + 1e-3f * it, Y = y0 - 0.29f * k + 7e-4f * it;
      if (KIND == 1) {
        const Sample sm = eval_profile<true, false>(e, AP_PROFILE_SERSIC, X, Y, 1.f);
        float t = sm.v;
#pragma unroll
        for (int q = 0; q < NGRAD; ++q) t += sm.g[q];
        acc[k] += t;
      } else if (KIND == 2) {
        float dI;
        const Sample sm = eval_profile_delta(e, d, AP_PROFILE_SERSIC, X, Y, 1.f, dI);
        acc[k] += sm.v + dI;
      } else {
        acc[k] += eval_profile<false, false>(e, AP_PROFILE_SERSIC, X, Y, 1.f).v;
      }
    }
  }
  const float r = acc[0] + acc[1] + acc[2] + acc[3];
  if (r == 123.456f) out[blockIdx.x * blockDim.x + threadIdx.x] = r;
}

cudaError_t launch_sample_probe(int kind, float* out, int iters, int blocks, cudaStream_t s) {
  if (kind == 1)
    k_sample_probe<1><<<blocks, 256, 0, s>>>(out, iters);
  else if (kind == 2)
    k_sample_probe<2><<<blocks, 256, 0, s>>>(out, iters);
  else
    k_sample_probe<0><<<blocks, 256, 0, s>>>(out, iters);
  return cudaGetLastError();
}

cudaError_t launch_fma_probe(float* out, int iters, int blocks, cudaStream_t s) {
  k_fma_probe<<<blocks, 256, 0, s>>>(out, iters);
  return cudaGetLastError();
}

int Profiler::begin(int k, cudaStream_t s) {
  if (used >= cap) {
    const int ncap = cap ? 2 * cap : 256;
    cudaEvent_t* nev = new cudaEvent_t[2 * ncap];
    int* nk = new int[ncap];
    for (int i = 0; i < cap; ++i) {
      nev[2 * i] = ev[2 * i];
      nev[2 * i + 1] = ev[2 * i + 1];
      nk[i] = kind[i];
    }
    for (int i = cap; i < ncap; ++i) {
      cudaEventCreate(&nev[2 * i]);
      cudaEventCreate(&nev[2 * i + 1]);
      nk[i] = 0;
    }
    delete[] ev;
    delete[] kind;
    ev = nev;
    kind = nk;
    cap = ncap;
  }
  const int idx = used++;
  kind[idx] = k;
  record(ev[2 * idx], s);
  return idx;
}

// External records become event-record nodes when the stream is being captured; outside a
// capture the flag is not accepted, and a plain record does the same job.
void Profiler::record(cudaEvent_t e, cudaStream_t s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(s, &cs);
  if (cs == cudaStreamCaptureStatusActive)
    cudaEventRecordWithFlags(e, s, cudaEventRecordExternal);
  else
    cudaEventRecord(e, s);
}

void Profiler::end(int idx, cudaStream_t s) { record(ev[2 * idx + 1], s); }

void Profiler::harvest(bool reset) {
  for (int i = 0; i < used; ++i) {
    float t = 0.f;
    if (cudaEventElapsedTime(&t, ev[2 * i], ev[2 * i + 1]) == cudaSuccess) {
      ms[kind[i]] += t;
      launches[kind[i]] += 1;
    }
  }
  (void)cudaGetLastError();  // a pair that never completed must not poison later checks
  if (reset) used = 0;
}

void Profiler::clear_totals() {
  for (int k = 0; k < KC_COUNT; ++k) {
    ms[k] = 0;
    launches[k] = 0;
  }
}

void Profiler::destroy() {
  for (int i = 0; i < cap; ++i) {
    cudaEventDestroy(ev[2 * i]);
    cudaEventDestroy(ev[2 * i + 1]);
  }
  delete[] ev;
  delete[] kind;
  ev = nullptr;
  kind = nullptr;
  cap = used = 0;
}

// grad[s][k] = accumulated VJP of stamp s (slot 0)
__global__ void k_gather_vjp(BatchArgs b, double* grad) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= b.n_stamps * b.n_free) return;
  const int s = t / b.n_free, k = t - s * b.n_free;
  grad[t] = b.acc[((int64_t)s * 2 + 0) * kNacc + 1 + k];
}

cudaError_t launch_gather_vjp(const BatchArgs& b, double* grad, cudaStream_t s) {
  const int n = b.n_stamps * b.n_free;
  if (n > 0) k_gather_vjp<<<(n + 127) / 128, 128, 0, s>>>(b, grad);
  return cudaGetLastError();
}

cudaError_t launch_chi2_only(const BatchArgs& b, const ConvIO& io, const float* model,
                             double* out, cudaStream_t s) {
  k_chi2<<<b.n_out_tiles, kConvThreads, 0, s>>>(b, io, model);
  k_chi2_reduce<<<(b.n_stamps + 127) / 128, 128, 0, s>>>(b, out);
  return cudaGetLastError();
}

cudaError_t launch_psf_only(const BatchArgs& b, const float* psf, cudaStream_t s) {
  k_build_lists<<<(b.n_stamps * 2 + 127) / 128, 128, 0, s>>>(b);
  k_psf_shift<<<std::max(1, std::min(2 * b.n_stamps, 1024)), 256, 0, s>>>(b, psf, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_damped_solve(int m, int p, const double* hess, const double* grad,
                                const double* L, double* h, cudaStream_t s) {
  k_damped_solve<<<(m + 63) / 64, 64, 0, s>>>(m, p, hess, grad, L, h);
  return cudaGetLastError();
}

cudaError_t launch_psf_export(const BatchArgs& b, float* out, float* d_out, int64_t stride,
                              cudaStream_t s) {
  k_psf_export<<<b.n_stamps, 256, 0, s>>>(b, out, d_out, stride);
  return cudaGetLastError();
}

}  // namespace apgb
