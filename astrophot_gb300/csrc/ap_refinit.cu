// The reference's initial-value heuristics for a Sérsic / exponential galaxy
// (``Model.initialize()`` with no parameter values), one CTA per stamp, float64 throughout.
//
// Reference (AstroPhot 0.x):
//   centre  : models/model_object.py:180-233, utils/initialize/center.py:8-49
//   PA      : models/galaxy_model_object.py:60-98, utils/angle_operations.py:35-56
//   q       : models/galaxy_model_object.py:99-113, utils/initialize/initialize.py:8-113,
//             utils/isophote/extract.py:10-218, utils/interpolate.py:232-273
//   n/Re/Ie : models/_shared_methods.py:71-166 (binned median profile + Nelder-Mead),
//             models/sersic_model.py:33-38, models/exponential_model.py:32-37,
//             utils/parametric_profiles.py:21-36,77-86
//   limits  : param/parameter.py:452-477 (soft-limit setter)
// Nelder-Mead follows scipy's default form of the method (Lagarias, Reeds, Wright & Wright
// 1998): reflection 1, expansion 2, contractions and shrink 1/2, first simplex x0 scaled by 1.05
// per coordinate (2.5e-4 where 0), xatol = fatol = 1e-4, at most 200 N iterations/evaluations.
//
// Reference quirks kept: the isophotes are centred on the transposed centre pixel, the centre of
// light runs on the raw data and returns the box centre of the step before convergence, and the
// exponential profile fit passes its two parameters to the profile in swapped order.
//
// This file is compiled without FMA contraction so its arithmetic rounds like numpy's.
#include <algorithm>
#include <cfloat>
#include <cmath>

#include "ap_internal.h"

namespace apgb {
namespace {

constexpr int kInitThreads = 128;
constexpr int kInitWarps = kInitThreads / 32;
constexpr int kBins = 10;
constexpr int kQSamples = 15;
constexpr double kNorth = kPi / 2.0;
constexpr double kTwoPi = 2 * kPi;

struct InitGeom {
  int32_t nx, ny;
  int64_t off;
  double s, ox, oy, area;
};

// one stamp of a chunk waiting for its profile fit (each warp fits one stamp of the chunk)
struct ChunkSlot {
  double R[kBins], I[kBins], x0[3];
  double cx, cy, q, PA;
  int st;        // stamp index, -1: empty
  int status;
  int need_fit;
};

struct InitShared {
  ChunkSlot slot[kInitWarps];
  double red[kInitWarps * 4];
  int ired[kInitWarps + 1];
  double d[8];
  int i[8];
  double prof_R[kBins], prof_I[kBins], edges[kBins + 1];
  int bin_cnt[kBins], bin_start[kBins];
  double amp[kQSamples];
  double sin5[10], cos5[10];  // sin, cos of pi k / 5, k = -4..5
};

// -- small helpers --------------------------------------------------------------------------

__device__ __forceinline__ bool lt_nan(double a, double b) {  // numpy order: NaN last
  return a < b || (isnan(b) && !isnan(a));
}

__device__ __forceinline__ double pymod(double a, double b) {  // Python / numpy float %
  double m = fmod(a, b);
  if (m != 0.0) {
    if ((b < 0) != (m < 0)) m += b;
  } else {
    m = copysign(0.0, b);
  }
  return m;
}

// numpy's 'linear' percentile of a sorted array (q in [0, 1])
__device__ double pct_sorted(const double* a, int n, double q) {
  const double vi = (n - 1) * q;
  const double lo = floor(vi);
  const int i = (int)lo;
  const int j = min(i + 1, n - 1);
  const double g = vi - lo;
  const double d = a[j] - a[i];
  return g >= 0.5 ? a[j] - d * (1.0 - g) : a[i] + d * g;
}

__device__ double median_sorted(const double* a, int n) {
  if (n <= 0) return nan("");
  if (n & 1) return a[(n - 1) / 2];
  return (a[n / 2 - 1] + a[n / 2]) / 2.0;
}

__device__ double iqr_half_sorted(const double* a, int n) {
  if (n <= 0) return nan("");
  return (pct_sorted(a, n, 0.84) - pct_sorted(a, n, 0.16)) / 2;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block sums of up to 4 values; every thread receives the totals
__device__ void block_sum4(InitShared& S, double* v, int k) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j = 0; j < k; ++j) {
    const double t = warp_sum(v[j]);
    if (lane == 0) S.red[w * 4 + j] = t;
  }
  __syncthreads();
  for (int j = 0; j < k; ++j) {
    double t = 0.0;
    for (int u = 0; u < kInitWarps; ++u) t += S.red[u * 4 + j];
    v[j] = t;
  }
  __syncthreads();
}

__device__ void block_minmax(InitShared& S, double& mn, double& mx) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  if (lane == 0) {
    S.red[w * 4] = mn;
    S.red[w * 4 + 1] = mx;
  }
  __syncthreads();
  mn = S.red[0];
  mx = S.red[1];
  for (int u = 1; u < kInitWarps; ++u) {
    mn = fmin(mn, S.red[u * 4]);
    mx = fmax(mx, S.red[u * 4 + 1]);
  }
  __syncthreads();
}

// order-preserving compaction: returns this thread's slot (or -1) and the chunk total
__device__ int block_compact(InitShared& S, bool flag, int& total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned b = __ballot_sync(0xffffffffu, flag);
  if (lane == 0) S.ired[w] = __popc(b);
  __syncthreads();
  int before = 0;
  total = 0;
  for (int u = 0; u < kInitWarps; ++u) {
    if (u < w) before += S.ired[u];
    total += S.ired[u];
  }
  __syncthreads();
  return flag ? before + __popc(b & ((1u << lane) - 1u)) : -1;
}

__device__ __forceinline__ int pow2_at_least(int n) {
  int p = 1;
  while (p < n) p <<= 1;
  return p;
}

// Sorting runs on order-preserving 64-bit integer keys of the doubles (integer compares keep the
// narrow FP64 pipe free): negative values map to ~bits, the rest to bits | sign; a positive NaN
// sorts after +inf, as numpy's NaN-last order.
__device__ __forceinline__ unsigned long long okey(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double okey_inv(unsigned long long k) {
  return __longlong_as_double((long long)((k >> 63) ? (k & 0x7fffffffffffffffull) : ~k));
}

__device__ void to_keys(double* a, int P) {
  unsigned long long* k = (unsigned long long*)a;
  for (int i = threadIdx.x; i < P; i += blockDim.x) k[i] = okey(a[i]);
  __syncthreads();
}
__device__ void from_keys(double* a, int P) {
  unsigned long long* k = (unsigned long long*)a;
  for (int i = threadIdx.x; i < P; i += blockDim.x) a[i] = okey_inv(k[i]);
  __syncthreads();
}

// ascending bitonic sort of a[0, P) (P a power of two), NaN last
__device__ void sort_keys(double* a, int P) {
  to_keys(a, P);
  unsigned long long* k = (unsigned long long*)a;
  for (int sz = 2; sz <= P; sz <<= 1)
    for (int j = sz >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < P; i += blockDim.x) {
        const int l = i ^ j;
        if (l > i) {
          const unsigned long long x = k[i], y = k[l];
          if (((i & sz) == 0) ? (y < x) : (x < y)) {
            k[i] = y;
            k[l] = x;
          }
        }
      }
      __syncthreads();
    }
  from_keys(a, P);
}

// ascending sort of (key, value) pairs by key
__device__ void sort_pairs(double* key, double* val, int P) {
  to_keys(key, P);
  unsigned long long* k = (unsigned long long*)key;
  for (int sz = 2; sz <= P; sz <<= 1)
    for (int j = sz >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < P; i += blockDim.x) {
        const int l = i ^ j;
        if (l > i) {
          const unsigned long long x = k[i], y = k[l];
          if (((i & sz) == 0) ? (y < x) : (x < y)) {
            k[i] = y;
            k[l] = x;
            const double t = val[i];
            val[i] = val[l];
            val[l] = t;
          }
        }
      }
      __syncthreads();
    }
  from_keys(key, P);
}

// ascending sort of (bin, value) pairs, bins first
__device__ void sort_binned(uint8_t* bin, double* val, int P) {
  to_keys(val, P);
  unsigned long long* k = (unsigned long long*)val;
  for (int sz = 2; sz <= P; sz <<= 1)
    for (int j = sz >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < P; i += blockDim.x) {
        const int l = i ^ j;
        if (l > i) {
          const uint8_t bx = bin[i], by = bin[l];
          const unsigned long long x = k[i], y = k[l];
          const bool lx = bx < by || (bx == by && x < y);  // (bx, x) < (by, y)
          const bool ly = by < bx || (by == bx && y < x);
          if (((i & sz) == 0) ? ly : lx) {
            bin[i] = by;
            bin[l] = bx;
            k[i] = y;
            k[l] = x;
          }
        }
      }
      __syncthreads();
    }
  from_keys(val, P);
}

// ``Sigma_Clip_Upper`` on sorted values (one thread): lim = median + nsigma iqr/2 of the
// values below lim, until lim repeats (10 iterations at most)
__device__ double sigma_clip_upper_sorted(const double* v, int n, double nsigma) {
  double old = 0.0, lim = INFINITY;
  for (int i = 0; i < 10 && old != lim; ++i) {
    // values < lim form a prefix of the sorted array
    int lo = 0, hi = n;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (v[mid] < lim) lo = mid + 1;
      else hi = mid;
    }
    const int m = isnan(lim) ? 0 : lo;
    const double med = median_sorted(v, m);
    const double rng = iqr_half_sorted(v, m);
    old = lim;
    lim = med + rng * nsigma;
  }
  return lim;
}

// ``np.interp`` on sorted (xp, fp) of m samples (non-periodic, clamped ends)
__device__ double interp_sorted(double x, const double* xp, const double* fp, int m) {
  if (!(x < xp[m - 1])) return fp[m - 1];
  if (x < xp[0]) return fp[0];
  int lo = 0, hi = m - 1;  // xp[lo] <= x < xp[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (xp[mid] <= x) lo = mid;
    else hi = mid;
  }
  if (xp[lo] == x) return fp[lo];
  const double slope = (fp[lo + 1] - fp[lo]) / (xp[lo + 1] - xp[lo]);
  double r = slope * (x - xp[lo]) + fp[lo];
  if (isnan(r)) {
    r = slope * (x - xp[lo + 1]) + fp[lo + 1];
    if (isnan(r) && fp[lo] == fp[lo + 1]) r = fp[lo];
  }
  return r;
}

// periodic ``np.interp`` (period 2 pi) on (xp, fp) sorted by xp, wrapped by one sample per end
__device__ double interp_periodic(double x, const double* xp, const double* fp, int m) {
  x = pymod(x, kTwoPi);
  const double xl = xp[m - 1] - kTwoPi, xr = xp[0] + kTwoPi;
  if (!(x < xr)) return fp[0];
  if (x < xl) return fp[m - 1];
  double x0, x1, f0, f1;
  if (x < xp[0]) {
    x0 = xl, x1 = xp[0], f0 = fp[m - 1], f1 = fp[0];
  } else if (!(x < xp[m - 1])) {
    x0 = xp[m - 1], x1 = xr, f0 = fp[m - 1], f1 = fp[0];
  } else {
    int lo = 0, hi = m - 1;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (xp[mid] <= x) lo = mid;
      else hi = mid;
    }
    x0 = xp[lo], x1 = xp[lo + 1], f0 = fp[lo], f1 = fp[lo + 1];
  }
  if (x0 == x) return f0;
  const double slope = (f1 - f0) / (x1 - x0);
  double r = slope * (x - x0) + f0;
  if (isnan(r)) {
    r = slope * (x - x1) + f1;
    if (isnan(r) && f0 == f1) r = f0;
  }
  return r;
}

// -- the isophote sampler -------------------------------------------------------------------

struct IsoBuf {
  double *x, *y, *t, *fl, *srt, *k2, *v2;  // [cap] each; t = ellipse parameter of the sample
  int cap;
};

// Python's a % 2pi for a in (-2pi, 4pi): fmod is exact there, so this is the same number
__device__ __forceinline__ double mod_2pi(double a) {
  if (a < 0) return a + kTwoPi;
  if (a >= kTwoPi) return a - kTwoPi;
  return a;
}

// the reference's isophote angle of ellipse parameter t: atan(q tan t) (+ pi where cos t < 0),
// rotated by pa, mod 2 pi (extract.py:136, 148)
__device__ __forceinline__ double iso_theta(double t, double q, double pa) {
  double st, ct;
  sincos(t, &st, &ct);
  const double th = atan(q * (st / ct)) + kPi * (ct < 0 ? 1.0 : 0.0);
  return mod_2pi(th + pa);
}

// normalised Lanczos (scale 5) at (X, Y) of the float64 image img (``interpolate_Lanczos``):
// separable weights sinc(u) sinc(u / 5), u = (k - X) + floor(X), k = -4..5, over the taps that
// fall inside the image.  sin(pi u) = -(-1)^k sin(pi f) and sin(pi u / 5) by angle addition; the
// ten reciprocals of one axis come from one division (running products).
__device__ double lanczos5(const InitShared& S, const double* img, int nx, int ny, double X, double Y) {
  const double fx = floor(X), fy = floor(Y);
  const int ix = (int)fx, iy = (int)fy;
  double L[2][10];
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    const double base = a == 0 ? X : Y;
    const double fl = a == 0 ? fx : fy;
    const double f = base - fl;
    const double sp = sinpi(f);
    double s5, c5;
    sincospi(f / 5.0, &s5, &c5);
    double num[10], den[10], pre[10];
    double run = 1.0;
#pragma unroll
    for (int k = 0; k < 10; ++k) {
      const double u = ((double)(k - 4) - base) + fl;
      const double sgn = ((k - 4) & 1) ? 1.0 : -1.0;  // -(-1)^k
      num[k] = (sgn * sp) * (S.sin5[k] * c5 - S.cos5[k] * s5);
      den[k] = u == 0.0 ? 1.0 : (kPi * u) * (kPi * (u / 5.0));
      if (u == 0.0) num[k] = 1.0;
      pre[k] = run;
      run *= den[k];
    }
    double inv = 1.0 / run;
#pragma unroll
    for (int k = 9; k >= 0; --k) {
      L[a][k] = num[k] * (inv * pre[k]);
      inv *= den[k];
    }
  }
  const int bx0 = max(0, ix - 4), bx1 = min(nx, ix + 6);
  const int by0 = max(0, iy - 4), by1 = min(ny, iy + 6);
  double sx = 0.0, sy = 0.0, acc = 0.0;
  for (int c = bx0; c < bx1; ++c) sx += L[0][c - (ix - 4)];
  for (int r = by0; r < by1; ++r) {
    const double* row = img + (int64_t)r * nx;
    double rs = 0.0;
    for (int c = bx0; c < bx1; ++c) rs = fma(L[0][c - (ix - 4)], row[c], rs);
    const double ly = L[1][r - (iy - 4)];
    acc = fma(ly, rs, acc);
    sy += ly;
  }
  return acc / (sx * sy);
}

// ``_iso_extract`` with sigma clipping (nsigma 3) on img = data - edge median (float64, row-major):
// fills B.fl[0, n) in ellipse order and B.srt[0, n) with the same fluxes sorted; returns n.
// *n_keep receives the number of values the reference keeps (those below the clip limit: a
// prefix of srt), or n when it keeps all.  With interp, clipped fluxes are replaced by periodic
// interpolation in angle (srt is then stale: callers sort again).  Sample points are
// sma (cos t, q sin t) rotated by pa, the reference's superellipse point for C = 2.
__device__ int iso_extract(InitShared& S, IsoBuf& B, const double* img, int nx, int ny, double sma, double q,
                           double pa, double cx, double cy, bool interp, int* n_keep) {
  const int N = max(15, (int)(((0.9 * 2) * kPi) * sma));
  const double stop = (2 * kPi) * (1.0 - 1.0 / N);
  const double step = stop / (double)(N - 1);
  const double sa = sin(pa), ca = cos(pa);
  int base = 0;
  for (int c0 = 0; c0 < N; c0 += blockDim.x) {
    const int k = c0 + threadIdx.x;
    bool keep = false;
    double X = 0, Y = 0, t = 0;
    if (k < N) {
      t = (k == N - 1) ? stop : (double)k * step;
      double st, ct;
      sincos(t, &st, &ct);
      const double x0 = sma * ct, y0 = sma * (q * st);
      X = (ca * x0 - sa * y0) + cx;
      Y = (ca * y0 + sa * x0) + cy;
      keep = X >= 0 && X < nx - 1 && Y >= 0 && Y < ny - 1;
    }
    int tot;
    const int slot = block_compact(S, keep, tot);
    if (keep) {
      B.x[base + slot] = X;
      B.y[base + slot] = Y;
      B.t[base + slot] = t;
    }
    base += tot;
  }
  __syncthreads();
  const int n = base;
  const int P = pow2_at_least(max(n, 1));
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    double f = INFINITY;
    if (i < n) {
      if (sma < 30)
        f = lanczos5(S, img, nx, ny, B.x[i], B.y[i]);
      else
        f = img[(int64_t)(int)rint(B.y[i]) * nx + (int)rint(B.x[i])];
      B.fl[i] = f;
    }
    B.srt[i] = f;
  }
  __syncthreads();
  sort_keys(B.srt, P);
  if (threadIdx.x == 0) {
    int keep_n = n;
    double lim = INFINITY;
    if (n > 30) {
      lim = sigma_clip_upper_sorted(B.srt, n, 3.0);
      int m = 0;
      while (m < n && B.srt[m] < lim) ++m;
      if (m > 0) keep_n = m;
      else lim = INFINITY;  // nothing below the limit: every flux is kept
    }
    S.i[0] = keep_n;
    S.d[0] = lim;
  }
  __syncthreads();
  const int keep_n = S.i[0];
  const double lim = S.d[0];
  __syncthreads();
  *n_keep = keep_n;
  if (interp && keep_n < n) {
    // kept (theta, flux) sorted by theta, then the clipped fluxes interpolated
    int base2 = 0;
    for (int c0 = 0; c0 < n; c0 += blockDim.x) {
      const int i = c0 + threadIdx.x;
      const bool kp = i < n && B.fl[i] < lim;
      int tot;
      const int slot = block_compact(S, kp, tot);
      if (kp) {
        B.k2[base2 + slot] = iso_theta(B.t[i], q, pa);
        B.v2[base2 + slot] = B.fl[i];
      }
      base2 += tot;
    }
    const int m = base2;
    const int P2 = pow2_at_least(max(m, 1));
    for (int i = m + threadIdx.x; i < P2; i += blockDim.x) {
      B.k2[i] = INFINITY;
      B.v2[i] = 0.0;
    }
    __syncthreads();
    sort_pairs(B.k2, B.v2, P2);
    for (int i = threadIdx.x; i < n; i += blockDim.x)
      if (!(B.fl[i] < lim)) B.fl[i] = interp_periodic(iso_theta(B.t[i], q, pa), B.k2, B.v2, m);
    __syncthreads();
  }
  return n;
}

// -- Nelder-Mead on the binned profile (one warp per stamp) --------------------------------
// The warp evaluates up to three simplex points at once: lanes 10 g .. 10 g + 9 hold the ten
// profile bins of point g (g = 0, 1, 2).  The points an iteration may need (reflection,
// expansion, outside contraction; the shrink's vertices) are evaluated side by side and used
// in the order the sequential method asks for them, so the path and the evaluation count are
// those of the sequential method.

__device__ __forceinline__ double sersic_b(double n) {
  // the n^3, n^4 terms are below 1e-4 of b(n): a last-bit difference there does not reach b(n)
  const double n2 = n * n;
  return 2 * n - 1.0 / 3 + 4 / (405 * n) + 46 / (25515 * n2) + 131 / (1148175 * (n2 * n)) -
         2194697 / (30690717750.0 * (n2 * n2));
}

// mean of the 8 smallest squared log residuals of this lane group's point x (numpy: sort,
// drop the 2 largest, pairwise mean); valid in the lanes of groups 0-2
__device__ double nm_objective3(int kind, double R, double I, const double* x) {
  const int lane = threadIdx.x & 31;
  const int g = lane / kBins, b = lane - g * kBins, base = g * kBins;
  const bool live = g < 3;
  double r = INFINITY;
  if (live) {
    double lp;
    if (kind == AP_PROFILE_SERSIC) {
      const double n = x[0], Re = x[1], Ie = pow(10.0, x[2]);
      if (n <= 0 || Re <= 0 || Ie <= 0) {
        lp = log10(1e6);
      } else {
        lp = log10(Ie * exp(-sersic_b(n) * (pow(R / Re, 1.0 / n) - 1)));
      }
    } else {
      const double amp = x[0], Rs = pow(10.0, x[1]);
      lp = log10(amp * exp(-sersic_b(1.0) * (R / Rs - 1.0)));
    }
    const double dlt = I - lp;
    r = dlt * dlt;
  }
  // rank within the group on order-preserving integer keys (NaN last), ties by lane
  const unsigned long long key = okey(r);
  int rank = 0;
  for (int m = 0; m < kBins; ++m) {
    const unsigned long long o = __shfl_sync(0xffffffffu, key, min(base + m, 31));
    if (live && (o < key || (o == key && m < b))) ++rank;
  }
  const unsigned gmask = live ? (0x3ffu << base) : 0u;
  double s[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const unsigned bal = __ballot_sync(0xffffffffu, live && rank == k) & gmask;
    s[k] = __shfl_sync(0xffffffffu, r, bal ? __ffs(bal) - 1 : lane);
  }
  return (((s[0] + s[1]) + (s[2] + s[3])) + ((s[4] + s[5]) + (s[6] + s[7]))) / 8.0;
}

struct NMResult {
  double x[3];
  bool success;
  int calls;
};

__device__ NMResult nelder_mead(int kind, int dim, double R, double I, const double* x0) {
  constexpr double xatol = 1e-4, fatol = 1e-4;
  const int maxiter = 200 * dim, maxfev = 200 * dim;
  const int g = (threadIdx.x & 31) / kBins;
  double sim[4][3], fs[4];
  int calls = 0;
  for (int j = 0; j <= dim; ++j)
    for (int k = 0; k < 3; ++k) sim[j][k] = k < dim ? x0[k] : 0.0;
  for (int k = 0; k < dim; ++k) sim[k + 1][k] = sim[k + 1][k] != 0 ? 1.05 * sim[k + 1][k] : 0.00025;
  double cand[3];
  // the first simplex: points 0-2 together, then point 3
  for (int k = 0; k < 3; ++k) cand[k] = sim[min(g, dim)][k];
  double f = nm_objective3(kind, R, I, cand);
  for (int j = 0; j <= min(dim, 2); ++j) fs[j] = __shfl_sync(0xffffffffu, f, j * kBins);
  if (dim == 3) {
    for (int k = 0; k < 3; ++k) cand[k] = sim[3][k];
    f = nm_objective3(kind, R, I, cand);
    fs[3] = __shfl_sync(0xffffffffu, f, 0);
  }
  calls = dim + 1;
  auto order = [&]() {  // stable insertion sort by value, NaN last
    for (int a = 1; a <= dim; ++a) {
      double fv = fs[a], xv[3];
      for (int k = 0; k < 3; ++k) xv[k] = sim[a][k];
      int b = a - 1;
      while (b >= 0 && lt_nan(fv, fs[b])) {
        fs[b + 1] = fs[b];
        for (int k = 0; k < 3; ++k) sim[b + 1][k] = sim[b][k];
        --b;
      }
      fs[b + 1] = fv;
      for (int k = 0; k < 3; ++k) sim[b + 1][k] = xv[k];
    }
  };
  order();
  int it = 1;
  double xr[3], xe[3], xc[3], xbar[3], nsim[4][3];
  while (calls < maxfev && it < maxiter) {
    // convergence (np.max propagates NaN: then not converged)
    double dx = 0.0, df = 0.0;
    bool nanx = false;
    for (int j = 1; j <= dim; ++j) {
      for (int k = 0; k < dim; ++k) {
        const double v = fabs(sim[j][k] - sim[0][k]);
        nanx |= isnan(v);
        dx = fmax(dx, v);
      }
      const double v = fabs(fs[0] - fs[j]);
      nanx |= isnan(v);
      df = fmax(df, v);
    }
    if (!nanx && dx <= xatol && df <= fatol) break;
    bool spent = false;
    for (int k = 0; k < 3; ++k) {
      if (k < dim) {
        double t = sim[0][k];
        for (int j = 1; j < dim; ++j) t += sim[j][k];
        xbar[k] = t / dim;
        xr[k] = (1 + 1) * xbar[k] - 1 * sim[dim][k];
        xe[k] = (1 + 1 * 2) * xbar[k] - 1 * 2 * sim[dim][k];
        xc[k] = (1 + 0.5 * 1) * xbar[k] - 0.5 * 1 * sim[dim][k];
      } else {
        xbar[k] = xr[k] = xe[k] = xc[k] = 0.0;
      }
    }
    for (int k = 0; k < 3; ++k) cand[k] = g == 0 ? xr[k] : (g == 1 ? xe[k] : xc[k]);
    f = nm_objective3(kind, R, I, cand);
    const double fr = __shfl_sync(0xffffffffu, f, 0);
    const double fe = __shfl_sync(0xffffffffu, f, kBins);
    const double fc = __shfl_sync(0xffffffffu, f, 2 * kBins);
    ++calls;
    if (fr < fs[0]) {
      if (calls >= maxfev) {
        spent = true;
      } else {
        ++calls;
        const bool take_e = fe < fr;
        for (int k = 0; k < 3; ++k) sim[dim][k] = take_e ? xe[k] : xr[k];
        fs[dim] = take_e ? fe : fr;
      }
    } else if (fr < fs[dim - 1]) {
      for (int k = 0; k < 3; ++k) sim[dim][k] = xr[k];
      fs[dim] = fr;
    } else {
      bool shrink = false;
      if (calls >= maxfev) {
        spent = true;
      } else if (fr < fs[dim]) {
        ++calls;
        if (fc <= fr) {
          for (int k = 0; k < 3; ++k) sim[dim][k] = xc[k];
          fs[dim] = fc;
        } else {
          shrink = true;
        }
      } else {
        double xcc[3];
        for (int k = 0; k < 3; ++k) xcc[k] = k < dim ? (1 - 0.5) * xbar[k] + 0.5 * sim[dim][k] : 0.0;
        f = nm_objective3(kind, R, I, xcc);
        const double fcc = __shfl_sync(0xffffffffu, f, 0);
        ++calls;
        if (fcc < fs[dim]) {
          for (int k = 0; k < 3; ++k) sim[dim][k] = xcc[k];
          fs[dim] = fcc;
        } else {
          shrink = true;
        }
      }
      if (shrink) {
        for (int j = 1; j <= dim; ++j)
          for (int k = 0; k < 3; ++k) nsim[j][k] = k < dim ? sim[0][k] + 0.5 * (sim[j][k] - sim[0][k]) : 0.0;
        for (int k = 0; k < 3; ++k) cand[k] = nsim[min(g, dim - 1) + 1][k];
        f = nm_objective3(kind, R, I, cand);
        for (int j = 1; j <= dim; ++j) {
          const double fj = __shfl_sync(0xffffffffu, f, (j - 1) * kBins);
          for (int k = 0; k < 3; ++k) sim[j][k] = nsim[j][k];
          if (calls >= maxfev) {
            spent = true;
            break;
          }
          fs[j] = fj;
          ++calls;
        }
      }
    }
    if (!spent) ++it;
    order();
  }
  NMResult res;
  for (int k = 0; k < 3; ++k) res.x[k] = sim[0][k];
  res.success = !(calls >= maxfev || it >= maxiter);
  res.calls = calls;
  return res;
}

__device__ __forceinline__ double soft_lo(double v, double lo) { return fmax(v, lo + 1e-3); }
__device__ __forceinline__ double soft_hi(double v, double hi) { return fmin(v, hi - 1e-3); }

// -- the kernel -----------------------------------------------------------------------------

struct InitArgs {
  const StampDev* stamps;
  int32_t n;
  int32_t kind;
  int32_t known;  // bit i: full-vector slot i given
  const float* data;
  const uint8_t* mask;
  double* params;  // [n][8]
  int32_t* status;
  int iso_cap;
  int pix_cap;           // power of two >= the largest stamp's pixel count and edge count
  bool pix_in_smem;
  double* pix_val_g;     // [grid][pix_cap] when not in shared memory
  uint8_t* pix_bin_g;    // [grid][pix_cap]
};

__global__ void __launch_bounds__(kInitThreads, 4) k_reference_init(InitArgs A) {
  __shared__ InitShared S;
  extern __shared__ __align__(16) unsigned char dyn[];
  IsoBuf B;
  B.cap = A.iso_cap;
  double* dp = (double*)dyn;
  B.x = dp;
  B.y = dp + B.cap;
  B.t = dp + 2 * B.cap;
  B.fl = dp + 3 * B.cap;
  B.srt = dp + 4 * B.cap;
  B.k2 = dp + 5 * B.cap;
  B.v2 = dp + 6 * B.cap;
  double* pv;
  uint8_t* pb;
  if (A.pix_in_smem) {
    pv = dp + 7 * B.cap;
    pb = (uint8_t*)(pv + A.pix_cap);
  } else {
    pv = A.pix_val_g + (int64_t)blockIdx.x * A.pix_cap;
    pb = A.pix_bin_g + (int64_t)blockIdx.x * A.pix_cap;
  }
  if (threadIdx.x < 10) {
    double s, c;
    sincospi((double)((int)threadIdx.x - 4) / 5.0, &s, &c);
    S.sin5[threadIdx.x] = s;
    S.cos5[threadIdx.x] = c;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;

  // chunks of kInitWarps stamps: every stage but the profile fit runs CTA-wide stamp by stamp,
  // then the chunk's fits run side by side, one warp per stamp
  for (int chunk = blockIdx.x; chunk * kInitWarps < A.n; chunk += gridDim.x) {
  for (int j = 0; j < kInitWarps; ++j) {
    const int st = chunk * kInitWarps + j;
    if (st >= A.n) {
      if (threadIdx.x == 0) S.slot[j].st = -1;
      continue;
    }
    const StampDev& sd = A.stamps[st];
    InitGeom g;
    g.nx = sd.nx;
    g.ny = sd.ny;
    g.off = sd.out_off;
    g.s = sd.P[0];
    g.ox = sd.ref_xy[0] - g.s * (sd.ref_ij[0] + 0.5);
    g.oy = sd.ref_xy[1] - g.s * (sd.ref_ij[1] + 0.5);
    g.area = sd.pixel_area;
    const int nx = g.nx, ny = g.ny, npix = nx * ny;
    const float* d = A.data + g.off;
    const uint8_t* msk = A.mask ? A.mask + g.off : nullptr;
    double* prm = A.params + (int64_t)st * NPARAM;
    int status = 0;
    double cx = prm[PX], cy = prm[PY], PA = prm[PPA], q = prm[PQ];
    const bool know_c = (A.known & 3) == 3, know_pa = (A.known >> PPA) & 1, know_q = (A.known >> PQ) & 1;

    // 1. centre: window centre, then the centre of light (warp 0)
    if (!know_c) {
      cx = g.ox + nx * g.s / 2;
      cy = g.oy + ny * g.s / 2;
      if (threadIdx.x < 32) {
        const double icx = (cx - g.ox) / g.s - 0.5, icy = (cy - g.oy) / g.s - 0.5;
        int w = max(min((int)(min(nx, ny) / 10.0), 30), 6);
        w += w % 2;
        double c0 = icy, c1 = icx;  // (row, col)
        bool edge = false;
        for (int it = 0; it < 100; ++it) {
          const int r0 = (int)rint(c0) - w / 2, r1 = (int)rint(c0) + w / 2;
          const int q0 = (int)rint(c1) - w / 2, q1 = (int)rint(c1) + w / 2;
          if (r0 < 0 || q0 < 0 || r1 >= ny || q1 >= nx) {
            edge = true;
            break;
          }
          double den = 0, sy = 0, sx = 0;
          for (int e = lane; e < w * w; e += 32) {
            const int rr = e / w, cc = e % w;
            const double v = (double)d[(int64_t)(r0 + rr) * nx + q0 + cc];
            den += v;
            sy += v * rr;
            sx += v * cc;
          }
          den = warp_sum(den);
          sy = warp_sum(sy);
          sx = warp_sum(sx);
          const double n0 = r0 + sy / den, n1 = q0 + sx / den;
          if (fabs(c0 - n0) + fabs(c1 - n1) < 0.1) break;
          c0 = n0;
          c1 = n1;
        }
        if (edge) {
          c0 = icy;
          c1 = icx;
        }
        if (lane == 0) {
          if (c0 < 0 || c1 < 0 || c0 >= ny || c1 >= nx) {
            S.d[0] = cx;
            S.d[1] = cy;
          } else {
            S.d[0] = (c1 + 0.5) * g.s + g.ox;
            S.d[1] = (c0 + 0.5) * g.s + g.oy;
          }
          S.i[0] = edge ? AP_INIT_CENTRE_EDGE : 0;
        }
      }
      __syncthreads();
      cx = S.d[0];
      cy = S.d[1];
      status |= S.i[0];
      __syncthreads();
    }

    // 2. mask fill value and edge statistics (data with masked pixels set to the median of the rest)
    double fill = 0.0;
    if (msk) {
      const int P = pow2_at_least(npix);
      double cnt[1] = {0.0};
      for (int i = threadIdx.x; i < P; i += blockDim.x) {
        const bool ok = i < npix && !msk[i];
        pv[i] = ok ? (double)d[i] : INFINITY;
        cnt[0] += ok ? 1.0 : 0.0;
      }
      block_sum4(S, cnt, 1);  // (also the barrier before the sort)
      sort_keys(pv, P);
      fill = median_sorted(pv, (int)cnt[0]);
      __syncthreads();
    }
    auto dat = [&](int r, int c) -> double {
      const int64_t i = (int64_t)r * nx + c;
      return (msk && msk[i]) ? fill : (double)d[i];
    };
    const int ne = 2 * (nx + ny);
    {
      const int P = pow2_at_least(ne);
      for (int i = threadIdx.x; i < P; i += blockDim.x) {
        double v = INFINITY;
        if (i < ny) v = dat(i, 0);
        else if (i < 2 * ny) v = dat(i - ny, nx - 1);
        else if (i < 2 * ny + nx) v = dat(0, i - 2 * ny);
        else if (i < ne) v = dat(ny - 1, i - 2 * ny - nx);
        pv[i] = v;
      }
      __syncthreads();
      sort_keys(pv, P);
    }
    const double edge_avg = median_sorted(pv, ne);
    const double edge_scatter = iqr_half_sorted(pv, ne);
    __syncthreads();

    // 3. PA: angular centre of light of (dat - edge median)
    if (!know_pa) {
      double v[3] = {0, 0, 0};
      for (int i = threadIdx.x; i < npix; i += blockDim.x) {
        if (msk && msk[i]) continue;
        const int r = i / nx, c = i % nx;
        const double X = ((c + 0.5) * g.s + g.ox) - cx, Y = ((r + 0.5) * g.s + g.oy) - cy;
        const double w = dat(r, c) - edge_avg;
        // cos 2θ, sin 2θ of θ = atan2(Y, X) as (X² - Y²) / r², 2XY / r² (θ = 0 at r = 0)
        const double r2 = X * X + Y * Y;
        const double c2 = r2 > 0 ? (X * X - Y * Y) / r2 : 1.0;
        const double s2 = r2 > 0 ? (2 * X * Y) / r2 : 0.0;
        v[0] += w * c2;
        v[1] += w * s2;
        v[2] += w;
      }
      block_sum4(S, v, 3);
      const double pa0 = pymod(atan2(v[1] / v[2], v[0] / v[2]) / 2, kPi);
      PA = pymod(pa0 + kNorth, kPi);
      PA = 0.0 + pymod(PA - 0.0, kPi);
    }
    const double pa = PA - kNorth;

    // 4. q: the flattest isophote at the radius where the light reaches 3 edge sigma
    if (!know_q) {
      const double icx = (cx - g.ox) / g.s - 0.5, icy = (cy - g.oy) / g.s - 0.5;
      const double ccx = icy, ccy = icx;  // the reference's transposed centre
      const double thr = 3 * edge_scatter;
      const double qmax = 0.9;
      // the isophotes read data - edge median (raw data: masked pixels keep their values)
      for (int i = threadIdx.x; i < npix; i += blockDim.x) pv[i] = (double)d[i] - edge_avg;
      __syncthreads();
      double r = 1.0;
      int count = 1;
      while (r < fmax((double)nx, (double)ny) / 2) {
        r = r * (1 + 0.2);
        ++count;
        int nk;
        const int n = iso_extract(S, B, pv, nx, ny, r, qmax, pa, ccx, ccy, false, &nk);
        if (nk < 3) continue;
        const double q80 = pct_sorted(B.srt, nk, 0.8);
        __syncthreads();
        (void)n;
        if (q80 < thr && count > 4) break;
      }
      const double R = r;
      const double qstep = (0.9 - 0.2) / 14.0;  // np.linspace(0.2, 0.9, 15)
      int good_last = -1;
      unsigned short_mask = 0;  // isophotes with fewer than 3 samples
      for (int qi = 0; qi < kQSamples; ++qi) {
        const double qv = qi == kQSamples - 1 ? 0.9 : qi * qstep + 0.2;
        int nk;
        const int n = iso_extract(S, B, pv, nx, ny, R, qv, pa, ccx, ccy, true, &nk);
        if (n < 3) {
          short_mask |= 1u << qi;
          continue;
        }
        good_last = qi;
        // second DFT coefficient over the ellipse order, median and iqr of the fluxes
        double v[2] = {0, 0};
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
          double s2, c2;
          sincospi((double)(2 * 2 * (int64_t)i % (2 * n)) / n, &s2, &c2);  // angle 2 pi 2 i / n
          v[0] += B.fl[i] * c2;
          v[1] -= B.fl[i] * s2;
        }
        block_sum4(S, v, 2);
        const int P = pow2_at_least(n);
        for (int i = threadIdx.x; i < P; i += blockDim.x) B.srt[i] = i < n ? B.fl[i] : INFINITY;
        __syncthreads();
        sort_keys(B.srt, P);
        if (threadIdx.x == 0) {
          const double med = median_sorted(B.srt, n);
          const double noise = iqr_half_sorted(B.srt, n);
          S.amp[qi] = hypot(v[0], v[1]) / (n * ((med > 0 ? med : 0.0) + noise));
        }
        __syncthreads();
      }
      if (threadIdx.x == 0) {
        int best = 0;
        if (good_last < 0) {
          S.i[1] = AP_INIT_NO_ISOPHOTE;
          best = kQSamples - 1;
        } else {
          S.i[1] = 0;
          // isophotes with fewer than 3 samples take the last good one's amplitude; np.argmin
          // returns the first minimum, or the first NaN
          double a[kQSamples];
          for (int qi = 0; qi < kQSamples; ++qi) a[qi] = ((short_mask >> qi) & 1) ? S.amp[good_last] : S.amp[qi];
          best = 0;
          for (int qi = 1; qi < kQSamples; ++qi) {
            if (isnan(a[best])) break;
            if (isnan(a[qi]) || a[qi] < a[best]) best = qi;
          }
        }
        const double qb = best == kQSamples - 1 ? 0.9 : best * qstep + 0.2;
        S.d[2] = soft_hi(soft_lo(qb, 0.0), 1.0);
      }
      __syncthreads();
      q = S.d[2];
      status |= S.i[1];
      __syncthreads();
    }

    // 5. n, Re, Ie: binned median profile of the inclined radius, then Nelder-Mead
    const int pslot[3] = {PN, PRE, PIE};
    const int dim = A.kind == AP_PROFILE_SERSIC ? 3 : 2;
    const int* fslot = A.kind == AP_PROFILE_SERSIC ? pslot : pslot + 1;
    bool need_fit = false;
    for (int k = 0; k < dim; ++k) need_fit |= !((A.known >> fslot[k]) & 1);
    if (need_fit) {
      const double ca = cos(-pa), sa = sin(-pa);
      constexpr double soft2 = 1e-3 * 1e-3;
      double mn = INFINITY, mx = -INFINITY;
      for (int i = threadIdx.x; i < npix; i += blockDim.x) {
        const int r = i / nx, c = i % nx;
        const double X = ((c + 0.5) * g.s + g.ox) - cx, Y = ((r + 0.5) * g.s + g.oy) - cy;
        const double Xr = ca * X - sa * Y, Yr = (sa * X + ca * Y) / q;
        const double R = sqrt((Xr * Xr + Yr * Yr) + soft2);
        pv[i] = R;  // read back by the binning pass (same thread, same index)
        mn = fmin(mn, R);
        mx = fmax(mx, R);
      }
      block_minmax(S, mn, mx);
      if (threadIdx.x == 0) {
        const double lo = log10(mn * 0.9), hi = log10(mx * 1.1);
        const double stp = (hi - lo) / 10;
        for (int k = 0; k < kBins; ++k) S.edges[k] = pow(10.0, k * stp + lo);
        S.edges[kBins] = pow(10.0, hi);
      }
      if (threadIdx.x < kBins) S.bin_cnt[threadIdx.x] = 0;
      __syncthreads();
      const int P = pow2_at_least(npix);
      for (int i = threadIdx.x; i < P; i += blockDim.x) {
        uint8_t b = 255;
        double v = INFINITY;
        if (i < npix) {
          const int r = i / nx, c = i % nx;
          const double R = pv[i];
          int k = 0;  // searchsorted(edges, R, 'right') - 1
          while (k < kBins && S.edges[k + 1] <= R) ++k;
          if (R < S.edges[0]) k = -1;
          if (k >= 0 && k < kBins) {
            b = (uint8_t)k;
            atomicAdd(&S.bin_cnt[k], 1);
          }
          v = dat(r, c) - edge_avg;
        }
        pb[i] = b;
        pv[i] = v;
      }
      __syncthreads();
      sort_binned(pb, pv, P);
      if (threadIdx.x == 0) {
        int acc = 0;
        for (int k = 0; k < kBins; ++k) {
          S.bin_start[k] = acc;
          acc += S.bin_cnt[k];
        }
        for (int k = 0; k < kBins; ++k) {
          S.prof_I[k] = median_sorted(pv + S.bin_start[k], S.bin_cnt[k]) / g.area;
          S.prof_R[k] = (S.edges[k] + S.edges[k + 1]) / 2;
        }
        double* I = S.prof_I;
        double mpos = INFINITY;
        bool any = false;
        for (int k = 0; k < kBins; ++k)
          if (isfinite(I[k]) && I[k] > 0) {
            mpos = fmin(mpos, I[k]);
            any = true;
          }
        int st2 = 0;
        if (!any) st2 |= AP_INIT_NO_PROFILE;
        for (int k = 0; k < kBins; ++k)
          if (I[k] <= 0) I[k] = mpos;
        for (int k = 5; k < kBins; ++k)
          if (I[k] >= I[k - 1] && isfinite(I[k - 1])) I[k] = I[k - 1] - fabs(I[k - 1] * 0.1);
        for (int k = 0; k < kBins; ++k) I[k] = log10(I[k]);
        // non-finite bins: linear interpolation over the finite ones
        double xr[kBins], fr[kBins];
        int m = 0;
        for (int k = 0; k < kBins; ++k)
          if (isfinite(I[k])) {
            xr[m] = S.prof_R[k];
            fr[m] = I[k];
            ++m;
          }
        if (m == 0) st2 |= AP_INIT_NO_PROFILE;
        for (int k = 0; k < kBins && m > 0; ++k)
          if (!isfinite(I[k])) I[k] = interp_sorted(S.prof_R[k], xr, fr, m);
        S.i[2] = st2;
      }
      __syncthreads();
      status |= S.i[2];
    }

    // 6. park the stamp until its chunk's fits run
    if (threadIdx.x == 0) {
      ChunkSlot& cs = S.slot[j];
      cs.st = st;
      cs.cx = cx;
      cs.cy = cy;
      cs.q = q;
      cs.PA = PA;
      cs.status = status;
      cs.need_fit = need_fit ? 1 : 0;
      if (need_fit) {
        for (int k = 0; k < kBins; ++k) {
          cs.R[k] = S.prof_R[k];
          cs.I[k] = S.prof_I[k];
        }
        if (A.kind == AP_PROFILE_SERSIC) {
          cs.x0[0] = 2.0;
          cs.x0[1] = S.prof_R[4];
          cs.x0[2] = S.prof_I[4];
        } else {
          cs.x0[0] = S.prof_R[4];
          cs.x0[1] = S.prof_I[4];
          cs.x0[2] = 0.0;
        }
        for (int k = 0; k < dim; ++k)
          if ((A.known >> fslot[k]) & 1) cs.x0[k] = prm[fslot[k]];
      }
    }
    __syncthreads();
  }

  __syncthreads();
  // 7. Nelder-Mead on the binned profiles, one warp per stamp, and the values written out
  {
    const int w = threadIdx.x >> 5;
    const ChunkSlot& cs = S.slot[w];
    if (cs.st >= 0) {
      const int dim = A.kind == AP_PROFILE_SERSIC ? 3 : 2;
      const int pslot[3] = {PN, PRE, PIE};
      const int* fslot = A.kind == AP_PROFILE_SERSIC ? pslot : pslot + 1;
      double* prm = A.params + (int64_t)cs.st * NPARAM;
      int status = cs.status;
      double fitv[3] = {0, 0, 0};
      if (cs.need_fit) {
        // lanes 10 g + b hold bin b for the point of lane group g
        const double Rb = lane < 3 * kBins ? cs.R[lane % kBins] : 0.0;
        const double Ib = lane < 3 * kBins ? cs.I[lane % kBins] : 0.0;
        const NMResult res = nelder_mead(A.kind, dim, Rb, Ib, cs.x0);
        double fit[3];
        for (int k = 0; k < 3; ++k) fit[k] = res.success ? res.x[k] : cs.x0[k];
        if (!res.success) status |= AP_INIT_FIT_LIMIT;
        if (A.kind == AP_PROFILE_SERSIC) {
          fitv[0] = soft_hi(soft_lo(fit[0], 0.36), 8.0);
          fitv[1] = soft_lo(fit[1], 0.0);
          fitv[2] = fit[2];
        } else {
          fitv[0] = soft_lo(fit[0], 0.0);
          fitv[1] = fit[1];
        }
      }
      if (lane == 0) {
        if ((A.known & 3) != 3) {
          prm[PX] = cs.cx;
          prm[PY] = cs.cy;
        }
        if (!((A.known >> PPA) & 1)) prm[PPA] = cs.PA;
        if (!((A.known >> PQ) & 1)) prm[PQ] = cs.q;
        if (cs.need_fit)
          for (int k = 0; k < dim; ++k)
            if (!((A.known >> fslot[k]) & 1)) prm[fslot[k]] = fitv[k];
        A.status[cs.st] = status;
      }
    }
  }
  __syncthreads();
  }
}

}  // namespace

// largest isophote length the sampler can see on an nx x ny stamp (the growth loop's last radius)
static int iso_cap_for(int nx, int ny) {
  double r = 1.0;
  while (r < std::fmax((double)nx, (double)ny) / 2) r = r * (1 + 0.2);
  const int N = std::max(15, (int)(((0.9 * 2) * kPi) * r));
  int p = 32;
  while (p < N) p <<= 1;
  return p;
}

RefInitPlan plan_reference_init(const StampDev* host_stamps, int32_t n) {
  RefInitPlan P{};
  int pix = 1, iso = 32;
  for (int i = 0; i < n; ++i) {
    const int nx = host_stamps[i].nx, ny = host_stamps[i].ny;
    pix = std::max(pix, std::max(nx * ny, 2 * (nx + ny)));
    iso = std::max(iso, iso_cap_for(nx, ny));
  }
  int p = 1;
  while (p < pix) p <<= 1;
  P.iso_cap = iso;
  P.pix_cap = p;
  const size_t iso_bytes = sizeof(double) * 7 * (size_t)iso;
  const size_t pix_bytes = (sizeof(double) + 1) * (size_t)p;
  P.pix_in_smem = iso_bytes + pix_bytes <= kRefInitSmemBudget;
  P.smem = iso_bytes + (P.pix_in_smem ? pix_bytes : 0);
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaFuncSetAttribute(k_reference_init, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P.smem);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_reference_init, kInitThreads, P.smem) != cudaSuccess ||
      per < 1)
    per = 1;
  if (sms < 1) sms = 1;
  const long long chunks = ((long long)n + kInitWarps - 1) / kInitWarps;
  P.grid = (int)std::max<long long>(1, std::min<long long>((long long)sms * per, chunks));
  P.scratch_bytes = P.pix_in_smem ? 0 : (int64_t)pix_bytes * P.grid;
  return P;
}

cudaError_t launch_reference_init(const RefInitPlan& P, const StampDev* stamps, int32_t n, int32_t kind,
                                  int32_t known, const float* data, const uint8_t* mask, double* params,
                                  int32_t* status, void* scratch, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  InitArgs A{};
  A.stamps = stamps;
  A.n = n;
  A.kind = kind;
  A.known = known;
  A.data = data;
  A.mask = mask;
  A.params = params;
  A.status = status;
  A.iso_cap = P.iso_cap;
  A.pix_cap = P.pix_cap;
  A.pix_in_smem = P.pix_in_smem;
  if (!P.pix_in_smem) {
    if (!scratch) return cudaErrorInvalidValue;
    A.pix_val_g = (double*)scratch;
    A.pix_bin_g = (uint8_t*)((char*)scratch + sizeof(double) * (size_t)P.pix_cap * P.grid);
  }
  cudaError_t e = cudaFuncSetAttribute(k_reference_init, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P.smem);
  if (e != cudaSuccess) return e;
  k_reference_init<<<P.grid, kInitThreads, P.smem, st>>>(A);
  return cudaGetLastError();
}

}  // namespace apgb
