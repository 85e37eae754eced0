// Scenes: many sources on one image fitted jointly (Group_Model + LM over the joint vector).
//
// Each source is rendered by an ap_batch stamp (its own window for the Jacobian, the group's
// window for the model image, as Group_Model.sample does).  These kernels combine the stamps:
//   forward   image = sky + sum of the sources' renders inside their own windows
//             (Group_Model.sample, astrophot/models/group_model_object.py:183-231)
//   hess      H = J^T W J over the joint vector, one block per pair of overlapping windows
//   jt        J^T v for an image v (gradient, geodesic-acceleration right-hand side)
//   jvp       J h as an image
//   chi2      sum of W (Y - M)^2 over unmasked pixels (LM._chi2, astrophot/fit/lm.py:374-378),
//             block partial sums added in a fixed order
//   solve     the damped system of LM._h (astrophot/fit/lm.py:361-371) for a dense P x P
//             matrix: blocked Cholesky in FP64 plus two triangular solves
// Linked parameters (one node shared by several sources) are one entry of the joint vector:
// every source slot names its joint index, so their Jacobian columns add up (the merge by
// identity of Jacobian_Image, astrophot/image/jacobian_image.py:36-37, 79-118).
#include <cuda_runtime.h>
#include <stdint.h>

#include "ap_internal.h"

using apgb::record_cuda;

namespace {

constexpr int kSceneTile = 32;
constexpr int kMaxSlots = 8;

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ bool in_window(const ap_scene_source& s, int x, int y) {
  return x >= s.x0 && x < s.x0 + s.wx && y >= s.y0 && y < s.y0 + s.wy;
}

// ---- forward: image = sky + sum over the tile's sources (fixed order: deterministic) -------------
__global__ void k_scene_forward(const ap_scene_source* __restrict__ src, const int32_t* __restrict__ tile_ptr,
                                const int32_t* __restrict__ tile_src, const float* __restrict__ fwd, float sky,
                                const double* __restrict__ sky_F, const double* __restrict__ sky_F0, double area,
                                int nx, int ny, float* __restrict__ image) {
  if (sky_F) {
    // a free flat sky: pixel_area 10^F counts per pixel, from the staged F (float64, then
    // rounded); for difference renders the sky's change area 10^F0 (10^(F - F0) - 1)
    __shared__ float s_sky;
    if (threadIdx.x == 0) {
      constexpr double kLn10 = 2.302585092994045684;
      s_sky = sky_F0 ? (float)(area * pow(10.0, *sky_F0) * expm1(kLn10 * (*sky_F - *sky_F0)))
                     : (float)(area * pow(10.0, *sky_F));
    }
    __syncthreads();
    sky = s_sky;
  }
  const int tx = blockIdx.x % ((nx + kSceneTile - 1) / kSceneTile);
  const int ty = blockIdx.x / ((nx + kSceneTile - 1) / kSceneTile);
  const int t = blockIdx.x;
  const int b = tile_ptr[t], e = tile_ptr[t + 1];
  for (int i = threadIdx.x; i < kSceneTile * kSceneTile; i += blockDim.x) {
    const int x = tx * kSceneTile + (i % kSceneTile), y = ty * kSceneTile + (i / kSceneTile);
    if (x >= nx || y >= ny) continue;
    float v = sky;
    for (int k = b; k < e; ++k) {
      const ap_scene_source& s = src[tile_src[k]];
      if (in_window(s, x, y)) v += fwd[s.fwd_off + (int64_t)(y - s.fwd_y0) * s.fwd_nx + (x - s.fwd_x0)];
    }
    image[(int64_t)y * nx + x] = v;
  }
}

// ---- jvp: out = J h on the image (own windows) -------------------------------------------------
__global__ void k_scene_jvp(const ap_scene_source* __restrict__ src, const int32_t* __restrict__ tile_ptr,
                            const int32_t* __restrict__ tile_src, const float* __restrict__ jac,
                            const double* __restrict__ h, int nx, int ny, float* __restrict__ out) {
  const int ntx = (nx + kSceneTile - 1) / kSceneTile;
  const int tx = blockIdx.x % ntx, ty = blockIdx.x / ntx;
  const int b = tile_ptr[blockIdx.x], e = tile_ptr[blockIdx.x + 1];
  for (int i = threadIdx.x; i < kSceneTile * kSceneTile; i += blockDim.x) {
    const int x = tx * kSceneTile + (i % kSceneTile), y = ty * kSceneTile + (i / kSceneTile);
    if (x >= nx || y >= ny) continue;
    float v = 0.f;
    for (int k = b; k < e; ++k) {
      const ap_scene_source& s = src[tile_src[k]];
      if (!in_window(s, x, y)) continue;
      const int64_t p = s.jac_off + (int64_t)(y - s.y0) * s.wx + (x - s.x0);
      for (int c = 0; c < s.n_free; ++c) v = fmaf(jac[p + c * s.jac_stride], (float)h[s.gidx[c]], v);
    }
    out[(int64_t)y * nx + x] = v;
  }
}

// ---- jt: out[g] += sum over the source's window of J_c(p) v(p) -----------------------------------
// With `part` (n_sources x kMaxSlots doubles), each source's sums go to its own slots instead
// of being added into out: ap_gather_sum then adds them in a fixed order.
__global__ void k_scene_jt(const ap_scene_source* __restrict__ src, const float* __restrict__ jac,
                           const float* __restrict__ v, int nx, double* __restrict__ out,
                           double* __restrict__ part) {
  const ap_scene_source& s = src[blockIdx.x];
  double acc[kMaxSlots];
#pragma unroll
  for (int c = 0; c < kMaxSlots; ++c) acc[c] = 0.0;
  const int64_t n = (int64_t)s.wx * s.wy;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const int lx = (int)(i % s.wx), ly = (int)(i / s.wx);
    const float vi = v[(int64_t)(s.y0 + ly) * nx + (s.x0 + lx)];
#pragma unroll
    for (int c = 0; c < kMaxSlots; ++c)
      if (c < s.n_free) acc[c] += (double)(jac[s.jac_off + i + c * s.jac_stride] * vi);
  }
  __shared__ double sh[kMaxSlots][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int c = 0; c < kMaxSlots; ++c) {
    const double r = warp_sum(acc[c]);
    if (lane == 0) sh[c][w] = r;
  }
  __syncthreads();
  if (threadIdx.x < s.n_free) {
    double t = 0.0;
    for (int k = 0; k < nw; ++k) t += sh[threadIdx.x][k];
    if (part) part[(int64_t)blockIdx.x * kMaxSlots + threadIdx.x] = t;
    else atomicAdd(out + s.gidx[threadIdx.x], t);
  }
}

// ---- hess: one block per overlapping pair (a <= b): H[ga][gb] += sum J_a W J_b --------------------
__global__ void __launch_bounds__(256) k_scene_hess(const ap_scene_source* __restrict__ src,
                                                    const int32_t* __restrict__ pairs, const float* __restrict__ jac,
                                                    const float* __restrict__ weight, const uint8_t* __restrict__ mask,
                                                    int nx, int P, double* __restrict__ H, double* __restrict__ part) {
  const ap_scene_source& A = src[pairs[2 * blockIdx.x]];
  const ap_scene_source& B = src[pairs[2 * blockIdx.x + 1]];
  const bool same = pairs[2 * blockIdx.x] == pairs[2 * blockIdx.x + 1];
  const int x0 = max(A.x0, B.x0), x1 = min(A.x0 + A.wx, B.x0 + B.wx);
  const int y0 = max(A.y0, B.y0), y1 = min(A.y0 + A.wy, B.y0 + B.wy);
  const int ow = x1 - x0, oh = y1 - y0;
  float acc[kMaxSlots][kMaxSlots];
#pragma unroll
  for (int i = 0; i < kMaxSlots; ++i)
#pragma unroll
    for (int j = 0; j < kMaxSlots; ++j) acc[i][j] = 0.f;
  if (ow > 0 && oh > 0) {
    const int64_t n = (int64_t)ow * oh;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
      const int x = x0 + (int)(i % ow), y = y0 + (int)(i / ow);
      const int64_t ip = (int64_t)y * nx + x;
      if (mask && mask[ip]) continue;
      const float w = weight ? weight[ip] : 1.f;
      const int64_t pa = A.jac_off + (int64_t)(y - A.y0) * A.wx + (x - A.x0);
      const int64_t pb = B.jac_off + (int64_t)(y - B.y0) * B.wx + (x - B.x0);
      float ja[kMaxSlots], jb[kMaxSlots];
#pragma unroll
      for (int c = 0; c < kMaxSlots; ++c) {
        ja[c] = c < A.n_free ? jac[pa + c * A.jac_stride] * w : 0.f;
        jb[c] = c < B.n_free ? jac[pb + c * B.jac_stride] : 0.f;
      }
#pragma unroll
      for (int a = 0; a < kMaxSlots; ++a)
#pragma unroll
        for (int c = 0; c < kMaxSlots; ++c) acc[a][c] = fmaf(ja[a], jb[c], acc[a][c]);
    }
  }
  __shared__ double sh[kMaxSlots * kMaxSlots][8];
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int a = 0; a < kMaxSlots; ++a)
#pragma unroll
    for (int c = 0; c < kMaxSlots; ++c) {
      const double r = warp_sum((double)acc[a][c]);
      if (lane == 0) sh[a * kMaxSlots + c][wp] = r;
    }
  __syncthreads();
  for (int k = threadIdx.x; k < kMaxSlots * kMaxSlots; k += blockDim.x) {
    const int a = k / kMaxSlots, c = k % kMaxSlots;
    if (a >= A.n_free || c >= B.n_free) continue;
    double t = 0.0;
    for (int q = 0; q < nw; ++q) t += sh[k][q];
    if (part) {  // the pair's block, summed into H by ap_gather_sum in a fixed order
      part[(int64_t)blockIdx.x * kMaxSlots * kMaxSlots + k] = t;
      continue;
    }
    const int ga = A.gidx[a], gb = B.gidx[c];
    atomicAdd(H + (int64_t)ga * P + gb, t);
    if (!same) atomicAdd(H + (int64_t)gb * P + ga, t);
  }
}

// out[entry[e]] = sum of part[contrib[k]], k in [ptr[e], ptr[e + 1]), in that order
__global__ void k_gather_sum(int64_t n_entries, const int64_t* __restrict__ entry, const int32_t* __restrict__ ptr,
                             const int32_t* __restrict__ contrib, const double* __restrict__ part,
                             double* __restrict__ out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n_entries;
       e += (int64_t)gridDim.x * blockDim.x) {
    double t = 0.0;
    for (int k = ptr[e]; k < ptr[e + 1]; ++k) t += part[contrib[k]];
    out[entry[e]] = t;
  }
}

// ---- chi2 and residual images --------------------------------------------------------------------
// chi^2 in two passes with a fixed summation order (the same bits on every run): block b sums
// the pixels [b chunk, (b + 1) chunk) into part[b], then one block sums the parts in order.  The
// float64 arithmetic per pixel is spread over the whole GPU (its float64 pipe is narrow).
// With `base`, model holds a difference dm to the model base and the sum is chi^2's change
// W dm (dm - 2 (data - base)), accurate relative to the change itself.
__global__ void __launch_bounds__(256) k_scene_chi2_part(const float* __restrict__ model, const float* __restrict__ base,
                                                         const float* __restrict__ data,
                                                         const float* __restrict__ weight,
                                                         const uint8_t* __restrict__ mask, int64_t n, int64_t chunk,
                                                         double* __restrict__ part) {
  const int64_t lo = (int64_t)blockIdx.x * chunk, hi = lo + chunk < n ? lo + chunk : n;
  double acc = 0.0;
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    if (mask && mask[i]) continue;
    const double w = weight ? (double)weight[i] : 1.0;
    if (base) {
      const double dm = (double)model[i], r = (double)data[i] - (double)base[i];
      acc += w * dm * (dm - 2.0 * r);
    } else {
      const double r = (double)data[i] - (double)model[i];
      acc += w * r * r;
    }
  }
  acc = warp_sum(acc);
  __shared__ double sh[8];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
    part[blockIdx.x] = t;
  }
}

__global__ void k_sum_parts(const double* __restrict__ part, int m, double* __restrict__ out) {
  double acc = 0.0;
  for (int k = threadIdx.x; k < m; k += blockDim.x) acc += part[k];
  acc = warp_sum(acc);
  __shared__ double sh[32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
    *out = t;
  }
}

// ---- a PSF finer than the image: fine renders summed back in u x u blocks ----------------------
// (Image.reduce after the crop of the working image, astrophot/image/image_object.py:348-376,
// models/model_object.py:346-350).  One thread per (plane, coarse pixel); the stamp of a coarse
// pixel by binary search over the coarse offsets.
__global__ void k_reduce_upscaled(int n_stamps, const int64_t* __restrict__ in_off, const int64_t* __restrict__ out_off,
                                  const int32_t* __restrict__ cnx, int u, int n_planes, const float* __restrict__ in,
                                  int64_t in_stride, float* __restrict__ out, int64_t out_stride, int64_t out_total) {
  const int64_t n = (int64_t)n_planes * out_total;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t pl = t / out_total, i = t - pl * out_total;
    int lo = 0, hi = n_stamps - 1;
    while (lo < hi) {  // last stamp whose coarse offset is <= i
      const int mid = (lo + hi + 1) >> 1;
      if (out_off[mid] <= i) lo = mid;
      else hi = mid - 1;
    }
    const int64_t local = i - out_off[lo];
    const int w = cnx[lo];
    const int64_t cy = local / w, cx = local - cy * w;
    const int64_t fw = (int64_t)w * u;
    const float* src = in + pl * in_stride + in_off[lo] + (cy * u) * fw + cx * u;
    float acc = 0.f;
    for (int b = 0; b < u; ++b)
      for (int a = 0; a < u; ++a) acc += src[(int64_t)b * fw + a];
    out[pl * out_stride + i] = acc;
  }
}

// r = W (Y - M) on unmasked pixels, 0 elsewhere (LM._r, astrophot/fit/lm.py:381-385)
__global__ void k_scene_residual(const float* __restrict__ model, const float* __restrict__ data,
                                 const float* __restrict__ weight, const uint8_t* __restrict__ mask, int64_t n,
                                 float* __restrict__ r) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const bool m = mask && mask[i];
    r[i] = m ? 0.f : (weight ? weight[i] : 1.f) * (data[i] - model[i]);
  }
}

// geodesic-acceleration right-hand side image (astrophot/fit/lm.py:286-291):
// out = (2/d) ((rh - r)/d - W (J h)) on unmasked pixels
__global__ void k_scene_rpp(const float* __restrict__ r, const float* __restrict__ rh, const float* __restrict__ jh,
                            const float* __restrict__ weight, const uint8_t* __restrict__ mask, double d, int64_t n,
                            float* __restrict__ out) {
  const float fd = (float)d;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const bool m = mask && mask[i];
    const float w = weight ? weight[i] : 1.f;
    out[i] = m ? 0.f : (2.f / fd) * ((rh[i] - r[i]) / fd - w * jh[i]);
  }
}

// ---- dense damped solve ----------------------------------------------------------------------------
// A = H o (I + D / (1 + L)) + L I (1 + diag H) (lower triangle written, used by the factorisation)
__global__ void k_damp(const double* __restrict__ H, double L, int n, double* __restrict__ A) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(k / n), j = (int)(k % n);
    const double h = H[k];
    A[k] = (i == j) ? h + L * (1.0 + h) : h / (1.0 + L);
  }
}

constexpr int kNB = 32;

__device__ __forceinline__ double warp_sum_d(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Factor the nb x nb diagonal block D (lower Cholesky, in shared memory) with one warp, lane =
// row.  A non-positive or non-finite pivot records info = 1 + row (the first one, when
// `report`) and continues with pivot 1.
__device__ void chol_diag_warp(double (*D)[kNB + 1], int nb, int k0, int* info, bool report) {
  const int lane = threadIdx.x & 31;
  for (int j = 0; j < nb; ++j) {
    if (lane == j) {
      const double d = D[j][j];
      if (!(d > 0.0) || !isfinite(d)) {
        if (report) atomicCAS(info, 0, 1 + k0 + j);
        D[j][j] = 1.0;
      } else {
        D[j][j] = sqrt(d);
      }
    }
    __syncwarp();
    const double djj = D[j][j];
    if (lane > j && lane < nb) D[lane][j] /= djj;
    __syncwarp();
    if (lane > j && lane < nb) {
      const double lij = D[lane][j];
      for (int c = j + 1; c <= lane; ++c) D[lane][c] -= lij * D[c][j];
    }
    __syncwarp();
  }
}

// Column step k0: every block (one warp) factors the diagonal block itself, from A, and solves
// its 32 rows of the panel below (X L^T = A[k0+nb:, k0:k0+nb], lane = row).  The factored
// diagonal block goes to dscr (block 0), copied into A by the trailing update, which reads no
// diagonal entry: A's diagonal block stays unmodified while the other blocks read it.  On the
// last step (no rows below, one block) it is written into A directly.
__global__ void __launch_bounds__(32) k_chol_panel(double* __restrict__ A, int n, int k0, int* __restrict__ info,
                                                   double* __restrict__ dscr) {
  __shared__ double D[kNB][kNB + 1];
  const int nb = min(kNB, n - k0);
  const int lane = threadIdx.x;
  for (int i = 0; i < nb; ++i)
    if (lane < nb) D[i][lane] = A[(int64_t)(k0 + i) * n + k0 + lane];
  __syncwarp();
  chol_diag_warp(D, nb, k0, info, blockIdx.x == 0);
  const bool last = (k0 + nb >= n);
  if (blockIdx.x == 0 && lane < nb) {
    for (int i = 0; i < nb; ++i) {
      const double v = lane <= i ? D[i][lane] : 0.0;
      if (last)
        A[(int64_t)(k0 + i) * n + k0 + lane] = v;
      else
        dscr[i * kNB + lane] = v;
    }
  }
  const int r = k0 + nb + blockIdx.x * 32 + lane;
  if (r >= n) return;
  double x[kNB];
  double* row = A + (int64_t)r * n + k0;
#pragma unroll
  for (int j = 0; j < kNB; ++j) {
    if (j >= nb) break;
    double v = row[j];
#pragma unroll
    for (int c = 0; c < j; ++c) v -= x[c] * D[j][c];
    x[j] = v / D[j][j];
  }
#pragma unroll
  for (int j = 0; j < kNB; ++j)
    if (j < nb) row[j] = x[j];
}

// trailing update: A[i][j] -= sum_c P[i][c] P[j][c] for k0 + nb <= j <= i (tiles of 32 x 32);
// block (0, 0) also stores the factored diagonal block of this step from dscr
__global__ void k_chol_update(double* __restrict__ A, int n, int k0, const double* __restrict__ dscr) {
  const int nb = min(kNB, n - k0);
  const int base = k0 + nb;
  const int ti = blockIdx.y, tj = blockIdx.x;
  if (tj > ti) return;
  if (ti == 0 && tj == 0) {
    for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {
      const int r = t / nb, c = t % nb;
      A[(int64_t)(k0 + r) * n + k0 + c] = dscr[r * kNB + c];
    }
  }
  __shared__ double Pi[kNB][kNB + 1], Pj[kNB][kNB + 1];
  const int i0 = base + ti * kNB, j0 = base + tj * kNB;
  for (int t = threadIdx.x; t < kNB * kNB; t += blockDim.x) {
    const int r = t / kNB, c = t % kNB;
    Pi[r][c] = (i0 + r < n && c < nb) ? A[(int64_t)(i0 + r) * n + k0 + c] : 0.0;
    Pj[r][c] = (j0 + r < n && c < nb) ? A[(int64_t)(j0 + r) * n + k0 + c] : 0.0;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < kNB * kNB; t += blockDim.x) {
    const int r = t / kNB, c = t % kNB;
    const int i = i0 + r, j = j0 + c;
    if (i >= n || j >= n || j > i) continue;
    double s = 0.0;
#pragma unroll 8
    for (int q = 0; q < kNB; ++q) s += Pi[r][q] * Pj[c][q];
    A[(int64_t)i * n + j] -= s;
  }
}

// the lower nb x nb diagonal block at kb into shared memory (upper part zero)
__device__ __forceinline__ void load_diag(const double* __restrict__ A, int n, int kb, int nb,
                                          double (*D)[kNB + 1]) {
  for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {
    const int i = t / nb, c = t % nb;
    D[i][c] = (c <= i) ? A[(int64_t)(kb + i) * n + kb + c] : 0.0;
  }
}

// Forward substitution L z = b, column block kb: every block solves the small triangle for
// z[kb..kb+nb) from y (warp 0, shuffles; block 0 stores it), then the rows below are updated,
// y[i] -= L[i][kb..kb+nb) . z_kb, one warp per row (coalesced row segments).  Blocks read only
// y[kb..kb+nb) and write only rows beyond it.
__global__ void __launch_bounds__(256) k_trsv_fwd(const double* __restrict__ A, int n, int kb,
                                                  double* __restrict__ y, double* __restrict__ z) {
  __shared__ double D[kNB][kNB + 1];
  __shared__ double zb[kNB];
  const int nb = min(kNB, n - kb);
  load_diag(A, n, kb, nb, D);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0) {
    double v = lane < nb ? y[kb + lane] : 0.0;
    for (int c = 0; c < nb; ++c) {
      if (lane == c) v = v / D[c][c];
      const double vc = __shfl_sync(0xffffffffu, v, c);
      if (lane > c && lane < nb) v -= D[lane][c] * vc;
    }
    if (lane < nb) {
      zb[lane] = v;
      if (blockIdx.x == 0) z[kb + lane] = v;
    }
  }
  __syncthreads();
  const int nw = blockDim.x >> 5;
  for (int i = kb + nb + blockIdx.x * nw + warp; i < n; i += gridDim.x * nw) {
    double p = lane < nb ? A[(int64_t)i * n + kb + lane] * zb[lane] : 0.0;
    p = warp_sum_d(p);
    if (lane == 0) y[i] -= p;
  }
}

// Back substitution L^T x = z (z updated in place as the right-hand side), column block kb
// from the last: x[kb..kb+nb) from z (warp 0; block 0 stores it), then z[i] -= sum_c
// L[kb+c][i] x_kb[c] for i < kb, one thread per row (coalesced over i).
__global__ void __launch_bounds__(256) k_trsv_bwd(const double* __restrict__ A, int n, int kb,
                                                  double* __restrict__ z, double* __restrict__ x) {
  __shared__ double D[kNB][kNB + 1];
  __shared__ double xb[kNB];
  const int nb = min(kNB, n - kb);
  load_diag(A, n, kb, nb, D);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0) {
    // L^T's diagonal block is upper triangular: rows from the bottom up
    double v = lane < nb ? z[kb + lane] : 0.0;
    for (int c = nb - 1; c >= 0; --c) {
      if (lane == c) v = v / D[c][c];
      const double vc = __shfl_sync(0xffffffffu, v, c);
      if (lane < c) v -= D[c][lane] * vc;
    }
    if (lane < nb) {
      xb[lane] = v;
      if (blockIdx.x == 0) x[kb + lane] = v;
    }
  }
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kb; i += gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int c = 0; c < nb; ++c) acc += A[(int64_t)(kb + c) * n + i] * xb[c];
    z[i] -= acc;
  }
}

inline int egrid(int64_t n) {
  int64_t g = (n + 255) / 256;
  return (int)(g < 1 ? 1 : (g > 4096 ? 4096 : g));
}

// ---- staged parameter rows from a device joint vector -------------------------------------------
// The value of full-vector slot `slot` at representation r, with the slot limits of the host maps
// (utils/conversions/optimization.py:6-54: tan/arctan for two-sided limits, v - 1/(v - lim) for
// one-sided ones, a modulo for the cyclic PA, identity otherwise), in numpy's operation order and
// without contraction (explicit _rn operations), so the staged rows equal the host staging's.
__device__ double stage_value(int slot, double r) {
  constexpr double kPi = 3.141592653589793;
  switch (slot) {
    case 2:  // q in (0, 1)
      return __dadd_rn(__ddiv_rn(__dmul_rn(__dadd_rn(atan(r), kPi / 2), 1.0 - 0.0), kPi), 0.0);
    case 4:  // n in (0.36, 8)
      return __dadd_rn(__ddiv_rn(__dmul_rn(__dadd_rn(atan(r), kPi / 2), 8.0 - 0.36), kPi), 0.36);
    case 5: {  // Re in (0, inf)
      const double t = __dsub_rn(r, 0.0);
      return __dmul_rn(__dadd_rn(__dadd_rn(r, 0.0), __dsqrt_rn(__dadd_rn(__dmul_rn(t, t), 4.0))), 0.5);
    }
    case 3: {  // PA: 0 + mod(r - 0, pi), numpy's floating modulo (fmod, then the divisor's sign)
      const double a = __dsub_rn(r, 0.0);
      double m = fmod(a, kPi);
      if (m != 0.0) {
        if (m < 0.0) m = __dadd_rn(m, kPi);
      } else {
        m = 0.0;
      }
      return __dadd_rn(0.0, m);
    }
    default:
      return r;
  }
}

// out[c] = base[c] (gidx[c] < 0) or the value of slot c % 8 at x[g] + alpha v[g]
__global__ void k_scene_stage(int n, const int32_t* __restrict__ gidx, const double* __restrict__ base,
                              const double* __restrict__ x, const double* __restrict__ v, double alpha,
                              double* __restrict__ out) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const int g = gidx[c];
    if (g < 0) {
      out[c] = base[c];
      continue;
    }
    const double r = v ? __dadd_rn(x[g], __dmul_rn(alpha, v[g])) : x[g];
    out[c] = stage_value(c % kMaxSlots, r);
  }
}

// ---- PSF model normalisation: K / sum K and its derivatives (one block) ---------------------------
__global__ void k_psf_normalize(int n, int m, const float* __restrict__ img, const float* __restrict__ dimg,
                                float* __restrict__ out, float* __restrict__ dout) {
  constexpr int kMaxDir = 8;
  double acc[1 + kMaxDir];
#pragma unroll
  for (int c = 0; c <= kMaxDir; ++c) acc[c] = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    acc[0] += (double)img[i];
#pragma unroll
    for (int c = 0; c < kMaxDir; ++c)
      if (c < m) acc[1 + c] += (double)dimg[(int64_t)c * n + i];
  }
  __shared__ double sh[1 + kMaxDir][32];
  __shared__ double tot[1 + kMaxDir];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int c = 0; c <= kMaxDir; ++c) {
    const double r = warp_sum(acc[c]);
    if (lane == 0) sh[c][w] = r;
  }
  __syncthreads();
  if (threadIdx.x <= kMaxDir) {
    double t = 0.0;
    for (int k = 0; k < nw; ++k) t += sh[threadIdx.x][k];
    tot[threadIdx.x] = t;
  }
  __syncthreads();
  const double S = tot[0];
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double k = (double)img[i] / S;
    out[i] = (float)k;
    for (int c = 0; c < m; ++c) dout[(int64_t)c * n + i] = (float)(((double)dimg[(int64_t)c * n + i] - k * tot[1 + c]) / S);
  }
}

}  // namespace

extern "C" {

int ap_psf_normalize(int32_t n_pix, int32_t n_dir, const float* img, const float* dimg, float* out, float* dout,
                     ap_stream_t stream) {
  if (n_pix <= 0 || n_dir < 0 || n_dir > 8 || !img || !out || (n_dir > 0 && (!dimg || !dout))) return AP_ERR_ARG;
  k_psf_normalize<<<1, 1024, 0, (cudaStream_t)stream>>>(n_pix, n_dir, img, dimg, out, dout);
  return record_cuda(cudaGetLastError());
}

int ap_scene_forward(const ap_scene_source* sources, const int32_t* tile_ptr, const int32_t* tile_src,
                     const float* fwd, float sky, const double* sky_F, const double* sky_F0, double area,
                     int32_t nx, int32_t ny, float* image, ap_stream_t stream) {
  if (!sources || !tile_ptr || !tile_src || !fwd || !image || nx <= 0 || ny <= 0) return AP_ERR_ARG;
  if (sky_F0 && !sky_F) return AP_ERR_ARG;
  const int tiles = ((nx + kSceneTile - 1) / kSceneTile) * ((ny + kSceneTile - 1) / kSceneTile);
  k_scene_forward<<<tiles, 256, 0, (cudaStream_t)stream>>>(sources, tile_ptr, tile_src, fwd, sky, sky_F, sky_F0, area,
                                                          nx, ny, image);
  return record_cuda(cudaGetLastError());
}

int ap_scene_jvp(const ap_scene_source* sources, const int32_t* tile_ptr, const int32_t* tile_src, const float* jac,
                 const double* h, int32_t nx, int32_t ny, float* out, ap_stream_t stream) {
  if (!sources || !tile_ptr || !tile_src || !jac || !h || !out || nx <= 0 || ny <= 0) return AP_ERR_ARG;
  const int tiles = ((nx + kSceneTile - 1) / kSceneTile) * ((ny + kSceneTile - 1) / kSceneTile);
  k_scene_jvp<<<tiles, 256, 0, (cudaStream_t)stream>>>(sources, tile_ptr, tile_src, jac, h, nx, ny, out);
  return record_cuda(cudaGetLastError());
}

int ap_scene_jt(const ap_scene_source* sources, int32_t n_sources, const float* jac, const float* v, int32_t nx,
                int32_t P, double* out, ap_stream_t stream) {
  if (!sources || !jac || !v || !out || n_sources < 0 || P <= 0) return AP_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  int rc = record_cuda(cudaMemsetAsync(out, 0, sizeof(double) * P, st));
  if (rc || n_sources == 0) return rc;
  k_scene_jt<<<n_sources, 256, 0, st>>>(sources, jac, v, nx, out, nullptr);
  return record_cuda(cudaGetLastError());
}

int ap_scene_hess(const ap_scene_source* sources, const int32_t* pairs, int32_t n_pairs, const float* jac,
                  const float* weight, const uint8_t* mask, int32_t nx, int32_t P, double* H, ap_stream_t stream) {
  if (!sources || !jac || !H || n_pairs < 0 || P <= 0 || (n_pairs > 0 && !pairs)) return AP_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  int rc = record_cuda(cudaMemsetAsync(H, 0, sizeof(double) * P * P, st));
  if (rc || n_pairs == 0) return rc;
  k_scene_hess<<<n_pairs, 256, 0, st>>>(sources, pairs, jac, weight, mask, nx, P, H, nullptr);
  return record_cuda(cudaGetLastError());
}

int ap_scene_hess_blocks(const ap_scene_source* sources, const int32_t* pairs, int32_t n_pairs, const float* jac,
                         const float* weight, const uint8_t* mask, int32_t nx, double* part, ap_stream_t stream) {
  if (!sources || !jac || !part || n_pairs < 0 || (n_pairs > 0 && !pairs)) return AP_ERR_ARG;
  if (n_pairs == 0) return AP_OK;
  k_scene_hess<<<n_pairs, 256, 0, (cudaStream_t)stream>>>(sources, pairs, jac, weight, mask, nx, 0, nullptr, part);
  return record_cuda(cudaGetLastError());
}

int ap_scene_jt_blocks(const ap_scene_source* sources, int32_t n_sources, const float* jac, const float* v,
                       int32_t nx, double* part, ap_stream_t stream) {
  if (!sources || !jac || !v || !part || n_sources < 0) return AP_ERR_ARG;
  if (n_sources == 0) return AP_OK;
  k_scene_jt<<<n_sources, 256, 0, (cudaStream_t)stream>>>(sources, jac, v, nx, nullptr, part);
  return record_cuda(cudaGetLastError());
}

int ap_gather_sum(int64_t n_entries, const int64_t* entry, const int32_t* ptr, const int32_t* contrib,
                  const double* part, double* out, int64_t out_n, ap_stream_t stream) {
  if (n_entries < 0 || !out || out_n <= 0 || (n_entries > 0 && (!entry || !ptr || !contrib || !part)))
    return AP_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  int rc = record_cuda(cudaMemsetAsync(out, 0, sizeof(double) * out_n, st));
  if (rc || n_entries == 0) return rc;
  k_gather_sum<<<egrid(n_entries), 256, 0, st>>>(n_entries, entry, ptr, contrib, part, out);
  return record_cuda(cudaGetLastError());
}

static int scene_chi2(const float* model, const float* base, const float* data, const float* weight,
                      const uint8_t* mask, int64_t n, double* out, double* parts, int32_t n_parts,
                      cudaStream_t st) {
  if (!model || !data || !out || !parts || n <= 0 || n_parts < 1) return AP_ERR_ARG;
  const int m = n_parts < 1024 ? n_parts : 1024;
  int64_t chunk = (n + m - 1) / m;
  chunk = (chunk + 255) / 256 * 256;
  const int blocks = (int)((n + chunk - 1) / chunk);
  k_scene_chi2_part<<<blocks, 256, 0, st>>>(model, base, data, weight, mask, n, chunk, parts);
  k_sum_parts<<<1, 256, 0, st>>>(parts, blocks, out);
  return record_cuda(cudaGetLastError());
}

int ap_scene_chi2(const float* model, const float* data, const float* weight, const uint8_t* mask, int64_t n,
                  double* out, double* parts, int32_t n_parts, ap_stream_t stream) {
  return scene_chi2(model, nullptr, data, weight, mask, n, out, parts, n_parts, (cudaStream_t)stream);
}

int ap_scene_chi2_change(const float* dm, const float* base, const float* data, const float* weight,
                         const uint8_t* mask, int64_t n, double* out, double* parts, int32_t n_parts,
                         ap_stream_t stream) {
  if (!base) return AP_ERR_ARG;
  return scene_chi2(dm, base, data, weight, mask, n, out, parts, n_parts, (cudaStream_t)stream);
}

int ap_reduce_upscaled(int32_t n_stamps, const int64_t* in_off, const int64_t* out_off, const int32_t* cnx, int32_t u,
                       int32_t n_planes, const float* in, int64_t in_stride, float* out, int64_t out_stride,
                       int64_t out_total, ap_stream_t stream) {
  if (n_stamps <= 0 || !in_off || !out_off || !cnx || u < 1 || n_planes < 1 || !in || !out || out_total <= 0 ||
      in_stride < 0 || out_stride < out_total)
    return AP_ERR_ARG;
  const int64_t n = (int64_t)n_planes * out_total;
  k_reduce_upscaled<<<egrid(n), 256, 0, (cudaStream_t)stream>>>(n_stamps, in_off, out_off, cnx, u, n_planes, in,
                                                               in_stride, out, out_stride, out_total);
  return record_cuda(cudaGetLastError());
}

int ap_scene_residual(const float* model, const float* data, const float* weight, const uint8_t* mask, int64_t n,
                      float* r, ap_stream_t stream) {
  if (!model || !data || !r || n <= 0) return AP_ERR_ARG;
  k_scene_residual<<<egrid(n), 256, 0, (cudaStream_t)stream>>>(model, data, weight, mask, n, r);
  return record_cuda(cudaGetLastError());
}

int ap_scene_rpp_image(const float* r, const float* rh, const float* jh, const float* weight, const uint8_t* mask,
                       double d, int64_t n, float* out, ap_stream_t stream) {
  if (!r || !rh || !jh || !out || n <= 0 || !(d > 0)) return AP_ERR_ARG;
  k_scene_rpp<<<egrid(n), 256, 0, (cudaStream_t)stream>>>(r, rh, jh, weight, mask, d, n, out);
  return record_cuda(cudaGetLastError());
}

int ap_scene_stage(int32_t n_cells, const int32_t* gidx, const double* base, const double* x, const double* v,
                   double alpha, double* out, ap_stream_t stream) {
  if (n_cells <= 0 || (n_cells % kMaxSlots) != 0 || !gidx || !base || !x || !out) return AP_ERR_ARG;
  k_scene_stage<<<egrid(n_cells), 256, 0, (cudaStream_t)stream>>>(n_cells, gidx, base, x, v, alpha, out);
  return record_cuda(cudaGetLastError());
}

size_t ap_dense_solve_workspace_bytes(int32_t n) {
  if (n <= 0) return 0;
  // the FP64 factorisation's region, then the mixed-precision solver's (ap_solve.cu)
  return apgb::align256(apgb::dense_fp64_ws_bytes(n)) + apgb::dense_mixed_ws_bytes(n);
}

namespace {
// both triangular solves on the factor in the workspace: L z = g, then L^T h = z
cudaError_t chol_solves(int n, const double* A, const double* g, double* h, double* y, double* z, cudaStream_t st) {
  cudaError_t e = cudaMemcpyAsync(y, g, sizeof(double) * n, cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) return e;
  for (int kb = 0; kb < n; kb += kNB) {
    const int rows = n - kb - (n - kb < kNB ? n - kb : kNB);
    int grid = (rows + 7) / 8;
    grid = grid < 1 ? 1 : (grid > 1024 ? 1024 : grid);
    k_trsv_fwd<<<grid, 256, 0, st>>>(A, n, kb, y, z);
  }
  for (int kb = ((n - 1) / kNB) * kNB; kb >= 0; kb -= kNB) {
    int grid = (kb + 255) / 256;
    grid = grid < 1 ? 1 : grid;
    k_trsv_bwd<<<grid, 256, 0, st>>>(A, n, kb, z, h);
  }
  return cudaGetLastError();
}
}  // namespace

int ap_dense_damped_solve(int32_t n, const double* H, const double* g, double L, double* h, void* ws,
                          size_t ws_bytes, int32_t* info, ap_stream_t stream) {
  if (n <= 0 || !H || !g || !h || !ws || !info) return AP_ERR_ARG;
  if (ws_bytes < ap_dense_solve_workspace_bytes(n)) return AP_ERR_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  double* A = (double*)ws;
  double* y = A + (size_t)n * n;
  double* z = y + n;
  double* dscr = z + n;
  int rc = record_cuda(cudaMemsetAsync(info, 0, sizeof(int32_t), st));
  if (rc) return rc;
  k_damp<<<egrid((int64_t)n * n), 256, 0, st>>>(H, L, n, A);
  for (int k0 = 0; k0 < n; k0 += kNB) {
    const int nb = n - k0 < kNB ? n - k0 : kNB;
    const int rest = n - k0 - nb;
    k_chol_panel<<<rest > 0 ? (rest + 31) / 32 : 1, 32, 0, st>>>(A, n, k0, info, dscr);
    if (rest > 0) {
      const int nt = (rest + kNB - 1) / kNB;
      k_chol_update<<<dim3(nt, nt), 256, 0, st>>>(A, n, k0, dscr);
    }
  }
  return record_cuda(chol_solves(n, A, g, h, y, z, st));
}

int ap_dense_factored_solve(int32_t n, const double* g, double* h, void* ws, size_t ws_bytes, ap_stream_t stream) {
  if (n <= 0 || !g || !h || !ws) return AP_ERR_ARG;
  if (ws_bytes < ap_dense_solve_workspace_bytes(n)) return AP_ERR_WORKSPACE;
  double* A = (double*)ws;
  double* y = A + (size_t)n * n;
  double* z = y + n;
  return record_cuda(chol_solves(n, A, g, h, y, z, (cudaStream_t)stream));
}

}  // extern "C"
