// Dense damped solve of LM._h (astrophot/fit/lm.py:361-371) in mixed precision.
//
// The reference solves (H o (I + D/(1+L)) + L I (1 + diag H)) h = g in float64 (torch.linalg.solve).
// This GPU's float64 pipe runs at 1/64 of its float32 rate, so the system is factored in float32
// (blocked right-looking Cholesky) and the float64 solution is reached by iterative refinement
// with float64 residuals of the exact damped matrix, the scheme of LAPACK's dsposv (Langou et al.,
// "Exploiting the performance of 32 bit floating point arithmetic in obtaining 64 bit accuracy",
// SC 2006): x <- x + solve32(g - A x) until ||g - A x||_inf <= ||x||_inf ||A||_inf eps sqrt(n)
// (with eps = 2^-53 and a factor 4 of slack for the residual's own rounding), at most kItMax
// rounds.  When the float32 factorisation meets a non-positive pivot or the refinement does not
// converge, the result is info = -1 and h = 0: the caller then takes the float64 factorisation
// (ap_dense_damped_solve).  The damped matrix is formed as the reference forms it: off-diagonal
// H_ij * fl(1 / (1 + L)), diagonal H_ii + L (1 + H_ii).
//
// Pieces:
//   k_damp32          float32 lower triangle of the damped matrix and ||A||_inf (float64)
//   k_chol32_diag     the first 32 x 32 diagonal block factored and inverted (one CTA)
//   k_chol32_panel    one 32-column step: the panel rows below as A_panel L_kk^-T
//   k_chol32_update   the trailing lower triangle minus the panel's rank-32 product, 64 x 64 tiles;
//                     the CTA holding the next diagonal block then factors and inverts it
//   k_trsv32          both triangular solves in one CTA, with the diagonal blocks' inverses
//   k_ir_residual     r = g - A x in float64 from H (a warp per row), the inf-norms of r and x
//   k_ir_check        the convergence test; every refinement kernel returns at once when done
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "ap_internal.h"

using apgb::record_cuda;

namespace {

constexpr int kB = 32;            // column block of the factorisation
constexpr int kPanelRows = 128;   // panel rows per CTA
constexpr int kTile = 64;         // trailing-update tile
constexpr int kItMax = 10;        // refinement rounds
constexpr int kTrsvThreads = 1024;
constexpr int kMaxMixedN = 8192;  // the triangular solve keeps the right-hand side in shared memory

struct MixedState {
  int info32;                       // 1 + first row with a non-positive float32 pivot, or 0
  int done;                         // 0 refining, 1 converged, 2 failed
  int iter;
  int pad;
  unsigned long long rnorm, xnorm;  // float64 bit patterns of non-negative norms (max by integer)
  double anorm;                     // ||A||_inf of the damped matrix
  double inv1L, L;
};

struct Layout {
  float* A32;     // n x n, lower triangle
  float* Linv;    // nblocks x 32 x 32 inverses of the diagonal blocks
  double* x;      // solution
  double* r;      // residual
  float* d;       // correction
  MixedState* st;
};

__host__ __device__ inline int nblocks(int n) { return (n + kB - 1) / kB; }

inline Layout layout(int n, void* ws) {
  char* p = (char*)ws + apgb::align256(apgb::dense_fp64_ws_bytes(n));
  Layout L;
  L.A32 = (float*)p;
  p += apgb::align256(sizeof(float) * (size_t)n * n);
  L.Linv = (float*)p;
  p += apgb::align256(sizeof(float) * (size_t)nblocks(n) * kB * kB);
  L.x = (double*)p;
  p += apgb::align256(sizeof(double) * (size_t)n);
  L.r = (double*)p;
  p += apgb::align256(sizeof(double) * (size_t)n);
  L.d = (float*)p;
  p += apgb::align256(sizeof(float) * (size_t)n);
  L.st = (MixedState*)p;
  return L;
}

__device__ __forceinline__ double warp_sumd(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_maxd(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// damped entry (i, j) of the reference's matrix
__device__ __forceinline__ double damped(double h, bool diag, double L, double inv1L) {
  return diag ? __dadd_rn(h, __dmul_rn(L, __dadd_rn(1.0, h))) : __dmul_rn(h, inv1L);
}

// float32 lower triangle of the damped matrix; ||A||_inf over full rows of H (symmetric)
__global__ void __launch_bounds__(256) k_damp32(int n, const double* __restrict__ H, float* __restrict__ A32,
                                                MixedState* __restrict__ st) {
  __shared__ double part[8];
  const double L = st->L, inv1L = st->inv1L;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double rmax = 0.0;
  for (int i = blockIdx.x; i < n; i += gridDim.x) {
    const double* row = H + (int64_t)i * n;
    float* arow = A32 + (int64_t)i * n;
    double s = 0.0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
      const double a = damped(row[j], i == j, L, inv1L);
      s += fabs(a);
      if (j <= i) arow[j] = (float)a;
    }
    s = warp_sumd(s);
    if (lane == 0) part[w] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += part[k];
      rmax = fmax(rmax, t);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicMax(&st->rnorm, (unsigned long long)__double_as_longlong(rmax));
}

__global__ void k_anorm_store(MixedState* st) {
  st->anorm = __longlong_as_double((long long)st->rnorm);
  st->rnorm = 0ull;
}

// The nb x nb diagonal block at kd (rows nb..31 the identity) factored and inverted by the 256
// threads of a CTA, in shared memory, with small code (loops over the 32 columns are not
// unrolled: this runs once per CTA, where a fully unrolled body would wait on instruction
// fetch).  Thread t owns the elements (t >> 3, (t & 7) + 8 q), q < 4.  Right-looking: at step j
// every thread updates its elements right of column j with the raw column scaled by 1/L_jj, one
// barrier, then column j itself is scaled.  The inverse of the factor: R = I; row k of L^-1 is
// R[k] / L_kk, subtracted from the rows below with L[i][k] as weight.  A non-positive or
// non-finite pivot records 1 + row in info32 and takes pivot 1.  Writes L^-1 (zeros above the
// diagonal) to Linv_blk.  S and R: shared [32][33]; uses every thread of the CTA (256).
__device__ void diag_factor_inv(const float* __restrict__ A, int n, int kd, float* __restrict__ Linv_blk,
                                int* info32, float (*S)[kB + 1], float (*R)[kB + 1], float* invd) {
  const int t = threadIdx.x, i = t >> 3, cb = t & 7;
  const int nb = min(kB, n - kd);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int c = cb + 8 * q;
    S[i][c] = (i < nb && c < nb) ? (c <= i ? A[(int64_t)(kd + i) * n + kd + c] : 0.f) : (i == c ? 1.f : 0.f);
    R[i][c] = (i == c) ? 1.f : 0.f;
  }
  __syncthreads();
  for (int j = 0; j < kB; ++j) {
    float piv = S[j][j];
    if (!(piv > 0.f) || !isfinite(piv)) {
      if (t == 0) atomicCAS(info32, 0, 1 + kd + j);
      piv = 1.f;
    }
    const float sj = sqrtf(piv), inv = 1.f / sj;
    const float lij = S[i][j] * inv;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int c = cb + 8 * q;
      if (c > j && c <= i) S[i][c] = fmaf(-lij, S[c][j] * inv, S[i][c]);
    }
    __syncthreads();
    if (cb == 0 && i >= j) S[i][j] = (i == j) ? sj : S[i][j] * inv;
    __syncthreads();
  }
  if (t < kB) invd[t] = 1.f / S[t][t];
  __syncthreads();
  for (int k = 0; k < kB; ++k) {
    const float wk = invd[k];
    if (i > k) {
      const float lik = S[i][k];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int c = cb + 8 * q;
        if (c <= k) R[i][c] = fmaf(-lik, R[k][c] * wk, R[i][c]);
      }
    }
    __syncthreads();
    if (i == k) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int c = cb + 8 * q;
        if (c <= k) R[k][c] *= wk;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int c = cb + 8 * q;
    Linv_blk[i * kB + c] = (c <= i) ? R[i][c] : 0.f;
  }
}

// the first diagonal block (the others are factored by the trailing update that finishes them)
__global__ void __launch_bounds__(256) k_chol32_diag(const float* __restrict__ A, int n, float* __restrict__ Linv,
                                                     MixedState* __restrict__ st) {
  __shared__ float S[kB][kB + 1], R[kB][kB + 1], invd[kB];
  diag_factor_inv(A, n, 0, Linv, &st->info32, S, R, invd);
}

// panel rows of step k0: row r (thread) becomes A[r][k0:k0+nb] L_kk^-T = sum_c a_c Linv[j][c]
__global__ void __launch_bounds__(kPanelRows) k_chol32_panel(float* __restrict__ A, int n, int k0,
                                                             const float* __restrict__ Linv) {
  __shared__ float Li[kB][kB + 1];
  const int nb = min(kB, n - k0);
  const float* Lb = Linv + (int64_t)(k0 / kB) * kB * kB;
  for (int e = threadIdx.x; e < kB * kB; e += blockDim.x) Li[e / kB][e % kB] = Lb[e];
  __syncthreads();
  const int r = k0 + nb + blockIdx.x * kPanelRows + threadIdx.x;
  if (r >= n) return;
  float* row = A + (int64_t)r * n + k0;
  float a[kB];
#pragma unroll
  for (int c = 0; c < kB; ++c) a[c] = c < nb ? row[c] : 0.f;
  for (int j = 0; j < nb; ++j) {
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kB; ++c) s = fmaf(a[c], Li[j][c], s);
    row[j] = s;
  }
}

// trailing update of the lower triangle: A[i][j] -= sum_c P[i][c] P[j][c], i >= j >= k0 + nb;
// the CTA of tile (0, 0), which holds the next diagonal block, then factors and inverts it
__global__ void __launch_bounds__(256) k_chol32_update(float* __restrict__ A, int n, int k0, float* __restrict__ Linv,
                                                       MixedState* __restrict__ st) {
  const int ti = blockIdx.y, tj = blockIdx.x;
  if (tj > ti) return;
  const int nb = min(kB, n - k0), base = k0 + nb;
  const int i0 = base + ti * kTile, j0 = base + tj * kTile;
  __shared__ __align__(16) float Pi[kB][kTile + 4];
  __shared__ __align__(16) float Pj[kB][kTile + 4];
  for (int t = threadIdx.x; t < kTile * kB; t += blockDim.x) {
    const int r = t / kB, c = t % kB;
    Pi[c][r] = (i0 + r < n && c < nb) ? A[(int64_t)(i0 + r) * n + k0 + c] : 0.f;
    Pj[c][r] = (j0 + r < n && c < nb) ? A[(int64_t)(j0 + r) * n + k0 + c] : 0.f;
  }
  __syncthreads();
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  float acc[4][4];
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[p][q] = 0.f;
#pragma unroll 8
  for (int c = 0; c < kB; ++c) {
    const float4 a4 = *reinterpret_cast<const float4*>(&Pi[c][ty * 4]);
    const float4 b4 = *reinterpret_cast<const float4*>(&Pj[c][tx * 4]);
    const float av[4] = {a4.x, a4.y, a4.z, a4.w}, bv[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[p][q] = fmaf(av[p], bv[q], acc[p][q]);
  }
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const int i = i0 + ty * 4 + p;
    if (i >= n) continue;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int j = j0 + tx * 4 + q;
      if (j < n && j <= i) A[(int64_t)i * n + j] -= acc[p][q];
    }
  }
  if (ti == 0 && tj == 0) {
    __syncthreads();  // this CTA's updates of the next diagonal block are written; Pi / Pj free
    float (*S)[kB + 1] = reinterpret_cast<float (*)[kB + 1]>(&Pi[0][0]);
    float (*R)[kB + 1] = reinterpret_cast<float (*)[kB + 1]>(&Pj[0][0]);
    __shared__ float invd[kB];
    diag_factor_inv(A, n, base, Linv + (int64_t)(base / kB) * kB * kB, &st->info32, S, R, invd);
  }
}

// x = 0, r = g; refinement state reset (failed at once when the float32 factorisation broke down)
__global__ void k_ir_init(int n, const double* __restrict__ g, double* __restrict__ x, double* __restrict__ r,
                          MixedState* __restrict__ st) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i] = 0.0;
    r[i] = g[i];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st->done = st->info32 ? 2 : 0;
    st->iter = 0;
    st->rnorm = 0ull;
    st->xnorm = 0ull;
  }
}

// d = (L L^T)^-1 r in float32 (one CTA; y in shared memory), then x += d
__global__ void __launch_bounds__(kTrsvThreads) k_trsv32(int n, const float* __restrict__ A,
                                                         const float* __restrict__ Linv,
                                                         const double* __restrict__ r, double* __restrict__ x,
                                                         MixedState* __restrict__ st) {
  extern __shared__ float y[];
  __shared__ float blk[kB];
  if (st->done) return;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const bool vec = (n & 3) == 0 && ((reinterpret_cast<uintptr_t>(A) & 15) == 0);
  for (int i = threadIdx.x; i < n; i += blockDim.x) y[i] = (float)r[i];
  __syncthreads();
  const int nbk = nblocks(n);
  // forward: L z = y
  for (int b = 0; b < nbk; ++b) {
    const int kb = b * kB, nb = min(kB, n - kb);
    if (w == 0) {
      // row `lane` of the block's inverse (zeros above the diagonal), as float4 loads
      const float4* Lr = reinterpret_cast<const float4*>(Linv + (int64_t)b * kB * kB + lane * kB);
      const float yv = lane < nb ? y[kb + lane] : 0.f;
      float v = 0.f;
#pragma unroll
      for (int q = 0; q < kB / 4; ++q) {
        const float4 l4 = Lr[q];
        v = fmaf(l4.x, __shfl_sync(0xffffffffu, yv, 4 * q + 0), v);
        v = fmaf(l4.y, __shfl_sync(0xffffffffu, yv, 4 * q + 1), v);
        v = fmaf(l4.z, __shfl_sync(0xffffffffu, yv, 4 * q + 2), v);
        v = fmaf(l4.w, __shfl_sync(0xffffffffu, yv, 4 * q + 3), v);
      }
      blk[lane] = v;
      if (lane < nb) y[kb + lane] = v;
    }
    __syncthreads();
    // rows below: a thread per row, its loads of the row segment in flight together (float4
    // when every row starts on a 16-byte boundary; a full block then has nb = 32)
    if (vec && nb == kB) {
      for (int i = kb + nb + threadIdx.x; i < n; i += blockDim.x) {
        const float4* row = reinterpret_cast<const float4*>(A + (int64_t)i * n + kb);
        float s = 0.f;
#pragma unroll
        for (int q = 0; q < kB / 4; ++q) {
          const float4 a4 = row[q];
          s = fmaf(a4.x, blk[4 * q + 0], s);
          s = fmaf(a4.y, blk[4 * q + 1], s);
          s = fmaf(a4.z, blk[4 * q + 2], s);
          s = fmaf(a4.w, blk[4 * q + 3], s);
        }
        y[i] -= s;
      }
    } else {
      for (int i = kb + nb + threadIdx.x; i < n; i += blockDim.x) {
        const float* row = A + (int64_t)i * n + kb;
        float s = 0.f;
#pragma unroll
        for (int c = 0; c < kB; ++c)
          if (c < nb) s = fmaf(row[c], blk[c], s);
        y[i] -= s;
      }
    }
    __syncthreads();
  }
  // backward: L^T d = z
  for (int b = nbk - 1; b >= 0; --b) {
    const int kb = b * kB, nb = min(kB, n - kb);
    if (w == 0) {
      const float* Lb = Linv + (int64_t)b * kB * kB;
      const float zv = lane < nb ? y[kb + lane] : 0.f;
      float v = 0.f;
#pragma unroll
      for (int c = 0; c < kB; ++c) {
        const float zc = __shfl_sync(0xffffffffu, zv, c);
        if (c >= lane) v = fmaf(Lb[c * kB + lane], zc, v);
      }
      blk[lane] = v;
      if (lane < nb) y[kb + lane] = v;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kb; i += blockDim.x) {
      float s = 0.f;
#pragma unroll
      for (int c = 0; c < kB; ++c)
        if (c < nb) s = fmaf(A[(int64_t)(kb + c) * n + i], blk[c], s);
      y[i] -= s;
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] += (double)y[i];
}

// r = g - A x (float64, A from H and the damping), ||r||_inf and ||x||_inf
__global__ void __launch_bounds__(256) k_ir_residual(int n, const double* __restrict__ H, const double* __restrict__ g,
                                                     const double* __restrict__ x, double* __restrict__ r,
                                                     MixedState* __restrict__ st) {
  if (st->done) return;
  const double L = st->L, inv1L = st->inv1L;
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  double rmax = 0.0, xmax = 0.0;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
    const double* row = H + (int64_t)i * n;
    double s = 0.0;
    for (int j = lane; j < n; j += 32) s = fma(damped(row[j], i == j, L, inv1L), x[j], s);
    s = warp_sumd(s);
    const double ri = g[i] - s;
    if (lane == 0) r[i] = ri;
    // a NaN entry counts as +inf (fmax would drop it), which fails the convergence test
    const double ar = fabs(ri), ax = fabs(x[i]);
    rmax = (ar == ar) ? fmax(rmax, ar) : INFINITY;
    xmax = (ax == ax) ? fmax(xmax, ax) : INFINITY;
  }
  rmax = warp_maxd(rmax);
  xmax = warp_maxd(xmax);
  if (lane == 0) {
    atomicMax(&st->rnorm, (unsigned long long)__double_as_longlong(rmax));
    atomicMax(&st->xnorm, (unsigned long long)__double_as_longlong(xmax));
  }
}

__global__ void k_ir_check(int n, MixedState* st) {
  if (st->done) return;
  const double rn = __longlong_as_double((long long)st->rnorm);
  const double xn = __longlong_as_double((long long)st->xnorm);
  const double cte = st->anorm * 4.0 * 1.1102230246251565e-16 * sqrt((double)n);
  st->iter += 1;
  if (isfinite(rn) && isfinite(xn) && rn <= xn * cte) {
    st->done = 1;
  } else if (st->iter >= kItMax || !isfinite(rn) || !isfinite(xn)) {
    st->done = 2;
  } else {
    st->rnorm = 0ull;
    st->xnorm = 0ull;
  }
}

// h = x and info = 0 when converged; else h = 0 and info = -1 (take the float64 path)
__global__ void k_ir_finish(int n, const double* __restrict__ x, double* __restrict__ h, const MixedState* st,
                            int32_t* info) {
  const bool ok = st->done == 1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) h[i] = ok ? x[i] : 0.0;
  if (blockIdx.x == 0 && threadIdx.x == 0) *info = ok ? 0 : -1;
}

__global__ void k_set_damping(MixedState* st, double L, double inv1L, int reset_info) {
  st->L = L;
  st->inv1L = inv1L;
  if (reset_info) {
    st->info32 = 0;
    st->rnorm = 0ull;
  }
}

inline int vgrid(int n) {
  int g = (n + 255) / 256;
  return g < 1 ? 1 : (g > 1024 ? 1024 : g);
}

cudaError_t refine(int n, const double* H, const double* g, double* h, int32_t* info, const Layout& Lw,
                   cudaStream_t st) {
  k_ir_init<<<vgrid(n), 256, 0, st>>>(n, g, Lw.x, Lw.r, Lw.st);
  const size_t smem = sizeof(float) * (size_t)n;
  const int rgrid = (int)((n * 32LL + 255) / 256 < 4096 ? (n * 32LL + 255) / 256 : 4096);
  for (int it = 0; it < kItMax; ++it) {
    k_trsv32<<<1, kTrsvThreads, smem, st>>>(n, Lw.A32, Lw.Linv, Lw.r, Lw.x, Lw.st);
    k_ir_residual<<<rgrid, 256, 0, st>>>(n, H, g, Lw.x, Lw.r, Lw.st);
    k_ir_check<<<1, 1, 0, st>>>(n, Lw.st);
  }
  k_ir_finish<<<vgrid(n), 256, 0, st>>>(n, Lw.x, h, Lw.st, info);
  return cudaGetLastError();
}

}  // namespace

namespace apgb {
size_t dense_mixed_ws_bytes(int32_t n) {
  if (n <= 0) return 0;
  return align256(sizeof(float) * (size_t)n * n) + align256(sizeof(float) * (size_t)nblocks(n) * kB * kB) +
         2 * align256(sizeof(double) * (size_t)n) + align256(sizeof(float) * (size_t)n) + align256(sizeof(MixedState));
}
}  // namespace apgb

extern "C" {

int ap_dense_damped_solve_mixed(int32_t n, const double* H, const double* g, double L, double* h, void* ws,
                                size_t ws_bytes, int32_t* info, ap_stream_t stream) {
  if (n <= 0 || !H || !g || !h || !ws || !info || !(L >= 0.0)) return AP_ERR_ARG;
  if (n > kMaxMixedN) return AP_ERR_UNSUPPORTED;
  if (ws_bytes < ap_dense_solve_workspace_bytes(n)) return AP_ERR_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  const Layout Lw = layout(n, ws);
  k_set_damping<<<1, 1, 0, st>>>(Lw.st, L, 1.0 / (1.0 + L), 1);
  k_damp32<<<n < 2048 ? n : 2048, 256, 0, st>>>(n, H, Lw.A32, Lw.st);
  k_anorm_store<<<1, 1, 0, st>>>(Lw.st);
  k_chol32_diag<<<1, 256, 0, st>>>(Lw.A32, n, Lw.Linv, Lw.st);
  for (int k0 = 0; k0 < n; k0 += kB) {
    const int nb = n - k0 < kB ? n - k0 : kB;
    const int rest = n - k0 - nb;
    if (rest <= 0) break;
    k_chol32_panel<<<(rest + kPanelRows - 1) / kPanelRows, kPanelRows, 0, st>>>(Lw.A32, n, k0, Lw.Linv);
    const int nt = (rest + kTile - 1) / kTile;
    k_chol32_update<<<dim3(nt, nt), 256, 0, st>>>(Lw.A32, n, k0, Lw.Linv, Lw.st);
  }
  return record_cuda(refine(n, H, g, h, info, Lw, st));
}

int ap_dense_factored_solve_mixed(int32_t n, const double* H, const double* g, double L, double* h, void* ws,
                                  size_t ws_bytes, int32_t* info, ap_stream_t stream) {
  if (n <= 0 || !H || !g || !h || !ws || !info || !(L >= 0.0)) return AP_ERR_ARG;
  if (n > kMaxMixedN) return AP_ERR_UNSUPPORTED;
  if (ws_bytes < ap_dense_solve_workspace_bytes(n)) return AP_ERR_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  const Layout Lw = layout(n, ws);
  k_set_damping<<<1, 1, 0, st>>>(Lw.st, L, 1.0 / (1.0 + L), 0);
  return record_cuda(refine(n, H, g, h, info, Lw, st));
}

}  // extern "C"
