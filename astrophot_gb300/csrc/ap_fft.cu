// PSF convolution by FFT for stamps with large kernels (the reference's default
// psf_convolve_mode "fft", models/_model_methods.py:245-257, utils/operations.py fft_convolve).
//
// The convolve pass (k_conv) convolves each working plane W with the shifted kernel K on the
// kept crop, out(i) = sum_u W(i + c - u) K(u), reading zeros outside the working window.  Here
// the same numbers come from complex 2-D FFTs of side N >= working window + kernel - 1 (powers
// of two up to 1024, so nothing wraps into the crop): the kernel is placed centred at index 0
// (position (u - c) mod N holds K(u)) and the circular convolution is taken.  Real planes are paired in one complex transform (A + iB): with a real kernel,
// the inverse transform of (A + iB)^ K^ is (A*K) + i (B*K).  The kernel and its two shift
// derivatives share transforms the same way, Z0 = (K + i dK/dsx)^ split by conjugate symmetry
// into K^ and dK/dsx^.  Buffers per (stamp, slot): K0 = K + i dKx, K1 = dKy, D = deep plane,
// P1..P3 = pairs of partial planes.  The convolved planes land in `preconv`, from which the
// convolve pass takes them instead of convolving directly (same Jacobian chain, chi^2 and
// accumulations afterwards).  A difference evaluation (OP_DIFF) transforms K1, dK, dS and the
// base's deep image S0 each on its own and returns the inverse of dS^ K1^ + S0^ dK^: a small
// difference never shares a transform with a large array, whose rounding it would take on.
//
// Transforms are radix-2, decimation in time, in shared memory after a bit-reversed load: one
// CTA per transform row (every active buffer of both evaluation slots in turn; the inputs are
// built in place), one CTA per group of 8 columns, the spectra products per row, the inverse
// columns, and the inverse rows only for the kept rows, written straight into the convolved
// planes.  FP32 with FP64-computed twiddles.
#include <cmath>
#include <vector>

#include "ap_internal.h"

namespace apgb {
namespace {

constexpr int kFftBufs = 6;
constexpr int kColGroup = 8;
constexpr int kFftThreads = 256;
enum FftBuf { FB_K0 = 0, FB_K1 = 1, FB_D = 2, FB_P1 = 3 };

__constant__ float2 c_tw[kFftMaxSide / 2];  // exp(-2 pi i m / kFftMaxSide), m < kFftMaxSide / 2

struct FftUse {
  bool jac, shift, diff;
  int npart;
  int part[NGRAD];
  unsigned fwd;  // buffers transformed forward
  unsigned inv;  // buffers transformed back
};

__device__ FftUse fft_use(const BatchArgs& b, int ops) {
  FftUse u;
  u.jac = (ops & OP_JAC) != 0;
  u.shift = b.psf_mode == AP_PSF_FULL;
  u.diff = (ops & OP_DIFF) != 0;
  u.npart = 0;
  if (u.diff) {
    // four real transforms, none paired (a small difference sharing a transform with a large
    // array would take on the large one's rounding): K0 <- K1, K1 <- dK, D <- dS, P1 <- S0 (the
    // base's deep image); D <- dS^ K1^ + S0^ dK^, whose inverse is the model difference
    u.fwd = (1u << FB_K0) | (1u << FB_D);
    if (u.shift) u.fwd |= (1u << FB_K1) | (1u << FB_P1);
    u.inv = 1u << FB_D;
    return u;
  }
  if (u.jac) {
    for (int q = 0; q < NGRAD; ++q) {
      if (u.shift && !(ops & OP_VJP_COORD) && (q == GX || q == GY)) continue;
      if (!profile_has_n(b.kind) && q == GN) continue;
      u.part[u.npart++] = q;
    }
  }
  const int pairs = (u.npart + 1) / 2;
  u.fwd = (1u << FB_K0) | (1u << FB_D);
  u.inv = 1u << FB_D;
  if (u.jac && u.shift) {
    u.fwd |= 1u << FB_K1;
    u.inv |= 1u << FB_K1;
  }
  for (int k = 0; k < pairs; ++k) {
    u.fwd |= 1u << (FB_P1 + k);
    u.inv |= 1u << (FB_P1 + k);
  }
  return u;
}

// stamp j of the FFT list whose [pre[j], pre[j+1]) holds item
__device__ __forceinline__ int fft_find(const int32_t* pre, int n, int item) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (pre[mid] <= item) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ float2* fft_buffer(const BatchArgs& b, const StampDev& st, int slot, int k) {
  return b.fft_buf + st.fft_off + (int64_t)(slot * kFftBufs + k) * st.fft_ny * st.fft_nx;
}

// in-place radix-2 DIT of rows bit-reversed rows of n points each, back to back in a (thread t of
// nt takes butterflies t, t + nt, ... over all rows); sign -1 forward, +1 inverse
__device__ void dit_rows(float2* a, int n, int rows, bool inverse, int t, int nt) {
  const int hn = n >> 1;
  for (int L = 2; L <= n; L <<= 1) {
    const int half = L >> 1;
    const int step = kFftMaxSide / L;
    for (int jj = t; jj < rows * hn; jj += nt) {
      const int r = jj / hn, j = jj - r * hn;
      const int g = j / half, k = j - g * half;
      float2* ar = a + r * n;
      const int i0 = g * L + k, i1 = i0 + half;
      float2 w = c_tw[k * step];
      if (inverse) w.y = -w.y;
      const float2 u = ar[i0], v = cmul(ar[i1], w);
      ar[i0] = make_float2(u.x + v.x, u.y + v.y);
      ar[i1] = make_float2(u.x - v.x, u.y - v.y);
    }
    __syncthreads();
  }
}

// value of buffer k at transform position (y, x) before the transforms (kernels centred at 0,
// planes at their working-window position, zero elsewhere)
__device__ __forceinline__ float2 fft_input(const BatchArgs& b, const StampDev& st, const FftUse& u, int slot, int k,
                                            int y, int x) {
  if (k == FB_K0 || k == FB_K1) {
    const int v = (y + st.kpy / 2) % st.fft_ny, uu = (x + st.kpx / 2) % st.fft_nx;  // y = (v - cy) mod Ny
    if (v >= st.kpy || uu >= st.kpx) return make_float2(0.f, 0.f);
    const int kp2 = st.kpx * st.kpy, ki = v * st.kpx + uu;
    const float* ksrc = b.spsf + st.spsf_off + (int64_t)slot * 3 * kp2;
    if (k == FB_K1) return make_float2(ksrc[(u.diff ? 1 : 2) * kp2 + ki], 0.f);
    return make_float2(ksrc[ki], (u.jac && u.shift) ? ksrc[kp2 + ki] : 0.f);
  }
  if (y >= st.wny || x >= st.wnx) return make_float2(0.f, 0.f);
  const int64_t wi = st.work_off + (int64_t)y * st.wnx + x;
  const float* w = b.work + wi;
  if (u.diff) return make_float2(k == FB_D ? w[work_plane(b, slot, 1)] : b.base_deep[wi], 0.f);
  if (k == FB_D) return make_float2(w[work_plane(b, slot, 0)], 0.f);
  const int p = k - FB_P1;
  const int qa = u.part[2 * p];
  const int qb = 2 * p + 1 < u.npart ? u.part[2 * p + 1] : -1;
  return make_float2(w[work_plane(b, slot, 1 + qa)], qb >= 0 ? w[work_plane(b, slot, 1 + qb)] : 0.f);
}

// -- forward row transforms, the inputs built in place: one CTA per (stamp, block of rows) ---
__global__ void __launch_bounds__(kFftThreads) k_fft_rows_fwd(BatchArgs b) {
  extern __shared__ float2 sm[];
  const int j = fft_find(b.fft_row_pre, b.n_fft, blockIdx.x);
  const int s = b.fft_stamp[j];
  const StampDev& st = b.stamps[s];
  const int Nx = st.fft_nx, bits = 31 - __clz(Nx);
  const int rb = fft_rows_per_block(Nx);
  const int y0 = (blockIdx.x - b.fft_row_pre[j]) * rb;
  const int rows = min(rb, st.fft_ny - y0);
  for (int slot = 0; slot < 2; ++slot) {
    const int ops = b.evals[s * 2 + slot].ops;
    if (!ops) continue;
    const FftUse u = fft_use(b, ops);
    for (int k = 0; k < kFftBufs; ++k) {
      if (!((u.fwd >> k) & 1u)) continue;
      float2* buf = fft_buffer(b, st, slot, k) + (int64_t)y0 * Nx;
      for (int e = threadIdx.x; e < rows * Nx; e += blockDim.x) {
        const int r = e / Nx, x = e - r * Nx;
        sm[r * Nx + (__brev(x) >> (32 - bits))] = fft_input(b, st, u, slot, k, y0 + r, x);
      }
      __syncthreads();
      dit_rows(sm, Nx, rows, false, threadIdx.x, blockDim.x);
      for (int e = threadIdx.x; e < rows * Nx; e += blockDim.x) buf[e] = sm[e];
      __syncthreads();
    }
  }
}

// -- column transforms: one CTA per (stamp, group of 8 columns), every active buffer ---------
__global__ void __launch_bounds__(kFftThreads) k_fft_cols(BatchArgs b, int inverse) {
  extern __shared__ float2 sm[];
  const int j = fft_find(b.fft_col_pre, b.n_fft, blockIdx.x);
  const int s = b.fft_stamp[j];
  const StampDev& st = b.stamps[s];
  const int x0 = (blockIdx.x - b.fft_col_pre[j]) * kColGroup;
  const int Nx = st.fft_nx, Ny = st.fft_ny;
  const int bits = 31 - __clz(Ny);
  const int c = threadIdx.x % kColGroup, t = threadIdx.x / kColGroup, nt = blockDim.x / kColGroup;
  for (int slot = 0; slot < 2; ++slot) {
    const int ops = b.evals[s * 2 + slot].ops;
    if (!ops) continue;
    const FftUse u = fft_use(b, ops);
    for (int k = 0; k < kFftBufs; ++k) {
      if (!(((inverse ? u.inv : u.fwd) >> k) & 1u)) continue;
      float2* buf = fft_buffer(b, st, slot, k);
      // column cc of the group lives at sm[cc * Ny ...], rows bit-reversed
      for (int e = threadIdx.x; e < kColGroup * Ny; e += blockDim.x) {
        const int r = e / kColGroup, cc = e - r * kColGroup;
        sm[cc * Ny + (__brev(r) >> (32 - bits))] = buf[(int64_t)r * Nx + x0 + cc];
      }
      __syncthreads();
      float2* a = sm + c * Ny;
      for (int L = 2; L <= Ny; L <<= 1) {
        const int half = L >> 1;
        const int step = kFftMaxSide / L;
        for (int jj = t; jj < Ny / 2; jj += nt) {
          const int g = jj / half, kk = jj - g * half;
          const int i0 = g * L + kk, i1 = i0 + half;
          float2 w = c_tw[kk * step];
          if (inverse) w.y = -w.y;
          const float2 p = a[i0], q = cmul(a[i1], w);
          a[i0] = make_float2(p.x + q.x, p.y + q.y);
          a[i1] = make_float2(p.x - q.x, p.y - q.y);
        }
        __syncthreads();
      }
      for (int e = threadIdx.x; e < kColGroup * Ny; e += blockDim.x) {
        const int r = e / kColGroup, cc = e - r * kColGroup;
        buf[(int64_t)r * Nx + x0 + cc] = sm[cc * Ny + r];
      }
      __syncthreads();
    }
  }
}

// -- spectra products: one CTA per (stamp, block of rows) ----------------------------------
__global__ void __launch_bounds__(kFftThreads) k_fft_mul(BatchArgs b) {
  const int j = fft_find(b.fft_row_pre, b.n_fft, blockIdx.x);
  const int s = b.fft_stamp[j];
  const StampDev& st = b.stamps[s];
  const int Nx = st.fft_nx, Ny = st.fft_ny;
  const int rb = fft_rows_per_block(Nx);
  const int y0 = (blockIdx.x - b.fft_row_pre[j]) * rb;
  const int rows = min(rb, Ny - y0);
  for (int slot = 0; slot < 2; ++slot) {
    const int ops = b.evals[s * 2 + slot].ops;
    if (!ops) continue;
    const FftUse u = fft_use(b, ops);
    const float2* K0 = fft_buffer(b, st, slot, FB_K0);
    float2* K1 = fft_buffer(b, st, slot, FB_K1);
    float2* D = fft_buffer(b, st, slot, FB_D);
    const bool two_k = u.jac && u.shift;
    const int pairs = (u.npart + 1) / 2;
    for (int e = threadIdx.x; e < rows * Nx; e += blockDim.x) {
      const int r = e / Nx, x = e - r * Nx;
      const int y = y0 + r;
      const int64_t i = (int64_t)y * Nx + x;
      const float2 z = K0[i];
      if (u.diff) {
        float2 r = cmul(D[i], z);
        if (u.shift) {
          const float2 c = cmul(fft_buffer(b, st, slot, FB_P1)[i], K1[i]);
          r = make_float2(r.x + c.x, r.y + c.y);
        }
        D[i] = r;
        continue;
      }
      float2 FK = z, FX = make_float2(0.f, 0.f);
      if (two_k) {
        const float2 zm = K0[(int64_t)((Ny - y) % Ny) * Nx + (Nx - x) % Nx];
        // K^ = (Z(k) + conj Z(-k)) / 2, dKx^ = (Z(k) - conj Z(-k)) / 2i
        FK = make_float2(0.5f * (z.x + zm.x), 0.5f * (z.y - zm.y));
        FX = make_float2(0.5f * (z.y + zm.y), -0.5f * (z.x - zm.x));
      }
      const float2 d = D[i];
      if (two_k) {
        K1[i] = cmul(d, K1[i]);
        D[i] = cmul(d, make_float2(FK.x - FX.y, FK.y + FX.x));  // d (K^ + i dKx^)
      } else {
        D[i] = cmul(d, FK);
      }
      for (int p = 0; p < pairs; ++p) {
        float2* P = fft_buffer(b, st, slot, FB_P1 + p);
        P[i] = cmul(P[i], FK);
      }
    }
  }
}

// -- inverse row transforms of the kept rows, written as convolved planes: one CTA per
// (stamp, block of output rows) ---------------------------------------------------------------
__global__ void __launch_bounds__(kFftThreads) k_fft_rows_inv(BatchArgs b) {
  extern __shared__ float2 sm[];
  const int j = fft_find(b.fft_out_pre, b.n_fft, blockIdx.x);
  const int s = b.fft_stamp[j];
  const StampDev& st = b.stamps[s];
  const int Nx = st.fft_nx, Ny = st.fft_ny, bits = 31 - __clz(Nx);
  const int rb = fft_rows_per_block(Nx);
  const int Y0 = (blockIdx.x - b.fft_out_pre[j]) * rb;
  const int rows = min(rb, st.ny - Y0);
  const float scale = 1.f / ((float)Nx * (float)Ny);
  const int64_t npix = (int64_t)st.nx * st.ny;
  for (int slot = 0; slot < 2; ++slot) {
    const int ops = b.evals[s * 2 + slot].ops;
    if (!ops) continue;
    const FftUse u = fft_use(b, ops);
    float* pre = b.preconv + st.pre_off + (int64_t)slot * (3 + NGRAD) * npix + (int64_t)Y0 * st.nx;
    for (int k = 0; k < kFftBufs; ++k) {
      if (!((u.inv >> k) & 1u)) continue;
      const float2* buf = fft_buffer(b, st, slot, k) + (int64_t)(Y0 + st.by) * Nx;
      for (int e = threadIdx.x; e < rows * Nx; e += blockDim.x) {
        const int r = e / Nx, x = e - r * Nx;
        sm[r * Nx + (__brev(x) >> (32 - bits))] = buf[e];
      }
      __syncthreads();
      dit_rows(sm, Nx, rows, true, threadIdx.x, blockDim.x);
      // planes: D -> model (re), d/dshift_x (im); K1 -> d/dshift_y (re); P -> a pair of partials
      int pr = -1, pi = -1;
      if (k == FB_D) {
        pr = 0;
        pi = (u.jac && u.shift) ? 1 : -1;
      } else if (k == FB_K1) {
        pr = 2;
      } else {
        const int p = k - FB_P1;
        pr = 3 + u.part[2 * p];
        pi = 2 * p + 1 < u.npart ? 3 + u.part[2 * p + 1] : -1;
      }
      for (int e = threadIdx.x; e < rows * st.nx; e += blockDim.x) {
        const int r = e / st.nx, X = e - r * st.nx;
        const float2 v = sm[r * Nx + X + st.bx];
        pre[(int64_t)pr * npix + (int64_t)r * st.nx + X] = v.x * scale;
        if (pi >= 0) pre[(int64_t)pi * npix + (int64_t)r * st.nx + X] = v.y * scale;
      }
      __syncthreads();
    }
  }
}

}  // namespace

cudaError_t fft_upload_twiddles(cudaStream_t st) {
  std::vector<float2> tw(kFftMaxSide / 2);
  for (int m = 0; m < kFftMaxSide / 2; ++m) {
    const double a = -2.0 * kPi * (double)m / (double)kFftMaxSide;
    tw[m] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  cudaError_t e = cudaMemcpyToSymbolAsync(c_tw, tw.data(), sizeof(float2) * tw.size(), 0, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(st);
}

cudaError_t set_fft_smem() {
  cudaError_t e = cudaFuncSetAttribute(k_fft_cols, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(sizeof(float2) * kColGroup * kFftMaxSide));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_fft_rows_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(sizeof(float2) * kFftMaxSide));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_fft_rows_inv, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)(sizeof(float2) * kFftMaxSide));
}

cudaError_t launch_fft_conv(const BatchArgs& b, int total_rows, int total_cols, int total_out, int max_nx,
                            int max_ny, cudaStream_t s) {
  if (b.n_fft <= 0) return cudaSuccess;
  const size_t row_smem = sizeof(float2) * (size_t)kFftMaxSide;  // fft_rows_per_block rows of max_nx
  const size_t col_smem = sizeof(float2) * kColGroup * (size_t)max_ny;
  k_fft_rows_fwd<<<total_rows, kFftThreads, row_smem, s>>>(b);
  k_fft_cols<<<total_cols, kFftThreads, col_smem, s>>>(b, 0);
  k_fft_mul<<<total_rows, kFftThreads, 0, s>>>(b);
  k_fft_cols<<<total_cols, kFftThreads, col_smem, s>>>(b, 1);
  k_fft_rows_inv<<<total_out, kFftThreads, row_smem, s>>>(b);
  return cudaGetLastError();
}

}  // namespace apgb
