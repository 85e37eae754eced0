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
// accumulations afterwards).
//
// Transforms are radix-2, decimation in time, in shared memory after a bit-reversed load: one
// CTA per row of one buffer, then one CTA per group of 8 columns.  FP32 with FP64-computed
// twiddles.
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
  bool jac, shift;
  int npart;
  int part[NGRAD];
  unsigned fwd;  // buffers transformed forward
  unsigned inv;  // buffers transformed back
};

__device__ FftUse fft_use(const BatchArgs& b, int ops) {
  FftUse u;
  u.jac = (ops & OP_JAC) != 0;
  u.shift = b.psf_mode == AP_PSF_FULL;
  u.npart = 0;
  if (u.jac) {
    for (int q = 0; q < NGRAD; ++q) {
      if (u.shift && !(ops & OP_VJP_COORD) && (q == GX || q == GY)) continue;
      if (b.kind != AP_PROFILE_SERSIC && q == GN) continue;
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

// in-place radix-2 DIT on n points of a bit-reversed array (one transform per block; thread t of
// nt takes butterflies t, t + nt, ...); sign -1 forward, +1 inverse
__device__ void dit_stages(float2* a, int n, bool inverse, int t, int nt) {
  for (int L = 2; L <= n; L <<= 1) {
    const int half = L >> 1;
    const int step = kFftMaxSide / L;
    for (int j = t; j < n / 2; j += nt) {
      const int g = j / half, k = j - g * half;
      const int i0 = g * L + k, i1 = i0 + half;
      float2 w = c_tw[k * step];
      if (inverse) w.y = -w.y;
      const float2 u = a[i0], v = cmul(a[i1], w);
      a[i0] = make_float2(u.x + v.x, u.y + v.y);
      a[i1] = make_float2(u.x - v.x, u.y - v.y);
    }
    __syncthreads();
  }
}

// -- pack the planes and kernels ------------------------------------------------------------
__global__ void __launch_bounds__(kFftThreads) k_fft_pack(BatchArgs b) {
  const int j = fft_find(b.fft_row_pre, b.n_fft, blockIdx.x);
  const int s = b.fft_stamp[j], slot = blockIdx.y;
  const int ops = b.evals[s * 2 + slot].ops;
  if (!ops) return;
  const StampDev& st = b.stamps[s];
  const FftUse u = fft_use(b, ops);
  const int y = blockIdx.x - b.fft_row_pre[j];
  const int Nx = st.fft_nx, Ny = st.fft_ny;
  const int kp2 = st.kpx * st.kpy;
  const float* ksrc = b.spsf + st.spsf_off + (int64_t)slot * 3 * kp2;
  const int cx = (st.kpx - 1) / 2, cy = (st.kpy - 1) / 2;
  const int v = (y + cy) % Ny;  // kernel row at this transform row: y = (v - cy) mod Ny
  const bool vrow = v < st.kpy;
  const bool wrow = y < st.wny;
  const float* work = b.work + st.work_off + (int64_t)y * st.wnx;
  float2* K0 = fft_buffer(b, st, slot, FB_K0) + (int64_t)y * Nx;
  float2* K1 = fft_buffer(b, st, slot, FB_K1) + (int64_t)y * Nx;
  float2* D = fft_buffer(b, st, slot, FB_D) + (int64_t)y * Nx;
  const bool two_k = u.jac && u.shift;
  for (int x = threadIdx.x; x < Nx; x += blockDim.x) {
    const int uu = (x + cx) % Nx;
    const bool kin = vrow && uu < st.kpx;
    const int ki = v * st.kpx + uu;
    K0[x] = kin ? make_float2(ksrc[ki], two_k ? ksrc[kp2 + ki] : 0.f) : make_float2(0.f, 0.f);
    if (two_k) K1[x] = make_float2(kin ? ksrc[2 * kp2 + ki] : 0.f, 0.f);
    const bool win = wrow && x < st.wnx;
    D[x] = make_float2(win ? work[work_plane(b, slot, 0) + x] : 0.f, 0.f);
    for (int p = 0; p < (u.npart + 1) / 2; ++p) {
      const int qa = u.part[2 * p];
      const int qb = 2 * p + 1 < u.npart ? u.part[2 * p + 1] : -1;
      float2* P = fft_buffer(b, st, slot, FB_P1 + p) + (int64_t)y * Nx;
      const float a = win ? work[work_plane(b, slot, 1 + qa) + x] : 0.f;
      const float c = (win && qb >= 0) ? work[work_plane(b, slot, 1 + qb) + x] : 0.f;
      P[x] = make_float2(a, c);
    }
  }
}

// -- row transforms: one CTA per (row, slot * kFftBufs + buffer) ----------------------------
__global__ void __launch_bounds__(kFftThreads) k_fft_rows(BatchArgs b, int inverse) {
  extern __shared__ float2 sm[];
  const int j = fft_find(b.fft_row_pre, b.n_fft, blockIdx.x);
  const int s = b.fft_stamp[j];
  const int slot = blockIdx.y / kFftBufs, k = blockIdx.y - slot * kFftBufs;
  const int ops = b.evals[s * 2 + slot].ops;
  if (!ops) return;
  const FftUse u = fft_use(b, ops);
  if (!(((inverse ? u.inv : u.fwd) >> k) & 1u)) return;
  const StampDev& st = b.stamps[s];
  const int y = blockIdx.x - b.fft_row_pre[j];
  const int Nx = st.fft_nx;
  const int bits = 31 - __clz(Nx);
  float2* row = fft_buffer(b, st, slot, k) + (int64_t)y * Nx;
  for (int x = threadIdx.x; x < Nx; x += blockDim.x) sm[__brev(x) >> (32 - bits)] = row[x];
  __syncthreads();
  dit_stages(sm, Nx, inverse != 0, threadIdx.x, blockDim.x);
  for (int x = threadIdx.x; x < Nx; x += blockDim.x) row[x] = sm[x];
}

// -- column transforms: one CTA per (group of 8 columns, slot * kFftBufs + buffer) ---------
__global__ void __launch_bounds__(kFftThreads) k_fft_cols(BatchArgs b, int inverse) {
  extern __shared__ float2 sm[];
  const int j = fft_find(b.fft_col_pre, b.n_fft, blockIdx.x);
  const int s = b.fft_stamp[j];
  const int slot = blockIdx.y / kFftBufs, k = blockIdx.y - slot * kFftBufs;
  const int ops = b.evals[s * 2 + slot].ops;
  if (!ops) return;
  const FftUse u = fft_use(b, ops);
  if (!(((inverse ? u.inv : u.fwd) >> k) & 1u)) return;
  const StampDev& st = b.stamps[s];
  const int x0 = (blockIdx.x - b.fft_col_pre[j]) * kColGroup;
  const int Nx = st.fft_nx, Ny = st.fft_ny;
  const int bits = 31 - __clz(Ny);
  float2* buf = fft_buffer(b, st, slot, k);
  // column c of the group lives at sm[c * Ny ...], rows bit-reversed
  for (int e = threadIdx.x; e < kColGroup * Ny; e += blockDim.x) {
    const int r = e / kColGroup, c = e - r * kColGroup;
    sm[c * Ny + (__brev(r) >> (32 - bits))] = buf[(int64_t)r * Nx + x0 + c];
  }
  __syncthreads();
  // the 8 columns' butterflies together: thread t takes column t % 8
  const int c = threadIdx.x % kColGroup, t = threadIdx.x / kColGroup, nt = blockDim.x / kColGroup;
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
}

// -- spectra products -----------------------------------------------------------------------
__global__ void __launch_bounds__(kFftThreads) k_fft_mul(BatchArgs b) {
  const int j = fft_find(b.fft_row_pre, b.n_fft, blockIdx.x);
  const int s = b.fft_stamp[j], slot = blockIdx.y;
  const int ops = b.evals[s * 2 + slot].ops;
  if (!ops) return;
  const StampDev& st = b.stamps[s];
  const FftUse u = fft_use(b, ops);
  const int y = blockIdx.x - b.fft_row_pre[j];
  const int Nx = st.fft_nx, Ny = st.fft_ny;
  const int ym = (Ny - y) % Ny;
  const float2* K0 = fft_buffer(b, st, slot, FB_K0);
  float2* K1 = fft_buffer(b, st, slot, FB_K1) + (int64_t)y * Nx;
  float2* D = fft_buffer(b, st, slot, FB_D) + (int64_t)y * Nx;
  const bool two_k = u.jac && u.shift;
  const int pairs = (u.npart + 1) / 2;
  for (int x = threadIdx.x; x < Nx; x += blockDim.x) {
    const int xm = (Nx - x) % Nx;
    const float2 z = K0[(int64_t)y * Nx + x];
    float2 FK = z, FX = make_float2(0.f, 0.f);
    if (two_k) {
      const float2 zm = K0[(int64_t)ym * Nx + xm];
      // K^ = (Z(k) + conj Z(-k)) / 2, dKx^ = (Z(k) - conj Z(-k)) / 2i
      FK = make_float2(0.5f * (z.x + zm.x), 0.5f * (z.y - zm.y));
      FX = make_float2(0.5f * (z.y + zm.y), -0.5f * (z.x - zm.x));
    }
    const float2 d = D[x];
    if (two_k) {
      K1[x] = cmul(d, K1[x]);
      const float2 m = make_float2(FK.x - FX.y, FK.y + FX.x);  // K^ + i dKx^
      D[x] = cmul(d, m);
    } else {
      D[x] = cmul(d, FK);
    }
    for (int p = 0; p < pairs; ++p) {
      float2* P = fft_buffer(b, st, slot, FB_P1 + p) + (int64_t)y * Nx;
      P[x] = cmul(P[x], FK);
    }
  }
}

// -- convolved planes on the output grid ----------------------------------------------------
__global__ void __launch_bounds__(kFftThreads) k_fft_extract(BatchArgs b) {
  const int j = fft_find(b.fft_out_pre, b.n_fft, blockIdx.x);
  const int s = b.fft_stamp[j], slot = blockIdx.y;
  const int ops = b.evals[s * 2 + slot].ops;
  if (!ops) return;
  const StampDev& st = b.stamps[s];
  const FftUse u = fft_use(b, ops);
  const int Y = blockIdx.x - b.fft_out_pre[j];
  const int Nx = st.fft_nx, Ny = st.fft_ny;
  const float scale = 1.f / ((float)Nx * (float)Ny);
  const int64_t npix = (int64_t)st.nx * st.ny;
  float* pre = b.preconv + st.pre_off + (int64_t)slot * (3 + NGRAD) * npix + (int64_t)Y * st.nx;
  const int64_t wrow = (int64_t)(Y + st.by) * Nx + st.bx;
  const float2* D = fft_buffer(b, st, slot, FB_D) + wrow;
  const float2* K1 = fft_buffer(b, st, slot, FB_K1) + wrow;
  const bool two_k = u.jac && u.shift;
  for (int X = threadIdx.x; X < st.nx; X += blockDim.x) {
    const float2 d = D[X];
    pre[X] = d.x * scale;
    if (two_k) {
      pre[npix + X] = d.y * scale;
      pre[2 * npix + X] = K1[X].x * scale;
    }
    for (int p = 0; p < u.npart; ++p) {
      const float2 v = fft_buffer(b, st, slot, FB_P1 + p / 2)[wrow + X];
      pre[(int64_t)(3 + u.part[p]) * npix + X] = ((p & 1) ? v.y : v.x) * scale;
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
  return cudaFuncSetAttribute(k_fft_rows, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)(sizeof(float2) * kFftMaxSide));
}

cudaError_t launch_fft_conv(const BatchArgs& b, int total_rows, int total_cols, int total_out, int max_nx,
                            int max_ny, cudaStream_t s) {
  if (b.n_fft <= 0) return cudaSuccess;
  const size_t row_smem = sizeof(float2) * (size_t)max_nx;
  const size_t col_smem = sizeof(float2) * kColGroup * (size_t)max_ny;
  k_fft_pack<<<dim3(total_rows, 2), kFftThreads, 0, s>>>(b);
  k_fft_rows<<<dim3(total_rows, 2 * kFftBufs), kFftThreads, row_smem, s>>>(b, 0);
  k_fft_cols<<<dim3(total_cols, 2 * kFftBufs), kFftThreads, col_smem, s>>>(b, 0);
  k_fft_mul<<<dim3(total_rows, 2), kFftThreads, 0, s>>>(b);
  k_fft_cols<<<dim3(total_cols, 2 * kFftBufs), kFftThreads, col_smem, s>>>(b, 1);
  k_fft_rows<<<dim3(total_rows, 2 * kFftBufs), kFftThreads, row_smem, s>>>(b, 1);
  k_fft_extract<<<dim3(total_out, 2), kFftThreads, 0, s>>>(b);
  return cudaGetLastError();
}

}  // namespace apgb
