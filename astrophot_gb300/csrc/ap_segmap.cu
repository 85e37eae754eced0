// Segment statistics of a segmentation map (the window and initial-value helpers of
// astrophot/utils/initialize/segmentation_map.py:33-180): per segment, the pixel bounding box,
// the flux-weighted centroid, the angular centre of light (PA) and the axis ratio of
// axis_ratio_com (utils/operations.py:77-91).
//
// Two passes over the pixels with float64 atomics into per-segment accumulators:
//   pass 1: sum f, sum f x, sum f y, bounding box;
//   pass 2: A = sum f cos 2t, B = sum f sin 2t with t = atan2(y - cy, x - cx), as
//           ((dx^2 - dy^2), 2 dx dy) / r^2 (t = 0 at r = 0).
// The axis ratio needs no third pass: with P = PA + north (the reference adds north twice),
// sum f cos^2(t - P) = (F + cos 2P A + sin 2P B) / 2 and sum f sin^2(t - P) = F - that.
#include <algorithm>
#include <climits>
#include <cmath>

#include "ap_internal.h"

namespace apgb {
namespace {

constexpr int kSegThreads = 256;
enum SegAcc { SA_F = 0, SA_FX = 1, SA_FY = 2, SA_A = 3, SA_B = 4, SA_N = 5 };

__global__ void k_seg_range(const int32_t* __restrict__ seg, int64_t n, int32_t* __restrict__ mm) {
  int lo = INT32_MAX, hi = INT32_MIN;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int v = seg[i];
    lo = min(lo, v);
    hi = max(hi, v);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(mm, lo);
    atomicMax(mm + 1, hi);
  }
}

__global__ void k_seg_mark(const int32_t* __restrict__ seg, int64_t n, uint8_t* __restrict__ present) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    present[seg[i]] = 1;
}

__global__ void k_seg_pass1(const int32_t* __restrict__ seg, const float* __restrict__ img, int nx, int64_t n,
                            const int32_t* __restrict__ index, double* __restrict__ acc, int32_t* __restrict__ bbox) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int k = index[seg[i]];
    if (k < 0) continue;
    const int y = (int)(i / nx), x = (int)(i - (int64_t)y * nx);
    const double f = (double)img[i];
    atomicAdd(acc + k * SA_N + SA_F, f);
    atomicAdd(acc + k * SA_N + SA_FX, f * x);
    atomicAdd(acc + k * SA_N + SA_FY, f * y);
    atomicMin(bbox + 4 * k + 0, x);
    atomicMax(bbox + 4 * k + 1, x);
    atomicMin(bbox + 4 * k + 2, y);
    atomicMax(bbox + 4 * k + 3, y);
  }
}

__global__ void k_seg_centroid(int n_seg, double* __restrict__ acc, const double* __restrict__ cen_in,
                               double* __restrict__ cen) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_seg) return;
  const double* a = acc + k * SA_N;
  cen[2 * k] = cen_in ? cen_in[2 * k] : a[SA_FX] / a[SA_F];
  cen[2 * k + 1] = cen_in ? cen_in[2 * k + 1] : a[SA_FY] / a[SA_F];
}

__global__ void k_seg_pass2(const int32_t* __restrict__ seg, const float* __restrict__ img, int nx, int64_t n,
                            const int32_t* __restrict__ index, const double* __restrict__ cen,
                            double* __restrict__ acc) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int k = index[seg[i]];
    if (k < 0) continue;
    const int y = (int)(i / nx), x = (int)(i - (int64_t)y * nx);
    const double f = (double)img[i];
    const double dx = x - cen[2 * k], dy = y - cen[2 * k + 1];
    const double r2 = dx * dx + dy * dy;
    const double c2 = r2 > 0 ? (dx * dx - dy * dy) / r2 : 1.0;
    const double s2 = r2 > 0 ? (2 * dx * dy) / r2 : 0.0;
    atomicAdd(acc + k * SA_N + SA_A, f * c2);
    atomicAdd(acc + k * SA_N + SA_B, f * s2);
  }
}

__device__ __forceinline__ double pymod_pos(double a, double b) {  // Python a % b, b > 0
  double m = fmod(a, b);
  if (m < 0) m += b;
  return m;
}

__global__ void k_seg_shape(int n_seg, double north, const double* __restrict__ acc, const double* __restrict__ pa_in,
                            double* __restrict__ pa, double* __restrict__ q) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_seg) return;
  const double* a = acc + k * SA_N;
  const double F = a[SA_F];
  const double PA = pa_in ? pa_in[k] : pymod_pos(atan2(a[SA_B] / F, a[SA_A] / F) / 2, kPi) + north;
  pa[k] = PA;
  const double P = PA + north;
  const double C = (F + cos(2 * P) * a[SA_A] + sin(2 * P) * a[SA_B]) / 2;
  const double S = F - C;
  q[k] = (S / F) / fmax(S / F, C / F);
}

// sum of the image over each window [[x0, x1), [y0, y1)] (filter_windows' flux), clipped to
// the image
__global__ void k_window_flux(const float* __restrict__ img, int nx, int ny, const int32_t* __restrict__ wins,
                              double* __restrict__ out) {
  const int w = blockIdx.x;
  const int x0 = min(max(wins[4 * w], 0), nx), x1 = min(max(wins[4 * w + 1], 0), nx);
  const int y0 = min(max(wins[4 * w + 2], 0), ny), y1 = min(max(wins[4 * w + 3], 0), ny);
  const int wx = max(0, x1 - x0), wy = max(0, y1 - y0);
  double s = 0.0;
  for (int64_t e = threadIdx.x; e < (int64_t)wx * wy; e += blockDim.x) {
    const int r = (int)(e / wx), c = (int)(e - (int64_t)r * wx);
    s += (double)img[(int64_t)(y0 + r) * nx + x0 + c];
  }
  __shared__ double red[kSegThreads / 32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < kSegThreads / 32; ++i) t += red[i];
    out[w] = t;
  }
}

__global__ void k_bbox_init(int n_seg, int32_t* bbox) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_seg) return;
  bbox[4 * k] = INT32_MAX;
  bbox[4 * k + 1] = INT32_MIN;
  bbox[4 * k + 2] = INT32_MAX;
  bbox[4 * k + 3] = INT32_MIN;
}

unsigned seg_grid(int64_t n) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t want = (n + kSegThreads - 1) / kSegThreads;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sms * 8));
}

}  // namespace

cudaError_t launch_seg_range(const int32_t* seg, int64_t n, int32_t* mm, cudaStream_t s) {
  const int32_t init[2] = {INT32_MAX, INT32_MIN};
  cudaError_t e = cudaMemcpyAsync(mm, init, sizeof(init), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return e;
  k_seg_range<<<seg_grid(n), kSegThreads, 0, s>>>(seg, n, mm);
  return cudaGetLastError();
}

cudaError_t launch_seg_mark(const int32_t* seg, int64_t n, uint8_t* present, int32_t max_id, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(present, 0, (size_t)max_id + 1, s);
  if (e != cudaSuccess) return e;
  k_seg_mark<<<seg_grid(n), kSegThreads, 0, s>>>(seg, n, present);
  return cudaGetLastError();
}

cudaError_t launch_seg_stats(const int32_t* seg, const float* img, int nx, int ny, const int32_t* index, int n_seg,
                             double north, const double* cen_in, const double* pa_in, double* acc, int32_t* bbox,
                             double* cen, double* pa, double* q, cudaStream_t s) {
  const int64_t n = (int64_t)nx * ny;
  cudaError_t e = cudaMemsetAsync(acc, 0, sizeof(double) * SA_N * (size_t)n_seg, s);
  if (e != cudaSuccess) return e;
  const unsigned g1 = (unsigned)((n_seg + 127) / 128);
  k_bbox_init<<<g1, 128, 0, s>>>(n_seg, bbox);
  k_seg_pass1<<<seg_grid(n), kSegThreads, 0, s>>>(seg, img, nx, n, index, acc, bbox);
  k_seg_centroid<<<g1, 128, 0, s>>>(n_seg, acc, cen_in, cen);
  k_seg_pass2<<<seg_grid(n), kSegThreads, 0, s>>>(seg, img, nx, n, index, cen, acc);
  k_seg_shape<<<g1, 128, 0, s>>>(n_seg, north, acc, pa_in, pa, q);
  return cudaGetLastError();
}

cudaError_t launch_window_flux(const float* img, int nx, int ny, const int32_t* wins, int n, double* out,
                               cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_window_flux<<<n, kSegThreads, 0, s>>>(img, nx, ny, wins, out);
  return cudaGetLastError();
}

}  // namespace apgb
