// Learned initial guess: a 6-layer CNN that maps a 64 x 64 stamp to the 7 Sersic parameters.
//
// No counterpart in the reference (its initial values come from the heuristics of
// models/galaxy_model_object.py:60-113 and models/_shared_methods.py:116-166); the network,
// its training kernels and the moments initialiser used as its fallback are this library's.
//
// Network (activations NHWC, bf16 between layers, fp32 accumulation):
//   L1 conv 3x3 s2 p1   1 ->  32   64x64 -> 32x32   ReLU
//   L2 conv 3x3 s2 p1  32 ->  64   32x32 -> 16x16   ReLU
//   L3 conv 3x3 s2 p1  64 -> 128   16x16 ->  8x8    ReLU
//   L4 conv 3x3 s2 p1 128 -> 256    8x8  ->  4x4    ReLU
//   L5 fc 4096 -> 192                               ReLU
//   L6 fc  192 ->   8 (stored as 16 output rows, rows 8..15 zero)
// 1,176,008 trainable parameters.  Every layer is one GEMM on the tensor cores, bf16 operands
// with fp32 accumulation.  Forward (default path): the tcgen05 kernels of ap_tcgemm.cu (TMEM
// accumulator, TMA-staged operands, bias + ReLU + bf16 in the epilogue); at inference the
// convolutions of layers 2-4 read the NHWC activations through strided TMA loads (implicit
// im2col), for training they run over the im2col matrices the weight gradients need.  The
// backward pass is two GEMMs per layer (weight gradient, input gradient) plus a col2im gather, on
// the ldmatrix + mma.sync tiles below (also the forward's second path, AP_CNN_MMA_SYNC).  Master
// weights, gradients and Adam moments are fp32; the GEMMs read a bf16 mirror of the weights.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <mutex>
#include <tuple>

#include "ap_internal.h"

using apgb::record_cuda;

namespace {

typedef __nv_bfloat16 bf16;

// ---------------------------------------------------------------------------------------------
// layer table
// ---------------------------------------------------------------------------------------------
constexpr int kImg = 64;
constexpr int kNumConv = 4;
constexpr int kOutPad = 16;  // rows of the last layer (8 used)

struct LayerDim {
  int cin, cout, hin, hout;  // conv: channels and square sizes; fc: hin = hout = 1
  int K;                     // reduction length (padded to a multiple of 16)
  int N;                     // output columns
};

__host__ __device__ constexpr LayerDim layer_dim(int l) {
  return l == 0   ? LayerDim{1, 32, 64, 32, 16, 32}
         : l == 1 ? LayerDim{32, 64, 32, 16, 288, 64}
         : l == 2 ? LayerDim{64, 128, 16, 8, 576, 128}
         : l == 3 ? LayerDim{128, 256, 8, 4, 1152, 256}
         : l == 4 ? LayerDim{4096, 192, 1, 1, 4096, 192}
                  : LayerDim{192, kOutPad, 1, 1, 192, kOutPad};
}
constexpr int kLayers = 6;

// parameter blocks: W[N][K] then b[N] per layer, in layer order
__host__ __device__ constexpr int64_t w_off(int l) {
  int64_t o = 0;
  for (int i = 0; i < l; ++i) o += (int64_t)layer_dim(i).N * layer_dim(i).K + layer_dim(i).N;
  return o;
}
__host__ __device__ constexpr int64_t b_off(int l) { return w_off(l) + (int64_t)layer_dim(l).N * layer_dim(l).K; }
constexpr int64_t kParamCount = w_off(kLayers);

// rows (GEMM M) of layer l for a batch of B stamps
__host__ __device__ inline int64_t layer_rows(int l, int64_t B) {
  const LayerDim d = layer_dim(l);
  return B * d.hout * d.hout;
}

// ---------------------------------------------------------------------------------------------
// workspace layout (per batch B); every block 256-byte aligned
// ---------------------------------------------------------------------------------------------
struct CnnWs {
  bf16* col[kLayers];   // GEMM A operand of each layer (col[4] = act[3] flattened, col[5] = act[4])
  float* pre[kLayers];  // GEMM output
  bf16* act[kLayers];   // bias + ReLU, bf16 (act[5] unused)
  float* out;           // [B][16] network output (pre + bias, no ReLU)
  float* dpre_f;        // fp32 scratch: d loss / d layer input (largest layer)
  float* dcol;          // fp32 dcol (largest layer)
  bf16* dpre;           // bf16 d loss / d pre-activation (largest layer)
  double* loss;         // [1]
  size_t act_off[kLayers], out_off;  // byte offsets of act[l] and out in the workspace
  size_t bytes;
};

inline size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

CnnWs cnn_layout(char* base, int64_t B) {
  CnnWs w{};
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* p = base ? base + off : nullptr;
    off += align256(bytes);
    return p;
  };
  size_t max_mn = 0, max_mk = 0;
  for (int l = 0; l < kLayers; ++l) {
    const LayerDim d = layer_dim(l);
    const int64_t M = (l < kNumConv) ? layer_rows(l, B) : B;
    if (l < kNumConv || l == 0) w.col[l] = (bf16*)take((size_t)M * d.K * sizeof(bf16));
    w.pre[l] = (float*)take((size_t)M * d.N * sizeof(float));
    w.act_off[l] = off;
    w.act[l] = (bf16*)take((size_t)M * d.N * sizeof(bf16));
    max_mn = (size_t)M * d.N > max_mn ? (size_t)M * d.N : max_mn;
    max_mk = (size_t)M * d.K > max_mk ? (size_t)M * d.K : max_mk;
  }
  w.col[4] = w.act[3];
  w.col[5] = w.act[4];
  w.out_off = off;
  w.out = (float*)take((size_t)B * kOutPad * sizeof(float));
  w.dpre_f = (float*)take(max_mk * sizeof(float));
  w.dcol = (float*)take(max_mk * sizeof(float));
  w.dpre = (bf16*)take(max_mn * sizeof(bf16));
  w.loss = (double*)take(sizeof(double) * 2);
  w.bytes = off;
  return w;
}

// ---------------------------------------------------------------------------------------------
// GEMM: C[r][s] (+)= sum_t A(r, t) * B(s, t), bf16 operands, fp32 accumulation on the tensor
// cores.  A(r, t) = A[r * lda + t] (A_T = false, reduction contiguous) or A[t * lda + r]
// (A_T = true); the same for B with s.  R, S multiples of 8, T a multiple of 16.
// ---------------------------------------------------------------------------------------------
constexpr int kBK = 32;
constexpr int kSK = kBK + 8;  // smem row stride (bf16): 80 bytes, ldmatrix rows stay 16B aligned

// Optional fused epilogue of a non-split GEMM: v = C + bias[s], ReLU, stored as bf16 into act
// (same row stride as C) instead of C; or, without act, v = C + bias stored into C.
struct GemmEpilogue {
  const float* bias = nullptr;  // null: plain store of C
  bf16* act = nullptr;
  int relu = 0;
};

__device__ __forceinline__ void ldsm_x4(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const void* p) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(a));
}

__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// one operand tile [ROWS][kBK] of rows [x0, x0 + ROWS) and reduction [t0, t1) into smem
template <int ROWS, bool TRANS, int NT>
__device__ __forceinline__ void load_tile(bf16 (*S)[kSK], const bf16* __restrict__ G, int ld, int x0, int X, int t0,
                                          int t1) {
  if (!TRANS) {
    constexpr int CH = ROWS * (kBK / 8);
    for (int c = threadIdx.x; c < CH; c += NT) {
      const int row = c / (kBK / 8), kc = (c % (kBK / 8)) * 8;
      const int x = x0 + row, t = t0 + kc;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (x < X && t + 8 <= t1) v = *reinterpret_cast<const uint4*>(G + (int64_t)x * ld + t);
      *reinterpret_cast<uint4*>(&S[row][kc]) = v;
    }
  } else {
    constexpr int CH = kBK * (ROWS / 8);
    for (int c = threadIdx.x; c < CH; c += NT) {
      const int tl = c / (ROWS / 8), rc = (c % (ROWS / 8)) * 8;
      const int t = t0 + tl, x = x0 + rc;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (t < t1 && x + 8 <= X) v = *reinterpret_cast<const uint4*>(G + (int64_t)t * ld + x);
      const bf16* e = reinterpret_cast<const bf16*>(&v);
#pragma unroll
      for (int i = 0; i < 8; ++i) S[rc + i][tl] = e[i];
    }
  }
}

template <int BM, int BN, int WM, int WN, bool A_T, bool B_T>
__global__ void __launch_bounds__(WM* WN * 32) k_gemm(const bf16* __restrict__ A, int lda, const bf16* __restrict__ B,
                                                      int ldb, float* __restrict__ C, int ldc, int R, int S, int T,
                                                      int t_split, int atomic, GemmEpilogue ep) {
  constexpr int NT = WM * WN * 32;
  constexpr int WTM = BM / WM, WTN = BN / WN;
  constexpr int TM = WTM / 16, TN = WTN / 8;
  static_assert(TN % 2 == 0, "B fragments are loaded in pairs of n8 tiles");
  __shared__ __align__(16) bf16 As[BM][kSK];
  __shared__ __align__(16) bf16 Bs[BN][kSK];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wm = warp / WN, wn = warp % WN;
  const int r0 = blockIdx.x * BM, s0 = blockIdx.y * BN;
  const int tb = blockIdx.z * t_split, te = min(T, tb + t_split);
  float acc[TM][TN][4];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j)
#pragma unroll
      for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.f;

  for (int t0 = tb; t0 < te; t0 += kBK) {
    load_tile<BM, A_T, NT>(As, A, lda, r0, R, t0, te);
    load_tile<BN, B_T, NT>(Bs, B, ldb, s0, S, t0, te);
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kBK; kk += 16) {
      uint32_t af[TM][4], bfr[TN][2];
#pragma unroll
      for (int i = 0; i < TM; ++i)
        ldsm_x4(af[i][0], af[i][1], af[i][2], af[i][3], &As[wm * WTM + i * 16 + (lane & 15)][kk + (lane >> 4) * 8]);
#pragma unroll
      for (int j = 0; j < TN; j += 2)
        ldsm_x4(bfr[j][0], bfr[j][1], bfr[j + 1][0], bfr[j + 1][1],
                &Bs[wn * WTN + j * 8 + (lane & 7) + ((lane >> 4) << 3)][kk + ((lane >> 3) & 1) * 8]);
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) mma_bf16(acc[i][j], af[i], bfr[j]);
    }
    __syncthreads();
  }
  const int g = lane >> 2, c2 = (lane & 3) * 2;
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r = r0 + wm * WTM + i * 16 + g + h * 8;
        const int s = s0 + wn * WTN + j * 8 + c2;
        if (r >= R) continue;
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          if (s + e >= S) continue;
          const int64_t o = (int64_t)r * ldc + s + e;
          float v = acc[i][j][h * 2 + e];
          if (atomic) {
            atomicAdd(C + o, v);
          } else if (ep.bias) {
            v += ep.bias[s + e];
            if (ep.relu) v = fmaxf(v, 0.f);
            if (ep.act)
              ep.act[o] = __float2bfloat16(v);
            else
              C[o] = v;
          } else {
            C[o] = v;
          }
        }
      }
}

int g_num_sms = 0;
int g_cnn_path = AP_CNN_TCGEN05;
bool g_gemm_tune = false;
std::mutex g_tune_mutex;
std::map<std::tuple<int, int, int, int, int>, int> g_tuned;  // (A_T, B_T, R, S, T) -> tile shape

// ep.bias set: the epilogue is fused when the reduction is not split; *fused tells the caller.
// allow_split = false keeps every reduction in one CTA (no float atomics: results independent of
// scheduling, as the forward pass needs for reproducible proposals)
template <bool A_T, bool B_T>
cudaError_t gemm(const bf16* A, int lda, const bf16* B, int ldb, float* C, int ldc, int R, int S, int T,
                 cudaStream_t st, GemmEpilogue ep = GemmEpilogue(), bool* fused = nullptr, bool allow_split = true) {
  if (fused) *fused = false;
  if (R <= 0 || S <= 0 || T <= 0) return cudaSuccess;
  if (!g_num_sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0) g_num_sms = 148;
  }
  auto run = [&](auto kern, int BM, int BN, int threads) {
    const int gx = (R + BM - 1) / BM, gy = (S + BN - 1) / BN;
    const int tiles = gx * gy;
    // split the reduction when the output tiles alone cannot fill the GPU
    int split = 1;
    const int want = 2 * g_num_sms;
    if (allow_split && tiles < want) {
      const int max_split = (T + 8 * kBK - 1) / (8 * kBK);  // at least 8 k-steps per split
      split = (want + tiles - 1) / tiles;
      if (split > max_split) split = max_split;
      if (split < 1) split = 1;
    }
    int t_split = (T + split - 1) / split;
    t_split = (t_split + kBK - 1) / kBK * kBK;
    split = (T + t_split - 1) / t_split;
    if (split > 1) {
      cudaError_t e = cudaMemsetAsync(C, 0, sizeof(float) * ((size_t)(R - 1) * ldc + S), st);
      if (e != cudaSuccess) return e;
    }
    const GemmEpilogue use = split > 1 ? GemmEpilogue() : ep;
    if (fused) *fused = (split == 1) && ep.bias != nullptr;
    kern<<<dim3(gx, gy, split), threads, 0, st>>>(A, lda, B, ldb, C, ldc, R, S, T, t_split, split > 1 ? 1 : 0, use);
    return cudaGetLastError();
  };
  auto run_cfg = [&](int cfg) {
    if (cfg == 0) return run(k_gemm<128, 128, 2, 4, A_T, B_T>, 128, 128, 256);
    if (cfg == 1) return run(k_gemm<128, 64, 4, 2, A_T, B_T>, 128, 64, 256);
    return run(k_gemm<128, 32, 4, 1, A_T, B_T>, 128, 32, 128);
  };
  const int heuristic = S >= 128 ? 0 : (S >= 64 ? 1 : 2);
  if (!g_gemm_tune) return run_cfg(heuristic);
  // in-project autotuner: the first call of each (layout, shape) times the three tile shapes
  // (outside stream capture) and keeps the fastest for the later calls
  const auto key = std::make_tuple((int)A_T, (int)B_T, R, S, T);
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) return run_cfg(it->second);
  }
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return run_cfg(heuristic);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int best = heuristic;
  float best_ms = 1e30f;
  cudaError_t err = cudaSuccess;
  for (int cfg = 0; cfg < 3 && err == cudaSuccess; ++cfg) {
    err = run_cfg(cfg);  // warm
    float ms_min = 1e30f;
    for (int rep = 0; rep < 2 && err == cudaSuccess; ++rep) {
      cudaEventRecord(e0, st);
      err = run_cfg(cfg);
      cudaEventRecord(e1, st);
      if (err == cudaSuccess) err = cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      ms_min = ms < ms_min ? ms : ms_min;
    }
    if (ms_min < best_ms) {
      best_ms = ms_min;
      best = cfg;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (err != cudaSuccess) return err;
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tuned[key] = best;
  }
  return run_cfg(best);
}

// ---------------------------------------------------------------------------------------------
// elementwise kernels
// ---------------------------------------------------------------------------------------------
// L1 im2col of the fp32 input stamps: col[m][0..8] = 3x3 window (zero outside), [9..15] = 0
__global__ void k_im2col_in(const float* __restrict__ x, bf16* __restrict__ col, int64_t B) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= B * 32 * 32) return;
  const int64_t b = m / 1024;
  const int p = (int)(m - b * 1024), oy = p / 32, ox = p % 32;
  __align__(16) bf16 v[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    float f = 0.f;
    if (k < 9) {
      const int iy = 2 * oy - 1 + k / 3, ix = 2 * ox - 1 + k % 3;
      if (iy >= 0 && iy < kImg && ix >= 0 && ix < kImg) f = x[b * kImg * kImg + iy * kImg + ix];
    }
    v[k] = __float2bfloat16(f);
  }
  uint4* dst = reinterpret_cast<uint4*>(col + m * 16);
  dst[0] = reinterpret_cast<const uint4*>(v)[0];
  dst[1] = reinterpret_cast<const uint4*>(v)[1];
}

// im2col of an NHWC bf16 activation, 3x3 stride 2 pad 1, k = (ky * 3 + kx) * C + c
__global__ void k_im2col(const bf16* __restrict__ act, bf16* __restrict__ col, int64_t B, int H, int C) {
  const int Ho = H / 2, C8 = C / 8;
  const int64_t n = B * Ho * Ho * 9 * C8;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int c8 = (int)(i % C8);
    const int64_t r = i / C8;
    const int tap = (int)(r % 9);
    const int64_t m = r / 9;
    const int64_t b = m / (Ho * Ho);
    const int p = (int)(m - b * Ho * Ho), oy = p / Ho, ox = p % Ho;
    const int iy = 2 * oy - 1 + tap / 3, ix = 2 * ox - 1 + tap % 3;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (iy >= 0 && iy < H && ix >= 0 && ix < H)
      v = *reinterpret_cast<const uint4*>(act + ((b * H + iy) * H + ix) * C + c8 * 8);
    *reinterpret_cast<uint4*>(col + m * 9 * C + tap * C + c8 * 8) = v;
  }
}

// dX[b][iy][ix][c] = sum of dcol over the (oy, ox, tap) that read it
__global__ void k_col2im(const float* __restrict__ dcol, float* __restrict__ dx, int64_t B, int H, int C) {
  const int Ho = H / 2;
  const int64_t n = B * H * H * C;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    const int64_t r = i / C;
    const int ix = (int)(r % H);
    const int64_t r2 = r / H;
    const int iy = (int)(r2 % H);
    const int64_t b = r2 / H;
    float s = 0.f;
#pragma unroll
    for (int ky = 0; ky < 3; ++ky) {
      const int ty = iy + 1 - ky;
      if (ty < 0 || (ty & 1)) continue;
      const int oy = ty >> 1;
      if (oy >= Ho) continue;
#pragma unroll
      for (int kx = 0; kx < 3; ++kx) {
        const int tx = ix + 1 - kx;
        if (tx < 0 || (tx & 1)) continue;
        const int ox = tx >> 1;
        if (ox >= Ho) continue;
        s += dcol[((b * Ho + oy) * Ho + ox) * 9 * C + (ky * 3 + kx) * C + c];
      }
    }
    dx[i] = s;
  }
}

// act = bf16(max(pre + bias, 0)) (relu) or out = pre + bias (fp32, last layer)
__global__ void k_bias_act(const float* __restrict__ pre, const float* __restrict__ bias, bf16* __restrict__ act,
                           float* __restrict__ out, int64_t M, int N, int relu) {
  const int64_t n = M * N;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float v = pre[i] + bias[i % N];
    if (relu) v = fmaxf(v, 0.f);
    if (act) act[i] = __float2bfloat16(v);
    if (out) out[i] = v;
  }
}

// dpre = bf16(dA * (act > 0)) (or no mask), db[n] += column sums; one block per row chunk
__global__ void k_act_back(const float* __restrict__ dA, const bf16* __restrict__ act, bf16* __restrict__ dpre,
                           float* __restrict__ db, int64_t M, int N, int rows_per_block) {
  const int64_t m0 = (int64_t)blockIdx.x * rows_per_block;
  const int64_t m1 = min(M, m0 + rows_per_block);
  for (int n = threadIdx.x; n < N; n += blockDim.x) {
    float s = 0.f;
    for (int64_t m = m0; m < m1; ++m) {
      const int64_t i = m * N + n;
      float v = dA[i];
      if (act && !(__bfloat162float(act[i]) > 0.f)) v = 0.f;
      dpre[i] = __float2bfloat16(v);
      s += v;
    }
    atomicAdd(db + n, s);
  }
}

// standardised targets t[B][8]; out[B][16]; dout = 2 (out - t) / (B * 8) on the 8 used columns
__global__ void k_mse(const float* __restrict__ out, const float* __restrict__ t, float* __restrict__ dout,
                      double* loss, int64_t B) {
  const int64_t n = B * kOutPad;
  double local = 0.0;
  const float inv = 2.f / (float)(B * 8);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / kOutPad;
    const int k = (int)(i % kOutPad);
    float g = 0.f;
    if (k < 8) {
      const float d = out[i] - t[b * 8 + k];
      g = d * inv;
      local += (double)d * d;
    }
    dout[i] = g;
  }
  for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, local / (double)(B * 8));
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                       float* __restrict__ m2, bf16* __restrict__ pb, int64_t n, float lr, float b1, float b2,
                       float eps, float c1, float c2, float wd) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float a = b1 * m1[i] + (1.f - b1) * gi;
    const float v = b2 * m2[i] + (1.f - b2) * gi * gi;
    m1[i] = a;
    m2[i] = v;
    const float mh = a / c1, vh = v / c2;
    const float q = p[i] * (1.f - lr * wd) - lr * mh / (sqrtf(vh) + eps);
    p[i] = q;
    pb[i] = __float2bfloat16(q);
  }
}

__global__ void k_to_bf16(const float* __restrict__ p, bf16* __restrict__ pb, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    pb[i] = __float2bfloat16(p[i]);
}

inline int grid_for(int64_t n, int threads = 256) {
  int64_t g = (n + threads - 1) / threads;
  const int64_t cap = (int64_t)(g_num_sms > 0 ? g_num_sms : 148) * 16;
  return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

// ---------------------------------------------------------------------------------------------
// input preparation, decoding, moments initialiser
// ---------------------------------------------------------------------------------------------
// x = asinh((d - sky) / (4 sigma)): pixel signal-to-noise, compressed; lscale = log10(sigma)
__global__ void k_prepare(const float* __restrict__ data, const float* __restrict__ sky,
                          const float* __restrict__ sigma, float* __restrict__ x, float* __restrict__ lscale,
                          int64_t B) {
  const int64_t b = blockIdx.x;
  if (b >= B) return;
  const float* d = data + b * kImg * kImg;
  const float sk = sky[b], sg = fmaxf(sigma[b], 1e-30f);
  const float inv = 0.25f / sg;
  if (threadIdx.x == 0) lscale[b] = log10f(sg);
  for (int i = threadIdx.x; i < kImg * kImg; i += blockDim.x) x[b * kImg * kImg + i] = asinhf((d[i] - sk) * inv);
}

// network output (standardised) -> full parameter vector [cx, cy, q, PA, n, Re, Ie, F]
// outputs: 0 cx - 32, 1 cy - 32, 2 q, 3 cos 2PA, 4 sin 2PA, 5 ln n, 6 ln Re, 7 log10 Ie - log10 s
__global__ void k_decode(const float* __restrict__ out, const float* __restrict__ lscale, const float* __restrict__ mean,
                         const float* __restrict__ stdv, const double* __restrict__ sky_F, double* __restrict__ params,
                         int64_t B) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  double y[8];
  for (int k = 0; k < 8; ++k) y[k] = (double)out[b * kOutPad + k] * stdv[k] + mean[k];
  double* p = params + b * 8;
  p[0] = kImg / 2 + y[0];
  p[1] = kImg / 2 + y[1];
  p[2] = fmin(fmax(y[2], 0.05), 0.995);
  double pa = 0.5 * atan2(y[4], y[3]);
  const double pi = 3.14159265358979323846;
  pa = fmod(pa + pi, pi);
  if (pa < 0) pa += pi;
  if (pa >= pi) pa = 0.0;
  p[3] = pa;
  p[4] = fmin(fmax(exp(y[5]), 0.4), 7.9);
  p[5] = fmax(exp(y[6]), 0.3);
  p[6] = y[7] + (double)lscale[b];
  p[7] = sky_F[b];
}

// Flux-weighted moments initial guess of one 64 x 64 stamp (one block per stamp):
// centre of light, PA and q from the second moments, Re as the elliptical radius holding half
// of the light, n = 2, Ie from the mean surface brightness of the annulus at Re.
constexpr int kMomBins = 64;
__global__ void k_moments_init(const float* __restrict__ data, const float* __restrict__ sky,
                               const float* __restrict__ sigma, const double* __restrict__ sky_F,
                               double* __restrict__ params, int64_t B) {
  const int64_t b = blockIdx.x;
  if (b >= B) return;
  const float* d = data + b * kImg * kImg;
  const float sk = sky[b], thr = 1.0f * sigma[b];
  __shared__ double red[6][8];
  __shared__ float hist_f[kMomBins], hist_n[kMomBins];
  __shared__ float whist_f[8][kMomBins], whist_n[8][kMomBins];  // per-warp histograms (256 threads)
  __shared__ double sh_par[6];
  double S = 0, Sx = 0, Sy = 0;
  for (int i = threadIdx.x; i < kImg * kImg; i += blockDim.x) {
    const float w = d[i] - sk;
    if (w > thr) {
      const double x = (i % kImg) + 0.5, y = (i / kImg) + 0.5;
      S += w;
      Sx += w * x;
      Sy += w * y;
    }
  }
  auto block_sum = [&](double v, int slot) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[slot][threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[slot][k];
    __syncthreads();
    return t;
  };
  S = block_sum(S, 0);
  Sx = block_sum(Sx, 1);
  Sy = block_sum(Sy, 2);
  const double cx = S > 0 ? Sx / S : kImg / 2, cy = S > 0 ? Sy / S : kImg / 2;
  double Mxx = 0, Myy = 0, Mxy = 0;
  for (int i = threadIdx.x; i < kImg * kImg; i += blockDim.x) {
    const float w = d[i] - sk;
    if (w > thr) {
      const double x = (i % kImg) + 0.5 - cx, y = (i / kImg) + 0.5 - cy;
      Mxx += w * x * x;
      Myy += w * y * y;
      Mxy += w * x * y;
    }
  }
  Mxx = block_sum(Mxx, 3);
  Myy = block_sum(Myy, 4);
  Mxy = block_sum(Mxy, 5);
  if (threadIdx.x == 0) {
    const double pi = 3.14159265358979323846;
    const double tr = Mxx + Myy, det = Mxx * Myy - Mxy * Mxy;
    const double disc = sqrt(fmax(tr * tr / 4 - det, 0.0));
    const double l1 = tr / 2 + disc, l2 = fmax(tr / 2 - disc, 1e-12);
    double q = (l1 > 0) ? sqrt(l2 / l1) : 0.7;
    q = fmin(fmax(q, 0.1), 0.95);
    // major axis angle from +x; the model's major axis lies at PA - pi/2 from +x
    const double theta = 0.5 * atan2(2 * Mxy, Mxx - Myy);
    double pa = fmod(theta + pi / 2 + 2 * pi, pi);
    sh_par[0] = cx;
    sh_par[1] = cy;
    sh_par[2] = q;
    sh_par[3] = pa;
  }
  for (int k = threadIdx.x; k < 8 * kMomBins; k += blockDim.x) {
    whist_f[k / kMomBins][k % kMomBins] = 0.f;
    whist_n[k / kMomBins][k % kMomBins] = 0.f;
  }
  __syncthreads();
  const double q = sh_par[2], pa = sh_par[3];
  const double ca = cos(pa - 1.5707963267948966), sa = sin(pa - 1.5707963267948966);
  const float rmax = 0.75f * kImg;
  // radial histogram in a fixed summation order (no float atomics): each warp walks its 512
  // pixels 32 at a time; the lanes of one bin sum their values in lane order and the lowest of
  // them adds the sum to the warp's histogram; the 8 warp histograms are then added in order
  {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int per_warp = kImg * kImg / 8;
    for (int base = warp * per_warp; base < (warp + 1) * per_warp; base += 32) {
      const int i = base + lane;
      const double x = (i % kImg) + 0.5 - sh_par[0], y = (i / kImg) + 0.5 - sh_par[1];
      const double u = x * ca + y * sa, v = (-x * sa + y * ca) / q;
      const float r = (float)sqrt(u * u + v * v);
      const int k = min(kMomBins - 1, (int)(r / rmax * kMomBins));
      const float val = d[i] - sk;
      const unsigned same = __match_any_sync(0xffffffffu, k);
      float acc = 0.f, cnt = 0.f;
      for (int src = 0; src < 32; ++src) {
        const float vs = __shfl_sync(0xffffffffu, val, src);
        if ((same >> src) & 1u) {
          acc += vs;
          cnt += 1.f;
        }
      }
      if (lane == __ffs(same) - 1) {
        whist_f[warp][k] += acc;
        whist_n[warp][k] += cnt;
      }
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < kMomBins; k += blockDim.x) {
    float f = 0.f, c = 0.f;
    for (int w = 0; w < 8; ++w) {
      f += whist_f[w][k];
      c += whist_n[w][k];
    }
    hist_f[k] = f;
    hist_n[k] = c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0;
    for (int k = 0; k < kMomBins; ++k) tot += hist_f[k];
    double cum = 0, re = 5.0;
    int kre = 0;
    for (int k = 0; k < kMomBins; ++k) {
      const double prev = cum;
      cum += hist_f[k];
      if (tot > 0 && cum >= 0.5 * tot) {
        const double frac = hist_f[k] > 0 ? (0.5 * tot - prev) / hist_f[k] : 0.5;
        re = (k + frac) * rmax / kMomBins;
        kre = k;
        break;
      }
    }
    re = fmax(re, 1.0);
    const double ie = (hist_n[kre] > 0 && hist_f[kre] > 0) ? hist_f[kre] / hist_n[kre] : fmax(tot, 1.0) / 1000.0;
    double* p = params + b * 8;
    p[0] = sh_par[0];
    p[1] = sh_par[1];
    p[2] = sh_par[2];
    p[3] = sh_par[3];
    p[4] = 2.0;
    p[5] = re;
    p[6] = log10(fmax(ie, 1e-6));
    p[7] = sky_F[b];
  }
}

// pick the initial vector with the lower chi2 per stamp (learned proposal vs fallback)
__global__ void k_select_init(const double* __restrict__ pa, const double* __restrict__ pb,
                              const double* __restrict__ ca, const double* __restrict__ cb, double* __restrict__ out,
                              int32_t* __restrict__ which, int64_t B) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B) return;
  const bool use_a = ca[i] <= cb[i];  // NaN chi2 of the proposal selects the fallback
  for (int k = 0; k < 8; ++k) out[i * 8 + k] = use_a ? pa[i * 8 + k] : pb[i * 8 + k];
  which[i] = use_a ? 0 : 1;
}

// ---------------------------------------------------------------------------------------------
// forward / backward drivers
// ---------------------------------------------------------------------------------------------
// tcgen05 forward: bias + ReLU + bf16 in every GEMM epilogue; the convolutions of layers 2-4
// read their inputs straight from the NHWC activations (implicit im2col by strided TMA loads)
// unless need_cols asks for the im2col matrices (kept for the weight gradients).
cudaError_t forward_tc(const float* params, const bf16* wb, const float* x, int64_t B, const CnnWs& w,
                       cudaStream_t st, bool need_cols) {
  cudaError_t e;
  k_im2col_in<<<(unsigned)((B * 1024 + 255) / 256), 256, 0, st>>>(x, w.col[0], B);
  for (int l = 0; l < kLayers; ++l) {
    const LayerDim d = layer_dim(l);
    const int64_t M = (l < kNumConv) ? layer_rows(l, B) : B;
    const bool last = (l == kLayers - 1);
    apgb::TcEpilogue ep;
    ep.bias = params + b_off(l);
    ep.act = last ? nullptr : w.act[l];
    ep.relu = last ? 0 : 1;
    float* cout = last ? w.out : nullptr;
    const int ldc = last ? kOutPad : d.N;
    if (l >= 1 && l < kNumConv && !need_cols) {
      const LayerDim dp = layer_dim(l - 1);
      e = apgb::tc_conv3x3s2(w.act[l - 1], B, dp.hout, d.cin, wb + w_off(l), d.N, cout, ldc, ep, st);
    } else {
      if (l >= 1 && l < kNumConv) {
        const LayerDim dp = layer_dim(l - 1);
        k_im2col<<<grid_for(M * 9 * (d.cin / 8)), 256, 0, st>>>(w.act[l - 1], w.col[l], B, dp.hout, d.cin);
      }
      e = apgb::tc_gemm(w.col[l], d.K, wb + w_off(l), d.K, cout, ldc, (int)M, d.N, d.K, ep, st);
    }
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

cudaError_t forward(const float* params, const bf16* wb, const float* x, int64_t B, const CnnWs& w, cudaStream_t st,
                    bool need_cols = false) {
  if (g_cnn_path == AP_CNN_TCGEN05) return forward_tc(params, wb, x, B, w, st, need_cols);
  cudaError_t e;
  k_im2col_in<<<(unsigned)((B * 1024 + 255) / 256), 256, 0, st>>>(x, w.col[0], B);
  for (int l = 0; l < kLayers; ++l) {
    const LayerDim d = layer_dim(l);
    const int64_t M = (l < kNumConv) ? layer_rows(l, B) : B;
    if (l >= 1 && l < kNumConv) {
      const LayerDim dp = layer_dim(l - 1);
      k_im2col<<<grid_for(M * 9 * (d.cin / 8)), 256, 0, st>>>(w.act[l - 1], w.col[l], B, dp.hout, d.cin);
    }
    const bool last = (l == kLayers - 1);
    // bias + ReLU + bf16 fused into the GEMM epilogue when the reduction is not split
    GemmEpilogue ep;
    ep.bias = params + b_off(l);
    ep.act = last ? nullptr : w.act[l];
    ep.relu = last ? 0 : 1;
    float* cout = last ? w.out : w.pre[l];
    bool fused = false;
    e = gemm<false, false>(w.col[l], d.K, wb + w_off(l), d.K, cout, d.N, (int)M, d.N, d.K, st, ep, &fused, false);
    if (e != cudaSuccess) return e;
    if (!fused)
      k_bias_act<<<grid_for(M * d.N), 256, 0, st>>>(cout, params + b_off(l), last ? nullptr : w.act[l],
                                                    last ? w.out : nullptr, M, d.N, last ? 0 : 1);
  }
  return cudaGetLastError();
}

// gradients (fp32, flat, same layout as the parameters) of the loss whose d/d out is dout
cudaError_t backward(const bf16* wb, const float* dout, float* grads, int64_t B, const CnnWs& w, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(grads, 0, sizeof(float) * kParamCount, st);
  if (e != cudaSuccess) return e;
  const float* dA = dout;
  for (int l = kLayers - 1; l >= 0; --l) {
    const LayerDim d = layer_dim(l);
    const int64_t M = (l < kNumConv) ? layer_rows(l, B) : B;
    const bool last = (l == kLayers - 1);
    // rows per block: enough blocks to fill the GPU, few enough atomics on the bias gradient
    const int64_t nblk_target = 4 * (g_num_sms > 0 ? g_num_sms : 148);
    const int64_t rpb_want = (M + nblk_target - 1) / nblk_target;
    const int rpb = (int)(rpb_want < 16 ? 16 : rpb_want);
    k_act_back<<<(unsigned)((M + rpb - 1) / rpb), 256, 0, st>>>(dA, last ? nullptr : w.act[l], w.dpre,
                                                               grads + b_off(l), M, d.N, rpb);
    // dW[N][K] = dpre^T . col   (reduction over the M rows)
    e = gemm<true, true>(w.dpre, d.N, w.col[l], d.K, grads + w_off(l), d.K, d.N, d.K, (int)M, st);
    if (e != cudaSuccess) return e;
    if (l == 0) break;
    // d input: dcol[M][K] = dpre . W
    float* dst = (l >= kNumConv) ? w.dpre_f : w.dcol;
    e = gemm<false, true>(w.dpre, d.N, wb + w_off(l), d.K, dst, d.K, (int)M, d.K, d.N, st);
    if (e != cudaSuccess) return e;
    if (l < kNumConv) {
      const LayerDim dp = layer_dim(l - 1);
      k_col2im<<<grid_for(B * dp.hout * dp.hout * dp.cout), 256, 0, st>>>(w.dcol, w.dpre_f, B, dp.hout, dp.cout);
    }
    dA = w.dpre_f;
  }
  return cudaGetLastError();
}

}  // namespace

extern "C" {

int64_t ap_cnn_param_count(void) { return kParamCount; }

int ap_cnn_autotune(int32_t enable, int32_t* tuned_shapes) {
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  g_gemm_tune = enable != 0;
  if (enable < 0) g_tuned.clear();
  if (tuned_shapes) *tuned_shapes = (int32_t)g_tuned.size();
  return AP_OK;
}

size_t ap_cnn_workspace_bytes(int64_t batch) {
  if (batch <= 0) return 0;
  return cnn_layout(nullptr, batch).bytes;
}

int ap_cnn_workspace_offsets(int64_t batch, int64_t* act_offsets, int64_t* out_offset) {
  if (batch <= 0 || !act_offsets || !out_offset) return AP_ERR_ARG;
  const CnnWs w = cnn_layout(nullptr, batch);
  for (int l = 0; l < kLayers; ++l) act_offsets[l] = (int64_t)w.act_off[l];
  *out_offset = (int64_t)w.out_off;
  return AP_OK;
}

int ap_cnn_layer_offsets(int64_t* w_offsets, int64_t* b_offsets, int32_t* dims) {
  if (!w_offsets || !b_offsets || !dims) return AP_ERR_ARG;
  for (int l = 0; l < kLayers; ++l) {
    w_offsets[l] = w_off(l);
    b_offsets[l] = b_off(l);
    const LayerDim d = layer_dim(l);
    dims[l * 6 + 0] = d.cin;
    dims[l * 6 + 1] = d.cout;
    dims[l * 6 + 2] = d.hin;
    dims[l * 6 + 3] = d.hout;
    dims[l * 6 + 4] = d.K;
    dims[l * 6 + 5] = d.N;
  }
  return AP_OK;
}

static int cnn_check(cudaError_t e) { return record_cuda(e); }

int ap_cnn_to_bf16(const float* params, void* params_bf16, ap_stream_t stream) {
  if (!params || !params_bf16) return AP_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  k_to_bf16<<<grid_for(kParamCount), 256, 0, st>>>(params, (bf16*)params_bf16, kParamCount);
  return cnn_check(cudaGetLastError());
}

int ap_cnn_forward(const float* params, const void* params_bf16, const float* x, int64_t batch, float* out,
                   void* ws, size_t ws_bytes, ap_stream_t stream) {
  if (!params || !params_bf16 || !x || !out || !ws || batch <= 0 || batch % 16) return AP_ERR_ARG;
  if (ws_bytes < ap_cnn_workspace_bytes(batch)) return AP_ERR_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  CnnWs w = cnn_layout((char*)ws, batch);
  // the im2col matrices stay in the workspace for a later ap_cnn_backward
  int rc = cnn_check(forward(params, (const bf16*)params_bf16, x, batch, w, st, true));
  if (rc) return rc;
  return cnn_check(cudaMemcpyAsync(out, w.out, sizeof(float) * batch * kOutPad, cudaMemcpyDeviceToDevice, st));
}

int ap_cnn_infer(const float* params, const void* params_bf16, const float* x, int64_t batch, float* out, void* ws,
                 size_t ws_bytes, ap_stream_t stream) {
  if (!params || !params_bf16 || !x || !out || !ws || batch <= 0 || batch % 16) return AP_ERR_ARG;
  if (ws_bytes < ap_cnn_workspace_bytes(batch)) return AP_ERR_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  CnnWs w = cnn_layout((char*)ws, batch);
  int rc = cnn_check(forward(params, (const bf16*)params_bf16, x, batch, w, st, false));
  if (rc) return rc;
  return cnn_check(cudaMemcpyAsync(out, w.out, sizeof(float) * batch * kOutPad, cudaMemcpyDeviceToDevice, st));
}

int ap_cnn_backward(const void* params_bf16, const float* dout, int64_t batch, float* grads, void* ws,
                    size_t ws_bytes, ap_stream_t stream) {
  if (!params_bf16 || !dout || !grads || !ws || batch <= 0 || batch % 16) return AP_ERR_ARG;
  if (ws_bytes < ap_cnn_workspace_bytes(batch)) return AP_ERR_WORKSPACE;
  CnnWs w = cnn_layout((char*)ws, batch);
  return cnn_check(backward((const bf16*)params_bf16, dout, grads, batch, w, (cudaStream_t)stream));
}

int ap_cnn_train_step(float* params, void* params_bf16, float* grads, float* adam_m, float* adam_v,
                      const float* x, const float* targets, int64_t batch, float lr, int32_t step,
                      float weight_decay, double* loss_out, void* ws, size_t ws_bytes, ap_stream_t stream) {
  if (!params || !params_bf16 || !grads || !adam_m || !adam_v || !x || !targets || batch <= 0 || batch % 16 ||
      step < 1 || !ws)
    return AP_ERR_ARG;
  if (ws_bytes < ap_cnn_workspace_bytes(batch)) return AP_ERR_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  CnnWs w = cnn_layout((char*)ws, batch);
  bf16* wb = (bf16*)params_bf16;
  int rc = cnn_check(forward(params, wb, x, batch, w, st, true));
  if (rc) return rc;
  rc = cnn_check(cudaMemsetAsync(w.loss, 0, sizeof(double), st));
  if (rc) return rc;
  // dout reuses the fp32 d-input scratch (free until the first layer's backward)
  float* dout = w.dcol;
  k_mse<<<grid_for(batch * kOutPad), 256, 0, st>>>(w.out, targets, dout, w.loss, batch);
  rc = cnn_check(backward(wb, dout, grads, batch, w, st));
  if (rc) return rc;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  k_adam<<<grid_for(kParamCount), 256, 0, st>>>(params, grads, adam_m, adam_v, wb, kParamCount, lr, b1, b2, 1e-8f,
                                               c1, c2, weight_decay);
  if (loss_out) {
    rc = cnn_check(cudaMemcpyAsync(loss_out, w.loss, sizeof(double), cudaMemcpyDeviceToDevice, st));
    if (rc) return rc;
  }
  return cnn_check(cudaGetLastError());
}

int ap_cnn_prepare(const float* data, const float* sky, const float* sigma, int64_t batch, float* x, float* lscale,
                   ap_stream_t stream) {
  if (!data || !sky || !sigma || !x || !lscale || batch <= 0) return AP_ERR_ARG;
  k_prepare<<<(unsigned)batch, 256, 0, (cudaStream_t)stream>>>(data, sky, sigma, x, lscale, batch);
  return cnn_check(cudaGetLastError());
}

int ap_cnn_decode(const float* out, const float* lscale, const float* mean, const float* stdv, const double* sky_F,
                  int64_t batch, double* params, ap_stream_t stream) {
  if (!out || !lscale || !mean || !stdv || !sky_F || !params || batch <= 0) return AP_ERR_ARG;
  k_decode<<<(unsigned)((batch + 127) / 128), 128, 0, (cudaStream_t)stream>>>(out, lscale, mean, stdv, sky_F, params,
                                                                            batch);
  return cnn_check(cudaGetLastError());
}

int ap_moments_init(const float* data, const float* sky, const float* sigma, const double* sky_F, int64_t batch,
                    double* params, ap_stream_t stream) {
  if (!data || !sky || !sigma || !sky_F || !params || batch <= 0) return AP_ERR_ARG;
  k_moments_init<<<(unsigned)batch, 256, 0, (cudaStream_t)stream>>>(data, sky, sigma, sky_F, params, batch);
  return cnn_check(cudaGetLastError());
}

int ap_select_init(const double* proposal, const double* fallback, const double* chi2_proposal,
                   const double* chi2_fallback, int64_t batch, double* out, int32_t* which, ap_stream_t stream) {
  if (!proposal || !fallback || !chi2_proposal || !chi2_fallback || !out || !which || batch <= 0) return AP_ERR_ARG;
  k_select_init<<<(unsigned)((batch + 127) / 128), 128, 0, (cudaStream_t)stream>>>(proposal, fallback, chi2_proposal,
                                                                                 chi2_fallback, out, which, batch);
  return cnn_check(cudaGetLastError());
}

// Plain bf16 GEMM entry (C[R][S] = sum_t A(r,t) B(s,t)), exposed for the numerics tests of
// the tensor-core kernel: a_trans / b_trans select the reduction-strided layouts.
int ap_gemm_bf16(const void* A, int32_t lda, int32_t a_trans, const void* B, int32_t ldb, int32_t b_trans, float* C,
                 int32_t ldc, int32_t R, int32_t S, int32_t T, ap_stream_t stream) {
  if (!A || !B || !C || R <= 0 || S <= 0 || T <= 0) return AP_ERR_ARG;
  if ((R % 8) || (S % 8) || (T % 16) || (lda % 8) || (ldb % 8)) return AP_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  const bf16* a = (const bf16*)A;
  const bf16* b = (const bf16*)B;
  cudaError_t e;
  if (!a_trans && !b_trans)
    e = gemm<false, false>(a, lda, b, ldb, C, ldc, R, S, T, st);
  else if (!a_trans && b_trans)
    e = gemm<false, true>(a, lda, b, ldb, C, ldc, R, S, T, st);
  else if (a_trans && b_trans)
    e = gemm<true, true>(a, lda, b, ldb, C, ldc, R, S, T, st);
  else
    e = gemm<true, false>(a, lda, b, ldb, C, ldc, R, S, T, st);
  return cnn_check(e);
}

int ap_cnn_set_path(int32_t path) {
  if (path != AP_CNN_MMA_SYNC && path != AP_CNN_TCGEN05) return AP_ERR_ARG;
  g_cnn_path = path;
  return AP_OK;
}

int ap_cnn_get_path(int32_t* path) {
  if (!path) return AP_ERR_ARG;
  *path = g_cnn_path;
  return AP_OK;
}

int ap_gemm_bf16_tc(const void* A, int32_t lda, const void* W, int32_t ldw, float* C, int32_t ldc, int32_t R,
                    int32_t S, int32_t T, const float* bias, void* act, int32_t relu, ap_stream_t stream) {
  if (!A || !W || (!C && !act) || R <= 0 || S <= 0 || T <= 0) return AP_ERR_ARG;
  apgb::TcEpilogue ep;
  ep.bias = bias;
  ep.act = (bf16*)act;
  ep.relu = relu;
  const cudaError_t e = apgb::tc_gemm((const bf16*)A, lda, (const bf16*)W, ldw, C, ldc, R, S, T, ep,
                                      (cudaStream_t)stream);
  if (e == cudaErrorInvalidValue) return AP_ERR_ARG;
  return cnn_check(e);
}

int ap_conv3x3s2_bf16_tc(const void* x, int64_t batch, int32_t H, int32_t cin, const void* W, int32_t S, float* C,
                         int32_t ldc, const float* bias, void* act, int32_t relu, ap_stream_t stream) {
  if (!x || !W || (!C && !act) || batch <= 0 || H <= 0 || cin <= 0 || S <= 0) return AP_ERR_ARG;
  apgb::TcEpilogue ep;
  ep.bias = bias;
  ep.act = (bf16*)act;
  ep.relu = relu;
  const cudaError_t e = apgb::tc_conv3x3s2((const bf16*)x, batch, H, cin, (const bf16*)W, S, C, ldc, ep,
                                           (cudaStream_t)stream);
  if (e == cudaErrorInvalidValue) return AP_ERR_ARG;
  return cnn_check(e);
}

int ap_tc_status(int32_t clear, uint32_t* code) {
  if (!code) return AP_ERR_ARG;
  const unsigned v = apgb::tc_error(clear != 0);
  if (v == 0xFFFFFFFFu) return cnn_check(cudaGetLastError());
  *code = v;
  return AP_OK;
}

}  // extern "C"
