// Blackwell tensor-core GEMM for the learned initial guess: tcgen05.mma (bf16 x bf16 -> fp32)
// with the accumulator in tensor memory (TMEM), operand tiles staged by TMA
// (cp.async.bulk.tensor) into swizzled shared memory through an mbarrier ring.
//
// C[r][s] = sum_t A(r, t) W(s, t), both operands reduction-contiguous (K-major):
//   dense: A(r, t) = A[r * lda + t], W(s, t) = W[s * ldw + t]
//   conv:  A(r, t) = row r of the implicit im2col matrix of a 3x3 stride-2 pad-1 convolution over
//          an NHWC bf16 activation [B][H][H][cin], t = (ky * 3 + kx) * cin + c.  One (tap,
//          channel-chunk) tile of A is ONE 4-D TMA load with traversal strides (1, 2, 2, 1) over
//          (c, x, y, stamp) starting at (c0, kx - 1, 2 * oy0 + ky - 1, b0): out-of-range
//          coordinates (the padding) read as zeros, and no im2col matrix is written or read.
// Epilogue: fp32 store of C, or bias (+ ReLU) and a bf16 store of the activation.
//
// Persistent CTAs of 192 threads over 128 x BN output tiles.  Warp 0 (one lane) issues the TMA
// loads through a ring of stages, warp 1 (one lane) the MMAs into one of two TMEM accumulators,
// warps 2-5 read the other accumulator back with tcgen05.ld (warp w owns TMEM lanes
// 32(w%4)..32(w%4)+31 = tile rows) while the next tile accumulates.  Every mbarrier wait is
// bounded by wall clock:
// on a timeout the kernel records an error code, stops issuing, waits (bounded) for its copies and
// MMAs in flight, frees its tensor memory and returns; later launches see the code and return at
// once.  ap_tc_status reads (and clears) the code.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "ap_internal.h"

namespace apgb {
namespace {

typedef __nv_bfloat16 bf16;

__device__ unsigned int g_tc_error;  // first error code of a tensor-core GEMM (0 = none)

enum TcError : unsigned { TC_ERR_EMPTY = 1, TC_ERR_FULL = 2, TC_ERR_DONE = 3, TC_ERR_TEMPTY = 4, TC_ERR_TFULL = 5 };

constexpr unsigned long long kWaitNs = 200ull * 1000 * 1000;   // one wait: 200 ms
constexpr unsigned long long kDrainNs = 20ull * 1000 * 1000;   // draining after an abort

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for the phase of the given parity.  false after `limit` ns (recording `code` when
// it is not 0) or, with watch_global, as soon as another CTA has recorded an error.
__device__ bool mbar_wait(uint32_t bar, uint32_t parity, unsigned code, unsigned long long limit, bool watch_global) {
  if (mbar_try(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (uint32_t it = 1;; ++it) {
    if (mbar_try(bar, parity)) return true;
    if ((it & 63u) == 0) {
      if (watch_global && *(volatile unsigned*)&g_tc_error) return false;
      if (global_ns() - t0 > limit) {
        if (code) atomicCAS(&g_tc_error, 0u, code);
        return false;
      }
    }
  }
}

__device__ __forceinline__ void tma_2d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void tma_4d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int x, int y, int z, int w) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(dst),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(w), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
// D[tmem] (+)= A[smem] . B[smem]^T, M = 128, N from the instruction descriptor, K = 16
__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(da), "l"(db), "r"(idesc), "r"(accumulate)
      : "memory");
}
// 16 consecutive fp32 columns of this thread's TMEM lane; the wait is in the same statement so
// that no use of the registers can be scheduled before the load has completed
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor of a K-major operand tile written by TMA with a SW-byte swizzle:
// rows of SW bytes, 8-row groups SBO = 8 * SW bytes apart, leading offset unused (16 B), layout
// code 2 / 4 / 6 for the 128 / 64 / 32-byte swizzle, descriptor version 1.
template <int SW>
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  constexpr uint64_t layout = SW == 128 ? 2 : (SW == 64 ? 4 : 6);
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)((8 * SW) >> 4) << 32) |
         ((uint64_t)1 << 46) | (layout << 61);
}

// Instruction descriptor of kind::f16: fp32 accumulator, bf16 A and B, both K-major, M = 128
template <int BN>
__host__ __device__ constexpr uint32_t instr_desc() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

struct TcArgs {
  float* C;           // fp32 output (act == nullptr)
  bf16* act;          // bf16 output of bias (+ ReLU)
  const float* bias;  // nullptr: none
  int ldc, R, relu;
  int ktiles;         // reduction tiles of BK elements
  int k16_last;       // K = 16 MMAs in the last tile
  int ntn, ntiles;    // output tiles along S, in all
  int conv;           // implicit convolution (else dense)
  int cin, cchunks;   // conv: input channels, channel chunks of BK per tap
  int hout;           // conv: output side
};

template <int SW, int BN>
struct TcCfg {
  static constexpr int BK = SW / 2;  // bf16 elements per stage row
  static constexpr int A_BYTES = 128 * SW;
  static constexpr int B_BYTES = BN * SW;
  static constexpr int STAGE = A_BYTES + B_BYTES;
  static constexpr int NCOLS = BN <= 32 ? 32 : (BN <= 64 ? 64 : (BN <= 128 ? 128 : 256));
  // two accumulators per CTA; two CTAs per SM when their 4 x NCOLS TMEM columns fit in 512
  static constexpr bool TWO_CTAS = 4 * NCOLS <= 512;
  static constexpr int TILE_BYTES = TWO_CTAS ? 100 * 1024 : 200 * 1024;
  static constexpr int STAGES_RAW = TILE_BYTES / STAGE;
  static constexpr int STAGES = STAGES_RAW < 2 ? 2 : (STAGES_RAW > 8 ? 8 : STAGES_RAW);
  static constexpr int SMEM = STAGES * STAGE + 1024;  // + slack to align the tiles to 1 KB
  static_assert(BN % 16 == 0 && BN >= 16 && BN <= 256, "M = 128 MMAs take N = 16..256 in steps of 16");
};

constexpr int kTcThreads = 192;  // warp 0 TMA, warp 1 MMA, warps 2-5 epilogue

// Persistent: CTA c takes output tiles c, c + gridDim.x, ...  The producer runs ahead through the
// stage ring across tiles; the MMA thread alternates between two TMEM accumulators, so the
// epilogue warps drain one tile while the next is accumulated.
template <int SW, int BN>
__global__ void __launch_bounds__(kTcThreads) k_gemm_tc(const __grid_constant__ CUtensorMap tmA,
                                                       const __grid_constant__ CUtensorMap tmB, const TcArgs a) {
  using G = TcCfg<SW, BN>;
  extern __shared__ uint8_t dsm[];
  __shared__ __align__(8) uint64_t bar_full[G::STAGES];
  __shared__ __align__(8) uint64_t bar_empty[G::STAGES];
  __shared__ __align__(8) uint64_t bar_tfull[2];   // accumulator j ready (tcgen05.commit)
  __shared__ __align__(8) uint64_t bar_tempty[2];  // accumulator j drained (4 epilogue warps)
  __shared__ __align__(8) uint64_t bar_drain;
  __shared__ uint32_t tmem_slot;
  __shared__ int aborted;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // another launch failed: return before anything is allocated (one read, shared by the CTA)
  if (threadIdx.x == 0) aborted = *(volatile unsigned*)&g_tc_error != 0;
  __syncthreads();
  if (aborted) return;
  const uint32_t tiles = (smem_u32(dsm) + 1023u) & ~1023u;
  if (threadIdx.x == 0) {
    for (int s = 0; s < G::STAGES; ++s) {
      mbar_init(smem_u32(&bar_full[s]), 1);
      mbar_init(smem_u32(&bar_empty[s]), 1);
    }
    for (int j = 0; j < 2; ++j) {
      mbar_init(smem_u32(&bar_tfull[j]), 1);
      mbar_init(smem_u32(&bar_tempty[j]), 4);
    }
    mbar_init(smem_u32(&bar_drain), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmA) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmB) : "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"((uint32_t)(2 * G::NCOLS))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // ---- TMA producer ----
      uint32_t it = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < a.ntiles && ok; t += gridDim.x) {
        const int m0 = (t / a.ntn) * 128, n0 = (t % a.ntn) * BN;
        int b0 = 0, y0 = 0;
        if (a.conv) {
          const int rps = a.hout * a.hout;  // output rows per stamp
          b0 = m0 / rps;
          y0 = 2 * ((m0 - b0 * rps) / a.hout);
        }
        for (int kt = 0; kt < a.ktiles; ++kt, ++it) {
          const int s = (int)(it % G::STAGES);
          const uint32_t ph = (it / G::STAGES) & 1u;
          if (!mbar_wait(smem_u32(&bar_empty[s]), ph ^ 1u, TC_ERR_EMPTY, kWaitNs, true)) {
            ok = false;
            break;
          }
          const uint32_t fb = smem_u32(&bar_full[s]);
          const uint32_t sa = tiles + (uint32_t)(s * G::STAGE), sb = sa + G::A_BYTES;
          mbar_expect_tx(fb, (uint32_t)G::STAGE);
          if (a.conv) {
            const int tap = kt / a.cchunks, c0 = (kt - tap * a.cchunks) * G::BK;
            const int ky = tap / 3, kx = tap - ky * 3;
            tma_4d(sa, &tmA, fb, c0, kx - 1, y0 + ky - 1, b0);
            tma_2d(sb, &tmB, fb, tap * a.cin + c0, n0);
          } else {
            tma_2d(sa, &tmA, fb, kt * G::BK, m0);
            tma_2d(sb, &tmB, fb, kt * G::BK, n0);
          }
        }
      }
      if (!ok) {
        aborted = 1;
        // let the copies already issued land before the shared memory is released
        for (uint32_t j = (it > (uint32_t)G::STAGES ? it - G::STAGES : 0); j < it; ++j)
          mbar_wait(smem_u32(&bar_full[j % G::STAGES]), (j / G::STAGES) & 1u, 0u, kDrainNs, false);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer ----
      constexpr uint32_t idesc = instr_desc<BN>();
      uint32_t it = 0, j = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < a.ntiles && ok; t += gridDim.x, ++j) {
        const uint32_t acc = j & 1u, aph = (j >> 1) & 1u;
        if (!mbar_wait(smem_u32(&bar_tempty[acc]), aph ^ 1u, TC_ERR_TEMPTY, kWaitNs, true)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t d = tmem + acc * (uint32_t)G::NCOLS;
        for (int kt = 0; kt < a.ktiles; ++kt, ++it) {
          const int s = (int)(it % G::STAGES);
          const uint32_t ph = (it / G::STAGES) & 1u;
          if (!mbar_wait(smem_u32(&bar_full[s]), ph, TC_ERR_FULL, kWaitNs, true)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t sa = tiles + (uint32_t)(s * G::STAGE), sb = sa + G::A_BYTES;
          const uint64_t da = smem_desc<SW>(sa), db = smem_desc<SW>(sb);
          const int nk = (kt == a.ktiles - 1) ? a.k16_last : SW / 32;
          for (int k = 0; k < nk; ++k)  // K = 16 step = 32 bytes along the swizzled row
            tc_mma(d, da + (uint64_t)(2 * k), db + (uint64_t)(2 * k), idesc, (uint32_t)((kt | k) != 0));
          tc_commit(smem_u32(&bar_empty[s]));  // frees the stage once these MMAs have read it
        }
        if (ok) tc_commit(smem_u32(&bar_tfull[acc]));
      }
      if (!ok) aborted = 1;
      // arrives once every MMA issued above has completed: wait for it before TMEM is freed
      tc_commit(smem_u32(&bar_drain));
      mbar_wait(smem_u32(&bar_drain), 0u, TC_ERR_DONE, kWaitNs, false);
    }
  } else {
    // ---- epilogue: TMEM -> registers -> bias / ReLU -> global ----
    const int q = warp & 3;  // TMEM lane quarter this warp may access
    uint32_t j = 0;
    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x, ++j) {
      const uint32_t acc = j & 1u, aph = (j >> 1) & 1u;
      int got = 0;
      if (lane == 0) got = mbar_wait(smem_u32(&bar_tfull[acc]), aph, TC_ERR_TFULL, kWaitNs, true) ? 1 : 0;
      got = __shfl_sync(0xffffffffu, got, 0);
      if (!got) break;
      tc_fence_after();
      const int m0 = (t / a.ntn) * 128, n0 = (t % a.ntn) * BN;
      const int row = m0 + q * 32 + lane;
      const uint32_t trow = tmem + acc * (uint32_t)G::NCOLS + ((uint32_t)(q * 32) << 16);
#pragma unroll 1
      for (int c = 0; c < BN; c += 16) {
        float v[16];
        tc_ld16(trow + (uint32_t)c, v);
        if (row < a.R) {
          const int col = n0 + c;
          if (a.bias) {
            const float4* bp = reinterpret_cast<const float4*>(a.bias + col);
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              const float4 bb = __ldg(bp + u);
              v[4 * u + 0] += bb.x;
              v[4 * u + 1] += bb.y;
              v[4 * u + 2] += bb.z;
              v[4 * u + 3] += bb.w;
            }
            if (a.relu) {
#pragma unroll
              for (int i = 0; i < 16; ++i) v[i] = fmaxf(v[i], 0.f);
            }
          }
          if (a.act) {
            uint32_t p[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) {
              const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
              p[i] = *reinterpret_cast<const uint32_t*>(&h);
            }
            uint4* dst = reinterpret_cast<uint4*>(a.act + (int64_t)row * a.ldc + col);
            dst[0] = make_uint4(p[0], p[1], p[2], p[3]);
            dst[1] = make_uint4(p[4], p[5], p[6], p[7]);
          } else {
            float4* dst = reinterpret_cast<float4*>(a.C + (int64_t)row * a.ldc + col);
#pragma unroll
            for (int u = 0; u < 4; ++u) dst[u] = make_float4(v[4 * u], v[4 * u + 1], v[4 * u + 2], v[4 * u + 3]);
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&bar_tempty[acc]));
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)(2 * G::NCOLS))
                 : "memory");
  }
}

// ---------------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;

bool have_encoder() {
  std::call_once(g_encode_once, [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  });
  return g_encode != nullptr;
}

bool encode_map(CUtensorMap* m, const void* base, int rank, const cuuint64_t* dims, const cuuint64_t* strides,
                const cuuint32_t* box, const cuuint32_t* estr, int sw) {
  const CUtensorMapSwizzle s = sw == 128 ? CU_TENSOR_MAP_SWIZZLE_128B
                               : sw == 64 ? CU_TENSOR_MAP_SWIZZLE_64B
                                          : CU_TENSOR_MAP_SWIZZLE_32B;
  return g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, (cuuint32_t)rank, const_cast<void*>(base), dims, strides, box,
                  estr, CU_TENSOR_MAP_INTERLEAVE_NONE, s, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// dynamic shared memory of each instantiation, per device: at least G::SMEM, raised until the
// CTAs resident on one SM need no more than the 512 TMEM columns (an allocation never waits);
// with it the resident CTAs per SM, which size the persistent grid
std::mutex g_cfg_mutex;
constexpr int kMaxDev = 64;

template <int SW, int BN>
cudaError_t launch_tc(const CUtensorMap& ta, const CUtensorMap& tb, const TcArgs& a, cudaStream_t st) {
  using G = TcCfg<SW, BN>;
  static int smem_for[kMaxDev] = {0};
  static int grid_for[kMaxDev] = {0};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDev) return cudaErrorInvalidDevice;
  int smem, resident;
  {
    std::lock_guard<std::mutex> lock(g_cfg_mutex);
    smem = smem_for[dev];
    resident = grid_for[dev];
    if (!smem) {
      int nsm = 0;
      e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess) return e;
      smem = G::SMEM;
      int nb = 0;
      for (;;) {
        e = cudaFuncSetAttribute(k_gemm_tc<SW, BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_gemm_tc<SW, BN>, kTcThreads, smem);
        if (e != cudaSuccess) return e;
        if (nb * 2 * G::NCOLS <= 512) break;
        smem += 4096;
      }
      if (nb < 1) return cudaErrorInvalidConfiguration;
      resident = nb * nsm;
      smem_for[dev] = smem;
      grid_for[dev] = resident;
    }
  }
  const int grid = a.ntiles < resident ? a.ntiles : resident;
  k_gemm_tc<SW, BN><<<(unsigned)grid, kTcThreads, smem, st>>>(ta, tb, a);
  return cudaGetLastError();
}

template <int SW>
cudaError_t launch_bn(int bn, const CUtensorMap& ta, const CUtensorMap& tb, const TcArgs& a, cudaStream_t st) {
  switch (bn) {
    case 16: return launch_tc<SW, 16>(ta, tb, a, st);
    case 32: return launch_tc<SW, 32>(ta, tb, a, st);
    case 64: return launch_tc<SW, 64>(ta, tb, a, st);
    case 128: return launch_tc<SW, 128>(ta, tb, a, st);
    case 256: return launch_tc<SW, 256>(ta, tb, a, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_sw(int sw, int bn, const CUtensorMap& ta, const CUtensorMap& tb, const TcArgs& a,
                      cudaStream_t st) {
  if (sw == 128) return launch_bn<128>(bn, ta, tb, a, st);
  if (sw == 64) return launch_bn<64>(bn, ta, tb, a, st);
  if (sw == 32) return launch_bn<32>(bn, ta, tb, a, st);
  return cudaErrorInvalidValue;
}

// widest output tile (16..256) dividing S
int pick_bn(int S) {
  for (int bn = 256; bn >= 16; bn >>= 1)
    if (S % bn == 0) return bn;
  return 0;
}

bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

bool epilogue_ok(const TcEpilogue& ep, const float* C, int ldc) {
  if (ep.act) return aligned16(ep.act) && ldc % 8 == 0 && (!ep.bias || aligned16(ep.bias));
  return C && aligned16(C) && ldc % 4 == 0 && (!ep.bias || aligned16(ep.bias));
}

}  // namespace

cudaError_t tc_gemm(const __nv_bfloat16* A, int lda, const __nv_bfloat16* W, int ldw, float* C, int ldc, int R, int S,
                    int T, const TcEpilogue& ep, cudaStream_t st) {
  if (R <= 0 || S <= 0 || T <= 0) return cudaSuccess;
  const int bn = pick_bn(S);
  if (!bn || T % 16 || lda % 8 || ldw % 8 || lda < T || ldw < T || ldc < S || !aligned16(A) || !aligned16(W) ||
      !epilogue_ok(ep, C, ldc))
    return cudaErrorInvalidValue;
  if (!have_encoder()) return cudaErrorNotSupported;
  const int sw = T >= 64 ? 128 : (T >= 32 ? 64 : 32);
  const int bk = sw / 2;
  CUtensorMap ta, tb;
  const cuuint32_t estr[2] = {1, 1};
  {
    const cuuint64_t dims[2] = {(cuuint64_t)T, (cuuint64_t)R};
    const cuuint64_t strides[1] = {(cuuint64_t)lda * 2};
    const cuuint32_t box[2] = {(cuuint32_t)bk, 128};
    if (!encode_map(&ta, A, 2, dims, strides, box, estr, sw)) return cudaErrorInvalidValue;
  }
  {
    const cuuint64_t dims[2] = {(cuuint64_t)T, (cuuint64_t)S};
    const cuuint64_t strides[1] = {(cuuint64_t)ldw * 2};
    const cuuint32_t box[2] = {(cuuint32_t)bk, (cuuint32_t)bn};
    if (!encode_map(&tb, W, 2, dims, strides, box, estr, sw)) return cudaErrorInvalidValue;
  }
  TcArgs a{};
  a.C = C;
  a.act = ep.act;
  a.bias = ep.bias;
  a.ldc = ldc;
  a.R = R;
  a.relu = ep.relu;
  a.ktiles = (T + bk - 1) / bk;
  a.k16_last = (T - (a.ktiles - 1) * bk) / 16;
  a.conv = 0;
  a.ntn = S / bn;
  const int64_t ntiles = (int64_t)((R + 127) / 128) * a.ntn;
  if (ntiles > INT32_MAX) return cudaErrorInvalidValue;
  a.ntiles = (int)ntiles;
  return launch_sw(sw, bn, ta, tb, a, st);
}

cudaError_t tc_conv3x3s2(const __nv_bfloat16* act_in, int64_t B, int H, int cin, const __nv_bfloat16* W, int S,
                         float* C, int ldc, const TcEpilogue& ep, cudaStream_t st) {
  if (B <= 0 || S <= 0) return cudaSuccess;
  const int hout = H / 2;
  const int bn = pick_bn(S);
  if (!bn || H < 2 || H % 2 || hout > 128 || ldc < S || !aligned16(act_in) || !aligned16(W) ||
      !epilogue_ok(ep, C, ldc))
    return cudaErrorInvalidValue;
  // 128 output rows per tile = nb stamps x ny output rows x hout columns
  int nb, ny;
  if (hout * hout <= 128) {
    if (128 % (hout * hout)) return cudaErrorInvalidValue;
    nb = 128 / (hout * hout);
    ny = hout;
  } else {
    if (128 % hout || hout % (128 / hout)) return cudaErrorInvalidValue;
    nb = 1;
    ny = 128 / hout;
  }
  int sw, cchunks;
  if (cin % 64 == 0) {
    sw = 128;
    cchunks = cin / 64;
  } else if (cin == 32) {
    sw = 64;
    cchunks = 1;
  } else if (cin == 16) {
    sw = 32;
    cchunks = 1;
  } else {
    return cudaErrorInvalidValue;
  }
  const int bk = sw / 2;
  const int64_t R64 = B * hout * hout;
  if (R64 > INT32_MAX - 128) return cudaErrorInvalidValue;
  if (!have_encoder()) return cudaErrorNotSupported;
  CUtensorMap ta, tb;
  {
    const cuuint64_t dims[4] = {(cuuint64_t)cin, (cuuint64_t)H, (cuuint64_t)H, (cuuint64_t)B};
    const cuuint64_t strides[3] = {(cuuint64_t)cin * 2, (cuuint64_t)H * cin * 2, (cuuint64_t)H * H * cin * 2};
    const cuuint32_t box[4] = {(cuuint32_t)bk, (cuuint32_t)(2 * hout), (cuuint32_t)(2 * ny), (cuuint32_t)nb};
    const cuuint32_t estr[4] = {1, 2, 2, 1};
    if (!encode_map(&ta, act_in, 4, dims, strides, box, estr, sw)) return cudaErrorInvalidValue;
  }
  {
    const int K = 9 * cin;
    const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)S};
    const cuuint64_t strides[1] = {(cuuint64_t)K * 2};
    const cuuint32_t box[2] = {(cuuint32_t)bk, (cuuint32_t)bn};
    const cuuint32_t estr[2] = {1, 1};
    if (!encode_map(&tb, W, 2, dims, strides, box, estr, sw)) return cudaErrorInvalidValue;
  }
  TcArgs a{};
  a.C = C;
  a.act = ep.act;
  a.bias = ep.bias;
  a.ldc = ldc;
  a.R = (int)R64;
  a.relu = ep.relu;
  a.ktiles = 9 * cchunks;
  a.k16_last = sw / 32;
  a.conv = 1;
  a.cin = cin;
  a.cchunks = cchunks;
  a.hout = hout;
  a.ntn = S / bn;
  const int64_t ntiles = ((R64 + 127) / 128) * a.ntn;
  if (ntiles > INT32_MAX) return cudaErrorInvalidValue;
  a.ntiles = (int)ntiles;
  return launch_sw(sw, bn, ta, tb, a, st);
}

unsigned tc_error(bool clear) {
  unsigned v = 0;
  if (cudaMemcpyFromSymbol(&v, g_tc_error, sizeof(v)) != cudaSuccess) return 0xFFFFFFFFu;
  if (clear && v) {
    const unsigned z = 0;
    cudaMemcpyToSymbol(g_tc_error, &z, sizeof(z));
  }
  return v;
}

}  // namespace apgb
