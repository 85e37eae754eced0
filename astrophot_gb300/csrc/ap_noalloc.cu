// ap_render_noalloc: the single-stamp render for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: a host application that reserves the
// whole device memory for its own pool and forbids other allocations, a plugin loaded into
// such a process with no handle on its allocator, or a latency-bound pipeline where an
// allocation (which can synchronise the device) would stall work on other streams.  This
// entry point gives them the model image of one stamp without any allocation: its scratch
// (plan tables, sample planes, integration queue, PSF kernels, counters) lives in the
// file-scope array below, which the CUDA module holds on every GPU that loads the library
// until the process exits.
//
// Rules of use
//   - At most AP_NOALLOC_SCRATCH_BYTES (8 MiB) of scratch: working windows up to about
//     80,000 pixels (e.g. a 256 x 256 stamp with a 21 x 21 PSF).  Larger stamps are rejected
//     with AP_ERR_WORKSPACE before any device work is queued.
//   - Stamp sides up to 65,536 pixels and PSF sides up to 4,095 are accepted (larger ones are
//     rejected with AP_ERR_ARG before any arithmetic on them).
//   - The first call on each device resolves the array's device address (cudaGetSymbolAddress,
//     with that device current); make that first call before any stream capture.
//   - The plan reaches the device as kernel arguments (no host-to-device copy), so a call only
//     enqueues work: it does not wait for the stream.
//   - The convolution is always direct (options.fft_min_kernel is not used).
//   - Every call on a device shares the one array and it keeps the last call's contents, so
//     calls that overlap on the GPU (different streams, or threads) race: serialise them.
//   - Nothing here calls cudaMalloc, cudaFree or any allocating routine; the caller passes the
//     parameters, the PSF and the output buffer.
#include <atomic>
#include <cmath>
#include <cstring>

#include "ap_internal.h"

using namespace apgb;

namespace {

constexpr size_t kScratchBytes = AP_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;
constexpr int64_t kAlignNA = 256;

// The scratch itself.  In host code this name is only a stand-in for the device symbol: its
// device address comes from cudaGetSymbolAddress, once per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// device address per device (nullptr until resolved; every thread that resolves it stores the
// same value)
std::atomic<void*> g_scratch_addr[kMaxDevices];

constexpr int32_t kMaxSide = 1 << 16;     // stamp side limit (keeps every index product in range)
constexpr int32_t kMaxPsfSide = 4095;     // PSF side limit

// The plan, passed by value, written into the scratch, and the state the render kernels expect
// at zero cleared there (the array keeps the previous call's contents): the tile -> stamp tables
// (a single stamp: index 0 everywhere), the evaluation slots, the counters.
struct NoallocOffsets {
  int64_t stamp, tab, wt, ot, evals, cnt, wctr;
};

__global__ void k_noalloc_setup(StampDev st, QuadTables T, NoallocOffsets o, char* ws) {
  const int t = threadIdx.x;
  if (t == 0) {
    *reinterpret_cast<StampDev*>(ws + o.stamp) = st;
    *reinterpret_cast<QuadTables*>(ws + o.tab) = T;
  }
  int32_t* wt = reinterpret_cast<int32_t*>(ws + o.wt);
  int32_t* ot = reinterpret_cast<int32_t*>(ws + o.ot);
  for (int i = t; i < st.ntw; i += blockDim.x) wt[i] = 0;
  for (int i = t; i < st.nto; i += blockDim.x) ot[i] = 0;
  uint32_t* ev = reinterpret_cast<uint32_t*>(ws + o.evals);
  for (int i = t; i < (int)(2 * sizeof(EvalDev) / sizeof(uint32_t)); i += blockDim.x) ev[i] = 0u;
  uint32_t* cnt = reinterpret_cast<uint32_t*>(ws + o.cnt);
  if (t < 16) cnt[t] = 0u;
  unsigned long long* wc = reinterpret_cast<unsigned long long*>(ws + o.wctr);
  if (t < 8) wc[t] = 0ull;
}
static_assert(sizeof(StampDev) + sizeof(QuadTables) + sizeof(NoallocOffsets) + sizeof(char*) <= 4000,
              "the plan must fit the kernel-argument space");
static_assert(sizeof(EvalDev) % sizeof(uint32_t) == 0, "evaluation slots are cleared by words");

int64_t na_align(int64_t v) { return (v + kAlignNA - 1) / kAlignNA * kAlignNA; }

// Gauss-Legendre nodes (ascending) and weights, 1..5 points, closed forms.
void na_gauss_legendre(int n, double* x, double* w) {
  const double r35 = std::sqrt(3.0 / 5.0);
  switch (n) {
    case 1:
      x[0] = 0.0;
      w[0] = 2.0;
      break;
    case 2:
      x[0] = -1.0 / std::sqrt(3.0);
      x[1] = -x[0];
      w[0] = w[1] = 1.0;
      break;
    case 3:
      x[0] = -r35;
      x[1] = 0.0;
      x[2] = r35;
      w[0] = w[2] = 5.0 / 9.0;
      w[1] = 8.0 / 9.0;
      break;
    case 4: {
      const double a = std::sqrt(3.0 / 7.0 - 2.0 / 7.0 * std::sqrt(6.0 / 5.0));
      const double b = std::sqrt(3.0 / 7.0 + 2.0 / 7.0 * std::sqrt(6.0 / 5.0));
      x[0] = -b;
      x[1] = -a;
      x[2] = a;
      x[3] = b;
      w[0] = w[3] = (18.0 - std::sqrt(30.0)) / 36.0;
      w[1] = w[2] = (18.0 + std::sqrt(30.0)) / 36.0;
      break;
    }
    default: {
      const double a = std::sqrt(5.0 - 2.0 * std::sqrt(10.0 / 7.0)) / 3.0;
      const double b = std::sqrt(5.0 + 2.0 * std::sqrt(10.0 / 7.0)) / 3.0;
      x[0] = -b;
      x[1] = -a;
      x[2] = 0.0;
      x[3] = a;
      x[4] = b;
      w[0] = w[4] = (322.0 - 13.0 * std::sqrt(70.0)) / 900.0;
      w[1] = w[3] = (322.0 + 13.0 * std::sqrt(70.0)) / 900.0;
      w[2] = 128.0 / 225.0;
      break;
    }
  }
}

void na_fill_quad(int n, double* ox, double* oy, double* ow) {
  double x[kMaxQuad], w[kMaxQuad];
  na_gauss_legendre(n, x, w);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      ox[j * n + i] = x[i] / 2.0;
      oy[j * n + i] = x[j] / 2.0;
      ow[j * n + i] = w[j] * w[i] / 4.0;
    }
}

bool na_options_ok(const ap_options* o) {
  if (o->profile != AP_PROFILE_SERSIC && o->profile != AP_PROFILE_EXPONENTIAL) return false;
  if (o->sampling_mode < AP_SAMPLING_MIDPOINT || o->sampling_mode > AP_SAMPLING_TRAPEZOID) return false;
  if (o->sampling_mode == AP_SAMPLING_QUAD && (o->sampling_quad_level < 1 || o->sampling_quad_level > kMaxQuad))
    return false;
  if (o->integrate_mode != AP_INTEGRATE_NONE && o->integrate_mode != AP_INTEGRATE_THRESHOLD) return false;
  if (o->psf_mode < AP_PSF_NONE || o->psf_mode > AP_PSF_FULL_NOSHIFT) return false;
  if (o->lanczos_order != 0) return false;  // the bilinear shift only
  if (o->integrate_mode == AP_INTEGRATE_THRESHOLD &&
      (o->integrate_max_depth < 1 || o->integrate_max_depth > kMaxDepth || o->integrate_gridding < 1 ||
       o->integrate_gridding > kMaxGrid || o->integrate_quad_level < 1 || o->integrate_quad_level > kMaxQuad))
    return false;
  return true;
}

}  // namespace

extern "C" int ap_render_noalloc(int32_t nx, int32_t ny, int32_t psf_kx, int32_t psf_ky,
                                 const double* geometry, const ap_options* options,
                                 const double* params, const float* psf, float* model,
                                 ap_stream_t stream) {
  if (!geometry || !options || !params || !model || nx <= 0 || ny <= 0) return AP_ERR_ARG;
  if (nx > kMaxSide || ny > kMaxSide) return AP_ERR_ARG;
  if (!na_options_ok(options)) return AP_ERR_UNSUPPORTED;
  if (options->free_mask & ~0xff) return AP_ERR_ARG;
  const bool with_psf = options->psf_mode != AP_PSF_NONE;
  if (with_psf && (!psf || psf_kx <= 0 || psf_ky <= 0 || psf_kx % 2 != 1 || psf_ky % 2 != 1 ||
                   psf_kx > kMaxPsfSide || psf_ky > kMaxPsfSide))
    return AP_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;

  // ---- single-stamp plan on the host stack -------------------------------------------------
  StampDev st;
  std::memset(&st, 0, sizeof(st));
  st.nx = nx;
  st.ny = ny;
  if (with_psf) {
    st.kx = psf_kx;
    st.ky = psf_ky;
    st.bx = (psf_kx + 2) / 2;  // psf_border_int = ceil((1 + k) / 2) for odd k
    st.by = (psf_ky + 2) / 2;
    const bool shift = options->psf_mode == AP_PSF_FULL;
    st.kpx = shift ? psf_kx + 2 : psf_kx;
    st.kpy = shift ? psf_ky + 2 : psf_ky;
  }
  st.wnx = nx + 2 * st.bx;
  st.wny = ny + 2 * st.by;
  const bool stencil = options->integrate_mode == AP_INTEGRATE_THRESHOLD &&
                       (options->sampling_mode == AP_SAMPLING_MIDPOINT ||
                        options->sampling_mode == AP_SAMPLING_TRAPEZOID);
  if (stencil && (st.wnx < 3 || st.wny < 3)) return AP_ERR_ARG;
  const double det = geometry[0] * geometry[3] - geometry[1] * geometry[2];
  if (!(std::fabs(det) > 0.0)) return AP_ERR_ARG;
  for (int k = 0; k < 4; ++k) st.P[k] = geometry[k];
  st.Pinv[0] = geometry[3] / det;
  st.Pinv[1] = -geometry[1] / det;
  st.Pinv[2] = -geometry[2] / det;
  st.Pinv[3] = geometry[0] / det;
  st.ref_ij[0] = geometry[4];
  st.ref_ij[1] = geometry[5];
  st.ref_xy[0] = geometry[6];
  st.ref_xy[1] = geometry[7];
  st.pixel_area = std::fabs(det);
  for (int k = 0; k < 4; ++k) {
    st.Pf[k] = (float)st.P[k];
    st.Pinvf[k] = (float)st.Pinv[k];
  }
  st.thr_numel = (double)st.wnx * (double)st.wny;
  st.ntw_x = (st.wnx + kTile - 1) / kTile;
  st.ntw = st.ntw_x * ((st.wny + kTile - 1) / kTile);
  st.nto_x = (nx + kOutTileX - 1) / kOutTileX;
  const bool large = with_psf && conv_kernel_large(st.kpx, st.kpy);
  st.nto = st.nto_x * ((ny + conv_tile_y(large) - 1) / conv_tile_y(large));
  const int64_t wp = (int64_t)st.wnx * st.wny;
  const int64_t kp2 = (int64_t)st.kpx * st.kpy;

  QuadTables T;
  std::memset(&T, 0, sizeof(T));
  T.quad_level = options->integrate_quad_level >= 1 && options->integrate_quad_level <= kMaxQuad
                     ? options->integrate_quad_level
                     : 3;
  T.gridding = options->integrate_gridding >= 1 && options->integrate_gridding <= kMaxGrid
                   ? options->integrate_gridding
                   : 5;
  na_fill_quad(T.quad_level, T.qx, T.qy, T.qw);
  const int g = T.gridding;
  for (int jj = 0; jj < g; ++jj)
    for (int ii = 0; ii < g; ++ii) {
      const double step = g == 1 ? 0.0 : ((g - 1) / (double)g) / (g - 1);
      T.gx[jj * g + ii] = g == 1 ? 0.0 : -(g - 1) / (2.0 * g) + ii * step;
      T.gy[jj * g + ii] = g == 1 ? 0.0 : -(g - 1) / (2.0 * g) + jj * step;
    }
  if (options->sampling_mode == AP_SAMPLING_MIDPOINT) {
    T.nsub = 1;
    T.sw[0] = 1.0;
  } else if (options->sampling_mode == AP_SAMPLING_TRAPEZOID) {
    T.nsub = 4;
    T.sub_center = -1;
    for (int v = 0; v < 2; ++v)
      for (int u = 0; u < 2; ++u) {
        T.sx[v * 2 + u] = u - 0.5;
        T.sy[v * 2 + u] = v - 0.5;
        T.sw[v * 2 + u] = 0.25;
      }
  } else if (options->sampling_mode == AP_SAMPLING_SIMPSONS) {
    static const double kw[9] = {1, 4, 1, 4, 16, 4, 1, 4, 1};
    T.nsub = 9;
    T.sub_center = 4;
    for (int v = 0; v < 3; ++v)
      for (int u = 0; u < 3; ++u) {
        T.sx[v * 3 + u] = 0.5 * (u - 1);
        T.sy[v * 3 + u] = 0.5 * (v - 1);
        T.sw[v * 3 + u] = kw[v * 3 + u] / 36.0;
      }
  } else {
    const int k = options->sampling_quad_level;
    T.nsub = k * k;
    T.sub_center = (k * k) / 2;
    na_fill_quad(k, T.sx, T.sy, T.sw);
  }

  quad_tables_fill_f32(T);

  // ---- scratch layout; refuse what does not fit ----------------------------------------------
  int64_t o = 0;
  auto take = [&o](int64_t bytes) {
    const int64_t at = o;
    o = na_align(o + bytes);
    return at;
  };
  const int64_t o_stamp = take(sizeof(StampDev));
  const int64_t o_evals = take(sizeof(EvalDev) * 2);
  const int64_t o_wt = take(sizeof(int32_t) * st.ntw);
  const int64_t o_ot = take(sizeof(int32_t) * st.nto);
  const int64_t o_tab = take(sizeof(QuadTables));
  const int64_t o_work = take(sizeof(float) * 2 * kNumPlanes * wp);
  const int64_t o_aux = take(sizeof(float) * 2 * 2 * wp);
  const int64_t o_spsf = take(sizeof(float) * (kp2 > 0 ? 6 * kp2 : 1));
  const int64_t o_queue = take(sizeof(int64_t) * 2 * wp);
  const int64_t o_recheck = take(sizeof(int64_t) * 2 * wp);
  const int64_t o_wlist = take(sizeof(int64_t) * 2 * st.ntw);
  const int64_t o_olist = take(sizeof(int64_t) * 2 * st.nto);
  const int64_t o_slist = take(sizeof(int32_t) * 2);
  const int64_t o_cnt = take(sizeof(uint32_t) * 16);
  const int64_t o_wctr = take(sizeof(unsigned long long) * 8);
  const int64_t o_mean = take(sizeof(double) * 2);
  const int64_t o_tacc = take(sizeof(double) * 2 * kNacc * st.nto);
  const int64_t o_acc = take(sizeof(double) * 2 * kNacc);
  if (o > (int64_t)kScratchBytes) return AP_ERR_WORKSPACE;
  size_t conv_smem = 0;
  if (with_psf)
    conv_smem = conv_smem_bytes(st.kpx, st.kpy, large);
  if (conv_smem > 200 * 1024) return AP_ERR_UNSUPPORTED;

  // ---- device address of the scratch, once per device ----------------------------------------
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return AP_ERR_CUDA;
  void* addr = g_scratch_addr[dev].load();
  if (!addr) {
    if (cudaGetSymbolAddress(&addr, g_noalloc_scratch) != cudaSuccess || !addr) return AP_ERR_CUDA;
    g_scratch_addr[dev].store(addr);
  }
  char* ws = (char*)addr;

  // ---- plan and zeroed state into the scratch (kernel arguments: nothing copied from host) ----
  const NoallocOffsets no{o_stamp, o_tab, o_wt, o_ot, o_evals, o_cnt, o_wctr};
  k_noalloc_setup<<<1, 256, 0, s>>>(st, T, no, ws);
  if (cudaGetLastError() != cudaSuccess) return AP_ERR_CUDA;
  if (conv_smem > 48 * 1024 && set_conv_smem(conv_smem) != cudaSuccess) return AP_ERR_CUDA;

  BatchArgs A{};
  std::memset(&A, 0, sizeof(A));
  A.n_stamps = 1;
  A.kind = options->profile;
  A.sampling = options->sampling_mode;
  A.integrate = options->integrate_mode;
  A.psf_mode = options->psf_mode;
  A.max_depth = options->integrate_max_depth;
  A.free_mask = options->free_mask;
  int nf = 0;
  for (int i = 0; i < NPARAM; ++i) nf += (options->free_mask >> i) & 1;
  A.n_free = nf;
  A.has_sky = options->has_sky;
  A.n_work_tiles = st.ntw;
  A.n_out_tiles = st.nto;
  A.max_kp2 = (int32_t)kp2;
  A.conv_large = large ? 1 : 0;
  A.tolerance = (float)options->sampling_tolerance;
  A.tolerance64 = options->sampling_tolerance;
  A.softening64 = options->softening;
  A.work_pixels = wp;
  A.out_pixels = (int64_t)nx * ny;
  A.stamps = (const StampDev*)(ws + o_stamp);
  A.evals = (EvalDev*)(ws + o_evals);
  A.work_tiles = (const int32_t*)(ws + o_wt);
  A.out_tiles = (const int32_t*)(ws + o_ot);
  A.tables = (const QuadTables*)(ws + o_tab);
  A.work = (float*)(ws + o_work);
  A.aux = (float*)(ws + o_aux);
  A.spsf = (float*)(ws + o_spsf);
  A.queue = (int64_t*)(ws + o_queue);
  A.recheck = (int64_t*)(ws + o_recheck);
  A.amb = nullptr;  // level-1 float64 decisions inline (no dense list in the fixed scratch)
  A.amb_cap = 0;
  A.wlist = (int64_t*)(ws + o_wlist);
  A.olist = (int64_t*)(ws + o_olist);
  A.slist = (int32_t*)(ws + o_slist);
  A.counters = (uint32_t*)(ws + o_cnt);
  A.work_ctr = (unsigned long long*)(ws + o_wctr);
  A.mean_acc = (double*)(ws + o_mean);
  A.tile_acc = (double*)(ws + o_tacc);
  A.acc = (double*)(ws + o_acc);

  if (launch_eval_setup(A, params, NPARAM, 0, nullptr, OP_FWD | OP_WRITE_MODEL, s) != cudaSuccess)
    return AP_ERR_CUDA;
  ConvIO io;
  std::memset(&io, 0, sizeof(io));
  io.psf = psf;
  io.model_out = model;
  if (launch_render_pass(A, io, conv_smem, false, s, nullptr) != cudaSuccess) return AP_ERR_CUDA;
  return AP_OK;
}
