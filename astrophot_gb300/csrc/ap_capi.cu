// The extern "C" boundary: host-side batch plan, workspace layout, and the launch
// sequences behind each entry point declared in include/astrophot_gb300.h.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "ap_internal.h"

using namespace apgb;

namespace {

constexpr int64_t kAlign = 256;

int64_t align_up(int64_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

struct Layout {
  int64_t stamps, evals, work_tiles, out_tiles, tables, work, aux, spsf, queue, recheck, amb, wlist,
      olist, slist, counters,
      work_ctr, mean_acc, tile_acc, acc, fft_lists, fft_buf, preconv, total;
};

// Gauss-Legendre nodes (ascending) and weights for 1..5 points, closed forms.
void gauss_legendre(int n, double* x, double* w) {
  switch (n) {
    case 1:
      x[0] = 0.0;
      w[0] = 2.0;
      break;
    case 2: {
      const double a = 1.0 / std::sqrt(3.0);
      x[0] = -a;
      x[1] = a;
      w[0] = w[1] = 1.0;
      break;
    }
    case 3: {
      const double a = std::sqrt(3.0 / 5.0);
      x[0] = -a;
      x[1] = 0.0;
      x[2] = a;
      w[0] = w[2] = 5.0 / 9.0;
      w[1] = 8.0 / 9.0;
      break;
    }
    case 4: {
      const double a = std::sqrt(3.0 / 7.0 - 2.0 / 7.0 * std::sqrt(6.0 / 5.0));
      const double b = std::sqrt(3.0 / 7.0 + 2.0 / 7.0 * std::sqrt(6.0 / 5.0));
      const double wa = (18.0 + std::sqrt(30.0)) / 36.0, wb = (18.0 - std::sqrt(30.0)) / 36.0;
      x[0] = -b;
      x[1] = -a;
      x[2] = a;
      x[3] = b;
      w[0] = w[3] = wb;
      w[1] = w[2] = wa;
      break;
    }
    case 5: {
      const double a = std::sqrt(5.0 - 2.0 * std::sqrt(10.0 / 7.0)) / 3.0;
      const double b = std::sqrt(5.0 + 2.0 * std::sqrt(10.0 / 7.0)) / 3.0;
      const double wa = (322.0 + 13.0 * std::sqrt(70.0)) / 900.0;
      const double wb = (322.0 - 13.0 * std::sqrt(70.0)) / 900.0;
      x[0] = -b;
      x[1] = -a;
      x[2] = 0.0;
      x[3] = a;
      x[4] = b;
      w[0] = w[4] = wb;
      w[1] = w[3] = wa;
      w[2] = 128.0 / 225.0;
      break;
    }
  }
}

// quad_table (utils/operations.py:105-120): k = j * n + i, offsets a/2, weights w_j w_i / 4
void fill_quad(int n, double* ox, double* oy, double* ow) {
  double x[kMaxQuad], w[kMaxQuad];
  gauss_legendre(n, x, w);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      ox[j * n + i] = x[i] / 2.0;
      oy[j * n + i] = x[j] / 2.0;
      ow[j * n + i] = w[j] * w[i] / 4.0;
    }
}

}  // namespace

struct ap_batch {
  ap_options opt{};
  int32_t n = 0;
  std::vector<StampDev> stamps;
  std::vector<int32_t> work_tiles, out_tiles;
  QuadTables tables{};
  int64_t out_pixels = 0, psf_pixels = 0, work_pixels = 0, spsf_total = 0;
  int32_t max_kp2 = 0;
  bool conv_large = false;  // k_conv's large flavour and its tile height
  size_t conv_smem = 0;
  std::vector<int32_t> fft_lists;  // stamp list, then the row / column-group / output-row prefixes
  int64_t fft_buf_elems = 0, preconv_elems = 0;
  Layout L{};
  BatchArgs args{};
  bool bound = false;
  char* ws = nullptr;
  int64_t stats[4] = {0, 0, 0, 0};
  // last LM run
  const double* hist_loss = nullptr;
  const double* hist_L = nullptr;
  const double* hist_x = nullptr;
  int32_t hist_len = 0;
  cudaStream_t cap_stream = nullptr;  // private stream the LM rounds are captured on
  Profiler prof;
  ~ap_batch() {
    if (cap_stream) cudaStreamDestroy(cap_stream);
    prof.destroy();
  }
};

namespace {

int validate_options(const ap_options* o) {
  if (!o) return AP_ERR_ARG;
  if (o->fft_min_kernel < 0) return AP_ERR_ARG;
  if (o->profile < AP_PROFILE_SERSIC || o->profile > AP_PROFILE_GAUSSIAN) return AP_ERR_UNSUPPORTED;
  if (o->sampling_mode < AP_SAMPLING_MIDPOINT || o->sampling_mode > AP_SAMPLING_MIDPOINT_CENTER)
    return AP_ERR_UNSUPPORTED;
  if ((o->sampling_mode == AP_SAMPLING_QUAD || o->sampling_mode == AP_SAMPLING_MIDPOINT_CENTER) &&
      (o->sampling_quad_level < 1 || o->sampling_quad_level > kMaxQuad))
    return AP_ERR_UNSUPPORTED;
  if (o->sampling_mode == AP_SAMPLING_MIDPOINT_CENTER) {
    if (o->integrate_mode != AP_INTEGRATE_NONE) return AP_ERR_UNSUPPORTED;
    if (!(o->center_radius >= 0.0) || !std::isfinite(o->center_radius)) return AP_ERR_ARG;
  }
  if (o->integrate_mode != AP_INTEGRATE_NONE && o->integrate_mode != AP_INTEGRATE_THRESHOLD)
    return AP_ERR_UNSUPPORTED;
  if (o->psf_mode < AP_PSF_NONE || o->psf_mode > AP_PSF_FULL_NOSHIFT) return AP_ERR_UNSUPPORTED;
  if (o->lanczos_order < 0 || o->lanczos_order > kMaxLanczos) return AP_ERR_UNSUPPORTED;
  if (o->lanczos_order > 0 && o->psf_mode != AP_PSF_FULL) return AP_ERR_UNSUPPORTED;
  if (o->integrate_mode == AP_INTEGRATE_THRESHOLD) {
    if (o->integrate_max_depth < 1 || o->integrate_max_depth > kMaxDepth) return AP_ERR_UNSUPPORTED;
    if (o->integrate_gridding < 1 || o->integrate_gridding > kMaxGrid) return AP_ERR_UNSUPPORTED;
    if (o->integrate_quad_level < 1 || o->integrate_quad_level > kMaxQuad) return AP_ERR_UNSUPPORTED;
  }
  if (o->free_mask & ~0xff) return AP_ERR_ARG;
  if (!profile_has_n(o->profile) && (o->free_mask & (1 << PN))) return AP_ERR_ARG;
  if (!o->has_sky && (o->free_mask & (1 << PF))) return AP_ERR_ARG;
  if (!(o->softening >= 0.0) || !(o->sampling_tolerance >= 0.0)) return AP_ERR_ARG;
  return AP_OK;
}

int check_cuda(cudaError_t e) { return record_cuda(e); }

}  // namespace

namespace apgb {
thread_local cudaError_t g_last_cuda_error = cudaSuccess;

int record_cuda(cudaError_t e) {
  if (e == cudaSuccess) return AP_OK;
  g_last_cuda_error = e;
  return AP_ERR_CUDA;
}
}  // namespace apgb

extern "C" {

const char* ap_version(void) { return "astrophot_gb300 0.1 (sm_103a)"; }

const char* ap_last_cuda_error(void) {
  return g_last_cuda_error == cudaSuccess ? "" : cudaGetErrorString(g_last_cuda_error);
}

int ap_batch_create(ap_batch** out, int32_t n, const int32_t* nx, const int32_t* ny,
                    const int32_t* psf_kx, const int32_t* psf_ky, const double* geometry,
                    const ap_options* options) {
  if (!out || n <= 0 || !nx || !ny || !geometry) return AP_ERR_ARG;
  *out = nullptr;
  int rc = validate_options(options);
  if (rc) return rc;
  const bool psf = options->psf_mode != AP_PSF_NONE;
  if (psf && (!psf_kx || !psf_ky)) return AP_ERR_ARG;
  ap_batch* b = new (std::nothrow) ap_batch();
  if (!b) return AP_ERR_ARG;
  b->opt = *options;
  b->n = n;
  b->stamps.resize(n);
  int64_t out_off = 0, work_off = 0, psf_off = 0, spsf_off = 0;
  int32_t tw = 0, to = 0;
  size_t smem = 0;
  const bool stencil = options->integrate_mode == AP_INTEGRATE_THRESHOLD &&
                       (options->sampling_mode == AP_SAMPLING_MIDPOINT ||
                        options->sampling_mode == AP_SAMPLING_TRAPEZOID);
  // k_conv's flavour (and with it the output tile height) for the whole batch: the large one
  // when some kernel is not covered by the register-blocked sizes
  bool large = false;
  // the shifted kernel grows by the shift's padding: 1 a side (bilinear), k a side (Lanczos k)
  const int shift_pad = options->psf_mode != AP_PSF_FULL ? 0 : (options->lanczos_order > 0 ? 2 * options->lanczos_order : 2);
  if (psf) {
    for (int s = 0; s < n; ++s)
      if (conv_kernel_large(psf_kx[s] + shift_pad, psf_ky[s] + shift_pad)) large = true;
  }
  b->conv_large = large;
  for (int s = 0; s < n; ++s) {
    StampDev& st = b->stamps[s];
    std::memset(&st, 0, sizeof(st));
    if (nx[s] <= 0 || ny[s] <= 0) {
      delete b;
      return AP_ERR_ARG;
    }
    st.nx = nx[s];
    st.ny = ny[s];
    if (psf) {
      st.kx = psf_kx[s];
      st.ky = psf_ky[s];
      if (st.kx <= 0 || st.ky <= 0 || (st.kx % 2) != 1 || (st.ky % 2) != 1) {
        delete b;
        return AP_ERR_ARG;
      }
      // psf_border_int = ceil((1 + shape) / 2)  (image/psf_image.py:71-93)
      st.bx = (st.kx + 2) / 2;
      st.by = (st.ky + 2) / 2;
      st.kpx = st.kx + shift_pad;
      st.kpy = st.ky + shift_pad;
    }
    st.wnx = st.nx + 2 * st.bx;
    st.wny = st.ny + 2 * st.by;
    if (stencil && (st.wnx < 3 || st.wny < 3)) {
      delete b;
      return AP_ERR_ARG;
    }
    const double* g = geometry + 8 * (int64_t)s;
    for (int k = 0; k < 4; ++k) st.P[k] = g[k];
    const double det = g[0] * g[3] - g[1] * g[2];
    if (!(std::fabs(det) > 0.0)) {
      delete b;
      return AP_ERR_ARG;
    }
    st.Pinv[0] = g[3] / det;
    st.Pinv[1] = -g[1] / det;
    st.Pinv[2] = -g[2] / det;
    st.Pinv[3] = g[0] / det;
    st.ref_ij[0] = g[4];
    st.ref_ij[1] = g[5];
    st.ref_xy[0] = g[6];
    st.ref_xy[1] = g[7];
    st.pixel_area = std::fabs(det);
    for (int k = 0; k < 4; ++k) {
      st.Pf[k] = (float)st.P[k];
      st.Pinvf[k] = (float)st.Pinv[k];
    }
    st.thr_numel = (double)st.wnx * (double)st.wny;
    st.out_off = out_off;
    st.work_off = work_off;
    st.psf_off = psf_off;
    st.spsf_off = spsf_off;
    out_off += (int64_t)st.nx * st.ny;
    work_off += (int64_t)st.wnx * st.wny;
    psf_off += (int64_t)st.kx * st.ky;
    const int32_t kp2 = st.kpx * st.kpy;
    spsf_off += 2 * 3 * (int64_t)kp2;
    b->max_kp2 = std::max(b->max_kp2, kp2);
    st.ntw_x = (st.wnx + kTile - 1) / kTile;
    st.ntw = st.ntw_x * ((st.wny + kTile - 1) / kTile);
    st.nto_x = (st.nx + kOutTileX - 1) / kOutTileX;
    st.nto = st.nto_x * ((st.ny + conv_tile_y(large) - 1) / conv_tile_y(large));
    st.tile_w0 = tw;
    st.tile_o0 = to;
    if ((int64_t)tw + st.ntw > (int64_t)INT32_MAX / 2 || (int64_t)to + st.nto > (int64_t)INT32_MAX / 2) {
      delete b;
      return AP_ERR_ARG;
    }
    for (int t = 0; t < st.ntw; ++t) b->work_tiles.push_back(s);
    for (int t = 0; t < st.nto; ++t) b->out_tiles.push_back(s);
    tw += st.ntw;
    to += st.nto;
    if (psf && options->fft_min_kernel > 0 && std::max(st.kpx, st.kpy) >= options->fft_min_kernel) {
      // FFT sides: powers of two >= working window + kernel - 1 (no wrap into the crop)
      auto pow2 = [](int v) {
        int p = 8;
        while (p < v) p <<= 1;
        return p;
      };
      const int fx = pow2(st.wnx + st.kpx - 1), fy = pow2(st.wny + st.kpy - 1);
      if (fx <= kFftMaxSide && fy <= kFftMaxSide) {
        st.fft_nx = fx;
        st.fft_ny = fy;
        st.fft_off = b->fft_buf_elems;
        st.pre_off = b->preconv_elems;
        b->fft_buf_elems += 2 * 6 * (int64_t)fx * fy;
        b->preconv_elems += 2 * (3 + NGRAD) * (int64_t)st.nx * st.ny;
        b->fft_lists.push_back(s);
      }
    }
    if (psf && st.fft_nx == 0) {
      const size_t need = conv_smem_bytes(st.kpx, st.kpy, large);
      smem = std::max(smem, need);
    }
    if ((int64_t)st.wnx * st.wny >= (int64_t)1 << 31) {
      delete b;
      return AP_ERR_ARG;
    }
  }
  if (smem > 200 * 1024) {
    delete b;
    return AP_ERR_UNSUPPORTED;
  }
  b->conv_smem = smem;
  b->out_pixels = out_off;
  b->work_pixels = work_off;
  b->psf_pixels = psf_off;
  b->spsf_total = spsf_off;
  // FFT work lists: [stamps (n_fft)] [row-block prefix (n_fft + 1)] [column-group prefix]
  // [output row-block prefix]
  const int32_t n_fft = (int32_t)b->fft_lists.size();
  int32_t fft_rows = 0, fft_cols = 0, fft_outs = 0, fft_max_nx = 0, fft_max_ny = 0;
  if (n_fft > 0) {
    std::vector<int32_t> lists(b->fft_lists);
    std::vector<int32_t> rp(1, 0), cp(1, 0), op(1, 0);
    for (int32_t s : b->fft_lists) {
      const StampDev& st = b->stamps[s];
      const int rb = fft_rows_per_block(st.fft_nx);
      rp.push_back(rp.back() + (st.fft_ny + rb - 1) / rb);
      cp.push_back(cp.back() + st.fft_nx / 8);
      op.push_back(op.back() + (st.ny + rb - 1) / rb);
      fft_max_nx = std::max(fft_max_nx, st.fft_nx);
      fft_max_ny = std::max(fft_max_ny, st.fft_ny);
    }
    fft_rows = rp.back();
    fft_cols = cp.back();
    fft_outs = op.back();
    lists.insert(lists.end(), rp.begin(), rp.end());
    lists.insert(lists.end(), cp.begin(), cp.end());
    lists.insert(lists.end(), op.begin(), op.end());
    b->fft_lists = lists;
  }

  // quadrature tables
  QuadTables& T = b->tables;
  T.quad_level = options->integrate_quad_level > 0 ? options->integrate_quad_level : 3;
  T.gridding = options->integrate_gridding > 0 ? options->integrate_gridding : 5;
  if (T.quad_level > kMaxQuad) T.quad_level = kMaxQuad;
  if (T.gridding > kMaxGrid) T.gridding = kMaxGrid;
  fill_quad(T.quad_level, T.qx, T.qy, T.qw);
  const int g = T.gridding;
  for (int jj = 0; jj < g; ++jj)
    for (int ii = 0; ii < g; ++ii) {
      // linspace(-(g-1)/(2g), (g-1)/(2g), g)  (utils/operations.py:94-95)
      auto lin = [g](int k) {
        return g == 1 ? 0.0 : -(g - 1) / (2.0 * g) + k * ((g - 1) / (double)g) / (g - 1);
      };
      T.gx[jj * g + ii] = lin(ii);
      T.gy[jj * g + ii] = lin(jj);
    }
  switch (options->sampling_mode) {
    case AP_SAMPLING_MIDPOINT:
      T.nsub = 1;
      T.sub_center = 0;
      T.sx[0] = T.sy[0] = 0.0;
      T.sw[0] = 1.0;
      break;
    case AP_SAMPLING_TRAPEZOID:
      // corner grid, 2x2 mean (models/_model_methods.py:125-132)
      T.nsub = 4;
      T.sub_center = -1;
      for (int v = 0; v < 2; ++v)
        for (int u = 0; u < 2; ++u) {
          T.sx[v * 2 + u] = u - 0.5;
          T.sy[v * 2 + u] = v - 0.5;
          T.sw[v * 2 + u] = 0.25;
        }
      break;
    case AP_SAMPLING_SIMPSONS: {
      // half-pixel grid with the Simpson kernel (utils/interpolate.py:346-355)
      static const double kw[9] = {1, 4, 1, 4, 16, 4, 1, 4, 1};
      T.nsub = 9;
      T.sub_center = 4;
      for (int v = 0; v < 3; ++v)
        for (int u = 0; u < 3; ++u) {
          T.sx[v * 3 + u] = 0.5 * (u - 1);
          T.sy[v * 3 + u] = 0.5 * (v - 1);
          T.sw[v * 3 + u] = kw[v * 3 + u] / 36.0;
        }
      break;
    }
    case AP_SAMPLING_QUAD:
    case AP_SAMPLING_MIDPOINT_CENTER: {  // (the latter: the table of its centre pixels)
      const int k = options->sampling_quad_level;
      T.nsub = k * k;
      T.sub_center = (k * k) / 2;
      fill_quad(k, T.sx, T.sy, T.sw);
      break;
    }
  }

  quad_tables_fill_f32(T);

  // workspace layout
  Layout& L = b->L;
  int64_t o = 0;
  auto take = [&o](int64_t bytes) {
    const int64_t at = o;
    o = align_up(o + bytes);
    return at;
  };
  L.stamps = take(sizeof(StampDev) * (int64_t)n);
  L.evals = take(sizeof(EvalDev) * 2 * (int64_t)n);
  L.work_tiles = take(sizeof(int32_t) * (int64_t)b->work_tiles.size());
  L.out_tiles = take(sizeof(int32_t) * (int64_t)b->out_tiles.size());
  L.tables = take(sizeof(QuadTables));
  L.work = take(sizeof(float) * 2 * kNumPlanes * b->work_pixels);
  L.aux = take(sizeof(float) * 2 * 2 * b->work_pixels);
  L.spsf = take(sizeof(float) * std::max<int64_t>(b->spsf_total, 1));
  L.queue = take(sizeof(int64_t) * 2 * b->work_pixels);
  L.recheck = take(sizeof(int64_t) * 2 * b->work_pixels);
  L.amb = take(sizeof(int64_t) * b->work_pixels);
  L.wlist = take(sizeof(int64_t) * 2 * (int64_t)b->work_tiles.size());
  L.olist = take(sizeof(int64_t) * 2 * (int64_t)b->out_tiles.size());
  L.slist = take(sizeof(int32_t) * 2 * (int64_t)n);
  L.counters = take(sizeof(uint32_t) * 16);
  L.work_ctr = take(sizeof(unsigned long long) * 8);
  L.mean_acc = take(sizeof(double) * 2 * (int64_t)n);
  L.tile_acc = take(sizeof(double) * 2 * kNacc * (int64_t)b->out_tiles.size());
  L.acc = take(sizeof(double) * 2 * kNacc * (int64_t)n);
  L.fft_lists = take(sizeof(int32_t) * std::max<int64_t>((int64_t)b->fft_lists.size(), 1));
  L.fft_buf = take(sizeof(float2) * std::max<int64_t>(b->fft_buf_elems, 1));
  L.preconv = take(sizeof(float) * std::max<int64_t>(b->preconv_elems, 1));
  L.total = o;

  BatchArgs& A = b->args;
  A.n_stamps = n;
  A.kind = options->profile;
  A.sampling = options->sampling_mode;
  A.integrate = options->integrate_mode;
  A.psf_mode = options->psf_mode;
  A.lanczos = options->psf_mode == AP_PSF_FULL ? options->lanczos_order : 0;
  A.max_depth = options->integrate_max_depth;
  A.free_mask = options->free_mask;
  int nf = 0;
  for (int i = 0; i < NPARAM; ++i) nf += (options->free_mask >> i) & 1;
  A.n_free = nf;
  A.has_sky = options->has_sky;
  A.n_work_tiles = (int32_t)b->work_tiles.size();
  A.n_out_tiles = (int32_t)b->out_tiles.size();
  A.max_kp2 = b->max_kp2;
  A.conv_large = b->conv_large ? 1 : 0;
  A.tolerance = (float)options->sampling_tolerance;
  A.tolerance64 = options->sampling_tolerance;
  A.softening64 = options->softening;
  A.center_r2 = (float)(options->center_radius * options->center_radius + 1e-6);
  A.work_pixels = b->work_pixels;
  A.out_pixels = b->out_pixels;
  A.n_fft = n_fft;
  A.fft_rows = fft_rows;
  A.fft_cols = fft_cols;
  A.fft_outs = fft_outs;
  A.fft_max_nx = fft_max_nx;
  A.fft_max_ny = fft_max_ny;
  *out = b;
  return AP_OK;
}

int ap_batch_destroy(ap_batch* b) {
  delete b;
  return AP_OK;
}

int ap_batch_sizes(const ap_batch* b, int64_t* out_pixels, int64_t* psf_pixels,
                   int64_t* workspace_bytes) {
  if (!b) return AP_ERR_ARG;
  if (out_pixels) *out_pixels = b->out_pixels;
  if (psf_pixels) *psf_pixels = b->psf_pixels;
  if (workspace_bytes) *workspace_bytes = b->L.total;
  return AP_OK;
}

int ap_batch_offsets(const ap_batch* b, int64_t* out_offsets, int64_t* psf_offsets) {
  if (!b) return AP_ERR_ARG;
  for (int s = 0; s < b->n; ++s) {
    if (out_offsets) out_offsets[s] = b->stamps[s].out_off;
    if (psf_offsets) psf_offsets[s] = b->stamps[s].psf_off;
  }
  return AP_OK;
}

int ap_batch_psf_stride(const ap_batch* b, int64_t* stride) {
  if (!b || !stride) return AP_ERR_ARG;
  *stride = b->max_kp2;
  return AP_OK;
}

int ap_batch_set_threshold_numel(ap_batch* b, const double* numel) {
  if (!b || !numel) return AP_ERR_ARG;
  for (int i = 0; i < b->n; ++i)
    if (!(numel[i] > 0)) return AP_ERR_ARG;
  for (int i = 0; i < b->n; ++i) b->stamps[i].thr_numel = numel[i];
  if (b->bound) {
    const Layout& L = b->L;
    return check_cuda(cudaMemcpy(b->ws + L.stamps, b->stamps.data(), sizeof(StampDev) * b->n, cudaMemcpyHostToDevice));
  }
  return AP_OK;
}

int ap_batch_set_threshold_window(ap_batch* b, const int32_t* windows) {
  if (!b || !windows) return AP_ERR_ARG;
  for (int i = 0; i < b->n; ++i)
    if (windows[4 * i + 2] < 0 || windows[4 * i + 3] < 0) return AP_ERR_ARG;
  int any = 0;
  for (int i = 0; i < b->n; ++i) {
    StampDev& st = b->stamps[i];
    st.gw_x0 = windows[4 * i + 0];
    st.gw_y0 = windows[4 * i + 1];
    st.gw_nx = windows[4 * i + 2];
    st.gw_ny = windows[4 * i + 3];
    if (st.gw_nx == 0 || st.gw_ny == 0) st.gw_nx = st.gw_ny = 0;
    any |= st.gw_nx > 0;
  }
  b->args.thr_window = any;
  if (b->bound) {
    const Layout& L = b->L;
    return check_cuda(cudaMemcpy(b->ws + L.stamps, b->stamps.data(), sizeof(StampDev) * b->n, cudaMemcpyHostToDevice));
  }
  return AP_OK;
}

int ap_batch_bind(ap_batch* b, void* workspace, int64_t bytes, ap_stream_t stream) {
  if (!b || !workspace) return AP_ERR_ARG;
  if (bytes < b->L.total) return AP_ERR_WORKSPACE;
  if (((uintptr_t)workspace) % kAlign) return AP_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  char* ws = (char*)workspace;
  const Layout& L = b->L;
  BatchArgs& A = b->args;
  A.stamps = (const StampDev*)(ws + L.stamps);
  A.evals = (EvalDev*)(ws + L.evals);
  A.work_tiles = (const int32_t*)(ws + L.work_tiles);
  A.out_tiles = (const int32_t*)(ws + L.out_tiles);
  A.tables = (const QuadTables*)(ws + L.tables);
  A.work = (float*)(ws + L.work);
  A.aux = (float*)(ws + L.aux);
  A.spsf = (float*)(ws + L.spsf);
  A.queue = (int64_t*)(ws + L.queue);
  A.recheck = (int64_t*)(ws + L.recheck);
  A.amb = (int64_t*)(ws + L.amb);
  A.amb_cap = b->work_pixels;
  A.wlist = (int64_t*)(ws + L.wlist);
  A.olist = (int64_t*)(ws + L.olist);
  A.slist = (int32_t*)(ws + L.slist);
  A.counters = (uint32_t*)(ws + L.counters);
  A.work_ctr = (unsigned long long*)(ws + L.work_ctr);
  A.mean_acc = (double*)(ws + L.mean_acc);
  A.tile_acc = (double*)(ws + L.tile_acc);
  A.acc = (double*)(ws + L.acc);
  if (A.n_fft > 0) {
    const int32_t* fl = (const int32_t*)(ws + L.fft_lists);
    A.fft_stamp = fl;
    A.fft_row_pre = fl + A.n_fft;
    A.fft_col_pre = fl + 2 * A.n_fft + 1;
    A.fft_out_pre = fl + 3 * A.n_fft + 2;
    A.fft_buf = (float2*)(ws + L.fft_buf);
    A.preconv = (float*)(ws + L.preconv);
  }
  int rc = AP_OK;
  rc = rc ? rc : check_cuda(cudaMemcpyAsync(ws + L.stamps, b->stamps.data(), sizeof(StampDev) * b->n, cudaMemcpyHostToDevice, s));
  rc = rc ? rc : check_cuda(cudaMemcpyAsync(ws + L.work_tiles, b->work_tiles.data(), sizeof(int32_t) * b->work_tiles.size(), cudaMemcpyHostToDevice, s));
  rc = rc ? rc : check_cuda(cudaMemcpyAsync(ws + L.out_tiles, b->out_tiles.data(), sizeof(int32_t) * b->out_tiles.size(), cudaMemcpyHostToDevice, s));
  rc = rc ? rc : check_cuda(cudaMemcpyAsync(ws + L.tables, &b->tables, sizeof(QuadTables), cudaMemcpyHostToDevice, s));
  rc = rc ? rc : check_cuda(cudaMemsetAsync(ws + L.counters, 0, sizeof(uint32_t) * 16, s));
  rc = rc ? rc : check_cuda(cudaMemsetAsync(ws + L.work_ctr, 0, sizeof(unsigned long long) * 8, s));
  rc = rc ? rc : check_cuda(cudaMemsetAsync(ws + L.evals, 0, sizeof(EvalDev) * 2 * b->n, s));
  if (A.n_fft > 0) {
    rc = rc ? rc : check_cuda(cudaMemcpyAsync(ws + L.fft_lists, b->fft_lists.data(),
                                              sizeof(int32_t) * b->fft_lists.size(), cudaMemcpyHostToDevice, s));
    rc = rc ? rc : check_cuda(fft_upload_twiddles(s));
    rc = rc ? rc : check_cuda(set_fft_smem());
  }
  rc = rc ? rc : check_cuda(cudaStreamSynchronize(s));
  if (!rc && b->conv_smem > 48 * 1024) rc = check_cuda(set_conv_smem(b->conv_smem));
  b->ws = ws;
  b->bound = (rc == AP_OK);
  return rc;
}

static int render_common(ap_batch* b, const double* params, const float* psf, float* model,
                         float* jac, int32_t ops, ap_stream_t stream) {
  if (!b || !params || !model) return AP_ERR_ARG;
  if (!b->bound) return AP_ERR_NOT_BOUND;
  if (b->opt.psf_mode != AP_PSF_NONE && !psf) return AP_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  int rc = check_cuda(launch_eval_setup(b->args, params, NPARAM, 0, nullptr, ops, s));
  if (rc) return rc;
  ConvIO io{};
  io.psf = psf;
  io.model_out = model;
  io.jac_out = jac;
  return check_cuda(launch_render_pass(b->args, io, b->conv_smem, false, s, &b->prof));
}

int ap_render(ap_batch* b, const double* params, const float* psf, float* model,
              ap_stream_t stream) {
  return render_common(b, params, psf, model, nullptr, OP_FWD | OP_WRITE_MODEL, stream);
}

int ap_jacobian(ap_batch* b, const double* params, const float* psf, float* model, float* jac,
                int32_t as_representation, ap_stream_t stream) {
  if (!jac) return AP_ERR_ARG;
  int32_t ops = OP_FWD | OP_JAC | OP_WRITE_MODEL | OP_WRITE_JAC;
  if (as_representation) ops |= OP_REP;
  return render_common(b, params, psf, model, jac, ops, stream);
}

// base point of difference renders outside the LM: evaluation constants, shifted kernel, deep
// image and integration pattern (the buffers the batched LM keeps in its own workspace)
namespace {
struct BaseLayout {
  int64_t eval, psf, deep, code, total;
};

BaseLayout base_layout(const ap_batch* b) {
  BaseLayout L{};
  int64_t o = 0;
  auto take = [&o](int64_t bytes) {
    const int64_t at = o;
    o = align_up(o + bytes);
    return at;
  };
  L.eval = take(sizeof(EvalDev) * b->n);
  L.psf = take(sizeof(float) * b->n * std::max<int64_t>(1, b->max_kp2));
  L.deep = take(sizeof(float) * b->work_pixels);
  L.code = take(sizeof(uint32_t) * b->work_pixels);
  L.total = o;
  return L;
}
}  // namespace

int ap_render_base_bytes(const ap_batch* b, int64_t* bytes) {
  if (!b || !bytes) return AP_ERR_ARG;
  *bytes = base_layout(b).total;
  return AP_OK;
}

int ap_render_precise(ap_batch* b, const double* params, const float* psf, float* model, void* base,
                      int64_t base_bytes, int32_t mode, ap_stream_t stream) {
  if (!b || !params || !model || !base) return AP_ERR_ARG;
  if (mode != AP_RENDER_BASE && mode != AP_RENDER_DIFFERENCE) return AP_ERR_ARG;
  if (((uintptr_t)base & 15u) != 0) return AP_ERR_ARG;
  if (!b->bound) return AP_ERR_NOT_BOUND;
  if (b->opt.psf_mode != AP_PSF_NONE && !psf) return AP_ERR_ARG;
  if (b->args.kind != AP_PROFILE_SERSIC && b->args.kind != AP_PROFILE_EXPONENTIAL) return AP_ERR_UNSUPPORTED;
  if (b->args.lanczos > 0) return AP_ERR_UNSUPPORTED;  // no difference form of a Lanczos shift
  const BaseLayout L = base_layout(b);
  if (base_bytes < L.total) return AP_ERR_WORKSPACE;
  char* w = (char*)base;
  BatchArgs A = b->args;
  A.base_eval = (EvalDev*)(w + L.eval);
  A.base_psf = (float*)(w + L.psf);
  A.base_deep = (float*)(w + L.deep);
  A.base_code = (uint32_t*)(w + L.code);
  cudaStream_t s = (cudaStream_t)stream;
  const int32_t ops = OP_FWD | OP_WRITE_MODEL | (mode == AP_RENDER_BASE ? OP_BASE : OP_DIFF);
  int rc = check_cuda(launch_eval_setup(A, params, NPARAM, 0, nullptr, ops, s));
  if (rc) return rc;
  ConvIO io{};
  io.psf = psf;
  io.model_out = model;
  return check_cuda(launch_render_pass(A, io, b->conv_smem, false, s, &b->prof));
}

int ap_render_psf_derivative(ap_batch* b, const double* params, const float* psf, const float* dpsf,
                             float* model, ap_stream_t stream) {
  if (!b || !params || !psf || !dpsf || !model) return AP_ERR_ARG;
  if (!b->bound) return AP_ERR_NOT_BOUND;
  if (b->opt.psf_mode == AP_PSF_NONE || b->opt.has_sky) return AP_ERR_ARG;
  if (b->args.lanczos > 0) return AP_ERR_UNSUPPORTED;  // the derivative's shift is bilinear
  cudaStream_t s = (cudaStream_t)stream;
  int rc = check_cuda(launch_eval_setup(b->args, params, NPARAM, 0, nullptr, OP_FWD | OP_WRITE_MODEL, s));
  if (rc) return rc;
  ConvIO io{};
  io.psf = dpsf;
  io.psf_base = psf;
  io.model_out = model;
  return check_cuda(launch_render_pass(b->args, io, b->conv_smem, false, s, &b->prof));
}

int ap_render_vjp(ap_batch* b, const double* params, const float* psf, const float* grad_model,
                  int32_t flags, double* grad_params, ap_stream_t stream) {
  if (!b || !params || !grad_model || !grad_params) return AP_ERR_ARG;
  if (flags & ~(AP_VJP_REPRESENTATION | AP_VJP_REFERENCE_CENTER)) return AP_ERR_ARG;
  if (!b->bound) return AP_ERR_NOT_BOUND;
  if (b->opt.psf_mode != AP_PSF_NONE && !psf) return AP_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  int32_t ops = OP_FWD | OP_JAC | OP_VJP;
  if (flags & AP_VJP_REPRESENTATION) ops |= OP_REP;
  if ((flags & AP_VJP_REFERENCE_CENTER) && b->opt.psf_mode == AP_PSF_FULL) ops |= OP_VJP_COORD;
  int rc = check_cuda(launch_eval_setup(b->args, params, NPARAM, 0, nullptr, ops, s));
  if (rc) return rc;
  ConvIO io{};
  io.psf = psf;
  io.vjp_in = grad_model;
  rc = check_cuda(launch_render_pass(b->args, io, b->conv_smem, true, s, &b->prof));
  if (rc) return rc;
  return check_cuda(launch_gather_vjp(b->args, grad_params, s));
}

int ap_batch_autotune(ap_batch* b, const double* params, const float* psf, int32_t jacobian, int32_t* chosen,
                      double* best_ms, ap_stream_t stream) {
  if (!b || !params || !chosen) return AP_ERR_ARG;
  if (!b->bound) return AP_ERR_NOT_BOUND;
  if (b->opt.psf_mode != AP_PSF_NONE && !psf) return AP_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return AP_ERR_ARG;
  const int32_t ops = jacobian ? (OP_FWD | OP_JAC) : OP_FWD;
  // candidates (blocks per SM) of each persistent grid, tuned one knob at a time
  static const int cand[GK_COUNT][5] = {{4, 8, 16, 0, 0}, {3, 6, 8, 12, 0}, {4, 8, 12, 16, 24}, {4, 8, 16, 0, 0}};
  const int defaults[GK_COUNT] = {8, 8, 16, 8};
  for (int k = 0; k < GK_COUNT; ++k) b->args.grid_mult[k] = defaults[k];
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return check_cuda(cudaGetLastError());
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return check_cuda(cudaGetLastError());
  }
  ConvIO io{};
  io.psf = psf;
  auto run = [&]() -> int {
    int rc = check_cuda(launch_eval_setup(b->args, params, NPARAM, 0, nullptr, ops, s));
    if (rc) return rc;
    return check_cuda(launch_render_pass(b->args, io, b->conv_smem, false, s, nullptr));
  };
  auto time_it = [&](double& ms) -> int {
    int rc = run();  // warm
    if (rc) return rc;
    float best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(e0, s);
      rc = run();
      if (rc) return rc;
      cudaEventRecord(e1, s);
      rc = check_cuda(cudaEventSynchronize(e1));
      if (rc) return rc;
      float t = 0.f;
      cudaEventElapsedTime(&t, e0, e1);
      best = t < best ? t : best;
    }
    ms = best;
    return AP_OK;
  };
  int rc = AP_OK;
  double ms_best = 0.0;
  rc = time_it(ms_best);
  for (int k = 0; k < GK_COUNT && !rc; ++k) {
    if (k == GK_PSF && b->opt.psf_mode == AP_PSF_NONE) continue;
    if (k == GK_INTEGRATE && b->opt.integrate_mode != AP_INTEGRATE_THRESHOLD) continue;
    int best = b->args.grid_mult[k];
    for (int c = 0; c < 5 && cand[k][c] > 0 && !rc; ++c) {
      if (cand[k][c] == best) continue;
      b->args.grid_mult[k] = cand[k][c];
      double ms = 0.0;
      rc = time_it(ms);
      if (!rc && ms < ms_best) {
        ms_best = ms;
        best = cand[k][c];
      }
    }
    b->args.grid_mult[k] = best;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  for (int k = 0; k < GK_COUNT; ++k) chosen[k] = b->args.grid_mult[k];
  if (best_ms) *best_ms = ms_best;
  return rc;
}

int ap_values_to_rep(const double* values, int32_t n, int32_t free_mask, double* rep, ap_stream_t stream) {
  if (!values || !rep || n < 0 || (free_mask & ~0xff)) return AP_ERR_ARG;
  return check_cuda(launch_values_to_rep(values, n, free_mask, rep, (cudaStream_t)stream));
}

namespace {
int refinit_geometry_ok(const ap_batch* b) {
  for (int i = 0; i < b->n; ++i) {
    const StampDev& s = b->stamps[i];
    if (!(s.P[0] > 0) || s.P[0] != s.P[3] || s.P[1] != 0 || s.P[2] != 0) return AP_ERR_UNSUPPORTED;
  }
  return AP_OK;
}
}  // namespace

int ap_reference_init_workspace_bytes(const ap_batch* b, int64_t* bytes) {
  if (!b || !bytes) return AP_ERR_ARG;
  const RefInitPlan P = plan_reference_init(b->stamps.data(), b->n);
  *bytes = P.scratch_bytes;
  return AP_OK;
}

int ap_reference_init(ap_batch* b, const float* data, const uint8_t* mask, int32_t known_mask, double* params,
                      int32_t* status, void* workspace, int64_t workspace_bytes, ap_stream_t stream) {
  if (!b || !data || !params || !status || (known_mask & ~0xff)) return AP_ERR_ARG;
  if (!b->bound) return AP_ERR_NOT_BOUND;
  if (b->opt.profile != AP_PROFILE_SERSIC && b->opt.profile != AP_PROFILE_EXPONENTIAL) return AP_ERR_UNSUPPORTED;
  if (int rc = refinit_geometry_ok(b)) return rc;
  const RefInitPlan P = plan_reference_init(b->stamps.data(), b->n);
  if (P.scratch_bytes > 0 && (!workspace || workspace_bytes < P.scratch_bytes)) return AP_ERR_WORKSPACE;
  return check_cuda(launch_reference_init(P, b->args.stamps, b->n, b->opt.profile, known_mask, data, mask, params,
                                          status, workspace, (cudaStream_t)stream));
}

int ap_segmap_range(const int32_t* seg, int64_t npix, int32_t* min_max, ap_stream_t stream) {
  if (!seg || !min_max || npix <= 0) return AP_ERR_ARG;
  return check_cuda(launch_seg_range(seg, npix, min_max, (cudaStream_t)stream));
}

int ap_segmap_present(const int32_t* seg, int64_t npix, int32_t max_id, uint8_t* present, ap_stream_t stream) {
  if (!seg || !present || npix <= 0 || max_id < 0) return AP_ERR_ARG;
  return check_cuda(launch_seg_mark(seg, npix, present, max_id, (cudaStream_t)stream));
}

int ap_segmap_stats(const int32_t* seg, const float* image, int32_t nx, int32_t ny, const int32_t* index,
                    int32_t n_seg, double north, const double* centroid_in, const double* pa_in, double* acc,
                    int32_t* bbox, double* centroid, double* pa, double* q, ap_stream_t stream) {
  if (!seg || !image || !index || !acc || !bbox || !centroid || !pa || !q || nx <= 0 || ny <= 0 || n_seg < 0)
    return AP_ERR_ARG;
  if (n_seg == 0) return AP_OK;
  return check_cuda(launch_seg_stats(seg, image, nx, ny, index, n_seg, north, centroid_in, pa_in, acc, bbox,
                                     centroid, pa, q, (cudaStream_t)stream));
}

int ap_window_flux(const float* image, int32_t nx, int32_t ny, const int32_t* windows, int32_t n, double* flux,
                   ap_stream_t stream) {
  if (!image || !windows || !flux || nx <= 0 || ny <= 0 || n < 0) return AP_ERR_ARG;
  return check_cuda(launch_window_flux(image, nx, ny, windows, n, flux, (cudaStream_t)stream));
}

int ap_batch_set_grid(ap_batch* b, const int32_t* blocks_per_sm) {
  if (!b || !blocks_per_sm) return AP_ERR_ARG;
  for (int k = 0; k < GK_COUNT; ++k)
    if (blocks_per_sm[k] < 1 || blocks_per_sm[k] > 64) return AP_ERR_ARG;
  for (int k = 0; k < GK_COUNT; ++k) b->args.grid_mult[k] = blocks_per_sm[k];
  return AP_OK;
}

int ap_psf_shift(ap_batch* b, const double* params, const float* psf, float* out, float* d_out,
                 ap_stream_t stream) {
  if (!b || !params || !psf || !out) return AP_ERR_ARG;
  if (!b->bound) return AP_ERR_NOT_BOUND;
  if (b->opt.psf_mode == AP_PSF_NONE) return AP_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int32_t ops = OP_FWD | (d_out ? OP_JAC : 0);
  int rc = check_cuda(launch_eval_setup(b->args, params, NPARAM, 0, nullptr, ops, s));
  if (rc) return rc;
  // only the PSF stage of the render pass
  const BatchArgs& A = b->args;
  rc = check_cuda(launch_psf_only(A, psf, s));
  if (rc) return rc;
  return check_cuda(launch_psf_export(A, out, d_out, b->max_kp2, s));
}

int ap_chi2(ap_batch* b, const float* data, const float* weight, const uint8_t* mask,
            const float* model, double* chi2_out, ap_stream_t stream) {
  if (!b || !data || !model || !chi2_out) return AP_ERR_ARG;
  if (!b->bound) return AP_ERR_NOT_BOUND;
  cudaStream_t s = (cudaStream_t)stream;
  ConvIO io{};
  io.data = data;
  io.weight = weight;
  io.mask = mask;
  return check_cuda(launch_chi2_only(b->args, io, model, chi2_out, s));
}

int ap_damped_solve(int32_t m, int32_t p, const double* hess, const double* grad, const double* L,
                    double* h_out, ap_stream_t stream) {
  if (m < 0 || p < 1 || p > NPARAM || !hess || !grad || !L || !h_out) return AP_ERR_ARG;
  if (m == 0) return AP_OK;
  return check_cuda(launch_damped_solve(m, p, hess, grad, L, h_out, (cudaStream_t)stream));
}

// ---------------------------------------------------------------------------
// batched LM
// ---------------------------------------------------------------------------
namespace {
struct LMLayout {
  int64_t st, params_next, ops_next, hvec, y0, jbase, base_eval, base_psf, base_deep, base_code, hist_loss, hist_L,
      hist_x, active, total;
};

LMLayout lm_layout(const ap_batch* b, const ap_lm_options* lm) {
  LMLayout L{};
  int64_t o = 0;
  auto take = [&o](int64_t bytes) {
    const int64_t at = o;
    o = align_up(o + bytes);
    return at;
  };
  const int64_t n = b->n, H = (int64_t)lm->max_iter + 1;
  L.st = take(sizeof(LMState) * n);
  L.params_next = take(sizeof(double) * n * 2 * NPARAM);
  L.ops_next = take(sizeof(int32_t) * n * 2);
  L.hvec = take(sizeof(double) * n * NPARAM);
  L.y0 = take(sizeof(float) * b->out_pixels);
  L.jbase = take(sizeof(float) * std::max<int64_t>(1, b->args.n_free) * b->out_pixels);
  // base point of the difference trials: evaluation constants, kernel, deep image, pattern
  L.base_eval = take(sizeof(EvalDev) * n);
  L.base_psf = take(sizeof(float) * n * std::max<int64_t>(1, b->max_kp2));
  L.base_deep = take(sizeof(float) * b->work_pixels);
  L.base_code = take(sizeof(uint32_t) * b->work_pixels);
  L.hist_loss = take(sizeof(double) * n * H);
  L.hist_L = take(sizeof(double) * n * H);
  L.hist_x = take(sizeof(double) * n * H * NPARAM);
  L.active = take(sizeof(uint32_t) * 4);
  L.total = o;
  return L;
}

int lm_validate(const ap_lm_options* lm) {
  if (!lm) return AP_ERR_ARG;
  if (lm->max_iter < 0 || lm->max_iter > 100000 || lm->max_step_iter < 1) return AP_ERR_ARG;
  if (lm->rounds_per_sync < 1) return AP_ERR_ARG;
  return AP_OK;
}
}  // namespace

int ap_lm_workspace_bytes(const ap_batch* b, const ap_lm_options* lm, int64_t* bytes) {
  if (!b || !bytes) return AP_ERR_ARG;
  int rc = lm_validate(lm);
  if (rc) return rc;
  *bytes = lm_layout(b, lm).total;
  return AP_OK;
}

int ap_lm_fit(ap_batch* b, const float* data, const float* weight, const uint8_t* mask,
              const float* psf, const double* fixed_params, double* state, const ap_lm_options* lm,
              void* lm_ws, int64_t lm_ws_bytes, double* chi2_out, int32_t* iters_out,
              int32_t* status_out, ap_stream_t stream) {
  if (!b || !data || !fixed_params || !state || !lm_ws || !chi2_out || !iters_out || !status_out)
    return AP_ERR_ARG;
  if (!b->bound) return AP_ERR_NOT_BOUND;
  // the device LM's representation maps carry the Sersic index limits (0.36, 8)
  if (b->opt.profile != AP_PROFILE_SERSIC && b->opt.profile != AP_PROFILE_EXPONENTIAL) return AP_ERR_UNSUPPORTED;
  int rc = lm_validate(lm);
  if (rc) return rc;
  if (b->opt.psf_mode != AP_PSF_NONE && !psf) return AP_ERR_ARG;
  const LMLayout L = lm_layout(b, lm);
  if (lm_ws_bytes < L.total) return AP_ERR_WORKSPACE;
  if (((uintptr_t)lm_ws) % kAlign) return AP_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  char* w = (char*)lm_ws;
  LMArgs a{};
  a.max_iter = lm->max_iter;
  a.max_step_iter = lm->max_step_iter;
  a.precise = lm->precise_trials ? 1 : 0;
  a.rel_tol = lm->relative_tolerance;
  a.curvature_limit = lm->curvature_limit;
  a.Lup = lm->Lup;
  a.Ldn = lm->Ldn;
  a.L0 = lm->L0;
  a.acceleration = lm->acceleration;
  a.st = (LMState*)(w + L.st);
  a.params_next = (double*)(w + L.params_next);
  a.ops_next = (int32_t*)(w + L.ops_next);
  a.hvec = (double*)(w + L.hvec);
  a.fixed = fixed_params;
  a.hist_loss = (double*)(w + L.hist_loss);
  a.hist_L = (double*)(w + L.hist_L);
  a.hist_x = (double*)(w + L.hist_x);
  a.state_out = state;
  a.chi2_out = chi2_out;
  a.iters_out = iters_out;
  a.status_out = status_out;
  a.active_count = (uint32_t*)(w + L.active);
  ConvIO io{};
  io.psf = psf;
  io.data = data;
  io.weight = weight;
  io.mask = mask;
  io.model_out = (float*)(w + L.y0);
  io.jac_out = (float*)(w + L.jbase);
  io.y0 = (const float*)(w + L.y0);
  io.jbase = (const float*)(w + L.jbase);
  io.hvec = a.hvec;
  io.rpp_d = 0.1;

  // the batch's arguments with the LM's base buffers (kept out of b->args: the other entry
  // points render without them)
  BatchArgs A = b->args;
  A.base_eval = (EvalDev*)(w + L.base_eval);
  A.base_psf = (float*)(w + L.base_psf);
  A.base_deep = (float*)(w + L.base_deep);
  A.base_code = (uint32_t*)(w + L.base_code);

  rc = check_cuda(cudaMemsetAsync(w + L.hist_loss, 0, L.active - L.hist_loss, s));
  if (rc) return rc;
  rc = check_cuda(launch_lm_init(A, a, state, mask, s));
  if (rc) return rc;

  Profiler* P = &b->prof;
  if (P->on) {
    // pairs recorded before this call (render entry points) are harvested first
    cudaStreamSynchronize(s);
    P->harvest(true);
  }
  auto one_round = [&](cudaStream_t st) -> cudaError_t {
    int t = P->on ? P->begin(KC_SETUP, st) : -1;
    cudaError_t e = launch_eval_setup(A, a.params_next, 2 * NPARAM, NPARAM, a.ops_next, 0, st);
    if (t >= 0) P->end(t, st);
    if (e != cudaSuccess) return e;
    e = launch_render_pass(A, io, b->conv_smem, true, st, P);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(a.active_count, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    t = P->on ? P->begin(KC_LM, st) : -1;
    e = launch_lm_update(A, a, st);
    if (t >= 0) P->end(t, st);
    return e;
  };

  // every LM phase finishes within (1 + max_iter * (1 + 2 * max_step_iter)) rounds
  const int64_t max_rounds = 2 + (int64_t)lm->max_iter * (2 + 2 * (int64_t)lm->max_step_iter);
  const int R = lm->rounds_per_sync;
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  if (lm->use_graph) {
    // capture on a private stream (the caller's may be the legacy default stream, which
    // cannot be captured); the instantiated graph is then launched on the caller's stream
    if (!b->cap_stream) rc = check_cuda(cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking));
    cudaStream_t cs = b->cap_stream;
    if (!rc) rc = check_cuda(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    if (!rc) {
      for (int r = 0; r < R && !rc; ++r) rc = check_cuda(one_round(cs));
      cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
      if (!rc) rc = check_cuda(e2);
    }
    if (!rc) rc = check_cuda(cudaGraphInstantiate(&exec, graph, 0));
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
  }
  int64_t rounds = 0;
  uint32_t active = 1;
  while (rounds < max_rounds && active > 0) {
    if (exec) {
      rc = check_cuda(cudaGraphLaunch(exec, s));
    } else {
      for (int r = 0; r < R && !rc; ++r) rc = check_cuda(one_round(s));
    }
    if (rc) break;
    rounds += R;
    rc = check_cuda(cudaMemcpyAsync(&active, a.active_count, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    if (!rc) rc = check_cuda(cudaStreamSynchronize(s));
    if (rc) break;
    if (P->on) P->harvest(!exec);  // graph: the captured pairs are re-recorded every replay
  }
  if (P->on && exec) P->used = 0;
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (rc) return rc;
  rc = check_cuda(launch_lm_finish(A, a, s));
  b->stats[3] = rounds;
  b->hist_loss = a.hist_loss;
  b->hist_L = a.hist_L;
  b->hist_x = a.hist_x;
  b->hist_len = lm->max_iter + 1;
  return rc;
}

int ap_lm_history(const ap_batch* b, const double** loss, const double** lambda_,
                  const double** states, int32_t* hist_len) {
  if (!b) return AP_ERR_ARG;
  if (loss) *loss = b->hist_loss;
  if (lambda_) *lambda_ = b->hist_L;
  if (states) *states = b->hist_x;
  if (hist_len) *hist_len = b->hist_len;
  return AP_OK;
}

int ap_batch_profile(ap_batch* b, int32_t enable) {
  if (!b) return AP_ERR_ARG;
  b->prof.on = enable != 0;
  b->prof.clear_totals();
  return AP_OK;
}

int ap_batch_kernel_times(ap_batch* b, double* ms_out, int64_t* launches_out) {
  if (!b) return AP_ERR_ARG;
  if (b->prof.on && b->prof.used > 0) {
    if (cudaDeviceSynchronize() != cudaSuccess) return AP_ERR_CUDA;
    b->prof.harvest(true);
  }
  for (int k = 0; k < KC_COUNT; ++k) {
    if (ms_out) ms_out[k] = b->prof.ms[k];
    if (launches_out) launches_out[k] = b->prof.launches[k];
  }
  return AP_OK;
}

int ap_batch_work_counters(ap_batch* b, uint64_t* out, int32_t reset, ap_stream_t stream) {
  if (!b || !out) return AP_ERR_ARG;
  if (!b->bound) return AP_ERR_NOT_BOUND;
  cudaStream_t s = (cudaStream_t)stream;
  unsigned long long c[6];
  if (cudaMemcpyAsync(c, b->args.work_ctr, sizeof(c), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return AP_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return AP_ERR_CUDA;
  for (int k = 0; k < 6; ++k) out[k] = c[k];
  if (reset && cudaMemsetAsync(b->args.work_ctr, 0, sizeof(c), s) != cudaSuccess) return AP_ERR_CUDA;
  return AP_OK;
}

int ap_fma_probe(float* scratch, int32_t iters, int32_t blocks, ap_stream_t stream) {
  if (!scratch || iters < 1 || blocks < 1) return AP_ERR_ARG;
  return check_cuda(launch_fma_probe(scratch, iters, blocks, (cudaStream_t)stream));
}

int ap_sample_probe(int32_t kind, float* scratch, int32_t iters, int32_t blocks, ap_stream_t stream) {
  if (!scratch || iters < 1 || blocks < 1 || kind < 0 || kind > 2) return AP_ERR_ARG;
  return check_cuda(launch_sample_probe(kind, scratch, iters, blocks, (cudaStream_t)stream));
}

int ap_batch_stats(const ap_batch* b, int64_t* stats_out) {
  if (!b || !stats_out) return AP_ERR_ARG;
  uint32_t c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (b->bound) {
    if (cudaMemcpy(c, b->args.counters, sizeof(c), cudaMemcpyDeviceToHost) != cudaSuccess)
      return AP_ERR_CUDA;
  }
  stats_out[0] = c[0];
  stats_out[1] = c[2];
  stats_out[2] = c[3];
  stats_out[3] = b->stats[3];
  stats_out[4] = c[6];
  return AP_OK;
}

}  // extern "C"
