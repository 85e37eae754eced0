// Host-side declarations shared by the kernel and C-ABI translation units.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "ap_device.cuh"

namespace apgb {

// Per-stamp LM state (float64), one thread per stamp updates it.
struct LMState {
  int32_t phase;      // LM_PH_*
  int32_t status;     // AP_LM_*
  int32_t iter;       // outer iterations done
  int32_t sub;        // inner (damping search) iteration
  int32_t direction;  // 0 none, 1 better, 2 worse
  int32_t nostep;
  int32_t scarry_valid;
  int32_t hist_len;
  double L;
  double chi2_cur;    // loss_history[-1]
  double init_chi2;
  double ndf;
  double best_chi2, best_L, scarry_chi2, scarry_L;
  double anchor_err;  // error bound of chi2_cur accumulated from trial differences since it was
                      // last taken from a full render
  double x[NPARAM], h[NPARAM], a[NPARAM], ha[NPARAM];
  double best_ha[NPARAM], scarry_ha[NPARAM];
  double H[NPARAM * NPARAM], g[NPARAM];
};

enum LMPhase { LM_PH_INIT = 0, LM_PH_JAC = 1, LM_PH_SUB = 2, LM_PH_SUB2 = 3, LM_PH_DONE = 4 };

struct LMArgs {
  int32_t max_iter, max_step_iter;
  int32_t precise;         // trials rendered as differences to the step's base point (OP_DIFF)
  double rel_tol, curvature_limit, Lup, Ldn, L0, acceleration;
  LMState* st;             // [n]
  double* params_next;     // [n][2][8]  value space
  int32_t* ops_next;       // [n][2]
  double* hvec;            // [n][8] h of the current trial (for OP_RPP)
  const double* fixed;     // [n][8] value-space parameters of locked slots
  double* hist_loss;       // [n][max_iter + 1]
  double* hist_L;          // [n][max_iter + 1]
  double* hist_x;          // [n][max_iter + 1][8]
  double* state_out;       // [n][n_free]
  double* chi2_out;        // [n]
  int32_t* iters_out;      // [n]
  int32_t* status_out;     // [n]
  uint32_t* active_count;  // device counter of stamps not done
};

// Optional CUDA-event timing of each kernel class (works inside captured graphs: every
// round captured gets its own event pairs, harvested after each replay).
enum KernelClass { KC_SETUP = 0, KC_PSF, KC_SAMPLE, KC_SELECT, KC_INTEGRATE, KC_CONV, KC_REDUCE,
                   KC_LM, KC_COUNT };

struct Profiler {
  bool on = false;
  int used = 0;              // event pairs in use
  int cap = 0;               // pairs created
  cudaEvent_t* ev = nullptr; // [cap][2]
  int* kind = nullptr;       // [cap]
  double ms[KC_COUNT] = {0};
  long long launches[KC_COUNT] = {0};
  int begin(int k, cudaStream_t s);
  void end(int idx, cudaStream_t s);
  void record(cudaEvent_t e, cudaStream_t s);
  void harvest(bool reset);  // after a synchronise: add elapsed times of the used pairs
  void clear_totals();
  void destroy();
};

// AP_OK for cudaSuccess, else remembers the error for ap_last_cuda_error and returns AP_ERR_CUDA
int record_cuda(cudaError_t e);
extern thread_local cudaError_t g_last_cuda_error;

// render-pass launches (ap_kernels.cu)
cudaError_t launch_eval_setup(const BatchArgs& b, const double* params, int64_t stamp_stride,
                              int64_t slot_stride, const int32_t* ops, int32_t ops_uniform,
                              cudaStream_t s);
cudaError_t launch_render_pass(const BatchArgs& b, const ConvIO& io, size_t conv_smem,
                               bool accumulate, cudaStream_t s, Profiler* prof = nullptr);
cudaError_t launch_fma_probe(float* out, int iters, int blocks, cudaStream_t s);
cudaError_t launch_sample_probe(int kind, float* out, int iters, int blocks, cudaStream_t s);
cudaError_t set_conv_smem(size_t bytes);
cudaError_t launch_chi2_only(const BatchArgs& b, const ConvIO& io, const float* model,
                             double* out, cudaStream_t s);
cudaError_t launch_psf_only(const BatchArgs& b, const float* psf, cudaStream_t s);
cudaError_t launch_gather_vjp(const BatchArgs& b, double* grad, cudaStream_t s);
cudaError_t launch_values_to_rep(const double* values, int32_t n, int32_t free_mask, double* rep, cudaStream_t st);
cudaError_t launch_damped_solve(int m, int p, const double* hess, const double* grad,
                                const double* L, double* h, cudaStream_t s);
cudaError_t launch_psf_export(const BatchArgs& b, float* out, float* d_out, int64_t stride,
                              cudaStream_t s);

// PSF convolution by FFT (ap_fft.cu)
constexpr int kFftMaxSide = 1024;  // largest transform side
cudaError_t fft_upload_twiddles(cudaStream_t st);
cudaError_t set_fft_smem();
cudaError_t launch_fft_conv(const BatchArgs& b, int total_rows, int total_cols, int total_out, int max_nx,
                            int max_ny, cudaStream_t s);

// segmentation-map statistics (ap_segmap.cu)
cudaError_t launch_seg_range(const int32_t* seg, int64_t n, int32_t* mm, cudaStream_t s);
cudaError_t launch_seg_mark(const int32_t* seg, int64_t n, uint8_t* present, int32_t max_id, cudaStream_t s);
cudaError_t launch_seg_stats(const int32_t* seg, const float* img, int nx, int ny, const int32_t* index, int n_seg,
                             double north, const double* cen_in, const double* pa_in, double* acc, int32_t* bbox,
                             double* cen, double* pa, double* q, cudaStream_t s);
cudaError_t launch_window_flux(const float* img, int nx, int ny, const int32_t* wins, int n, double* out,
                               cudaStream_t s);

// the reference's initial-value heuristics (ap_refinit.cu)
constexpr size_t kRefInitSmemBudget = 200 * 1024;  // dynamic shared memory per CTA at most
struct RefInitPlan {
  int iso_cap = 0;         // isophote samples per CTA (power of two)
  int pix_cap = 0;         // pixel sort buffer (power of two >= pixels and edge pixels per stamp)
  bool pix_in_smem = false;
  size_t smem = 0;         // dynamic shared memory per CTA
  int grid = 0;            // persistent CTAs
  int64_t scratch_bytes = 0;  // global pixel buffers when they do not fit in shared memory
};
RefInitPlan plan_reference_init(const StampDev* host_stamps, int32_t n);
cudaError_t launch_reference_init(const RefInitPlan& P, const StampDev* stamps, int32_t n, int32_t kind,
                                  int32_t known, const float* data, const uint8_t* mask, double* params,
                                  int32_t* status, void* scratch, cudaStream_t st);

// LM launches (ap_lm.cu)
cudaError_t launch_lm_init(const BatchArgs& b, const LMArgs& lm, const double* state0,
                           const uint8_t* mask, cudaStream_t s);
cudaError_t launch_lm_update(const BatchArgs& b, const LMArgs& lm, cudaStream_t s);
cudaError_t launch_lm_finish(const BatchArgs& b, const LMArgs& lm, cudaStream_t s);

// Tensor-core (tcgen05 + TMA) GEMMs of the learned initial guess (ap_tcgemm.cu).
// C[r][s] = sum_t A(r, t) W(s, t), bf16 operands, fp32 accumulation in tensor memory.
struct TcEpilogue {
  const float* bias = nullptr;     // added per output column when set
  __nv_bfloat16* act = nullptr;    // set: bf16 store of (bias, ReLU) into act, row stride ldc
  int relu = 0;
};
// dense: A[r * lda + t], W[s * ldw + t]; S a multiple of 16, T of 16, lda / ldw of 8
cudaError_t tc_gemm(const __nv_bfloat16* A, int lda, const __nv_bfloat16* W, int ldw, float* C, int ldc, int R, int S,
                    int T, const TcEpilogue& ep, cudaStream_t st);
// 3x3 stride-2 pad-1 convolution of an NHWC activation [B][H][H][cin] (cin 16, 32 or a multiple
// of 64) with W[S][9 * cin] (t = (ky * 3 + kx) * cin + c); rows r = (b * H/2 + oy) * H/2 + ox
cudaError_t tc_conv3x3s2(const __nv_bfloat16* act_in, int64_t B, int H, int cin, const __nv_bfloat16* W, int S,
                         float* C, int ldc, const TcEpilogue& ep, cudaStream_t st);
// first error code recorded by a tensor-core GEMM (0 none; 1-5 a wait that ran out), cleared on
// request; reading it synchronises the device
unsigned tc_error(bool clear);

// Dense damped solves (ap_scene.cu: FP64 Cholesky; ap_solve.cu: FP32 Cholesky + FP64 iterative
// refinement).  One workspace serves both: the FP64 region first, the mixed region after it.
inline size_t dense_fp64_ws_bytes(int32_t n) {
  // A (n x n), y and z (n each), the factored 32 x 32 diagonal block of the current step
  return sizeof(double) * ((size_t)n * n + 2 * (size_t)n + 32 * 32) + sizeof(int) * 4;
}
inline size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }
size_t dense_mixed_ws_bytes(int32_t n);

}  // namespace apgb
