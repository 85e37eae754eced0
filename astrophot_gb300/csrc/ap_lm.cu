// Batched Levenberg-Marquardt: one thread per stamp runs the reference's damping search
// (LM.step, astrophot/fit/lm.py:249-357) and outer loop (LM.fit, :428-493) as a state
// machine.  Each device round renders, for every active stamp, the parameter vectors its
// state asks for (slot 0 / slot 1 of the render pass), then this kernel consumes the
// reduced chi^2, J^T W J, J^T W r and rpp sums and schedules the next round.
//
//   phase INIT : chi^2 at the initial state            -> loss_history[0]
//   phase JAC  : model, Jacobian, hess, grad at x       -> first damping trial
//   phase SUB  : slot 0 at x + 0.1 h (rpp), slot 1 at x + h + acceleration a (chi^2)
//                (acceleration != 0 needs a first, so slot 1 runs one round later: SUB2)
#include <cmath>

#include "ap_internal.h"

namespace apgb {

// representation -> value (utils/conversions/optimization.py:17-25,50-54); false when the
// value is not strictly inside the limits (Parameter_Node._set_val_self would raise).
__device__ __forceinline__ bool rep_to_value(int slot, double r, double& v) {
  switch (slot) {
    case PQ:
      v = (atan(r) + kPi / 2) * (1.0 - 0.0) / kPi + 0.0;
      return v > 0.0 && v < 1.0;
    case PN:
      v = (atan(r) + kPi / 2) * (8.0 - 0.36) / kPi + 0.36;
      return v > 0.36 && v < 8.0;
    case PRE:
      v = (r + 0.0 + sqrt((r - 0.0) * (r - 0.0) + 4)) * 0.5;
      return v > 0.0;
    case PPA: {
      v = 0.0 + (r - 0.0) - kPi * floor((r - 0.0) / kPi);
      v = 0.0 + (v - 0.0) - kPi * floor((v - 0.0) / kPi);
      return true;
    }
    default:
      v = r;
      return true;
  }
}

// value -> representation (utils/conversions/optimization.py:6-16,42-48): the inverse of
// rep_to_value for the fitted slots
__device__ __forceinline__ double value_to_rep(int slot, double v) {
  switch (slot) {
    case PQ:
      return tan((v - 0.0) * kPi / (1.0 - 0.0) - kPi / 2);
    case PN:
      return tan((v - 0.36) * kPi / (8.0 - 0.36) - kPi / 2);
    case PRE:
      return v - 1.0 / (v - 0.0);
    case PPA:
      return 0.0 + (v - 0.0) - kPi * floor((v - 0.0) / kPi);
    default:
      return v;
  }
}

__global__ void k_values_to_rep(const double* __restrict__ values, int32_t n, int32_t free_mask,
                                double* __restrict__ rep) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  int k = 0;
  const int nf = __popc(free_mask & 0xff);
  for (int i = 0; i < NPARAM; ++i)
    if (free_mask & (1 << i)) rep[(int64_t)s * nf + k++] = value_to_rep(i, values[(int64_t)s * NPARAM + i]);
}

cudaError_t launch_values_to_rep(const double* values, int32_t n, int32_t free_mask, double* rep, cudaStream_t st) {
  if (n > 0) k_values_to_rep<<<(n + 127) / 128, 128, 0, st>>>(values, n, free_mask, rep);
  return cudaGetLastError();
}

__device__ bool write_eval(const BatchArgs& b, const LMArgs& lm, int s, int slot, const double* x,
                           int32_t ops) {
  double* out = lm.params_next + ((int64_t)s * 2 + slot) * NPARAM;
  const double* fixed = lm.fixed + (int64_t)s * NPARAM;
  int k = 0;
  bool ok = true;
  for (int i = 0; i < NPARAM; ++i) {
    if (b.free_mask & (1 << i)) {
      double v;
      ok = rep_to_value(i, x[k++], v) && ok;
      out[i] = v;
    } else {
      out[i] = fixed[i];
    }
  }
  lm.ops_next[s * 2 + slot] = ops;
  return ok;
}

__device__ void finish(const BatchArgs& b, const LMArgs& lm, int s, LMState& S, int status) {
  S.phase = LM_PH_DONE;
  S.status = status;
  lm.ops_next[s * 2 + 0] = 0;
  lm.ops_next[s * 2 + 1] = 0;
}

// Trials rendered as differences to the step's base point (k_eval_setup drops OP_DIFF for the
// same stamps): their chi^2 is chi^2(x) + the accumulated change, and rpp uses the precise
// model difference, so the damping search compares chi^2 values that differ by far less
// than the FP32 rendering error of a single model.
__device__ __forceinline__ bool trials_as_diff(const BatchArgs& b, const LMArgs& lm, int s) {
  return lm.precise && diff_capable(b, b.stamps[s]);
}

// Relative error bounds of a chi^2 change accumulated from a difference render, and of a
// chi^2 accumulated from a full FP32 render.  A chain of trial differences drifts by the
// first times the sizes of its steps; the next Jacobian render of the base point (which
// accumulates chi^2 too) re-anchors the chain once that drift exceeds the second.
constexpr double kDiffRelErr = 2e-6;
constexpr double kFullRelErr = 2e-8;

__device__ void schedule_jac(const BatchArgs& b, const LMArgs& lm, int s, LMState& S) {
  S.phase = LM_PH_JAC;
  if (!write_eval(b, lm, s, 0, S.x,
                  OP_FWD | OP_JAC | OP_HG | OP_WRITE_MODEL | OP_WRITE_JAC | OP_REP |
                      (lm.precise ? OP_BASE : 0))) {
    finish(b, lm, s, S, AP_LM_LIMIT);
    return;
  }
  lm.ops_next[s * 2 + 1] = 0;
}

__device__ void start_sub(const BatchArgs& b, const LMArgs& lm, int s, LMState& S) {
  const int P = b.n_free;
  if (S.sub > lm.max_step_iter / 2.0 && S.L < 1e-3) S.L = 1.0;
  damped_solve_dev(P, S.H, S.g, S.L, S.h);
  for (int k = 0; k < P; ++k) lm.hvec[(int64_t)s * NPARAM + k] = S.h[k];
  double xa[NPARAM];
  for (int k = 0; k < P; ++k) xa[k] = S.x[k] + 0.1 * S.h[k];
  const int32_t dop = trials_as_diff(b, lm, s) ? OP_DIFF : 0;
  bool ok = write_eval(b, lm, s, 0, xa, OP_FWD | OP_RPP | dop);
  // The reference renders x + 0.1 h for the geodesic term but uses it only when L > 1e-4 (the
  // term is zero below, fit/lm.py:283-286) or with acceleration: skip that render there (the
  // value-space check of x + 0.1 h, which can end the fit, is kept).
  if (!(S.L > 1e-4) && lm.acceleration == 0.0) lm.ops_next[s * 2 + 0] = 0;
  if (lm.acceleration == 0.0) {
    double xb[NPARAM];
    for (int k = 0; k < P; ++k) xb[k] = S.x[k] + S.h[k];
    ok = write_eval(b, lm, s, 1, xb, OP_FWD | OP_CHI2 | dop) && ok;
  } else {
    lm.ops_next[s * 2 + 1] = 0;
  }
  S.phase = LM_PH_SUB;
  if (!ok) finish(b, lm, s, S, AP_LM_LIMIT);
}

__device__ void record(const LMArgs& lm, int s, LMState& S, double chi2) {
  const int n = lm.max_iter + 1;
  if (S.hist_len < n) {
    lm.hist_loss[(int64_t)s * n + S.hist_len] = chi2;
    lm.hist_L[(int64_t)s * n + S.hist_len] = S.L;
    for (int k = 0; k < NPARAM; ++k)
      lm.hist_x[((int64_t)s * n + S.hist_len) * NPARAM + k] = S.x[k];
    S.hist_len++;
  }
}

__device__ void end_step(const BatchArgs& b, const LMArgs& lm, int s, LMState& S) {
  const int P = b.n_free;
  const double* rha;
  double rchi2, rL;
  if (S.nostep) {
    if (!S.scarry_valid) {  // OptimizeStop (fit/lm.py:348-355)
      finish(b, lm, s, S, AP_LM_NO_STEP);
      return;
    }
    rha = S.scarry_ha;
    rchi2 = S.scarry_chi2;
    rL = S.scarry_L;
  } else {
    rha = S.best_ha;
    rchi2 = S.best_chi2;
    rL = S.best_L;
  }
  // LM.fit bookkeeping (fit/lm.py:461-482)
  S.L = rL;
  for (int k = 0; k < P; ++k) S.x[k] = S.x[k] + rha[k];
  S.chi2_cur = rchi2;
  if (trials_as_diff(b, lm, s)) S.anchor_err += kDiffRelErr * fabs(rchi2 - S.init_chi2);
  record(lm, s, S, rchi2);
  S.L = fmax(1e-9, S.L / lm.Ldn);
  S.iter++;
  const int n = lm.max_iter + 1;
  const double* hl = lm.hist_loss + (int64_t)s * n;
  const int len = S.hist_len;
  if (len >= 3 && (hl[len - 3] - hl[len - 1]) / hl[len - 1] < lm.rel_tol && S.L < 0.1) {
    finish(b, lm, s, S, AP_LM_SUCCESS);
    return;
  }
  if (len > 10 && (hl[len - 10] - hl[len - 1]) / hl[len - 1] < lm.rel_tol) {
    finish(b, lm, s, S, AP_LM_IMMOBILE);
    return;
  }
  if (S.iter >= lm.max_iter) {
    finish(b, lm, s, S, AP_LM_MAX_ITER);
    return;
  }
  schedule_jac(b, lm, s, S);
}

// tail of one damping-search iteration once chi^2 of the trial is known
__device__ void decide_step(const BatchArgs& b, const LMArgs& lm, int s, LMState& S, double chi2) {
  const int P = b.n_free;
  bool brk = false;
  if (!isfinite(chi2)) {
    S.L = fmin(1e9, S.L * lm.Lup);
    if (S.direction == 1)
      brk = true;
    else
      S.direction = 2;
  } else {
    if (chi2 <= S.scarry_chi2) {
      for (int k = 0; k < P; ++k) S.scarry_ha[k] = S.ha[k];
      S.scarry_chi2 = chi2;
      S.scarry_L = S.L;
      S.scarry_valid = 1;
    }
    double na = 0, nh = 0;
    for (int k = 0; k < P; ++k) {
      na += S.a[k] * S.a[k];
      nh += S.h[k] * S.h[k];
    }
    const double rho = sqrt(na) / sqrt(nh);
    if (rho > lm.curvature_limit) {
      S.L = fmin(1e9, S.L * lm.Lup);
      if (S.direction == 1)
        brk = true;
      else
        S.direction = 2;
    } else {
      if (chi2 < S.best_chi2) {
        for (int k = 0; k < P; ++k) S.best_ha[k] = S.ha[k];
        S.best_chi2 = chi2;
        S.best_L = S.L;
        S.nostep = 0;
        S.L = fmax(1e-9, S.L / lm.Ldn);
        if (S.L <= 1e-8 || S.direction == 2)
          brk = true;
        else
          S.direction = 1;
      } else if (chi2 > S.best_chi2 && (S.direction == 0 || S.direction == 2)) {
        S.L = fmin(1e9, S.L * lm.Lup);
        if (S.L == 1e9)
          brk = true;
        else
          S.direction = 2;
      } else {
        brk = true;
      }
      if (!brk && (S.best_chi2 - S.init_chi2) / S.init_chi2 < -0.1) brk = true;
    }
  }
  if (!brk) {
    S.sub++;
    if (S.sub < lm.max_step_iter) {
      start_sub(b, lm, s, S);
      return;
    }
  }
  end_step(b, lm, s, S);
}

// chi^2 / ndf of a trial from its accumulated sum (the change to the base point's when the
// trial was rendered as a difference)
__device__ __forceinline__ double trial_chi2(const BatchArgs& b, const LMArgs& lm, int s, const LMState& S,
                                             double acc) {
  return trials_as_diff(b, lm, s) ? S.init_chi2 + acc / S.ndf : acc / S.ndf;
}

__global__ void k_lm_count(BatchArgs b, const uint8_t* mask, LMArgs lm) {
  const int s = blockIdx.x;
  const StampDev& st = b.stamps[s];
  const int64_t n = (int64_t)st.nx * st.ny;
  int64_t c = 0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) c += (mask && mask[st.out_off + i]) ? 0 : 1;
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  __shared__ int64_t sh[8];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
    lm.st[s].ndf = fmax(1.0, (double)t - (double)b.n_free);
  }
}

__global__ void k_lm_init(BatchArgs b, LMArgs lm, const double* state0) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= b.n_stamps) return;
  LMState& S = lm.st[s];
  const int P = b.n_free;
  S.iter = 0;
  S.sub = 0;
  S.direction = 0;
  S.nostep = 1;
  S.scarry_valid = 0;
  S.hist_len = 0;
  S.anchor_err = 0.0;
  S.L = lm.L0;
  S.status = AP_LM_RUNNING;
  for (int k = 0; k < NPARAM; ++k) S.x[k] = (k < P) ? state0[(int64_t)s * P + k] : 0.0;
  if (P == 0) {
    finish(b, lm, s, S, AP_LM_SUCCESS);
    return;
  }
  S.phase = LM_PH_INIT;
  if (!write_eval(b, lm, s, 0, S.x, OP_FWD | OP_CHI2)) {
    finish(b, lm, s, S, AP_LM_LIMIT);
    return;
  }
  lm.ops_next[s * 2 + 1] = 0;
}

__global__ void k_lm_update(BatchArgs b, LMArgs lm) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= b.n_stamps) return;
  LMState& S = lm.st[s];
  const int P = b.n_free;
  const double* acc0 = b.acc + ((int64_t)s * 2 + 0) * kNacc;
  const double* acc1 = b.acc + ((int64_t)s * 2 + 1) * kNacc;
  switch (S.phase) {
    case LM_PH_DONE:
      return;
    case LM_PH_INIT: {
      const double chi2 = acc0[0] / S.ndf;
      S.chi2_cur = chi2;
      record(lm, s, S, chi2);
      if (lm.max_iter <= 0) {
        finish(b, lm, s, S, AP_LM_MAX_ITER);
        break;
      }
      schedule_jac(b, lm, s, S);
      break;
    }
    case LM_PH_JAC: {
      // hess = J^T W J, grad = -J^T r = J^T W (Y - Y0)   (fit/lm.py:388-399)
      for (int a = 0; a < P; ++a) S.g[a] = acc0[1 + a];
      int idx = 1 + P;
      for (int a = 0; a < P; ++a)
        for (int c = a; c < P; ++c) {
          S.H[a * P + c] = acc0[idx];
          S.H[c * P + a] = acc0[idx];
          ++idx;
        }
      if (trials_as_diff(b, lm, s) && S.anchor_err > kFullRelErr * S.chi2_cur) {
        // the chain of differences drifted more than a full render's rounding: take chi^2 of
        // this base point from its render (loss_history[-1] too; at this size of step no
        // convergence test is near its threshold)
        S.chi2_cur = acc0[0] / S.ndf;
        S.anchor_err = 0.0;
        const int n = lm.max_iter + 1;
        if (S.hist_len > 0) lm.hist_loss[(int64_t)s * n + S.hist_len - 1] = S.chi2_cur;
      }
      S.init_chi2 = S.chi2_cur;
      S.nostep = 1;
      S.best_chi2 = S.init_chi2;
      S.best_L = S.L;
      for (int k = 0; k < P; ++k) S.best_ha[k] = 0.0;
      S.scarry_valid = 0;
      S.scarry_chi2 = S.init_chi2;
      S.scarry_L = S.L;
      S.direction = 0;
      S.sub = 0;
      start_sub(b, lm, s, S);
      break;
    }
    case LM_PH_SUB: {
      // geodesic term (fit/lm.py:277-290)
      double rpp[NPARAM];
      for (int k = 0; k < P; ++k) rpp[k] = acc0[1 + k];
      if (S.L > 1e-4) {
        damped_solve_dev(P, S.H, rpp, S.L, S.a);
        for (int k = 0; k < P; ++k) S.a[k] = -S.a[k] / 2;
      } else {
        for (int k = 0; k < P; ++k) S.a[k] = 0.0;
      }
      for (int k = 0; k < P; ++k) S.ha[k] = S.h[k] + S.a[k] * lm.acceleration;
      if (lm.acceleration == 0.0) {
        decide_step(b, lm, s, S, trial_chi2(b, lm, s, S, acc1[0]));
      } else {
        double xb[NPARAM];
        for (int k = 0; k < P; ++k) xb[k] = S.x[k] + S.ha[k];
        lm.ops_next[s * 2 + 0] = 0;
        S.phase = LM_PH_SUB2;
        if (!write_eval(b, lm, s, 1, xb, OP_FWD | OP_CHI2 | (trials_as_diff(b, lm, s) ? OP_DIFF : 0)))
          finish(b, lm, s, S, AP_LM_LIMIT);
      }
      break;
    }
    case LM_PH_SUB2: {
      decide_step(b, lm, s, S, trial_chi2(b, lm, s, S, acc1[0]));
      break;
    }
    default:
      break;
  }
  if (S.phase != LM_PH_DONE) atomicAdd(lm.active_count, 1u);
}

__global__ void k_lm_finish(BatchArgs b, LMArgs lm) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= b.n_stamps) return;
  LMState& S = lm.st[s];
  const int P = b.n_free;
  const int n = lm.max_iter + 1;
  // BaseOptimizer.res (fit/base.py:113-124): state of the lowest finite loss
  int best = -1;
  double bl = 0;
  for (int i = 0; i < S.hist_len; ++i) {
    const double l = lm.hist_loss[(int64_t)s * n + i];
    if (isfinite(l) && (best < 0 || l < bl)) {
      best = i;
      bl = l;
    }
  }
  for (int k = 0; k < P; ++k)
    lm.state_out[(int64_t)s * P + k] =
        best >= 0 ? lm.hist_x[((int64_t)s * n + best) * NPARAM + k] : S.x[k];
  lm.chi2_out[s] = best >= 0 ? bl : NAN;
  lm.iters_out[s] = S.iter;
  lm.status_out[s] = (S.phase == LM_PH_DONE) ? S.status : AP_LM_RUNNING;
}

cudaError_t launch_lm_init(const BatchArgs& b, const LMArgs& lm, const double* state0,
                           const uint8_t* mask, cudaStream_t s) {
  k_lm_init<<<(b.n_stamps + 127) / 128, 128, 0, s>>>(b, lm, state0);
  k_lm_count<<<b.n_stamps, 256, 0, s>>>(b, mask, lm);
  return cudaGetLastError();
}

cudaError_t launch_lm_update(const BatchArgs& b, const LMArgs& lm, cudaStream_t s) {
  k_lm_update<<<(b.n_stamps + 127) / 128, 128, 0, s>>>(b, lm);
  return cudaGetLastError();
}

cudaError_t launch_lm_finish(const BatchArgs& b, const LMArgs& lm, cudaStream_t s) {
  k_lm_finish<<<(b.n_stamps + 127) / 128, 128, 0, s>>>(b, lm);
  return cudaGetLastError();
}

}  // namespace apgb
