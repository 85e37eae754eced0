"""Levenberg-Marquardt with the reference's interface (``astrophot/fit/lm.py``,
``astrophot/fit/base.py``), run entirely on the GPU by ``ap_lm_fit``.

``LM(model, initial_state=None, max_iter=100, relative_tolerance=1e-5, **kwargs).fit()``
keeps the reference's knobs (``max_step_iter``, ``curvature_limit``, ``Lup``, ``Ldn``, ``L0``,
``acceleration``), its outputs (``loss_history``, ``L_history``, ``lambda_history``,
``message``, ``res()``, ``covariance_matrix``, ``update_uncertainty()``) and its messages.
``BatchLM(models)`` fits many independent models (cutouts) in one device run.
``Iter_LM(model, chunks=50, method="random")`` runs LM on chunks of the parameter vector in
turn (``astrophot/fit/iterative.py:177-338``).
"""

from __future__ import annotations

from typing import List, Optional, Sequence

import numpy as np
import torch

from . import config
from .errors import OptimizeStop
from .models import _Structure, _make_scene, _needs_scene, _plan

__all__ = ("LM", "BatchLM", "Iter_LM")


def _setup(model, initial_state):
    struct = _Structure(model, list(model.models.values()) if hasattr(model, "models") else [model])
    if initial_state is None:
        model.initialize()
        initial_state = model.parameters.vector_representation()
    state = torch.as_tensor(initial_state, dtype=config.ap_dtype).flatten()
    window = model.window
    target = model.target[window]
    return struct, window, target, state


class _Fit:
    """Shared bookkeeping of one model inside a batched device run."""

    def __init__(self, model, initial_state):
        self.model = model
        self.struct, self.window, self.target, self.current_state = _setup(model, initial_state)
        self.order = self.struct.vector_order()  # model vector element -> full-vector slot
        self.message = ""
        self.loss_history = []
        self.L_history = []
        self.lambda_history = []


def _run(fits: List[_Fit], lm_kwargs):
    """One ``ap_lm_fit`` over all fits (they must share their structure and options)."""
    from . import _native as N

    first = fits[0]
    opts = first.struct.options()
    psfs = []
    for f in fits:
        g = f.struct.gal
        psfs.append(g.psf if (g is not None and g.psf_mode == "full") else None)
    batch = N.StampBatch([tuple(f.window.pixel_shape) for f in fits],
                         None if psfs[0] is None else [(p.data.shape[1], p.data.shape[0]) for p in psfs],
                         np.stack([f.window.geometry_row() for f in fits]), opts, config.ap_device)
    compact = [i for i in range(8) if opts.free_mask & (1 << i)]
    for f in fits:
        if sorted(f.order) != compact:
            raise ValueError("models of one batch must fit the same parameters")
    data = batch.pack([f.target.data.numpy() for f in fits])
    weight = batch.pack([f.target.weight.numpy() for f in fits])
    has_mask = any(f.target.has_mask for f in fits)
    mask = batch.pack([f.target.mask.numpy().astype(np.uint8) for f in fits], torch.uint8) if has_mask else None
    psf = None if psfs[0] is None else batch.pack_psf([p.data.numpy() for p in psfs])
    fixed = torch.tensor(np.stack([f.struct.full_params() for f in fits]))
    # model vector order -> compact (full-vector slot) order
    perms = [[f.order.index(sl) for sl in compact] for f in fits]
    state0 = torch.tensor(np.stack([f.current_state.numpy()[p] for f, p in zip(fits, perms)])) if compact else torch.zeros((len(fits), 0))
    lmo = N.make_lm_options(
        max_iter=lm_kwargs.get("max_iter", 100),
        max_step_iter=lm_kwargs.get("max_step_iter", 10),
        relative_tolerance=lm_kwargs.get("relative_tolerance", 1e-5),
        curvature_limit=lm_kwargs.get("curvature_limit", 1.0),
        Lup=lm_kwargs.get("Lup", 11.0),
        Ldn=lm_kwargs.get("Ldn", 9.0),
        L0=lm_kwargs.get("L0", 1.0),
        acceleration=lm_kwargs.get("acceleration", 0.0),
        rounds_per_sync=lm_kwargs.get("rounds_per_sync", 4),
        use_graph=lm_kwargs.get("use_graph", True),
    )
    state, chi2, iters, status = batch.lm_fit(data, weight, mask, psf, fixed, state0, lmo)
    loss, lam, xs = batch.lm_history()
    loss, lam, xs = loss.cpu().numpy(), lam.cpu().numpy(), xs.cpu().numpy()
    state, chi2, iters, status = state.cpu().numpy(), chi2.cpu().numpy(), iters.cpu().numpy(), status.cpu().numpy()
    for k, (f, p) in enumerate(zip(fits, perms)):
        n = min(int(iters[k]) + 1, loss.shape[1])  # the initial loss + one per accepted step
        inv = np.argsort(p)  # compact -> model order
        f.loss_history = [float(v) for v in loss[k, :n]]
        f.L_history = [float(v) for v in lam[k, :n]]
        f.lambda_history = [xs[k, i, : len(compact)][inv] for i in range(n)]
        f.current_state = torch.tensor(f.lambda_history[-1] if f.lambda_history else f.current_state.numpy())
        f.iterations = int(iters[k])
        f.status = int(status[k])
        f.message = N.LM_MESSAGES[int(status[k])]
        f.res_state = torch.tensor(state[k][inv])
        f.model.parameters.vector_set_representation(f.res_state)
    return batch


class LM:
    """``LM`` (fit/lm.py:15-539) on the CUDA path."""

    def __init__(self, model, initial_state: Sequence = None, max_iter: int = 100, relative_tolerance: float = 1e-5,
                 ndf=None, **kwargs):
        self.model = model
        self.verbose = kwargs.get("verbose", 0)
        self.max_iter = max_iter
        self.relative_tolerance = relative_tolerance
        self.kwargs = dict(kwargs, max_iter=max_iter, relative_tolerance=relative_tolerance)
        comps = list(model.models.values()) if hasattr(model, "models") else [model]
        self._scene = None
        if _needs_scene(model, comps):
            # several galaxies on one image: joint LM over the scene (fit/lm.py over a Group_Model)
            if initial_state is None:
                model.initialize()
                initial_state = model.parameters.vector_representation()
            self._scene = _make_scene(model, comps)
            self._scene_ndf = ndf
            self.current_state = torch.as_tensor(initial_state, dtype=config.ap_dtype).flatten()
            self.ndf = self._scene.ndf if ndf is None else ndf
            self.message = ""
            self.loss_history, self.L_history, self.lambda_history = [], [], []
            self._covariance_matrix = None
            tgt = model.target[model.window]
            self.W = tgt.flatten("weight")
            self.mask = None if not tgt.has_mask else torch.logical_not(tgt.flatten("mask"))
            return
        self._fit = _Fit(model, initial_state)
        self.current_state = self._fit.current_state
        tgt = self._fit.target
        if tgt.has_mask and not bool(torch.any(torch.logical_not(tgt.mask))):
            raise OptimizeStop("No data to fit. All pixels are masked")
        self.Y = tgt.flatten("data")
        self.W = tgt.flatten("weight")
        self.mask = None if not tgt.has_mask else torch.logical_not(tgt.flatten("mask"))
        n = len(self.Y) if self.mask is None else int(self.mask.sum())
        self.ndf = max(1.0, n - len(self.current_state)) if ndf is None else ndf
        self._covariance_matrix = None
        self.message = ""
        self.loss_history, self.L_history, self.lambda_history = [], [], []

    def fit(self):
        if len(self.current_state) == 0:
            return self
        self._covariance_matrix = None
        if self._scene is not None:
            from .scene import SceneLM

            kw = {k: self.kwargs[k] for k in ("max_step_iter", "curvature_limit", "Lup", "Ldn", "L0", "acceleration")
                  if k in self.kwargs}
            lm = SceneLM(self._scene, initial_state=self.current_state.numpy(), max_iter=self.max_iter,
                         relative_tolerance=self.relative_tolerance, ndf=self._scene_ndf, **kw).fit()
            self.loss_history, self.L_history = list(lm.loss_history), list(lm.L_history)
            self.lambda_history = [np.array(v) for v in lm.lambda_history]
            self.current_state = torch.tensor(lm.x)
            self.message = self.message + lm.message
            self.iterations = lm.iterations
            self.model.parameters.vector_set_representation(torch.tensor(lm.res()))
            return self
        _run([self._fit], self.kwargs)
        f = self._fit
        self.loss_history, self.L_history, self.lambda_history = f.loss_history, f.L_history, f.lambda_history
        self.current_state = f.current_state
        self.message = self.message + f.message
        self.iterations = f.iterations
        return self

    def res(self):
        """``BaseOptimizer.res`` (fit/base.py:113-124): the state of the lowest loss."""
        hist = np.array(self.loss_history)
        N = np.isfinite(hist)
        if len(hist) == 0 or not N.any():
            return self.current_state.numpy()
        return np.array(self.lambda_history)[N][np.argmin(hist[N])]

    def res_loss(self):
        hist = np.array(self.loss_history)
        return float(np.min(hist[np.isfinite(hist)]))

    def chi2min(self):
        return float(np.nanmin(self.loss_history))

    @property
    def covariance_matrix(self):
        """(J^T W J)^-1 in value space at the current parameters (fit/lm.py:497-519)."""
        if self._covariance_matrix is not None:
            return self._covariance_matrix
        J = self.model.jacobian(as_representation=False).flatten("data")
        W = self.W
        if self.mask is not None:
            J, W = J[self.mask], W[self.mask]
        hess = J.T @ (W[:, None] * J)
        try:
            cov = torch.linalg.inv(hess)
        except RuntimeError:
            hess = hess + torch.eye(len(hess), dtype=hess.dtype) * (torch.diag(hess) == 0)
            cov = torch.linalg.inv(hess)
        self._covariance_matrix = cov
        return cov

    def update_uncertainty(self):
        cov = self.covariance_matrix
        if torch.all(torch.isfinite(cov)):
            self.model.parameters.vector_set_uncertainty(torch.sqrt(torch.abs(torch.diag(cov))))
        else:
            config.ap_logger.warning("Unable to update uncertainty due to non finite covariance matrix")


class BatchLM:
    """Many independent models (each galaxy [+ flat sky] on its own target) fitted together:
    one ``ap_lm_fit`` device run, one LM per model with the reference's semantics."""

    def __init__(self, models, initial_states: Optional[Sequence] = None, **kwargs):
        self.models = list(models)
        states = initial_states if initial_states is not None else [None] * len(self.models)
        self.fits = [_Fit(m, s) for m, s in zip(self.models, states)]
        self.kwargs = kwargs

    def fit(self):
        # one device run per group of models that share their options (sampling, integration,
        # PSF mode and fitted parameters); most batches are one group
        groups = {}
        for f in self.fits:
            key = (bytes(f.struct.options()), f.struct.gal is not None and f.struct.gal.psf_mode == "full")
            groups.setdefault(key, []).append(f)
        for fits in groups.values():
            _run(fits, self.kwargs)
        return self

    @property
    def messages(self):
        return [f.message for f in self.fits]

    @property
    def loss_histories(self):
        return [f.loss_history for f in self.fits]

    def res(self):
        return [f.res_state.numpy() for f in self.fits]


class Iter_LM:
    """``Iter_LM`` (fit/iterative.py:177-338) on the CUDA path: sweeps of LMs on chunks of the
    model's parameter vector, the other entries held, each chunk's LM with the whole problem's
    degrees of freedom, until the sweep loss settles twice or ``max_iter`` sweeps.  ``chunks``:
    an int (chunks of that many entries, drawn by ``random.sample`` with ``method="random"`` or
    taken in order with ``"sequential"``) or a tuple of index tuples into the vector.  Runs over
    the model's scene (its galaxies with their windows and the locked sky); ``LM_kwargs`` go to
    each chunk's LM."""

    def __init__(self, model, initial_state: Sequence = None, chunks=50, max_iter: int = 100, method: str = "random",
                 LM_kwargs: Optional[dict] = None, relative_tolerance: float = 1e-3, **kwargs):
        if method not in ("random", "sequential"):
            raise ValueError(f"unrecognized Iter_LM method: {method}")
        if not isinstance(chunks, (int, tuple, list)):
            raise ValueError(f"Unrecognized chunks value, should be one of int, tuple. not: {type(chunks)}")
        self.model = model
        comps = list(model.models.values()) if hasattr(model, "models") else [model]
        if initial_state is None:
            model.initialize()
            initial_state = model.parameters.vector_representation()
        self.current_state = torch.as_tensor(initial_state, dtype=config.ap_dtype).flatten()
        self._scene = _make_scene(model, comps)
        self.chunks, self.method, self.max_iter = chunks, method, max_iter
        self.relative_tolerance = relative_tolerance
        self.LM_kwargs = dict(LM_kwargs or {})
        self.loss_history, self.lambda_history = [], []
        self.message = ""
        self.iteration = 0
        self.ndf = None

    def fit(self):
        from .scene import SceneIterLM

        it = SceneIterLM(self._scene, initial_state=self.current_state.numpy(), chunks=self.chunks,
                         max_iter=self.max_iter, method=self.method, relative_tolerance=self.relative_tolerance,
                         LM_kwargs=self.LM_kwargs).fit()
        self.ndf = it.ndf
        self.loss_history = list(it.loss_history)
        self.lambda_history = [np.array(v) for v in it.lambda_history]
        self.iteration = it.iteration
        self.message = self.message + it.message
        self.current_state = torch.tensor(it.x)
        self.model.parameters.vector_set_representation(torch.tensor(it.res()))
        return self

    def res(self):
        hist = np.array(self.loss_history)
        N = np.isfinite(hist)
        if len(hist) == 0 or not N.any():
            return self.current_state.numpy()
        return np.array(self.lambda_history)[N][np.argmin(hist[N])]

    def res_loss(self):
        hist = np.array(self.loss_history)
        return float(np.min(hist[np.isfinite(hist)]))

    def chi2min(self):
        return float(np.nanmin(self.loss_history))
