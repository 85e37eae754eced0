"""float64 numpy restatement of AstroPhot's Levenberg-Marquardt fitter
(``astrophot/fit/lm.py``, ``astrophot/fit/base.py``).  TEST INFRASTRUCTURE
ONLY (see ``oracle/__init__``)."""

from __future__ import annotations

import copy
from dataclasses import dataclass
from typing import List, Optional

import numpy as np

from .render import (
    Component,
    PSF,
    Window,
    check_limits,
    drep_dvalue,
    rep_to_value,
    sample_group,
    value_to_rep,
)


class OptimizeStop(Exception):
    """``astrophot/errors/fit.py:6``."""


@dataclass
class GroupProblem:
    """Components rendered on one window against data ``Y`` with weights ``W`` (1/variance)
    and an optional boolean ``mask`` (True = ignored), as ``LM.__init__`` sets them up
    (fit/lm.py:191-222)."""

    components: List[Component]
    window: Window
    psf: Optional[PSF]
    Y: np.ndarray
    W: Optional[np.ndarray] = None
    mask: Optional[np.ndarray] = None
    # (component, name) -> (component, name) of the node it points at (see ``sample_group``)
    links: Optional[dict] = None

    def __post_init__(self):
        self.components = [copy.deepcopy(c) for c in self.components]
        self.links = dict(self.links or {})
        self.slots = [(ci, name, k) for ci, c in enumerate(self.components) for (name, k) in c.free_slots()
                      if (ci, name) not in self.links]

    # vector_values / vector_representation (param/parameter.py:169-214)
    def values(self):
        return np.array([np.atleast_1d(self.components[ci].params[name])[k] for ci, name, k in self.slots])

    def representation(self):
        return np.array(
            [value_to_rep(name, np.atleast_1d(self.components[ci].params[name])[k]) for ci, name, k in self.slots]
        )

    def set_representation(self, rep):
        """``vector_set_representation`` (param/parameter.py:323-328) with the limit checks of
        ``_set_val_self`` (:422-450)."""
        for (ci, name, k), r in zip(self.slots, rep):
            v = rep_to_value(name, r)
            check_limits(name, v)
            for cj in [ci] + [a for (a, n), t in self.links.items() if t == (ci, name)]:
                c = self.components[cj]
                if name == "center":
                    arr = np.array(c.params["center"], dtype=float).copy()
                    arr[k] = v
                    c.params["center"] = arr
                else:
                    c.params[name] = np.asarray(v, dtype=float)

    def forward(self, rep):
        self.set_representation(rep)
        model, _ = sample_group(self.components, self.window, self.psf, grad=False)
        return model.reshape(-1)

    def jacobian(self, rep):
        """Representation-space Jacobian ``[N, P]`` (models/_model_methods.py:260-347)."""
        self.set_representation(rep)
        _, J = sample_group(self.components, self.window, self.psf, grad=True, links=self.links)
        scale = np.array([drep_dvalue(name, r) for (ci, name, k), r in zip(self.slots, rep)])
        return J.reshape(-1, J.shape[-1]) * scale[None, :]


class LMOracle:
    """``LM`` (fit/lm.py:15-539) on a :class:`GroupProblem`."""

    def __init__(
        self,
        problem: GroupProblem,
        initial_state=None,
        max_iter: int = 100,
        relative_tolerance: float = 1e-5,
        ndf=None,
        **kwargs,
    ):
        self.problem = problem
        if initial_state is None:
            initial_state = problem.representation()
        self.current_state = np.array(initial_state, dtype=np.float64)
        self.max_iter = max_iter
        self.relative_tolerance = relative_tolerance
        self.max_step_iter = kwargs.get("max_step_iter", 10)
        self.curvature_limit = kwargs.get("curvature_limit", 1.0)
        self._Lup = kwargs.get("Lup", 11.0)
        self._Ldn = kwargs.get("Ldn", 9.0)
        self.L = kwargs.get("L0", 1.0)
        self.acceleration = kwargs.get("acceleration", 0.0)
        self.Y = problem.Y.reshape(-1).astype(np.float64)
        self.W = np.ones_like(self.Y) if problem.W is None else problem.W.reshape(-1).astype(np.float64)
        if problem.mask is not None and np.any(problem.mask):
            self.mask = np.logical_not(problem.mask.reshape(-1))
            if np.sum(self.mask) == 0:
                raise OptimizeStop("No data to fit. All pixels are masked")
        else:
            self.mask = None
        if ndf is None:
            n = len(self.Y) if self.mask is None else int(np.sum(self.mask))
            self.ndf = max(1.0, n - len(self.current_state))
        else:
            self.ndf = ndf
        self.lambda_history = []
        self.loss_history = []
        self.L_history = []
        self.message = ""
        self.iterations = 0
        self.n_forward = 0
        self.n_jacobian = 0

    def Lup(self):
        self.L = min(1e9, self.L * self._Lup)

    def Ldn(self):
        self.L = max(1e-9, self.L / self._Ldn)

    def forward(self, x):
        self.n_forward += 1
        return self.problem.forward(x)

    def _m(self, a):
        return a if self.mask is None else a[self.mask]

    def _r(self, Y, Ypred, W):  # lm.py:381-385
        return self._m(W) * (self._m(Y) - self._m(Ypred))

    def _chi2(self, Ypred):  # lm.py:374-378
        return float(np.sum(self._m(self.W * (self.Y - Ypred) ** 2)) / self.ndf)

    @staticmethod
    def damped(L, hess):
        """The matrix of ``_h`` (lm.py:361-371)."""
        P = hess.shape[0]
        I = np.eye(P)
        D = np.ones_like(hess) - I
        return hess * (I + D / (1 + L)) + L * I * (1 + np.diag(hess))

    @classmethod
    def _h(cls, L, grad, hess):
        return np.linalg.solve(cls.damped(L, hess), grad)

    def step(self, chi2):
        """``LM.step``, fit/lm.py:249-357."""
        x = self.current_state
        Y0 = self.forward(x)
        self.n_jacobian += 1
        J = self.problem.jacobian(x)
        Jm = self._m(J)
        Wm = self._m(self.W)
        r = self._r(Y0, self.Y, self.W)
        self.hess = Jm.T @ (Wm[:, None] * Jm)
        self.grad = -Jm.T @ r
        init_chi2 = chi2
        nostep = True
        best = (np.zeros_like(x), init_chi2, self.L)
        scarry_best = (None, init_chi2, self.L)
        direction = "none"
        d = 0.1
        for iteration in range(self.max_step_iter):
            if iteration > self.max_step_iter / 2 and self.L < 1e-3:
                self.L = 1.0
            h = self._h(self.L, self.grad, self.hess)
            Y1 = self.forward(x + d * h)
            rh = self._r(Y1, self.Y, self.W)
            rpp = Jm.T @ ((2 / d) * ((rh - r) / d - Wm * (Jm @ h)))
            if self.L > 1e-4:
                a = -self._h(self.L, rpp, self.hess) / 2
            else:
                a = np.zeros_like(h)
            ha = h + a * self.acceleration
            Y1 = self.forward(x + ha)
            chi2 = self._chi2(Y1)
            if not np.isfinite(chi2):
                self.Lup()
                if direction == "better":
                    break
                direction = "worse"
                continue
            if chi2 <= scarry_best[1]:
                scarry_best = (ha, chi2, self.L)
            rho = np.linalg.norm(a) / np.linalg.norm(h)
            if rho > self.curvature_limit:
                self.Lup()
                if direction == "better":
                    break
                direction = "worse"
                continue
            if chi2 < best[1]:
                best = (ha, chi2, self.L)
                nostep = False
                self.Ldn()
                if self.L <= 1e-8 or direction == "worse":
                    break
                direction = "better"
            elif chi2 > best[1] and direction in ["none", "worse"]:
                self.Lup()
                if self.L == 1e9:
                    break
                direction = "worse"
            else:
                break
            if (best[1] - init_chi2) / init_chi2 < -0.1:
                break
        if nostep:
            if scarry_best[0] is not None:
                return scarry_best
            raise OptimizeStop("Could not find step to improve chi^2")
        return best

    def fit(self):
        """``LM.fit``, fit/lm.py:428-493."""
        if len(self.current_state) == 0:
            return self
        self.loss_history = [self._chi2(self.forward(self.current_state))]
        self.L_history = [self.L]
        self.lambda_history = [self.current_state.copy()]
        for iteration in range(self.max_iter):
            self.iterations = iteration + 1
            try:
                res = self.step(chi2=self.loss_history[-1])
            except OptimizeStop:
                self.message = self.message + "fail. Could not find step to improve Chi^2"
                break
            self.L = res[2]
            self.current_state = self.current_state + res[0]
            self.L_history.append(self.L)
            self.loss_history.append(res[1])
            self.lambda_history.append(self.current_state.copy())
            self.Ldn()
            if len(self.loss_history) >= 3:
                if (self.loss_history[-3] - self.loss_history[-1]) / self.loss_history[
                    -1
                ] < self.relative_tolerance and self.L < 0.1:
                    self.message = self.message + "success"
                    break
            if len(self.loss_history) > 10:
                if (self.loss_history[-10] - self.loss_history[-1]) / self.loss_history[-1] < self.relative_tolerance:
                    self.message = self.message + "success by immobility. Convergence not guaranteed"
                    break
        else:
            self.message = self.message + "fail. Maximum iterations"
        self.problem.set_representation(self.res())
        return self

    def res(self):
        """``BaseOptimizer.res`` (fit/base.py:113-124)."""
        hist = np.array(self.loss_history)
        N = np.isfinite(hist)
        if np.sum(N) == 0:
            return self.current_state.copy()
        return np.array(self.lambda_history)[N][np.argmin(hist[N])]

    def res_loss(self):
        hist = np.array(self.loss_history)
        return float(np.min(hist[np.isfinite(hist)]))


class ChunkProblem:
    """A :class:`GroupProblem` restricted to the joint-vector entries ``idx``, the others held at
    their current values: what ``Param_Mask(parameters, chunk)`` shows the LM
    (param/param_context.py:62-90, fit/iterative.py:291-296)."""

    def __init__(self, problem: GroupProblem, idx):
        self.problem = problem
        self.idx = np.asarray(idx, dtype=np.int64)
        self.base = np.array(problem.representation(), dtype=np.float64)
        self.Y, self.W, self.mask = problem.Y, problem.W, problem.mask

    def full(self, sub):
        x = self.base.copy()
        x[self.idx] = sub
        return x

    def representation(self):
        return self.base[self.idx].copy()

    def set_representation(self, sub):
        self.problem.set_representation(self.full(sub))
        self.base = np.array(self.problem.representation(), dtype=np.float64)

    def forward(self, sub):
        return self.problem.forward(self.full(sub))

    def jacobian(self, sub):
        return self.problem.jacobian(self.full(sub))[:, self.idx]


class IterLMOracle:
    """``Iter_LM`` (fit/iterative.py:177-338): LM on chunks of the joint vector in turn, the
    rest held, until the loss of two successive sweeps settles (or ``max_iter`` sweeps).
    ``chunks`` an int: chunks of that many entries, in order (``method="sequential"``) or drawn
    with ``random.sample`` (``"random"``, Python's ``random`` module as the reference uses it);
    or a tuple of index lists.  Each chunk's LM uses the full problem's degrees of freedom."""

    def __init__(self, problem: GroupProblem, initial_state=None, chunks=50, max_iter=100, method="random",
                 relative_tolerance=1e-3, LM_kwargs=None):
        self.problem = problem
        if initial_state is not None:
            problem.set_representation(np.asarray(initial_state, dtype=np.float64))
        self.current_state = np.array(problem.representation(), dtype=np.float64)
        self.chunks, self.method, self.max_iter = chunks, method, max_iter
        self.relative_tolerance = relative_tolerance
        self.LM_kwargs = dict(LM_kwargs or {})
        n = problem.Y.size
        self.ndf = n - len(self.current_state)
        if problem.mask is not None:
            self.ndf -= int(np.sum(problem.mask))
        self.loss_history, self.lambda_history = [], []
        self.message = ""
        self.iteration = 0
        self._count_finish = 0

    def _chunk_list(self):
        P = len(self.current_state)
        if isinstance(self.chunks, int):
            import random

            ids = list(range(P))
            while ids:
                take = random.sample(ids, min(len(ids), self.chunks)) if self.method == "random" else ids[: self.chunks]
                for t in sorted(take):
                    ids.pop(ids.index(t))
                yield sorted(take)
        else:
            import random

            order = list(range(len(self.chunks)))
            while order:
                k = random.choice(order) if self.method == "random" else order[0]
                order.pop(order.index(k))
                yield sorted(self.chunks[k])

    def step(self):
        res = None
        for chunk in self._chunk_list():
            res = LMOracle(ChunkProblem(self.problem, chunk), ndf=self.ndf, **self.LM_kwargs).fit()
        self.loss_history.append(res.res_loss())
        self.lambda_history.append(np.array(self.problem.representation(), dtype=np.float64))
        if self.iteration >= 2 and (
            (-self.relative_tolerance * 1e-3)
            < ((self.loss_history[-2] - self.loss_history[-1]) / self.loss_history[-1])
            < (self.relative_tolerance / 10)
        ):
            self._count_finish += 1
        else:
            self._count_finish = 0
        self.iteration += 1

    def fit(self):
        while True:
            self.step()
            if self.iteration > 2 and self._count_finish >= 2:
                self.message = self.message + "success"
                break
            if self.iteration >= self.max_iter:
                self.message = self.message + f"fail max iterations reached: {self.iteration}"
                break
        self.problem.set_representation(self.res())
        return self

    def res(self):
        hist = np.array(self.loss_history)
        N = np.isfinite(hist)
        if not N.any():
            return self.current_state.copy()
        return np.array(self.lambda_history)[N][np.argmin(hist[N])]
