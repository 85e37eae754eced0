"""Scenes: many galaxies on one image, rendered and fitted jointly on the GPU.

``Group_Model.sample`` / ``jacobian`` (models/group_model_object.py:183-283) and ``LM``
(fit/lm.py) over the joint parameter vector when the sources share an image:

* every source is a stamp of an ``ap_batch``: its Jacobian on its own pixel window
  (``self.window & window``, models/_model_methods.py:293-298), its model image on the group's
  window and then cropped to its own window (inside a group ``model(window=group window)``
  makes the group window the working window, models/model_object.py:290-296, while only the
  model's own window is added, core_model.py:193-204);
* ``ap_scene_forward`` / ``ap_scene_hess`` / ``ap_scene_jt`` / ``ap_scene_jvp`` combine the
  stamps over the image; ``ap_dense_damped_solve`` solves the joint damped system;
* a source's centre may be linked to another source's centre (``value = node``,
  param/parameter.py:480-496): one entry of the joint vector, Jacobian columns summed.

``SceneLM`` is ``LM.fit`` / ``LM.step`` (fit/lm.py:249-357, 428-493) with these primitives:
the damping search, geodesic right-hand side, curvature test, convergence rules and
``res()`` of the reference, with all images, Jacobians and reductions on the device.

Every evaluation stages its parameters (all renders' value rows, a live PSF's row) in one
host-to-device copy; the forward and the Jacobian then read device memory only, so each is
captured as a CUDA graph at its second call and replayed (``graphs=False``: launched one by
one).  The LM's
geodesic-term solve reuses the Cholesky factor of its step solve (``ap_dense_factored_solve``).
Without a live PSF the LM keeps its vectors on the device: parameters are staged there from the
joint vector (``ap_scene_stage``), a damping trial reads back one packed status (factorisation
status, chi^2, the step and geodesic vectors) on which the host takes the reference's decisions,
and the next step's base image is the accepted trial's render.

A scene's PSF may be a live Moffat PSF model (``set_aux_psf``, models/model_object.py:133-149)
instead of a fixed image: :class:`LivePSF` samples it on its PSF image at every evaluation, its
free parameters lead the joint vector (the linked PSF node comes before the galaxy's own
parameters), and their Jacobian columns are image-wide: every source's pre-convolution image
convolved with the derivative of its shifted, renormalised kernel (``ap_render_psf_derivative``),
summed over the image like the model.
"""

from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import _native as N
from .transforms import SLOT_LIMITS, drep_dvalue, to_rep, to_value

__all__ = ("SceneSource", "Scene", "SceneLM", "LivePSF", "fit_scenes", "SceneRenderFunction", "render")

TILE = 32
_SLOTS_OF = {"sersic": (0, 1, 2, 3, 4, 5, 6), "exponential": (0, 1, 2, 3, 5, 6)}

# PSF model parameters per kind: limits (Moffat_PSF models/moffat_model.py:88-92, Gaussian_PSF
# models/gaussian_model.py:272-275) and their slots in the render
PSF_MODEL_LIMITS = {
    "moffat": {"n": ((0.1, 10.0), False), "Rd": ((0.0, None), False), "I0": ((None, None), False)},
    "gaussian": {"sigma": ((0.0, None), False), "flux": ((None, None), False)},
}
_PSF_SLOT = {"moffat": {"n": 4, "Rd": 5, "I0": 6}, "gaussian": {"sigma": 5, "flux": 6}}
_PSF_DEFAULT_FREE = {"moffat": ("n", "Rd"), "gaussian": ("sigma",)}
# PSF_Model class knobs (models/psf_model_object.py:50-80)
PSF_MODEL_KNOBS = dict(sampling_mode="simpsons", sampling_tolerance=1e-3, integrate_mode="threshold",
                       integrate_max_depth=3, integrate_gridding=5, integrate_quad_level=3, softening=1e-3)


class LivePSF:
    """A PSF model centred on its PSF image -- ``kind`` "moffat" (I0 / (1 + (R/Rd)^2)^n) or
    "gaussian" (10^flux / sqrt(2 pi sigma^2) exp(-R^2 / (2 sigma^2))) -- sampled on the device as
    ``PSF_Model.sample`` does (models/psf_model_object.py:180-264: sampling and threshold
    integration, then ``normalize_psf``), with the derivatives of the normalised image with
    respect to its ``free`` parameters (``ap_psf_normalize``)."""

    def __init__(self, params: dict, shape, scale: float = 1.0, free=None, knobs: Optional[dict] = None,
                 device="cuda", kind: str = "moffat"):
        if kind not in _PSF_SLOT:
            raise ValueError(f"unsupported PSF model kind {kind}")
        self.kind = kind
        self.limits = PSF_MODEL_LIMITS[kind]
        self.params = {k: float(params.get(k, 0.0)) for k in _PSF_SLOT[kind]}
        self.ky, self.kx = int(shape[0]), int(shape[1])
        self.scale = float(scale)
        self.free = tuple(_PSF_DEFAULT_FREE[kind] if free is None else free)
        if any(f not in _PSF_SLOT[kind] for f in self.free):
            raise ValueError(f"unknown {kind} PSF parameter in {self.free}")
        kn = dict(PSF_MODEL_KNOBS)
        kn.update(knobs or {})
        mask = sum(1 << _PSF_SLOT[kind][f] for f in self.free)
        o = N.make_options(profile=kind, psf_mode="none", free_mask=mask, has_sky=False, **kn)
        origin = (-self.kx * self.scale / 2, -self.ky * self.scale / 2)  # the image centred on (0, 0)
        self.device = torch.device(device)
        self.batch = N.StampBatch([(self.kx, self.ky)], None, N.scale_geometry(1, self.scale, origin), o, self.device)
        self.npix = self.kx * self.ky
        self.K = torch.empty(self.npix, dtype=torch.float32, device=self.device)
        self.dK = torch.empty((max(len(self.free), 1), self.npix), dtype=torch.float32, device=self.device)
        self.row_d = torch.zeros((1, 8), dtype=torch.float64, device=self.device)  # staged parameter row
        self.lib = N.lib()

    def _row(self):
        row = [0.0, 0.0, 1.0, math.pi / 2, 1.0, 1.0, 0.0, 0.0]  # q = 1, PA = pi/2: no inclination
        for k, v in self.params.items():
            row[_PSF_SLOT[self.kind][k]] = v
        return torch.tensor([row], dtype=torch.float64)

    def representation(self):
        return np.array([to_rep(*self.limits[f], self.params[f]) for f in self.free])

    def set_representation(self, rep):
        for f, r in zip(self.free, rep):
            self.params[f] = float(to_value(*self.limits[f], r))

    def drep(self, rep):
        """d value / d representation of the free parameters."""
        return np.array([float(drep_dvalue(*self.limits[f], r)) for f, r in zip(self.free, rep)])

    def stage(self):
        """Copy the current parameter row to the device (``render(staged=True)`` reads it)."""
        self.row_d.copy_(self._row())

    def render(self, grad: bool = False, staged: bool = False):
        """(K [ky * kx], dK [n_free][ky * kx] or None): the normalised PSF image and its
        value-space derivatives; ``staged`` reads the parameters :meth:`stage` copied (no
        host-to-device copy, so the call can be captured in a CUDA graph)."""
        m = len(self.free) if grad else 0
        row = self.row_d if staged else self._row()
        if m:
            model, jac = self.batch.jacobian(row, None, as_representation=False)
        else:
            model, jac = self.batch.render(row, None), None
        N.check(self.lib.ap_psf_normalize(self.npix, m, N._ptr(model), N._ptr(jac), N._ptr(self.K), N._ptr(self.dK),
                                          N._stream()), "ap_psf_normalize")
        return self.K, (self.dK[:m] if m else None)

    def image(self) -> np.ndarray:
        return self.render(False)[0].cpu().numpy().reshape(self.ky, self.kx).astype(np.float64)


class ApSceneSource(ctypes.Structure):
    _fields_ = [
        ("fwd_off", ctypes.c_int64),
        ("jac_off", ctypes.c_int64),
        ("jac_stride", ctypes.c_int64),
        ("x0", ctypes.c_int32),
        ("y0", ctypes.c_int32),
        ("wx", ctypes.c_int32),
        ("wy", ctypes.c_int32),
        ("n_free", ctypes.c_int32),
        ("gidx", ctypes.c_int32 * 8),
        ("fwd_x0", ctypes.c_int32),
        ("fwd_y0", ctypes.c_int32),
        ("fwd_nx", ctypes.c_int32),
    ]


@dataclass
class SceneSource:
    """One galaxy: ``kind`` "sersic" or "exponential", value-space ``params``
    [cx, cy, q, PA, n, Re, Ie] (n ignored for exponential), pixel ``window``
    ((x0, x1), (y0, y1)) or None for the whole image, ``link_center`` = index of the source
    whose centre node this one shares, ``locked`` = full-vector slots held fixed, ``options`` =
    this source's own sampling settings over the scene's (sampling_mode, integrate_mode, ...:
    each model of a reference group samples with its own, models/model_object.py:64-95)."""

    kind: str
    params: Sequence[float]
    window: Optional[tuple] = None
    link_center: Optional[int] = None
    locked: tuple = ()
    options: Optional[dict] = None


class Scene:
    """Sources on one ``nx`` x ``ny`` image (pixel scale ``scale``, the (0, 0) pixel corner at the
    origin) with a locked flat sky ``sky`` (counts per pixel) or, with ``sky_F`` given, a free
    flat sky of pixel_area * 10^F (``Flat_Sky``, models/flatsky_model.py:13-55) whose F sits in
    the joint vector after the free slots of the first ``sky_after`` sources (after all of them
    by default), one PSF (None: no convolution) or a live PSF
    model ``psf_model`` (:class:`LivePSF`, its free parameters first in the joint vector), data /
    weight (1 / variance) / mask (True = ignored).  ``graphs``: replay the forward and the
    Jacobian from CUDA graphs captured at their second call."""

    def __init__(self, nx: int, ny: int, sources: List[SceneSource], psf: Optional[np.ndarray], data, weight,
                 mask=None, sky: float = 0.0, scale: float = 1.0, options: Optional[dict] = None,
                 fwd_chunk: int = 64, device="cuda", origin=(0.0, 0.0), psf_model: Optional[LivePSF] = None,
                 graphs: bool = True, sky_F: Optional[float] = None, sky_after: Optional[int] = None,
                 psf_upscale: int = 1):
        self.nx, self.ny, self.scale = int(nx), int(ny), float(scale)
        # psf_upscale u: the PSF image has pixels u times finer than the image's; every source is
        # sampled, integrated and convolved on a u-times finer window and summed back in u x u
        # blocks (models/model_object.py:308-350)
        self.upscale = int(psf_upscale)
        if self.upscale < 1:
            raise ValueError("psf_upscale must be a positive integer")
        if self.upscale > 1 and (psf is None or psf_model is not None):
            raise NotImplementedError("psf_upscale needs a fixed PSF image (no live PSF model)")
        self.origin = (float(origin[0]), float(origin[1]))
        self.sources = list(sources)
        self.device = torch.device(device)
        self.sky_free = sky_F is not None
        self.sky_F = float(sky_F) if self.sky_free else None
        self.pixel_area = self.scale * self.scale
        self.sky = self.pixel_area * 10.0 ** self.sky_F if self.sky_free else float(sky)
        self.live_psf = psf_model
        if psf_model is not None:
            if psf is not None:
                raise ValueError("a scene takes a fixed PSF image or a live PSF model, not both")
            psf = psf_model.image()
        self.psf_np = None if psf is None else np.asarray(psf, dtype=np.float64)
        opts_kw = dict(options or {})
        dev = self.device
        self.data = torch.as_tensor(np.asarray(data, dtype=np.float32).reshape(-1), device=dev).contiguous()
        self.weight = torch.as_tensor(np.asarray(weight, dtype=np.float32).reshape(-1), device=dev).contiguous()
        self.mask = None
        if mask is not None and np.any(mask):
            self.mask = torch.as_tensor(np.asarray(mask, dtype=np.uint8).reshape(-1), device=dev).contiguous()
        n_used = self.nx * self.ny if self.mask is None else int((self.mask == 0).sum().item())

        # ---- joint vector: a live PSF's free parameters, then the sources in order and their
        # free slots in parameter order --------------------------------------------------------
        self.n_psf = 0 if psf_model is None else len(psf_model.free)
        # per joint index: (source, full-vector slot), (-1, PSF parameter name) for the live PSF,
        # (-2, "F") for a free sky
        self.slot_of = [(-1, f) for f in (psf_model.free if psf_model is not None else ())]
        self.gidx = []     # per source: {slot: joint index}
        self.sky_g = None
        n_src = len(self.sources)
        sky_pos = n_src if sky_after is None else int(sky_after)
        if self.sky_free and not 0 <= sky_pos <= n_src:
            raise ValueError("sky_after must lie between 0 and the number of sources")
        for si, src in enumerate(self.sources):
            if self.sky_free and si == sky_pos:
                self.sky_g = len(self.slot_of)
                self.slot_of.append((-2, "F"))
            if src.kind not in _SLOTS_OF:
                raise ValueError(f"unsupported source kind {src.kind}")
            g = {}
            for sl in _SLOTS_OF[src.kind]:
                if sl in src.locked:
                    continue
                if sl in (0, 1) and src.link_center is not None:
                    lead = src.link_center
                    if lead >= si or sl not in self.gidx[lead]:
                        raise ValueError("a linked centre must point at an earlier source's free centre")
                    g[sl] = self.gidx[lead][sl]
                    continue
                g[sl] = len(self.slot_of)
                self.slot_of.append((si, sl))
            self.gidx.append(g)
        if self.sky_free and self.sky_g is None:
            self.sky_g = len(self.slot_of)
            self.slot_of.append((-2, "F"))
        self.P = len(self.slot_of)
        # image-wide Jacobian columns: a live PSF's free parameters, then a free sky's F
        self.n_img = self.n_psf + (1 if self.sky_free else 0)
        self.ndf = max(1.0, n_used - self.P)

        # ---- stamp batches, one per (kind, fitted slots, sampling settings) --------------------
        self.groups = {}
        for si, src in enumerate(self.sources):
            free = tuple(sl for sl in _SLOTS_OF[src.kind] if sl not in src.locked)
            own = tuple(sorted((src.options or {}).items()))
            if any(k == "psf_mode" for k, _ in own):
                raise ValueError("a scene's sources share its PSF: psf_mode is not a per-source option")
            self.groups.setdefault((src.kind, free, own), []).append(si)
        kpsf = None if psf is None else (self.psf_np.shape[1], self.psf_np.shape[0])
        self._jac_parts = []
        jac_total = 0
        for (kind, free, own), members in self.groups.items():
            mask_bits = sum(1 << sl for sl in free)
            o = N.make_options(profile=kind, psf_mode="full" if psf is not None else "none", free_mask=mask_bits,
                               has_sky=False, **{**opts_kw, **dict(own)})
            shapes, geoms = self._fine_windows(members)
            jb = N.StampBatch(shapes, None if kpsf is None else [kpsf] * len(members), np.array(geoms), o, dev)
            jpsf = None if psf is None else jb.pack_psf([self.psf_np] * len(members))
            nf = len(free)
            part = dict(kind=kind, free=free, members=members, batch=jb, psf=jpsf, off=jac_total, nf=nf,
                        **self._coarse_layout(jb, members, nf))
            self._jac_parts.append(part)
            jac_total += nf * part["cpix"]
        # image-wide columns: one [ny * nx] plane per free PSF parameter, then a free sky's
        self.psf_jac_off = jac_total
        jac_total += self.n_img * self.nx * self.ny
        self.jac = torch.zeros(max(jac_total, 1), dtype=torch.float32, device=dev)

        # model renders.  The reference evaluates a windowed source of a group on the group's
        # window and keeps its own window.  Each source is rendered on its own window with the
        # group's working pixel count in its integration threshold, which gives the same pixels;
        # an exponential source's threshold also sums its samples over the whole group working
        # window, which a separate sampling pass of the render takes (set_threshold_window).
        self._fwd_parts = []
        self.fwd_chunk = max(1, int(fwd_chunk))
        bx = by = 0
        if psf is not None:
            ky_, kx_ = self.psf_np.shape
            bx, by = int(math.ceil((1 + kx_) / 2)), int(math.ceil((1 + ky_) / 2))
        u = self.upscale
        group_numel = float((u * self.nx + 2 * bx) * (u * self.ny + 2 * by))
        fwd_total = 0
        for (kind, free, own), members in self.groups.items():
            fo = N.make_options(profile=kind, psf_mode="full" if psf is not None else "none",
                                free_mask=sum(1 << sl for sl in _SLOTS_OF[kind]), has_sky=False,
                                **{**opts_kw, **dict(own)})
            if kind in ("sersic", "exponential"):
                shapes, geoms = self._fine_windows(members)
                # the group's working window in each source's working-pixel indices
                gwin = []
                for si in members:
                    (x0, x1), (y0, y1) = self._window(si)
                    gwin.append((-u * x0, -u * y0, u * self.nx + 2 * bx, u * self.ny + 2 * by))
                fb = N.StampBatch(shapes, None if kpsf is None else [kpsf] * len(members), np.array(geoms), fo, dev)
                fb.set_threshold_numel(group_numel)
                if kind == "exponential":
                    fb.set_threshold_window(np.array(gwin))
                fpsf = None if psf is None else fb.pack_psf([self.psf_np] * len(members))
                part = dict(kind=kind, members=members, batch=fb, psf=fpsf, off=fwd_total, m=len(members), own=True,
                            **self._coarse_layout(fb, members, 1))
                self._fwd_parts.append(part)
                fwd_total += part["cpix"]
            else:
                m = min(self.fwd_chunk, len(members))
                fb = N.StampBatch([(self.nx, self.ny)] * m, None if kpsf is None else [kpsf] * m,
                                  N.scale_geometry(m, self.scale, self.origin), fo, dev)
                fpsf = None if psf is None else fb.pack_psf([self.psf_np] * m)
                self._fwd_parts.append(dict(kind=kind, members=members, batch=fb, psf=fpsf, off=fwd_total, m=m,
                                            own=False))
                fwd_total += len(members) * self.nx * self.ny
        self.fwd = torch.zeros(max(fwd_total, 1), dtype=torch.float32, device=dev)
        self.fwd_d = torch.zeros_like(self.fwd) if psf_model is not None else None

        # staged parameters: every render's value rows, the live PSF's row and its column scales
        # in one float64 buffer (one host-to-device copy per evaluation, by _stage); the render
        # bodies read only device memory, so each is captured once and replayed as a CUDA graph
        rows = 0
        for part in self._jac_parts:
            part["srow"] = (rows, len(part["members"]))
            rows += len(part["members"])
        for part in self._fwd_parts:
            n_chunks = 1 if part["own"] else (len(part["members"]) + part["m"] - 1) // part["m"]
            part["srow"] = [(rows + c * part["m"], len(part["members"]) if part["own"] else part["m"])
                            for c in range(n_chunks)]
            rows += n_chunks * (len(part["members"]) if part["own"] else part["m"])
        self._psf_row = rows
        rows += 1
        # then the PSF columns' d value / d rep, and the sky row (cell 0: a free sky's F)
        self._scale_row, self._sky_row = rows, rows + 1
        self._stage_h = np.zeros((rows + 2, 8))
        self._stage_d = torch.zeros((rows + 2, 8), dtype=torch.float64, device=dev)
        self._sky_F_d = self._stage_d[self._sky_row, 0:1]
        for part in self._jac_parts:
            r0, n = part["srow"]
            part["dpar"] = self._stage_d[r0 : r0 + n]
        for part in self._fwd_parts:
            part["dpar"] = [self._stage_d[r0 : r0 + n] for r0, n in part["srow"]]
        if psf_model is not None:
            psf_model.row_d = self._stage_d[self._psf_row : self._psf_row + 1]
        self._img = torch.empty(self.nx * self.ny, dtype=torch.float32, device=dev)
        self._dimg = torch.empty_like(self._img)   # difference renders
        self._bases = None                          # their base points, allocated at first use
        self._sky_F0_d = torch.zeros(1, dtype=torch.float64, device=dev)
        self.use_graphs = bool(graphs)
        self._graphs, self._graph_failed, self._graph_calls = {}, set(), {}

        # ---- source descriptors (+ one whole-image entry carrying the image-wide columns) ------
        ns = len(self.sources)
        desc = (ApSceneSource * (ns + (1 if self.n_img else 0)))()
        if self.n_img:
            d = desc[ns]
            d.jac_off, d.jac_stride = self.psf_jac_off, self.nx * self.ny
            d.x0, d.y0, d.wx, d.wy = 0, 0, self.nx, self.ny
            d.n_free = self.n_img
            for c in range(self.n_psf):
                d.gidx[c] = c
            if self.sky_free:
                d.gidx[self.n_psf] = self.sky_g
        for part in self._fwd_parts:
            for k, si in enumerate(part["members"]):
                d = desc[si]
                if part["own"]:
                    (x0, x1), (y0, y1) = self._window(si)
                    d.fwd_off = part["off"] + int(part["coff"][k])
                    d.fwd_x0, d.fwd_y0, d.fwd_nx = x0, y0, x1 - x0
                else:
                    d.fwd_off = part["off"] + k * self.nx * self.ny
                    d.fwd_x0, d.fwd_y0, d.fwd_nx = 0, 0, self.nx
        for part in self._jac_parts:
            b = part["batch"]
            for k, si in enumerate(part["members"]):
                d = desc[si]
                (x0, x1), (y0, y1) = self._window(si)
                d.jac_off = part["off"] + int(part["coff"][k])
                d.jac_stride = int(part["cpix"])
                d.x0, d.y0, d.wx, d.wy = x0, y0, x1 - x0, y1 - y0
                d.n_free = part["nf"]
                for c, sl in enumerate(part["free"]):
                    d.gidx[c] = self.gidx[si][sl]
        raw = bytes(desc)
        self.desc = torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(dev)

        # ---- tile lists and overlapping pairs (windows are fixed for the scene) -------------
        ntx, nty = (self.nx + TILE - 1) // TILE, (self.ny + TILE - 1) // TILE
        lists = [[] for _ in range(ntx * nty)]
        for si in range(len(self.sources)):
            (x0, x1), (y0, y1) = self._window(si)
            for ty in range(y0 // TILE, (y1 - 1) // TILE + 1):
                for tx in range(x0 // TILE, (x1 - 1) // TILE + 1):
                    lists[ty * ntx + tx].append(si)
        ptr = np.zeros(len(lists) + 1, dtype=np.int32)
        ptr[1:] = np.cumsum([len(l) for l in lists])
        flat = np.array([s for l in lists for s in l] or [0], dtype=np.int32)
        self.tile_ptr = torch.tensor(ptr, device=dev)
        self.tile_src = torch.tensor(flat, device=dev)
        # J h also sums the image-wide columns: the whole-image entry in every tile
        self.jtile_ptr, self.jtile_src = self.tile_ptr, self.tile_src
        if self.n_img:
            jl = [l + [ns] for l in lists]
            jptr = np.zeros(len(jl) + 1, dtype=np.int32)
            jptr[1:] = np.cumsum([len(l) for l in jl])
            self.jtile_ptr = torch.tensor(jptr, device=dev)
            self.jtile_src = torch.tensor(np.array([x for l in jl for x in l], dtype=np.int32), device=dev)
        pairs = []
        wins = [self._window(si) for si in range(len(self.sources))]
        for a in range(len(self.sources)):
            (ax0, ax1), (ay0, ay1) = wins[a]
            for b in range(a, len(self.sources)):
                (bx0, bx1), (by0, by1) = wins[b]
                if max(ax0, bx0) < min(ax1, bx1) and max(ay0, by0) < min(ay1, by1):
                    pairs.append((a, b))
        if self.n_img:
            pairs += [(a, ns) for a in range(ns)] + [(ns, ns)]
        self.n_pairs = len(pairs)
        self.pairs = torch.tensor(np.array(pairs, dtype=np.int32).reshape(-1, 2), device=dev).contiguous()

        # fixed-order sums of J^T W J and J^T v: every block (a pair, a source) writes its own
        # partial sums and each entry adds its blocks' in one order (linked centres make several
        # blocks meet in one entry, where atomic adds would depend on the order blocks run in)
        n_desc = ns + (1 if self.n_img else 0)
        nf = np.array([desc[i].n_free for i in range(n_desc)], dtype=np.int64)
        gid = np.array([[desc[i].gidx[c] for c in range(8)] for i in range(n_desc)], dtype=np.int64)
        self._jt_table = self._gather_table(*jt_contributions(nf, gid))
        self._jt_part = torch.empty(max(n_desc, 1) * 8, dtype=torch.float64, device=dev)
        self._hess_table = self._gather_table(*hess_contributions(nf, gid, pairs, self.P))
        self._hess_part = torch.empty(max(self.n_pairs, 1) * 64, dtype=torch.float64, device=dev)

        self.lib = N.lib()
        self._solve_ws = torch.empty(int(self.lib.ap_dense_solve_workspace_bytes(self.P)), dtype=torch.uint8,
                                     device=dev)
        self._info = torch.zeros(1, dtype=torch.int32, device=dev)
        self._info2 = torch.zeros(1, dtype=torch.int32, device=dev)
        self._last_mixed = False
        self._d64 = torch.zeros(1, dtype=torch.float64, device=dev)
        self._chi2_parts = torch.zeros(1024, dtype=torch.float64, device=dev)

    # ---- geometry and parameters -----------------------------------------------------------
    def _window(self, si):
        w = self.sources[si].window
        if w is None:
            return (0, self.nx), (0, self.ny)
        (x0, x1), (y0, y1) = w
        x0, y0 = max(0, int(x0)), max(0, int(y0))
        x1, y1 = min(self.nx, int(x1)), min(self.ny, int(y1))
        if x1 <= x0 or y1 <= y0:
            raise ValueError(f"source {si} window lies outside the image")
        return (x0, x1), (y0, y1)

    def _fine_windows(self, members):
        """Render shapes and geometry rows of the sources ``members``: their own windows, on
        the u-times finer grid of the PSF (the same corner, pixel scale / u)."""
        u = self.upscale
        shapes, geoms = [], []
        for si in members:
            (x0, x1), (y0, y1) = self._window(si)
            shapes.append((u * (x1 - x0), u * (y1 - y0)))
            geoms.append(N.scale_geometry(1, self.scale / u, (self.origin[0] + x0 * self.scale,
                                                              self.origin[1] + y0 * self.scale))[0])
        return shapes, geoms

    def _coarse_layout(self, batch, members, n_planes):
        """The image-pixel layout of a batch's renders: per member its window's offset ``coff``,
        the total ``cpix``; with psf_upscale, a fine scratch of ``n_planes`` planes for the
        batch's output and the tables of the block sums into the coarse layout."""
        if self.upscale == 1:
            return dict(coff=np.asarray(batch.out_offsets, dtype=np.int64), cpix=int(batch.out_pixels), fine=None)
        sizes = []
        cnx = []
        for si in members:
            (x0, x1), (y0, y1) = self._window(si)
            sizes.append((x1 - x0) * (y1 - y0))
            cnx.append(x1 - x0)
        coff = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
        dev = self.device
        return dict(coff=coff, cpix=int(np.sum(sizes)),
                    fine=torch.zeros(n_planes * int(batch.out_pixels), dtype=torch.float32, device=dev),
                    foff_d=torch.tensor(np.asarray(batch.out_offsets, dtype=np.int64), device=dev),
                    coff_d=torch.tensor(coff, device=dev),
                    cnx_d=torch.tensor(np.asarray(cnx, dtype=np.int32), device=dev))

    def _reduce(self, part, fine, out, n_planes):
        """out (coarse layout, planes cpix apart) = u x u block sums of ``fine`` (the batch's
        layout, planes out_pixels apart)."""
        N.check(self.lib.ap_reduce_upscaled(len(part["members"]), N._ptr(part["foff_d"]), N._ptr(part["coff_d"]),
                                            N._ptr(part["cnx_d"]), self.upscale, n_planes, N._ptr(fine),
                                            int(part["batch"].out_pixels), N._ptr(out), int(part["cpix"]),
                                            int(part["cpix"]), N._stream()), "ap_reduce_upscaled")

    def values_matrix(self, rep: np.ndarray) -> np.ndarray:
        """[n_sources, 8] value-space rows from a joint representation vector."""
        V = np.zeros((len(self.sources), 8))
        for si, src in enumerate(self.sources):
            p = np.asarray(src.params, dtype=np.float64)
            V[si, : len(p)] = p
            if src.kind == "exponential":
                V[si, 4] = 1.0
            for sl, g in self.gidx[si].items():
                V[si, sl] = to_value(*SLOT_LIMITS[sl], rep[g])
        return V

    def representation(self) -> np.ndarray:
        rep = np.zeros(self.P)
        for g, (si, sl) in enumerate(self.slot_of):
            if si < 0:
                continue
            rep[g] = to_rep(*SLOT_LIMITS[sl], self.sources[si].params[sl])
        if self.n_psf:
            rep[: self.n_psf] = self.live_psf.representation()
        if self.sky_free:
            rep[self.sky_g] = self.sky_F  # no limits: F is its own representation
        return rep

    def set_representation(self, rep):
        rep = np.asarray(rep, dtype=np.float64)
        V = self.values_matrix(rep)
        for si, src in enumerate(self.sources):
            src.params = list(V[si, :7])
        if self.n_psf:
            self.live_psf.set_representation(rep[: self.n_psf])
        if self.sky_free:
            self.sky_F = float(rep[self.sky_g])
            self.sky = self.pixel_area * 10.0 ** self.sky_F

    def _stage(self, rep, as_representation: bool = True):
        """Every render's parameter rows (and a live PSF's row and column scales) at ``rep`` into
        the device staging buffer, in one copy."""
        rep = np.asarray(rep, dtype=np.float64)
        V = self.values_matrix(rep)
        H = self._stage_h
        for part in self._jac_parts:
            r0, n = part["srow"]
            H[r0 : r0 + n] = V[part["members"]]
        for part in self._fwd_parts:
            mem, m = part["members"], part["m"]
            if part["own"]:
                r0, n = part["srow"][0]
                H[r0 : r0 + n] = V[mem]
                continue
            for (r0, n), c0 in zip(part["srow"], range(0, len(mem), m)):
                chunk = mem[c0 : c0 + m]
                H[r0 : r0 + n] = V[chunk[0]]
                H[r0 : r0 + len(chunk)] = V[chunk]
        if self.n_psf:
            live = self.live_psf
            live.set_representation(rep[: self.n_psf])
            H[self._psf_row] = live._row().numpy()[0]
            H[self._scale_row, : self.n_psf] = live.drep(rep[: self.n_psf]) if as_representation else 1.0
        if self.sky_free:
            H[self._sky_row, 0] = rep[self.sky_g]
        self._stage_d.copy_(torch.from_numpy(H))
        return V

    # ---- parameters staged from a device vector (the LM's vectors stay on the device) --------
    def _stage_rows(self) -> np.ndarray:
        """Source index of every staged row (-1: the live PSF's rows), as ``_stage`` fills them."""
        if getattr(self, "_row_src", None) is None:
            row_src = np.full(self._stage_h.shape[0], -1, dtype=np.int64)
            for part in self._jac_parts:
                r0, n = part["srow"]
                row_src[r0 : r0 + n] = part["members"]
            for part in self._fwd_parts:
                mem, m = part["members"], part["m"]
                if part["own"]:
                    r0, n = part["srow"][0]
                    row_src[r0 : r0 + n] = mem
                    continue
                for (r0, n), c0 in zip(part["srow"], range(0, len(mem), m)):
                    chunk = mem[c0 : c0 + m]
                    row_src[r0 : r0 + n] = chunk[0]
                    row_src[r0 : r0 + len(chunk)] = chunk
            g = np.full(self._stage_h.shape, -1, dtype=np.int32)
            for r, si in enumerate(row_src):
                if si >= 0:
                    for sl, gi in self.gidx[si].items():
                        g[r, sl] = gi
            if self.sky_free:
                g[self._sky_row, 0] = self.sky_g  # slot 0's map is the identity, as F's
            self._row_src = row_src
            self._stage_gidx = torch.tensor(g.reshape(-1), device=self.device)
            self._stage_base = torch.zeros(g.size, dtype=torch.float64, device=self.device)
        return self._row_src

    @property
    def device_staging(self) -> bool:
        """Whether renders can take their parameters from a device vector (no live PSF)."""
        return self.n_psf == 0

    def set_stage_base(self, rep):
        """The constant cells of device staging (locked slots, an exponential's n) from the
        sources' current values; the free cells are computed from the vector at every call."""
        row_src = self._stage_rows()
        V = self.values_matrix(np.asarray(rep, dtype=np.float64))
        base = np.zeros(self._stage_h.shape)
        used = row_src >= 0
        base[used] = V[row_src[used]]
        self._stage_base.copy_(torch.from_numpy(base.reshape(-1)))

    def _stage_dev(self, x: torch.Tensor, v: Optional[torch.Tensor] = None, alpha: float = 0.0):
        """Every render's parameter rows at the device joint vector x + alpha v (float64)."""
        if not self.device_staging:
            raise NotImplementedError("device staging of a scene with a live PSF model")
        self._stage_rows()
        N.check(self.lib.ap_scene_stage(self._stage_d.numel(), N._ptr(self._stage_gidx), N._ptr(self._stage_base),
                                        N._ptr(x), N._ptr(v) if v is not None else None, float(alpha),
                                        N._ptr(self._stage_d), N._stream()), "ap_scene_stage")

    def forward_device(self, x: torch.Tensor, v: Optional[torch.Tensor] = None, alpha: float = 0.0) -> torch.Tensor:
        """Model image [ny * nx] at the device joint vector x + alpha v (``set_stage_base`` first).
        Returns the scene's image buffer, which the next render overwrites."""
        self._stage_dev(x, v, alpha)
        self._run("forward", self._forward_body)
        return self._img

    def jacobian_device(self, x: torch.Tensor) -> torch.Tensor:
        """:meth:`jacobian` (representation space) at the device joint vector x."""
        self._stage_dev(x)
        self._run(("jacobian", True), lambda: self._jacobian_body(True))
        return self.jac

    def chi2_into(self, model: torch.Tensor, out: torch.Tensor):
        """chi^2 of ``model`` into the device float64 ``out[0]`` (no host read)."""
        N.check(self.lib.ap_scene_chi2(N._ptr(model), N._ptr(self.data), N._ptr(self.weight), N._ptr(self.mask),
                                       self.nx * self.ny, N._ptr(out), N._ptr(self._chi2_parts),
                                       self._chi2_parts.numel(), N._stream()), "ap_scene_chi2")

    def solve_device(self, H: torch.Tensor, g: torch.Tensor, L: float, info: torch.Tensor, mixed: bool = True,
                     reuse: bool = False) -> torch.Tensor:
        """:meth:`solve` without a host read: the status goes to the device int ``info`` (0
        solved; > 0 the damped matrix is not positive definite; -1 the mixed-precision solve did
        not converge) and h is zero unless solved, so that nothing downstream renders a failed
        step.  ``reuse``: another right-hand side on the factor of the previous call of the same
        precision."""
        n = int(H.shape[0])
        h = torch.empty(n, dtype=torch.float64, device=self.device)
        self._solve_call(H, g, L, h, info, mixed, reuse)
        return torch.where(info == 0, h, torch.zeros_like(h))

    def _psf_body(self, grad: bool):
        """Sample the live PSF from the staged row and copy it into every batch's packed PSF;
        returns its value-space derivatives when ``grad``."""
        K, dK = self.live_psf.render(grad, staged=True)
        for part in self._jac_parts + self._fwd_parts:
            if part["psf"] is not None:
                part["psf"].view(-1, K.numel()).copy_(K.expand(part["psf"].numel() // K.numel(), -1))
        return dK

    def _run(self, key, body):
        """``body()`` (device work only, reading staged parameters): eager at its first call,
        captured as a CUDA graph at its second and replayed from then on when graphs are on;
        eager for good if the capture fails."""
        calls = self._graph_calls.get(key, 0) + 1
        self._graph_calls[key] = calls
        if not self.use_graphs or key in self._graph_failed or calls < 2:
            body()
            return
        g = self._graphs.get(key)
        if g is None:
            g = torch.cuda.CUDAGraph()
            try:
                with torch.cuda.graph(g, capture_error_mode="thread_local"):
                    body()
            except Exception:
                self._graph_failed.add(key)
                body()
                return
            self._graphs[key] = g
        g.replay()

    # ---- device primitives -----------------------------------------------------------------
    def _render_sources(self, buf, render, base_mode: int = 0):
        """Every source's model render into ``buf`` (the layout of ``self.fwd``) by
        ``render(batch, staged params, packed psf, out)``, or, with ``base_mode`` (RENDER_BASE /
        RENDER_DIFFERENCE), by the batch's precise render against the base buffer of that call."""
        bases = self._base_buffers() if base_mode else None

        def call(pi, c, b, p, k, out):
            if base_mode:
                b.render_precise(p, k, bases[pi][c], base_mode, out=out)
            else:
                render(b, p, k, out)

        for pi, part in enumerate(self._fwd_parts):
            b, m, mem = part["batch"], part["m"], part["members"]
            if part["own"]:
                dst = buf[part["off"] : part["off"] + part["cpix"]]
                if part["fine"] is None:
                    call(pi, 0, b, part["dpar"][0], part["psf"], dst)
                else:  # rendered on the PSF's finer grid, then summed back in blocks
                    call(pi, 0, b, part["dpar"][0], part["psf"], part["fine"])
                    self._reduce(part, part["fine"], dst, 1)
                continue
            for c, c0 in enumerate(range(0, len(mem), m)):
                out = buf[part["off"] + c0 * self.nx * self.ny : part["off"] + (c0 + m) * self.nx * self.ny]
                if out.numel() == m * self.nx * self.ny:
                    call(pi, c, b, part["dpar"][c], part["psf"], out)
                else:
                    tmp = torch.empty(b.out_pixels, dtype=torch.float32, device=self.device)
                    call(pi, c, b, part["dpar"][c], part["psf"], tmp)
                    out.copy_(tmp[: out.numel()])

    def _combine(self, buf, sky, img, with_sky: bool = True, difference: bool = False):
        """img = the sources' renders in ``buf`` + the sky: ``sky`` (counts per pixel) when locked,
        pixel_area * 10^F from the staged F when free (``with_sky`` False: no sky).  With
        ``difference``, ``buf`` holds differences to the base renders and the sky term is the free
        sky's change since the base (a locked sky's is zero)."""
        sky_F = self._sky_F_d if (self.sky_free and with_sky) else None
        sky_F0 = self._sky_F0_d if (difference and sky_F is not None) else None
        locked = 0.0 if (difference or not with_sky) else sky
        N.check(self.lib.ap_scene_forward(N._ptr(self.desc), N._ptr(self.tile_ptr), N._ptr(self.tile_src),
                                          N._ptr(buf), ctypes.c_float(locked), N._ptr(sky_F), N._ptr(sky_F0),
                                          ctypes.c_double(self.pixel_area), self.nx, self.ny, N._ptr(img),
                                          N._stream()), "ap_scene_forward")
        return img

    # ---- difference renders: the joint LM's damping trials near its optimum ---------------
    def _base_buffers(self):
        """One base-point buffer per render call of the forward (a part, or one chunk of it)."""
        if self._bases is None:
            self._bases = {}
            for pi, part in enumerate(self._fwd_parts):
                n = 1 if part["own"] else (len(part["members"]) + part["m"] - 1) // part["m"]
                self._bases[pi] = [part["batch"].base_buffer() for _ in range(n)]
        return self._bases

    @property
    def precise_capable(self) -> bool:
        """Whether trials can be rendered as differences (device staging: no live PSF; no
        Lanczos sub-pixel shift, which has no kernel-difference form)."""
        return self.device_staging and not any(p["batch"].options.lanczos_order > 0 for p in self._fwd_parts)

    def _forward_base_body(self):
        self._render_sources(self.fwd, None, base_mode=N.StampBatch.RENDER_BASE)
        self._combine(self.fwd, self.sky, self._img)
        if self.sky_free:
            self._sky_F0_d.copy_(self._sky_F_d)

    def _forward_diff_body(self):
        self._render_sources(self.fwd, None, base_mode=N.StampBatch.RENDER_DIFFERENCE)
        self._combine(self.fwd, self.sky, self._dimg, difference=True)

    def forward_base_device(self, x: torch.Tensor) -> torch.Tensor:
        """:meth:`forward_device` at x, recording x as the base point of difference renders."""
        self._stage_dev(x)
        self._run("forward_base", self._forward_base_body)
        return self._img

    def forward_diff_device(self, x: torch.Tensor, v: torch.Tensor, alpha: float) -> torch.Tensor:
        """model(x + alpha v) - model(base point), accurate relative to the change (float32
        image, overwritten by the next call)."""
        self._stage_dev(x, v, alpha)
        self._run("forward_diff", self._forward_diff_body)
        return self._dimg

    def chi2_change_into(self, dm: torch.Tensor, base: torch.Tensor, out: torch.Tensor):
        """chi^2(base + dm) - chi^2(base) into the device float64 ``out[0]``."""
        N.check(self.lib.ap_scene_chi2_change(N._ptr(dm), N._ptr(base), N._ptr(self.data), N._ptr(self.weight),
                                              N._ptr(self.mask), self.nx * self.ny, N._ptr(out),
                                              N._ptr(self._chi2_parts), self._chi2_parts.numel(), N._stream()),
                "ap_scene_chi2_change")

    def _forward_body(self):
        if self.n_psf:
            self._psf_body(False)
        self._render_sources(self.fwd, lambda b, p, k, out: b.render(p, k, out=out))
        self._combine(self.fwd, self.sky, self._img)

    def forward(self, rep: np.ndarray) -> torch.Tensor:
        """Model image [ny * nx] (float32) at the joint representation vector."""
        self._stage(rep)
        self._run("forward", self._forward_body)
        return self._img.clone()

    def _psf_column(self, dK, j, out):
        """Image-wide column ``j`` of a live PSF into ``out`` [ny * nx]: every source rendered
        with the derivative of its kernel along d psf / d theta_j (scaled by the staged
        d value / d representation), summed like the model."""
        D = dK[j] * self._stage_d[self._scale_row, j].to(torch.float32)
        self._render_sources(self.fwd_d, lambda b, p, k, o: b.render_psf_derivative(
            p, k, D.repeat(k.numel() // D.numel()), out=o))
        return self._combine(self.fwd_d, 0.0, out, with_sky=False)

    def _sky_column(self, out):
        """The free sky's image-wide column, d image / d F = ln(10) pixel_area 10^F everywhere
        (F is unbounded: the same in representation space), from the staged F."""
        c = (math.log(10.0) * self.pixel_area) * torch.pow(10.0, self._sky_F_d)
        out.copy_(c.to(torch.float32).expand(out.numel()))

    def _jacobian_body(self, as_representation: bool):
        dK = self._psf_body(True) if self.n_psf else None
        for part in self._jac_parts:
            b, nf = part["batch"], part["nf"]
            jac = self.jac[part["off"] : part["off"] + nf * part["cpix"]]
            if part["fine"] is None:
                b.jacobian(part["dpar"], part["psf"], as_representation=as_representation,
                           jac=jac.view(nf, b.out_pixels))
            else:  # on the PSF's finer grid, each plane summed back in blocks (the sum is linear)
                b.jacobian(part["dpar"], part["psf"], as_representation=as_representation,
                           jac=part["fine"].view(nf, b.out_pixels))
                self._reduce(part, part["fine"], jac, nf)
        npx = self.nx * self.ny
        for j in range(self.n_psf):
            self._psf_column(dK, j, self.jac[self.psf_jac_off + j * npx : self.psf_jac_off + (j + 1) * npx])
        if self.sky_free:
            j = self.n_psf
            self._sky_column(self.jac[self.psf_jac_off + j * npx : self.psf_jac_off + (j + 1) * npx])

    def jacobian(self, rep: np.ndarray, as_representation: bool = True):
        """Own-window Jacobians of every source (representation or value space) into ``self.jac``,
        and the image-wide columns of a live PSF's parameters."""
        as_representation = bool(as_representation)
        self._stage(rep, as_representation)
        self._run(("jacobian", as_representation), lambda: self._jacobian_body(as_representation))
        return self.jac

    def jacobian_image(self, rep: np.ndarray, as_representation: bool = True) -> np.ndarray:
        """Dense [ny, nx, P] Jacobian (linked columns summed)."""
        self.jacobian(rep, as_representation)
        out = np.zeros((self.ny, self.nx, self.P))
        jac = self.jac.cpu().numpy()
        for part in self._jac_parts:
            cp = part["cpix"]
            for k, si in enumerate(part["members"]):
                (x0, x1), (y0, y1) = self._window(si)
                o = int(part["coff"][k])
                for c, sl in enumerate(part["free"]):
                    col = jac[part["off"] + c * cp + o : part["off"] + c * cp + o + (x1 - x0) * (y1 - y0)]
                    out[y0:y1, x0:x1, self.gidx[si][sl]] += col.reshape(y1 - y0, x1 - x0)
        npx = self.nx * self.ny
        for j in range(self.n_img):
            g = j if j < self.n_psf else self.sky_g
            out[:, :, g] += jac[self.psf_jac_off + j * npx : self.psf_jac_off + (j + 1) * npx].reshape(self.ny, self.nx)
        return out

    def _vjp_index(self, part):
        """For an own-window forward batch: image index of every packed output pixel (with
        psf_upscale, of the image pixel whose block holds the fine pixel: the block sum passes
        the image's gradient to each of its pixels unchanged)."""
        if "vjp_idx" not in part:
            b, u = part["batch"], self.upscale
            idx = np.zeros(b.out_pixels, dtype=np.int64)
            for k, si in enumerate(part["members"]):
                (x0, x1), (y0, y1) = self._window(si)
                yy, xx = np.mgrid[u * y0 : u * y1, u * x0 : u * x1] // u
                o = int(b.out_offsets[k])
                idx[o : o + u * u * (x1 - x0) * (y1 - y0)] = (yy * self.nx + xx).ravel()
            part["vjp_idx"] = torch.tensor(idx, device=self.device)
        return part["vjp_idx"]

    def vjp(self, rep: np.ndarray, grad_image: torch.Tensor, as_representation: bool = True,
            reference_center: bool = False) -> torch.Tensor:
        """Adjoint of :meth:`forward`: [P] float64 = sum_pixels grad_image d image / d theta, by
        ``ap_render_vjp`` of every source's model render (PSF-convolved derivative tiles are
        recomputed and reduced on the fly, no Jacobian is stored).  ``reference_center`` gives
        the centre entries the reference's reverse-mode autograd gives under PSF shift."""
        g_img = grad_image.to(self.device, torch.float32).reshape(-1).contiguous()
        out = np.zeros(self.P)
        if self.n_psf:
            # a live PSF's entries: the upstream gradient against each image-wide PSF column
            # (the render's derivative along d psf / d theta); the sources below see the current PSF
            self._stage(rep, as_representation)
            dK = self._psf_body(True)
            col = torch.empty(self.nx * self.ny, dtype=torch.float32, device=self.device)
            for j in range(self.n_psf):
                self._psf_column(dK, j, col)
                out[j] = float(torch.dot(col.to(torch.float64), g_img.to(torch.float64)).item())
        V = self.values_matrix(rep)
        for part in self._fwd_parts:
            b, m, mem = part["batch"], part["m"], part["members"]
            slots = [sl for sl in range(8) if b.options.free_mask & (1 << sl)]
            if part["own"]:
                gp = g_img[self._vjp_index(part)].contiguous()
                res = b.vjp(torch.tensor(V[mem]), part["psf"], gp, as_representation=as_representation,
                            reference_center=reference_center).cpu().numpy()
                rows = list(zip(mem, res))
            else:
                rows = []
                img2 = g_img.view(self.ny, self.nx)
                for c0 in range(0, len(mem), m):
                    chunk = mem[c0 : c0 + m]
                    gp = torch.zeros((m, self.ny, self.nx), dtype=torch.float32, device=self.device)
                    for k, si in enumerate(chunk):
                        (x0, x1), (y0, y1) = self._window(si)
                        gp[k, y0:y1, x0:x1] = img2[y0:y1, x0:x1]
                    params = np.zeros((m, 8))
                    params[:, :] = V[chunk[0]]
                    params[: len(chunk)] = V[chunk]
                    res = b.vjp(torch.tensor(params), part["psf"], gp.reshape(-1), as_representation=as_representation,
                                reference_center=reference_center).cpu().numpy()
                    rows += list(zip(chunk, res[: len(chunk)]))
            for si, r in rows:
                for c, sl in enumerate(slots):
                    gi = self.gidx[si].get(sl)
                    if gi is not None:
                        out[gi] += r[c]
        if self.sky_free:
            # d image / d F = ln(10) pixel_area 10^F in every pixel (F unbounded: rep = value)
            F = float(rep[self.sky_g])
            out[self.sky_g] = (math.log(10.0) * self.pixel_area * 10.0 ** F
                               * float(g_img.to(torch.float64).sum().item()))
        return torch.tensor(out, dtype=torch.float64)

    def _gather_table(self, entries, contribs):
        """The device tables (entry, ptr, contrib, n) of ap_gather_sum."""
        uniq, ptr, c = gather_table(entries, contribs)
        dev = self.device
        return (torch.tensor(uniq, device=dev), torch.tensor(ptr, device=dev), torch.tensor(c, device=dev),
                len(uniq))

    def _gather(self, table, part, out):
        entry, ptr, contrib, n = table
        N.check(self.lib.ap_gather_sum(n, N._ptr(entry), N._ptr(ptr), N._ptr(contrib), N._ptr(part), N._ptr(out),
                                       out.numel(), N._stream()), "ap_gather_sum")
        return out

    def hess(self) -> torch.Tensor:
        """J^T W J [P, P] (float64), the same bits on every run."""
        H = torch.empty((self.P, self.P), dtype=torch.float64, device=self.device)
        N.check(self.lib.ap_scene_hess_blocks(N._ptr(self.desc), N._ptr(self.pairs), self.n_pairs, N._ptr(self.jac),
                                              N._ptr(self.weight), N._ptr(self.mask), self.nx, N._ptr(self._hess_part),
                                              N._stream()), "ap_scene_hess_blocks")
        return self._gather(self._hess_table, self._hess_part, H)

    def jt(self, img: torch.Tensor) -> torch.Tensor:
        """J^T img [P] (float64), the same bits on every run."""
        out = torch.empty(self.P, dtype=torch.float64, device=self.device)
        N.check(self.lib.ap_scene_jt_blocks(N._ptr(self.desc), len(self.sources) + (1 if self.n_img else 0),
                                            N._ptr(self.jac), N._ptr(img), self.nx, N._ptr(self._jt_part),
                                            N._stream()), "ap_scene_jt_blocks")
        return self._gather(self._jt_table, self._jt_part, out)

    def jvp(self, h: torch.Tensor) -> torch.Tensor:
        out = torch.empty(self.nx * self.ny, dtype=torch.float32, device=self.device)
        N.check(self.lib.ap_scene_jvp(N._ptr(self.desc), N._ptr(self.jtile_ptr), N._ptr(self.jtile_src),
                                      N._ptr(self.jac), N._ptr(h.contiguous()), self.nx, self.ny, N._ptr(out),
                                      N._stream()), "ap_scene_jvp")
        return out

    def chi2(self, model: torch.Tensor) -> float:
        N.check(self.lib.ap_scene_chi2(N._ptr(model), N._ptr(self.data), N._ptr(self.weight), N._ptr(self.mask),
                                       self.nx * self.ny, N._ptr(self._d64), N._ptr(self._chi2_parts),
                                       self._chi2_parts.numel(), N._stream()), "ap_scene_chi2")
        return float(self._d64.item())

    def residual(self, model: torch.Tensor, data: Optional[torch.Tensor] = None) -> torch.Tensor:
        """W (data - model) on unmasked pixels."""
        r = torch.empty(self.nx * self.ny, dtype=torch.float32, device=self.device)
        d = self.data if data is None else data
        N.check(self.lib.ap_scene_residual(N._ptr(model), N._ptr(d), N._ptr(self.weight), N._ptr(self.mask),
                                           self.nx * self.ny, N._ptr(r), N._stream()), "ap_scene_residual")
        return r

    def rpp_image(self, r, rh, jh, d) -> torch.Tensor:
        out = torch.empty(self.nx * self.ny, dtype=torch.float32, device=self.device)
        N.check(self.lib.ap_scene_rpp_image(N._ptr(r), N._ptr(rh), N._ptr(jh), N._ptr(self.weight),
                                            N._ptr(self.mask), float(d), self.nx * self.ny, N._ptr(out),
                                            N._stream()), "ap_scene_rpp_image")
        return out

    def _solve_call(self, H, g, L, h, info, mixed: bool, reuse: bool):
        n = int(H.shape[0])
        ws, wsn = N._ptr(self._solve_ws), self._solve_ws.numel()
        Hp, gp, hp = N._ptr(H.contiguous()), N._ptr(g.contiguous()), N._ptr(h)
        if mixed and reuse:
            N.check(self.lib.ap_dense_factored_solve_mixed(n, Hp, gp, float(L), hp, ws, wsn, N._ptr(info), N._stream()),
                    "ap_dense_factored_solve_mixed")
        elif mixed:
            N.check(self.lib.ap_dense_damped_solve_mixed(n, Hp, gp, float(L), hp, ws, wsn, N._ptr(info), N._stream()),
                    "ap_dense_damped_solve_mixed")
        elif reuse:
            N.check(self.lib.ap_dense_factored_solve(n, gp, hp, ws, wsn, N._stream()), "ap_dense_factored_solve")
            info.zero_()
        else:
            N.check(self.lib.ap_dense_damped_solve(n, Hp, gp, float(L), hp, ws, wsn, N._ptr(info), N._stream()),
                    "ap_dense_damped_solve")

    def solve(self, H: torch.Tensor, g: torch.Tensor, L: float, reuse: bool = False, mixed: bool = True):
        """Damped solve of the n x n system H (n = H's side, at most P); None when the damped
        matrix is not positive definite.  ``reuse``: the same H and L as the previous (successful)
        call, another right-hand side: only the solves on its factor run.  ``mixed``: float32
        factorisation + float64 refinement (``ap_dense_damped_solve_mixed``) first, the float64
        factorisation when that does not converge."""
        n = int(H.shape[0])
        h = torch.empty(n, dtype=torch.float64, device=self.device)
        if mixed and (not reuse or self._last_mixed):
            self._solve_call(H, g, L, h, self._info, True, reuse)
            if int(self._info.item()) == 0:
                self._last_mixed = not reuse or self._last_mixed
                return h
            if reuse:  # the float32 factor did not serve this right-hand side: factor in float64
                reuse = False
        self._solve_call(H, g, L, h, self._info, False, reuse)
        self._last_mixed = False
        if not reuse and int(self._info.item()) != 0:
            return None
        return h


def gather_table(entries, contribs):
    """ap_gather_sum's tables: the distinct entries (ascending, int64), ptr (int32, one past each
    entry's last contribution) and the contributions of each entry in ascending order (int32)."""
    entries = np.asarray(entries, dtype=np.int64)
    contribs = np.asarray(contribs, dtype=np.int64)
    order = np.lexsort((contribs, entries))
    e, c = entries[order], contribs[order]
    uniq, start = np.unique(e, return_index=True)
    return uniq, np.append(start, len(e)).astype(np.int32), c.astype(np.int32)


def jt_contributions(nf, gid):
    """(entry, contribution) pairs of J^T v: source s's sum for its compact slot c (part index
    8 s + c) goes to the joint-vector entry gid[s][c].  nf[s]: the source's fitted slots."""
    nf, gid = np.asarray(nf, dtype=np.int64), np.asarray(gid, dtype=np.int64)
    src_i, c_i = np.nonzero(np.arange(8)[None, :] < nf[:, None])
    return gid[src_i, c_i], src_i * 8 + c_i


def hess_contributions(nf, gid, pairs, P):
    """(entry, contribution) pairs of J^T W J over a [P, P] row-major matrix: pair p = (A, B)'s
    block element (a, c) (part index 64 p + 8 a + c) goes to (gid[A][a], gid[B][c]) and, for two
    sources, to its transpose too; a source's own block gives its upper triangle, mirrored, so
    the matrix comes out exactly symmetric."""
    nf, gid = np.asarray(nf, dtype=np.int64), np.asarray(gid, dtype=np.int64)
    pa = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
    if len(pa) * 64 >= 2**31:
        raise ValueError("too many overlapping source pairs for int32 contribution indices")
    slot = np.arange(8)
    p_i, a_i, c_i = np.nonzero((slot[None, :, None] < nf[pa[:, 0]][:, None, None])
                               & (slot[None, None, :] < nf[pa[:, 1]][:, None, None]))
    two = pa[p_i, 0] != pa[p_i, 1]
    keep = two | (a_i <= c_i)
    p_i, a_i, c_i, two = p_i[keep], a_i[keep], c_i[keep], two[keep]
    ga, gb = gid[pa[p_i, 0], a_i], gid[pa[p_i, 1], c_i]
    contrib = p_i * 64 + a_i * 8 + c_i
    mirror = two | (a_i < c_i)
    return (np.concatenate([ga * P + gb, gb[mirror] * P + ga[mirror]]),
            np.concatenate([contrib, contrib[mirror]]))


class OptimizeStop(Exception):
    pass


class SceneLM:
    """``LM`` (fit/lm.py:15-539) over a scene's joint vector, or over the entries ``free`` of
    it with the others held (the LM ``Iter_LM`` runs under ``Param_Mask``,
    fit/iterative.py:291-296)."""

    # relative error bounds of a chi^2 change summed from a difference render, and of a chi^2
    # summed from a full float32 render: a chain of accepted changes drifts by the first times
    # their sizes, and the next base render's chi^2 re-anchors it once that exceeds the second
    DIFF_REL_ERR = 2e-6
    FULL_REL_ERR = 2e-8

    def __init__(self, scene: Scene, initial_state=None, max_iter: int = 100, relative_tolerance: float = 1e-5,
                 max_step_iter: int = 10, curvature_limit: float = 1.0, Lup: float = 11.0, Ldn: float = 9.0,
                 L0: float = 1.0, acceleration: float = 0.0, ndf=None, free=None, device_loop: bool = True,
                 precise_trials: bool = True, precise_below: float = 1e-2):
        self.scene = scene
        # device_loop: the vectors stay on the device, parameters are staged there, each damping
        # trial reads one status back (scenes without a live PSF); else the host loop below
        self.device_loop = bool(device_loop) and scene.device_staging
        # precise_trials (device loop): once an accepted step lowers chi^2 by less than
        # precise_below (relative; inf: from the first step) or finds no better trial, every step
        # renders its base point once more, recording it, and each trial (and the geodesic render)
        # as its difference to that base, so chi^2 changes far below one float32 render's rounding
        # (~1e-7 relative) still order the trials as the reference's float64 chi^2 does; the trial
        # chi^2 is then the step's chi^2 plus the change.  Before, trials are full float32 renders:
        # while steps gain more than 1 % the damping is large enough that its trials' chi^2 differ
        # by far more than the rounding, and the accepted trial's render is the next base image.
        self.precise = bool(precise_trials) and self.device_loop and scene.precise_capable
        self.precise_below = float(precise_below)
        self._diff = False   # trials rendered as differences in the current step
        self.x = np.array(scene.representation() if initial_state is None else initial_state, dtype=np.float64)
        self.free = None if free is None else np.asarray(free, dtype=np.int64)
        self._free_t = None if free is None else torch.as_tensor(self.free, device=scene.device)
        self.max_iter, self.relative_tolerance = int(max_iter), float(relative_tolerance)
        self.max_step_iter, self.curvature_limit = int(max_step_iter), float(curvature_limit)
        self._Lup, self._Ldn, self.L, self.acceleration = float(Lup), float(Ldn), float(L0), float(acceleration)
        self.ndf = scene.ndf if ndf is None else ndf
        self.loss_history, self.L_history, self.lambda_history = [], [], []
        self.message = ""
        self.iterations = 0

    def Lup(self):
        self.L = min(1e9, self.L * self._Lup)

    def Ldn(self):
        self.L = max(1e-9, self.L / self._Ldn)

    def _chi2(self, model):
        return self.scene.chi2(model) / self.ndf

    def _sub(self, v):  # entries of the fitted chunk
        return v if self._free_t is None else v[self._free_t]

    def _full(self, v):  # a chunk vector as a joint vector (zeros elsewhere)
        if self._free_t is None:
            return v
        out = torch.zeros(self.scene.P, dtype=v.dtype, device=v.device)
        out[self._free_t] = v
        return out

    def step(self, chi2):
        sc = self.scene
        x = self.x
        Y0 = sc.forward(x)
        sc.jacobian(x)
        hess = sc.hess()
        if self._free_t is not None:
            hess = hess[self._free_t][:, self._free_t].contiguous()
        resid = sc.residual(Y0)             # W (Y - Y0) = -r
        grad = self._sub(sc.jt(resid))      # -J^T r
        r = sc.residual(sc.data, Y0)        # W (Y0 - Y)
        init_chi2 = chi2
        nostep = True
        best = (np.zeros_like(x), init_chi2, self.L)
        scarry_best = (None, init_chi2, self.L)
        direction = "none"
        d = 0.1
        for iteration in range(self.max_step_iter):
            if iteration > self.max_step_iter / 2 and self.L < 1e-3:
                self.L = 1.0
            h = sc.solve(hess, grad, self.L)
            if h is None:
                self.Lup()
                if direction == "better":
                    break
                direction = "worse"
                continue
            h = self._full(h)
            h_np = h.cpu().numpy()
            if self.L > 1e-4:
                # the geodesic term from the render at x + d h; at L <= 1e-4 it is zero and that
                # render (computed and then discarded by fit/lm.py:277-286) is skipped
                Y1 = sc.forward(x + d * h_np)
                rh = sc.residual(sc.data, Y1)   # W (Y1 - Y)
                rpp = self._sub(sc.jt(sc.rpp_image(r, rh, sc.jvp(h), d)))
                a_d = sc.solve(hess, rpp, self.L, reuse=True)  # the factor of the h solve above
                a = np.zeros_like(h_np) if a_d is None else -self._full(a_d).cpu().numpy() / 2
            else:
                a = np.zeros_like(h_np)
            ha = h_np + a * self.acceleration
            Y1 = sc.forward(x + ha)
            chi2 = self._chi2(Y1)
            if not np.isfinite(chi2):
                self.Lup()
                if direction == "better":
                    break
                direction = "worse"
                continue
            if chi2 <= scarry_best[1]:
                scarry_best = (ha, chi2, self.L)
            rho = np.linalg.norm(a) / np.linalg.norm(h_np)
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
            elif chi2 > best[1] and direction in ("none", "worse"):
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

    # ---- the same LM with its vectors on the device -------------------------------------------
    def _trial(self, hess, grad, r, d, mixed: bool):
        """One damping trial at the current L on the device: the step h, the geodesic term a (when
        L > 1e-4), the render at x + h + a * acceleration and its chi^2.  Returns (h + a acc, the
        render (with precise trials its difference to the base render), the packed status
        [solve status, chi^2 (precise: its change from the base), geodesic solve status, the base
        render's chi^2, a, h] read back)."""
        sc = self.scene
        x = self._xd
        P = sc.P
        h = self._full(sc.solve_device(hess, grad, self.L, sc._info, mixed=mixed))
        if self.L > 1e-4:
            # the geodesic term from the render at x + d h (skipped at L <= 1e-4, where
            # fit/lm.py:277-286 computes it and then discards it); it needs only W (Y1 - Y0)
            if self._diff:
                rh = sc.residual(self._zero, sc.forward_diff_device(x, h, d))   # W (Y1 - Y0)
                rpp = self._sub(sc.jt(sc.rpp_image(self._zero, rh, sc.jvp(h), d)))
                self.diff_renders += 1
            else:
                self.full_renders += 1
                Y1 = sc.forward_device(x, h, d)
                rh = sc.residual(sc.data, Y1)   # W (Y1 - Y)
                rpp = self._sub(sc.jt(sc.rpp_image(r, rh, sc.jvp(h), d)))
            a_d = self._full(sc.solve_device(hess, rpp, self.L, sc._info2, mixed=mixed, reuse=True))
            a = torch.where((sc._info == 0) & (sc._info2 == 0), torch.neg(a_d) / 2, torch.zeros_like(a_d))
        else:
            a = torch.zeros_like(h)
            sc._info2.zero_()
        ha = torch.add(h, torch.mul(a, self.acceleration))
        st = self._status
        if self._diff:
            Y1 = sc.forward_diff_device(x, ha, 1.0)      # Y(x + ha) - Y0
            sc.chi2_change_into(Y1, self._Y0, st[1:2])
            self.diff_renders += 1
        else:
            self.full_renders += 1
            Y1 = sc.forward_device(x, ha, 1.0)
            sc.chi2_into(Y1, st[1:2])
        st[0:1].copy_(sc._info)
        st[2:3].copy_(sc._info2)
        st[4 : 4 + P].copy_(a)
        st[4 + P :].copy_(h)
        return ha, Y1, st.cpu().numpy()

    def _step_device(self, chi2, have_y0: bool):
        """:meth:`step` with x, h, a and the images on the device: parameters are staged from
        device vectors, a failed factorisation zeroes h on the device, and each damping trial
        reads back one packed status (factorisation status, chi^2, a, h), from which the host takes
        the reference's decisions in its order.  Returns (step vector on the device, chi^2, L,
        whether the model at the step is in ``self._Yb``)."""
        sc = self.scene
        x = self._xd
        P = sc.P
        if self._diff:
            # the base point of this step's difference trials; its full chi^2 travels with the
            # first trial's status and re-anchors the chain of changes once that has drifted
            self._Y0.copy_(sc.forward_base_device(x))
            sc.chi2_into(self._Y0, self._status[3:4])
            self.base_renders += 1
        elif not have_y0:
            self._Y0.copy_(sc.forward_device(x))
            self.base_renders += 1
        Y0 = self._Y0
        sc.jacobian_device(x)
        hess = sc.hess()
        if self._free_t is not None:
            hess = hess[self._free_t][:, self._free_t].contiguous()
        resid = sc.residual(Y0)             # W (Y - Y0) = -r
        grad = self._sub(sc.jt(resid))      # -J^T r
        r = sc.residual(sc.data, Y0)        # W (Y0 - Y)
        init_chi2 = chi2
        nostep = True
        best = (None, init_chi2, self.L)
        scarry_best = (None, init_chi2, self.L)
        direction = "none"
        d = 0.1
        for iteration in range(self.max_step_iter):
            if iteration > self.max_step_iter / 2 and self.L < 1e-3:
                self.L = 1.0
            self.trials += 1
            if self.L > 1e-4:
                self.geodesic_trials += 1
            ha, Y1, s = self._trial(hess, grad, r, d, mixed=True)
            if int(s[0]) == -1 or int(s[2]) == -1:
                # the mixed-precision solve did not converge: the trial again, in float64
                self.fp64_retries += 1
                ha, Y1, s = self._trial(hess, grad, r, d, mixed=False)
            if self._diff and iteration == 0:
                full = float(s[3]) / self.ndf
                if self._drift > self.FULL_REL_ERR * full:
                    init_chi2 = full
                    best = (None, full, self.L)
                    scarry_best = (None, full, self.L)
                    self._drift = 0.0
            if int(s[0]) != 0:   # the damped matrix was not positive definite
                self.Lup()
                if direction == "better":
                    break
                direction = "worse"
                continue
            chi2 = init_chi2 + float(s[1]) / self.ndf if self._diff else float(s[1]) / self.ndf
            a_np, h_np = s[4 : 4 + P], s[4 + P :]
            if not np.isfinite(chi2):
                self.Lup()
                if direction == "better":
                    break
                direction = "worse"
                continue
            if chi2 <= scarry_best[1]:
                scarry_best = (ha, chi2, self.L)
            rho = np.linalg.norm(a_np) / np.linalg.norm(h_np)
            if rho > self.curvature_limit:
                self.Lup()
                if direction == "better":
                    break
                direction = "worse"
                continue
            if chi2 < best[1]:
                best = (ha, chi2, self.L)
                if not self._diff:
                    self._Yb.copy_(Y1)
                nostep = False
                self.Ldn()
                if self.L <= 1e-8 or direction == "worse":
                    break
                direction = "better"
            elif chi2 > best[1] and direction in ("none", "worse"):
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
                self._drift += self.DIFF_REL_ERR * abs(scarry_best[1] - init_chi2)
                return scarry_best[0], scarry_best[1], scarry_best[2], False
            raise OptimizeStop("Could not find step to improve chi^2")
        self._drift += self.DIFF_REL_ERR * abs(best[1] - init_chi2)
        return best[0], best[1], best[2], not self._diff

    def _fit_device(self):
        sc = self.scene
        dev = sc.device
        sc.set_stage_base(self.x)
        self._xd = torch.tensor(self.x, dtype=torch.float64, device=dev)
        self._Y0 = torch.empty(sc.nx * sc.ny, dtype=torch.float32, device=dev)
        self._Yb = torch.empty_like(self._Y0)
        self._status = torch.zeros(4 + 2 * sc.P, dtype=torch.float64, device=dev)
        self._zero = torch.zeros(sc.nx * sc.ny, dtype=torch.float32, device=dev)
        self._drift = 0.0
        self._diff = self.precise and self.precise_below == float("inf")
        self.diff_steps = self.diff_renders = self.full_renders = 0
        self.trials = self.geodesic_trials = self.base_renders = self.fp64_retries = 0
        self._Y0.copy_(sc.forward_device(self._xd))
        sc.chi2_into(self._Y0, self._status[1:2])
        self.loss_history = [float(self._status[1].item()) / self.ndf]
        self.L_history = [self.L]
        self.lambda_history = [self.x.copy()]
        have_y0 = True
        for iteration in range(self.max_iter):
            self.iterations = iteration + 1
            try:
                self.diff_steps += int(self._diff)
                step, chi2, L, at_best = self._step_device(self.loss_history[-1], have_y0)
            except OptimizeStop:
                self.message = self.message + "fail. Could not find step to improve Chi^2"
                break
            if self.precise and not self._diff and (
                    not at_best or (self.loss_history[-1] - chi2) < self.precise_below * chi2):
                self._diff = True   # from the next step on, trials as differences
            self.L = L
            self._xd = self._xd + step
            if at_best:  # the model at the new x is the accepted trial's render
                self._Y0, self._Yb = self._Yb, self._Y0
            have_y0 = at_best
            self.x = self._xd.cpu().numpy().copy()
            self.L_history.append(self.L)
            self.loss_history.append(chi2)
            self.lambda_history.append(self.x.copy())
            self.Ldn()
            if len(self.loss_history) >= 3:
                if (self.loss_history[-3] - self.loss_history[-1]) / self.loss_history[-1] < self.relative_tolerance \
                        and self.L < 0.1:
                    self.message = self.message + "success"
                    break
            if len(self.loss_history) > 10:
                if (self.loss_history[-10] - self.loss_history[-1]) / self.loss_history[-1] < self.relative_tolerance:
                    self.message = self.message + "success by immobility. Convergence not guaranteed"
                    break
        else:
            self.message = self.message + "fail. Maximum iterations"
        self.scene.set_representation(self.res())
        return self

    def fit(self):
        if self.scene.P == 0 or (self.free is not None and len(self.free) == 0):
            return self
        if self.device_loop:
            return self._fit_device()
        self.loss_history = [self._chi2(self.scene.forward(self.x))]
        self.L_history = [self.L]
        self.lambda_history = [self.x.copy()]
        for iteration in range(self.max_iter):
            self.iterations = iteration + 1
            try:
                res = self.step(chi2=self.loss_history[-1])
            except OptimizeStop:
                self.message = self.message + "fail. Could not find step to improve Chi^2"
                break
            self.L = res[2]
            self.x = self.x + res[0]
            self.L_history.append(self.L)
            self.loss_history.append(res[1])
            self.lambda_history.append(self.x.copy())
            self.Ldn()
            if len(self.loss_history) >= 3:
                if (self.loss_history[-3] - self.loss_history[-1]) / self.loss_history[-1] < self.relative_tolerance \
                        and self.L < 0.1:
                    self.message = self.message + "success"
                    break
            if len(self.loss_history) > 10:
                if (self.loss_history[-10] - self.loss_history[-1]) / self.loss_history[-1] < self.relative_tolerance:
                    self.message = self.message + "success by immobility. Convergence not guaranteed"
                    break
        else:
            self.message = self.message + "fail. Maximum iterations"
        self.scene.set_representation(self.res())
        return self

    def res(self):
        hist = np.array(self.loss_history)
        ok = np.isfinite(hist)
        if not ok.any():
            return self.x.copy()
        return np.array(self.lambda_history)[ok][np.argmin(hist[ok])]


def fit_scenes(scenes: Sequence[Scene], initial_states=None, workers: int = 8, **lm_kwargs) -> List[SceneLM]:
    """Independent scene LMs (``LM(model).fit()`` of separate models) run concurrently: each of
    ``workers`` host threads drives its share of the scenes on its own CUDA stream, so that one
    fit's host round trips (damped-solve status, chi^2) overlap the kernels of the others.
    Every scene must own its batches (no scene shared between two entries).  Returns the
    :class:`SceneLM` of every scene, in order; each fit is the same as run alone."""
    import concurrent.futures as cf

    n = len(scenes)
    if len({id(sc) for sc in scenes}) != n:
        raise ValueError("fit_scenes needs distinct scenes")
    inits = [None] * n if initial_states is None else list(initial_states)
    nw = max(1, min(int(workers), n))
    streams = [torch.cuda.Stream(device=scenes[0].device) for _ in range(nw)] if n else []
    out: List[Optional[SceneLM]] = [None] * n
    caller = torch.cuda.current_stream()
    for st in streams:
        st.wait_stream(caller)

    def work(w):
        with torch.cuda.stream(streams[w]):
            for i in range(w, n, nw):
                x0 = None if inits[i] is None else np.array(inits[i], dtype=np.float64)
                out[i] = SceneLM(scenes[i], initial_state=x0, **lm_kwargs).fit()
        streams[w].synchronize()

    with cf.ThreadPoolExecutor(max_workers=nw) as ex:
        list(ex.map(work, range(nw)))
    for st in streams:
        caller.wait_stream(st)
    return out


class SceneIterLM:
    """``Iter_LM`` (fit/iterative.py:177-338) over a scene: sweeps of LMs on chunks of the joint
    vector (the rest held, the full problem's degrees of freedom), until the sweep loss settles
    twice (relative change in (-tol 1e-3, tol / 10)) or ``max_iter`` sweeps.  ``chunks`` an int:
    chunks of that many entries in order (``method="sequential"``) or drawn by ``random.sample``
    (``"random"``, Python's ``random`` module, as the reference draws them); or a sequence of
    index lists."""

    def __init__(self, scene: Scene, initial_state=None, chunks=50, max_iter: int = 100, method: str = "random",
                 relative_tolerance: float = 1e-3, LM_kwargs: Optional[dict] = None):
        self.scene = scene
        self.x = np.array(scene.representation() if initial_state is None else initial_state, dtype=np.float64)
        self.chunks, self.method, self.max_iter = chunks, method, int(max_iter)
        self.relative_tolerance = float(relative_tolerance)
        self.LM_kwargs = dict(LM_kwargs or {})
        n_used = scene.nx * scene.ny if scene.mask is None else int((scene.mask == 0).sum().item())
        self.ndf = n_used - scene.P
        self.loss_history, self.lambda_history = [], []
        self.message = ""
        self.iteration = 0
        self._count_finish = 0

    def _chunk_list(self):
        import random

        if isinstance(self.chunks, int):
            ids = list(range(self.scene.P))
            while ids:
                take = random.sample(ids, min(len(ids), self.chunks)) if self.method == "random" else ids[: self.chunks]
                for t in sorted(take):
                    ids.pop(ids.index(t))
                yield sorted(take)
        else:
            order = list(range(len(self.chunks)))
            while order:
                k = random.choice(order) if self.method == "random" else order[0]
                order.pop(order.index(k))
                yield sorted(int(i) for i in self.chunks[k])

    def step(self):
        res = None
        for chunk in self._chunk_list():
            res = SceneLM(self.scene, initial_state=self.x, ndf=self.ndf, free=chunk, **self.LM_kwargs).fit()
            self.x = np.array(res.res(), dtype=np.float64)
        self.loss_history.append(min(v for v in res.loss_history if np.isfinite(v)))
        self.lambda_history.append(self.x.copy())
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
        if self.scene.P == 0:
            return self
        while True:
            self.step()
            if self.iteration > 2 and self._count_finish >= 2:
                self.message = self.message + "success"
                break
            if self.iteration >= self.max_iter:
                self.message = self.message + f"fail max iterations reached: {self.iteration}"
                break
        self.scene.set_representation(self.res())
        return self

    def res(self):
        hist = np.array(self.loss_history)
        ok = np.isfinite(hist)
        if not ok.any():
            return self.x.copy()
        return np.array(self.lambda_history)[ok][np.argmin(hist[ok])]


class SceneRenderFunction(torch.autograd.Function):
    """image = scene.forward(rep) with the scene's adjoint as its backward."""

    @staticmethod
    def forward(ctx, rep, scene, reference_center):
        ctx.scene, ctx.reference_center = scene, reference_center
        ctx.save_for_backward(rep)
        return scene.forward(rep.detach().cpu().numpy())

    @staticmethod
    def backward(ctx, grad_image):
        (rep,) = ctx.saved_tensors
        g = ctx.scene.vjp(rep.detach().cpu().numpy(), grad_image, reference_center=ctx.reference_center)
        return g.to(rep.device, rep.dtype), None, None


def render(scene: Scene, rep: torch.Tensor, reference_center: bool = False) -> torch.Tensor:
    """Differentiable scene render from a joint representation vector (float64 tensor)."""
    return SceneRenderFunction.apply(rep, scene, reference_center)
