"""ctypes binding of ``libastrophot_gb300.so`` (declared in ``include/astrophot_gb300.h``)
and :class:`StampBatch`, the thin owner of one batch plan and its device workspace.

PyTorch is used only for device memory and the current CUDA stream.  There is no CPU
fallback: importing this module fails loudly when the library has not been built, and
every call needs a CUDA device.
"""

from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence

import numpy as np
import torch

from .errors import InvalidParameter, SpecificationConflict

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libastrophot_gb300.so")

AP_OK = 0
AP_ERR_ARG = 1
AP_ERR_UNSUPPORTED = 2
AP_ERR_CUDA = 3
AP_ERR_WORKSPACE = 4
AP_ERR_LIMIT = 5
AP_ERR_NOT_BOUND = 6
_ERR_NAMES = {
    AP_ERR_ARG: "bad argument",
    AP_ERR_UNSUPPORTED: "unsupported option",
    AP_ERR_CUDA: "CUDA error",
    AP_ERR_WORKSPACE: "workspace too small",
    AP_ERR_LIMIT: "parameter outside its limits",
    AP_ERR_NOT_BOUND: "batch not bound to a workspace",
}

PROFILE = {"sersic": 0, "exponential": 1, "moffat": 2, "gaussian": 3}
SAMPLING = {"midpoint": 0, "simpsons": 1, "quad": 2, "trapezoid": 3, "midpoint_center": 4}
INTEGRATE = {"none": 0, "threshold": 1}
PSF_NONE, PSF_FULL, PSF_FULL_NOSHIFT = 0, 1, 2
VJP_REPRESENTATION, VJP_REFERENCE_CENTER = 1, 2
# psf_convolve_mode "fft": stamps whose convolution kernel side (PSF side + 2 with the bilinear
# shift) is at least this are convolved by FFT, smaller ones directly (same numbers either way;
# measured on 200-source 1024² scenes, one Jacobian + two renders per LM iteration: direct is
# faster up to 65² PSFs, FFT from about 73²)
FFT_MIN_KERNEL = 75
# ap_reference_init status bits
INIT_CENTRE_EDGE, INIT_FIT_LIMIT, INIT_NO_ISOPHOTE, INIT_NO_PROFILE = 1, 2, 4, 8

LM_RUNNING, LM_SUCCESS, LM_IMMOBILE, LM_MAX_ITER, LM_NO_STEP, LM_LIMIT = range(6)
LM_MESSAGES = {
    LM_RUNNING: "running",
    LM_SUCCESS: "success",
    LM_IMMOBILE: "success by immobility. Convergence not guaranteed",
    LM_MAX_ITER: "fail. Maximum iterations",
    LM_NO_STEP: "fail. Could not find step to improve Chi^2",
    LM_LIMIT: "fail. A parameter left its limits",
}

# full parameter-vector slots
SLOTS = ("cx", "cy", "q", "PA", "n", "Re", "Ie", "F")


class ApOptions(ctypes.Structure):
    _fields_ = [
        ("profile", ctypes.c_int32),
        ("sampling_mode", ctypes.c_int32),
        ("sampling_quad_level", ctypes.c_int32),
        ("integrate_mode", ctypes.c_int32),
        ("psf_mode", ctypes.c_int32),
        ("integrate_max_depth", ctypes.c_int32),
        ("integrate_gridding", ctypes.c_int32),
        ("integrate_quad_level", ctypes.c_int32),
        ("sampling_tolerance", ctypes.c_double),
        ("softening", ctypes.c_double),
        ("free_mask", ctypes.c_int32),
        ("has_sky", ctypes.c_int32),
        ("fft_min_kernel", ctypes.c_int32),
        ("center_radius", ctypes.c_double),
        ("lanczos_order", ctypes.c_int32),
    ]


class ApLMOptions(ctypes.Structure):
    _fields_ = [
        ("max_iter", ctypes.c_int32),
        ("max_step_iter", ctypes.c_int32),
        ("relative_tolerance", ctypes.c_double),
        ("curvature_limit", ctypes.c_double),
        ("Lup", ctypes.c_double),
        ("Ldn", ctypes.c_double),
        ("L0", ctypes.c_double),
        ("acceleration", ctypes.c_double),
        ("rounds_per_sync", ctypes.c_int32),
        ("use_graph", ctypes.c_int32),
        ("precise_trials", ctypes.c_int32),
    ]


_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_PI32 = ctypes.POINTER(ctypes.c_int32)
_PI64 = ctypes.POINTER(ctypes.c_int64)
_PD = ctypes.POINTER(ctypes.c_double)

# (name, argtypes) of every exported symbol, in header order
EXPORTS = [
    ("ap_batch_create", [ctypes.POINTER(_P), _I32, _PI32, _PI32, _PI32, _PI32, _PD, ctypes.POINTER(ApOptions)]),
    ("ap_batch_destroy", [_P]),
    ("ap_batch_sizes", [_P, _PI64, _PI64, _PI64]),
    ("ap_batch_offsets", [_P, _PI64, _PI64]),
    ("ap_batch_bind", [_P, _P, _I64, _P]),
    ("ap_batch_set_threshold_numel", [_P, _PD]),
    ("ap_batch_set_threshold_window", [_P, _PI32]),
    ("ap_render", [_P, _P, _P, _P, _P]),
    ("ap_jacobian", [_P, _P, _P, _P, _P, _I32, _P]),
    ("ap_render_psf_derivative", [_P, _P, _P, _P, _P, _P]),
    ("ap_render_base_bytes", [_P, _PI64]),
    ("ap_render_precise", [_P, _P, _P, _P, _P, _I64, _I32, _P]),
    ("ap_psf_normalize", [_I32, _I32, _P, _P, _P, _P, _P]),
    ("ap_render_vjp", [_P, _P, _P, _P, _I32, _P, _P]),
    ("ap_batch_autotune", [_P, _P, _P, _I32, _PI32, _PD, _P]),
    ("ap_batch_set_grid", [_P, _PI32]),
    ("ap_values_to_rep", [_P, _I32, _I32, _P, _P]),
    ("ap_reference_init_workspace_bytes", [_P, _PI64]),
    ("ap_segmap_range", [_P, _I64, _P, _P]),
    ("ap_segmap_present", [_P, _I64, _I32, _P, _P]),
    ("ap_segmap_stats", [_P, _P, _I32, _I32, _P, _I32, ctypes.c_double, _P, _P, _P, _P, _P, _P, _P, _P]),
    ("ap_window_flux", [_P, _I32, _I32, _P, _I32, _P, _P]),
    ("ap_reference_init", [_P, _P, _P, _I32, _P, _P, _P, _I64, _P]),
    ("ap_batch_psf_stride", [_P, _PI64]),
    ("ap_psf_shift", [_P, _P, _P, _P, _P, _P]),
    ("ap_chi2", [_P, _P, _P, _P, _P, _P, _P]),
    ("ap_damped_solve", [_I32, _I32, _P, _P, _P, _P, _P]),
    ("ap_lm_workspace_bytes", [_P, ctypes.POINTER(ApLMOptions), _PI64]),
    ("ap_lm_fit", [_P, _P, _P, _P, _P, _P, _P, ctypes.POINTER(ApLMOptions), _P, _I64, _P, _P, _P, _P]),
    ("ap_lm_history", [_P, ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(_P), _PI32]),
    ("ap_batch_profile", [_P, _I32]),
    ("ap_batch_kernel_times", [_P, _PD, _PI64]),
    ("ap_batch_work_counters", [_P, ctypes.POINTER(ctypes.c_uint64), _I32, _P]),
    ("ap_fma_probe", [_P, _I32, _I32, _P]),
    ("ap_sample_probe", [_I32, _P, _I32, _I32, _P]),
    ("ap_batch_stats", [_P, _PI64]),
    ("ap_render_noalloc", [_I32, _I32, _I32, _I32, _PD, ctypes.POINTER(ApOptions), _P, _P, _P, _P]),
    ("ap_scene_forward", [_P, _P, _P, _P, ctypes.c_float, _P, _P, ctypes.c_double, _I32, _I32, _P, _P]),
    ("ap_scene_jvp", [_P, _P, _P, _P, _P, _I32, _I32, _P, _P]),
    ("ap_scene_jt", [_P, _I32, _P, _P, _I32, _I32, _P, _P]),
    ("ap_scene_hess", [_P, _P, _I32, _P, _P, _P, _I32, _I32, _P, _P]),
    ("ap_scene_chi2", [_P, _P, _P, _P, _I64, _P, _P, _I32, _P]),
    ("ap_scene_chi2_change", [_P, _P, _P, _P, _P, _I64, _P, _P, _I32, _P]),
    ("ap_reduce_upscaled", [_I32, _P, _P, _P, _I32, _I32, _P, _I64, _P, _I64, _I64, _P]),
    ("ap_scene_hess_blocks", [_P, _P, _I32, _P, _P, _P, _I32, _P, _P]),
    ("ap_scene_jt_blocks", [_P, _I32, _P, _P, _I32, _P, _P]),
    ("ap_gather_sum", [_I64, _P, _P, _P, _P, _P, _I64, _P]),
    ("ap_scene_residual", [_P, _P, _P, _P, _I64, _P, _P]),
    ("ap_scene_rpp_image", [_P, _P, _P, _P, _P, ctypes.c_double, _I64, _P, _P]),
    ("ap_scene_stage", [_I32, _P, _P, _P, _P, ctypes.c_double, _P, _P]),
    ("ap_dense_solve_workspace_bytes", [_I32]),
    ("ap_dense_damped_solve", [_I32, _P, _P, ctypes.c_double, _P, _P, ctypes.c_size_t, _P, _P]),
    ("ap_dense_factored_solve", [_I32, _P, _P, _P, ctypes.c_size_t, _P]),
    ("ap_dense_damped_solve_mixed", [_I32, _P, _P, ctypes.c_double, _P, _P, ctypes.c_size_t, _P, _P]),
    ("ap_dense_factored_solve_mixed", [_I32, _P, _P, ctypes.c_double, _P, _P, ctypes.c_size_t, _P, _P]),
    ("ap_cnn_param_count", []),
    ("ap_cnn_autotune", [_I32, _PI32]),
    ("ap_cnn_workspace_bytes", [_I64]),
    ("ap_cnn_layer_offsets", [_PI64, _PI64, _PI32]),
    ("ap_cnn_workspace_offsets", [_I64, _PI64, _PI64]),
    ("ap_cnn_to_bf16", [_P, _P, _P]),
    ("ap_cnn_forward", [_P, _P, _P, _I64, _P, _P, ctypes.c_size_t, _P]),
    ("ap_cnn_infer", [_P, _P, _P, _I64, _P, _P, ctypes.c_size_t, _P]),
    ("ap_cnn_backward", [_P, _P, _I64, _P, _P, ctypes.c_size_t, _P]),
    ("ap_cnn_train_step", [_P, _P, _P, _P, _P, _P, _P, _I64, ctypes.c_float, _I32, ctypes.c_float, _P, _P,
                           ctypes.c_size_t, _P]),
    ("ap_cnn_prepare", [_P, _P, _P, _I64, _P, _P, _P]),
    ("ap_cnn_decode", [_P, _P, _P, _P, _P, _I64, _P, _P]),
    ("ap_moments_init", [_P, _P, _P, _P, _I64, _P, _P]),
    ("ap_select_init", [_P, _P, _P, _P, _I64, _P, _P, _P]),
    ("ap_gemm_bf16", [_P, _I32, _I32, _P, _I32, _I32, _P, _I32, _I32, _I32, _I32, _P]),
    ("ap_cnn_set_path", [_I32]),
    ("ap_cnn_get_path", [_PI32]),
    ("ap_gemm_bf16_tc", [_P, _I32, _P, _I32, _P, _I32, _I32, _I32, _I32, _P, _P, _I32, _P]),
    ("ap_conv3x3s2_bf16_tc", [_P, _I64, _I32, _I32, _P, _I32, _P, _I32, _P, _P, _I32, _P]),
    ("ap_tc_status", [_I32, ctypes.POINTER(ctypes.c_uint32)]),
    ("ap_version", []),
    ("ap_last_cuda_error", []),
]

_RESTYPES = {
    "ap_version": ctypes.c_char_p,
    "ap_last_cuda_error": ctypes.c_char_p,
    "ap_cnn_param_count": ctypes.c_int64,
    "ap_cnn_workspace_bytes": ctypes.c_size_t,
    "ap_dense_solve_workspace_bytes": ctypes.c_size_t,
}


def load_library(path: str = LIB_PATH) -> ctypes.CDLL:
    if not os.path.exists(path):
        raise ImportError(
            f"{path} is missing: build the CUDA library first "
            "(python -m astrophot_gb300._build, or __graft_entry__.build())"
        )
    lib = ctypes.CDLL(path)
    for name, argtypes in EXPORTS:
        fn = getattr(lib, name)
        fn.argtypes = argtypes
        fn.restype = _RESTYPES.get(name, ctypes.c_int)
    return lib


_lib: Optional[ctypes.CDLL] = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        _lib = load_library()
    return _lib


def check(rc: int, what: str) -> None:
    if rc == AP_OK:
        return
    if rc == AP_ERR_LIMIT:
        raise InvalidParameter(f"{what}: {_ERR_NAMES[rc]}")
    if rc == AP_ERR_UNSUPPORTED:
        raise SpecificationConflict(f"{what}: {_ERR_NAMES[rc]}")
    detail = ""
    if rc == AP_ERR_CUDA and _lib is not None:
        detail = ": " + _lib.ap_last_cuda_error().decode()
    raise RuntimeError(f"{what} failed: {_ERR_NAMES.get(rc, rc)} (status {rc}){detail}")


def _ptr(t: Optional[torch.Tensor]):
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("astrophot_gb300 kernels need CUDA tensors")
    if not t.is_contiguous():
        raise ValueError("astrophot_gb300 kernels need contiguous tensors")
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def lanczos_order(psf_subpixel_shift: str) -> int:
    """k of a "lanczos:k" sub-pixel shift (models/_model_methods.py:209-210), else 0."""
    if not isinstance(psf_subpixel_shift, str) or "lanczos" not in psf_subpixel_shift:
        return 0
    try:
        k = int(psf_subpixel_shift[psf_subpixel_shift.find(":") + 1 :])
    except ValueError:
        raise SpecificationConflict(f"unrecognized subpixel shift method: {psf_subpixel_shift}") from None
    if not 1 <= k <= 8:
        raise SpecificationConflict(f"Lanczos order {k} outside 1..8 on the CUDA path")
    return k


def make_options(
    profile="sersic",
    sampling_mode="midpoint",
    integrate_mode="threshold",
    psf_mode="none",
    psf_subpixel_shift="bilinear",
    integrate_max_depth=3,
    integrate_gridding=5,
    integrate_quad_level=3,
    sampling_tolerance=1e-2,
    softening=1e-3,
    free_mask=0x7F,
    has_sky=False,
    psf_convolve_mode="direct",
    fft_min_kernel=None,
    center_quad_level=3,
    center_radius=2.0,
) -> ApOptions:
    o = ApOptions()
    if profile not in PROFILE:
        raise SpecificationConflict(f"unsupported profile {profile}")
    o.profile = PROFILE[profile]
    if sampling_mode.startswith("quad"):
        o.sampling_mode = SAMPLING["quad"]
        o.sampling_quad_level = int(sampling_mode[sampling_mode.find(":") + 1 :])
    elif sampling_mode == "midpoint_center":
        # midpoint + center_quad_level^2 Gauss-Legendre points on the pixels within center_radius
        # pixels of the centre (no adaptive integration)
        if integrate_mode != "none":
            raise SpecificationConflict("sampling_mode midpoint_center needs integrate_mode none")
        o.sampling_mode = SAMPLING[sampling_mode]
        o.sampling_quad_level = int(center_quad_level)
    elif sampling_mode in SAMPLING:
        o.sampling_mode = SAMPLING[sampling_mode]
        o.sampling_quad_level = 0
    else:
        raise SpecificationConflict(
            f"unknown sampling mode: {sampling_mode}. Should be one of: midpoint, simpsons, quad:level, trapezoid, "
            "midpoint_center"
        )
    if integrate_mode not in INTEGRATE:
        raise SpecificationConflict(
            f"unknown integration mode: {integrate_mode}. Should be one of: none, threshold"
        )
    o.integrate_mode = INTEGRATE[integrate_mode]
    if psf_mode == "none":
        o.psf_mode = PSF_NONE
    elif psf_mode == "full":
        o.lanczos_order = lanczos_order(psf_subpixel_shift)
        if psf_subpixel_shift == "bilinear" or o.lanczos_order > 0:
            o.psf_mode = PSF_FULL
        elif psf_subpixel_shift == "none":
            o.psf_mode = PSF_FULL_NOSHIFT
        else:
            raise SpecificationConflict(f"unrecognized subpixel shift method: {psf_subpixel_shift}")
    else:
        raise SpecificationConflict(f"unsupported psf_mode {psf_mode}")
    o.integrate_max_depth = int(integrate_max_depth)
    o.integrate_gridding = int(integrate_gridding)
    o.integrate_quad_level = int(integrate_quad_level)
    o.sampling_tolerance = float(sampling_tolerance)
    o.softening = float(softening)
    o.free_mask = int(free_mask)
    o.has_sky = 1 if has_sky else 0
    if psf_convolve_mode not in ("fft", "direct"):
        raise SpecificationConflict(f"unrecognized psf_convolve_mode: {psf_convolve_mode}")
    if fft_min_kernel is None:
        fft_min_kernel = FFT_MIN_KERNEL if psf_convolve_mode == "fft" else 0
    o.fft_min_kernel = int(fft_min_kernel)
    o.center_radius = float(center_radius)
    return o


def make_lm_options(
    max_iter=100,
    max_step_iter=10,
    relative_tolerance=1e-5,
    curvature_limit=1.0,
    Lup=11.0,
    Ldn=9.0,
    L0=1.0,
    acceleration=0.0,
    rounds_per_sync=4,
    use_graph=True,
    precise_trials=True,
) -> ApLMOptions:
    o = ApLMOptions()
    o.max_iter = int(max_iter)
    o.max_step_iter = int(max_step_iter)
    o.relative_tolerance = float(relative_tolerance)
    o.curvature_limit = float(curvature_limit)
    o.Lup = float(Lup)
    o.Ldn = float(Ldn)
    o.L0 = float(L0)
    o.acceleration = float(acceleration)
    o.rounds_per_sync = int(rounds_per_sync)
    o.use_graph = 1 if use_graph else 0
    o.precise_trials = 1 if precise_trials else 0
    return o


def scale_geometry(n: int, scale: float = 1.0, origin=(0.0, 0.0)) -> np.ndarray:
    """Geometry rows for ``n`` windows with pixel scale ``scale`` whose (0, 0) pixel corner
    sits at ``origin`` (reference pixel (-0.5, -0.5), as ``PPCS`` defaults)."""
    g = np.zeros((n, 8))
    g[:, 0] = scale
    g[:, 3] = scale
    g[:, 4] = -0.5
    g[:, 5] = -0.5
    g[:, 6] = origin[0]
    g[:, 7] = origin[1]
    return g


class StampBatch:
    """A planned batch of stamps bound to a device workspace."""

    def __init__(
        self,
        shapes: Sequence[tuple],
        psf_shapes: Optional[Sequence[tuple]],
        geometry: np.ndarray,
        options: ApOptions,
        device=None,
    ):
        self.lib = lib()
        self.device = torch.device(device if device is not None else "cuda")
        n = len(shapes)
        self.n = n
        self.options = options
        nx = (ctypes.c_int32 * n)(*[int(s[0]) for s in shapes])
        ny = (ctypes.c_int32 * n)(*[int(s[1]) for s in shapes])
        self.shapes = [(int(s[0]), int(s[1])) for s in shapes]
        if psf_shapes is not None:
            kx = (ctypes.c_int32 * n)(*[int(s[0]) for s in psf_shapes])
            ky = (ctypes.c_int32 * n)(*[int(s[1]) for s in psf_shapes])
            self.psf_shapes = [(int(s[0]), int(s[1])) for s in psf_shapes]
        else:
            kx = ky = None
            self.psf_shapes = None
        geom = np.ascontiguousarray(geometry, dtype=np.float64).reshape(n, 8)
        self.geometry = geom
        h = ctypes.c_void_p()
        check(
            self.lib.ap_batch_create(
                ctypes.byref(h), n, nx, ny, kx, ky, geom.ctypes.data_as(_PD), ctypes.byref(options)
            ),
            "ap_batch_create",
        )
        self.handle = h
        out_px, psf_px, ws = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        check(self.lib.ap_batch_sizes(h, ctypes.byref(out_px), ctypes.byref(psf_px), ctypes.byref(ws)), "sizes")
        self.out_pixels = out_px.value
        self.psf_pixels = psf_px.value
        self.workspace_bytes = ws.value
        oo = (ctypes.c_int64 * n)()
        po = (ctypes.c_int64 * n)()
        check(self.lib.ap_batch_offsets(h, oo, po), "offsets")
        self.out_offsets = np.array(oo[:], dtype=np.int64)
        self.psf_offsets = np.array(po[:], dtype=np.int64)
        stride = ctypes.c_int64()
        check(self.lib.ap_batch_psf_stride(h, ctypes.byref(stride)), "psf stride")
        self.psf_stride = stride.value
        self.n_free = bin(options.free_mask).count("1")
        self.workspace = torch.empty(max(self.workspace_bytes, 256), dtype=torch.uint8, device=self.device)
        check(self.lib.ap_batch_bind(h, _ptr(self.workspace), self.workspace_bytes, _stream()), "ap_batch_bind")
        self._lm_ws = None

    def __del__(self):
        try:
            if getattr(self, "handle", None) is not None:
                self.lib.ap_batch_destroy(self.handle)
                self.handle = None
        except Exception:
            pass

    # ---- packing helpers --------------------------------------------------------------
    def pack(self, images, dtype=torch.float32) -> torch.Tensor:
        """Pack a list of [ny, nx] arrays into one device vector in the output layout."""
        flat = np.concatenate([np.asarray(im).reshape(-1) for im in images])
        np_dtype = {torch.float32: np.float32, torch.uint8: np.uint8, torch.float64: np.float64}[dtype]
        return torch.from_numpy(flat.astype(np_dtype)).to(self.device)

    def pack_psf(self, psfs) -> torch.Tensor:
        flat = np.concatenate([np.asarray(p, dtype=np.float32).reshape(-1) for p in psfs])
        return torch.from_numpy(flat).to(self.device)

    def unpack(self, packed: torch.Tensor):
        host = packed.detach().cpu().numpy()
        out = []
        for s, (nx, ny) in enumerate(self.shapes):
            o = self.out_offsets[s]
            out.append(host[o : o + nx * ny].reshape(ny, nx))
        return out

    # ---- entry points -------------------------------------------------------------------
    def render(self, params: torch.Tensor, psf: Optional[torch.Tensor], out: Optional[torch.Tensor] = None):
        params = params.to(self.device, torch.float64).contiguous()
        if out is None:
            out = torch.empty(self.out_pixels, dtype=torch.float32, device=self.device)
        check(self.lib.ap_render(self.handle, _ptr(params), _ptr(psf), _ptr(out), _stream()), "ap_render")
        return out

    RENDER_BASE, RENDER_DIFFERENCE = 1, 2

    def base_buffer(self) -> torch.Tensor:
        """A device buffer for the base point of :meth:`render_precise` (ap_render_base_bytes)."""
        n = ctypes.c_int64()
        check(self.lib.ap_render_base_bytes(self.handle, ctypes.byref(n)), "ap_render_base_bytes")
        return torch.empty(int(n.value), dtype=torch.uint8, device=self.device)

    def render_precise(self, params: torch.Tensor, psf: Optional[torch.Tensor], base: torch.Tensor, mode: int,
                       out: Optional[torch.Tensor] = None):
        """RENDER_BASE: the model, recorded in ``base``; RENDER_DIFFERENCE: the model minus the
        recorded base model, accurate relative to the difference (ap_render_precise)."""
        params = params.to(self.device, torch.float64).contiguous()
        if out is None:
            out = torch.empty(self.out_pixels, dtype=torch.float32, device=self.device)
        check(self.lib.ap_render_precise(self.handle, _ptr(params), _ptr(psf), _ptr(out), _ptr(base), base.numel(),
                                         int(mode), _stream()), "ap_render_precise")
        return out

    def render_psf_derivative(self, params: torch.Tensor, psf: torch.Tensor, dpsf: torch.Tensor,
                              out: Optional[torch.Tensor] = None):
        """d model / d theta for a PSF change dpsf = d psf / d theta (ap_render_psf_derivative)."""
        params = params.to(self.device, torch.float64).contiguous()
        if out is None:
            out = torch.empty(self.out_pixels, dtype=torch.float32, device=self.device)
        check(self.lib.ap_render_psf_derivative(self.handle, _ptr(params), _ptr(psf), _ptr(dpsf.contiguous()),
                                                _ptr(out), _stream()), "ap_render_psf_derivative")
        return out

    GRID_KNOBS = ("sample", "integrate", "conv", "psf")

    def autotune(self, params: torch.Tensor, psf: Optional[torch.Tensor], jacobian: bool = True):
        """Pick the persistent-grid sizes of the render pass by timing it (ap_batch_autotune)."""
        params = params.to(self.device, torch.float64).contiguous()
        chosen = (ctypes.c_int32 * 4)()
        ms = ctypes.c_double()
        check(self.lib.ap_batch_autotune(self.handle, _ptr(params), _ptr(psf), 1 if jacobian else 0, chosen,
                                         ctypes.byref(ms), _stream()), "ap_batch_autotune")
        return {"blocks_per_sm": dict(zip(self.GRID_KNOBS, list(chosen))), "render_pass_ms": ms.value}

    def set_grid(self, blocks_per_sm):
        arr = (ctypes.c_int32 * 4)(*[int(blocks_per_sm[k]) for k in self.GRID_KNOBS])
        check(self.lib.ap_batch_set_grid(self.handle, arr), "ap_batch_set_grid")

    def set_threshold_window(self, windows):
        """Window [x0, y0, nx, ny] per stamp (working-pixel indices) whose samples an exponential
        stamp's integration threshold sums (see ap_batch_set_threshold_window)."""
        arr = np.ascontiguousarray(np.broadcast_to(np.asarray(windows, dtype=np.int32), (self.n, 4)))
        check(self.lib.ap_batch_set_threshold_window(self.handle, arr.ctypes.data_as(_PI32)), "threshold window")

    def set_threshold_numel(self, numel):
        """Pixel count of each stamp's integration threshold (see ap_batch_set_threshold_numel)."""
        arr = np.ascontiguousarray(np.broadcast_to(np.asarray(numel, dtype=np.float64), (self.n,)))
        check(self.lib.ap_batch_set_threshold_numel(self.handle, arr.ctypes.data_as(_PD)), "threshold numel")

    def jacobian(self, params: torch.Tensor, psf: Optional[torch.Tensor], as_representation=True,
                 model: Optional[torch.Tensor] = None, jac: Optional[torch.Tensor] = None):
        """(model [out_pixels], jac [n_free][out_pixels]); ``model`` / ``jac`` may be given
        (contiguous float32 of those sizes) to be written in place."""
        params = params.to(self.device, torch.float64).contiguous()
        if model is None:
            model = torch.empty(self.out_pixels, dtype=torch.float32, device=self.device)
        if jac is None:
            jac = torch.empty((max(self.n_free, 1), self.out_pixels), dtype=torch.float32, device=self.device)
        check(
            self.lib.ap_jacobian(
                self.handle, _ptr(params), _ptr(psf), _ptr(model), _ptr(jac), 1 if as_representation else 0, _stream()
            ),
            "ap_jacobian",
        )
        return model, jac[: self.n_free]

    def vjp(self, params: torch.Tensor, psf: Optional[torch.Tensor], grad_model: torch.Tensor, as_representation=False,
            reference_center=False):
        """Adjoint of :meth:`render`: [n, n_free] float64 = sum_pixels grad_model * d model / d theta.
        ``reference_center`` adds the sampling-coordinate path to the center entries under
        PSF shift, as the reference's reverse-mode autograd does."""
        params = params.to(self.device, torch.float64).contiguous()
        g = grad_model.to(self.device, torch.float32).contiguous()
        out = torch.empty((self.n, max(self.n_free, 1)), dtype=torch.float64, device=self.device)
        flags = (VJP_REPRESENTATION if as_representation else 0) | (VJP_REFERENCE_CENTER if reference_center else 0)
        check(self.lib.ap_render_vjp(self.handle, _ptr(params), _ptr(psf), _ptr(g), flags,
                                     _ptr(out), _stream()), "ap_render_vjp")
        return out[:, : self.n_free]

    def reference_init(self, data: torch.Tensor, mask: Optional[torch.Tensor] = None,
                       params: Optional[torch.Tensor] = None, known_mask: int = 0):
        """The reference's ``initialize()`` values of every stamp (see ap_reference_init):
        returns (params [n, 8] float64 value space, status [n] int32 of AP_INIT_* bits).
        ``params`` supplies the slots whose bit is set in ``known_mask``."""
        data = data.to(self.device, torch.float32).contiguous()
        if mask is not None:
            mask = mask.to(self.device, torch.uint8).contiguous()
        out = (torch.zeros((self.n, 8), dtype=torch.float64, device=self.device) if params is None
               else params.to(self.device, torch.float64).clone().contiguous())
        status = torch.zeros(self.n, dtype=torch.int32, device=self.device)
        nbytes = ctypes.c_int64(0)
        check(self.lib.ap_reference_init_workspace_bytes(self.handle, ctypes.byref(nbytes)), "init workspace")
        ws = torch.empty(max(int(nbytes.value), 1), dtype=torch.uint8, device=self.device)
        check(self.lib.ap_reference_init(self.handle, _ptr(data), _ptr(mask), int(known_mask), _ptr(out), _ptr(status),
                                         _ptr(ws), ws.numel(), _stream()), "ap_reference_init")
        return out, status

    def psf_shift(self, params: torch.Tensor, psf: torch.Tensor, derivatives=True):
        params = params.to(self.device, torch.float64).contiguous()
        out = torch.zeros((self.n, self.psf_stride), dtype=torch.float32, device=self.device)
        dout = torch.zeros((self.n, 2, self.psf_stride), dtype=torch.float32, device=self.device) if derivatives else None
        check(self.lib.ap_psf_shift(self.handle, _ptr(params), _ptr(psf), _ptr(out), _ptr(dout), _stream()), "ap_psf_shift")
        return out, dout

    def chi2(self, data, weight, mask, model) -> torch.Tensor:
        out = torch.empty(self.n, dtype=torch.float64, device=self.device)
        check(
            self.lib.ap_chi2(self.handle, _ptr(data), _ptr(weight), _ptr(mask), _ptr(model), _ptr(out), _stream()),
            "ap_chi2",
        )
        return out

    def lm_fit(self, data, weight, mask, psf, fixed_params, state0, lm_options: ApLMOptions):
        """Batched LM.  Returns (state [n, n_free] rep space, chi2/ndf [n], iters [n], status [n])."""
        nbytes = ctypes.c_int64()
        check(self.lib.ap_lm_workspace_bytes(self.handle, ctypes.byref(lm_options), ctypes.byref(nbytes)), "lm ws")
        if self._lm_ws is None or self._lm_ws.numel() < nbytes.value:
            self._lm_ws = torch.empty(max(nbytes.value, 256), dtype=torch.uint8, device=self.device)
        self._lm_max_iter = lm_options.max_iter
        state = state0.to(self.device, torch.float64).contiguous().clone()
        fixed = fixed_params.to(self.device, torch.float64).contiguous()
        chi2 = torch.empty(self.n, dtype=torch.float64, device=self.device)
        iters = torch.empty(self.n, dtype=torch.int32, device=self.device)
        status = torch.empty(self.n, dtype=torch.int32, device=self.device)
        check(
            self.lib.ap_lm_fit(
                self.handle,
                _ptr(data),
                _ptr(weight),
                _ptr(mask),
                _ptr(psf),
                _ptr(fixed),
                _ptr(state),
                ctypes.byref(lm_options),
                _ptr(self._lm_ws),
                nbytes.value,
                _ptr(chi2),
                _ptr(iters),
                _ptr(status),
                _stream(),
            ),
            "ap_lm_fit",
        )
        return state, chi2, iters, status

    def lm_history(self):
        """(loss [n, H], L [n, H], states [n, H, 8]) of the last :meth:`lm_fit` (device views)."""
        loss, lam, xs = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        hl = ctypes.c_int32()
        check(self.lib.ap_lm_history(self.handle, ctypes.byref(loss), ctypes.byref(lam), ctypes.byref(xs), ctypes.byref(hl)), "history")
        H = hl.value
        base = self._lm_ws
        def view(ptr, shape):
            off = ptr.value - base.data_ptr()
            count = int(np.prod(shape))
            return base[off : off + 8 * count].view(torch.float64).view(*shape)
        return view(loss, (self.n, H)), view(lam, (self.n, H)), view(xs, (self.n, H, 8))

    KERNEL_CLASSES = ("setup", "psf_shift", "sample", "select", "integrate", "conv", "reduce", "lm_update")

    def profile(self, enable=True):
        check(self.lib.ap_batch_profile(self.handle, 1 if enable else 0), "profile")

    def kernel_times(self):
        ms = (ctypes.c_double * 8)()
        n = (ctypes.c_int64 * 8)()
        check(self.lib.ap_batch_kernel_times(self.handle, ms, n), "kernel times")
        return {k: (ms[i], n[i]) for i, k in enumerate(self.KERNEL_CLASSES)}

    def work_counters(self, reset=False):
        out = (ctypes.c_uint64 * 6)()
        check(self.lib.ap_batch_work_counters(self.handle, out, 1 if reset else 0, _stream()), "work counters")
        return {"conv_flops": out[0], "integrate_samples": out[1], "sample_samples": out[2],
                "integrate_samples_diff": out[3], "integrate_samples_jacobian": out[4]}

    def stats(self):
        out = (ctypes.c_int64 * 5)()
        check(self.lib.ap_batch_stats(self.handle, out), "stats")
        return {"queue": out[0], "fp64_redecisions": out[1], "overflow": out[2], "rounds": out[3],
                "fp64_integrate": out[4]}


def sample_probe_rate(kind: int, iters=2048, blocks=None) -> float:
    """Measured samples/s of the integration's sample arithmetic (:func:`ap_sample_probe`; kind
    0 plain, 1 with partials, 2 as a difference) on this GPU."""
    dev = torch.cuda.current_device()
    nsm = torch.cuda.get_device_properties(dev).multi_processor_count
    blocks = blocks or nsm * 8
    scratch = torch.empty(blocks * 256, dtype=torch.float32, device="cuda")
    L = lib()
    s = _stream()
    for _ in range(2):
        check(L.ap_sample_probe(kind, _ptr(scratch), 32, blocks, s), "sample probe")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = 0.0
    for _ in range(5):
        e0.record()
        check(L.ap_sample_probe(kind, _ptr(scratch), iters, blocks, s), "sample probe")
        e1.record()
        torch.cuda.synchronize()
        best = max(best, blocks * 256 * 4 * iters / (e0.elapsed_time(e1) * 1e-3))
    return best


def fma_probe_tflops(iters=4096, blocks=None) -> float:
    """Measured FP32 FMA throughput (TFLOP/s) of this GPU from :func:`ap_fma_probe`."""
    dev = torch.cuda.current_device()
    nsm = torch.cuda.get_device_properties(dev).multi_processor_count
    blocks = blocks or nsm * 8
    scratch = torch.empty(blocks * 256, dtype=torch.float32, device="cuda")
    L = lib()
    s = _stream()
    for _ in range(2):
        check(L.ap_fma_probe(_ptr(scratch), 64, blocks, s), "fma probe")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = 0.0
    for _ in range(5):
        e0.record()
        check(L.ap_fma_probe(_ptr(scratch), iters, blocks, s), "fma probe")
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        flops = 2.0 * 8 * 16 * iters * blocks * 256
        best = max(best, flops / (ms * 1e-3) / 1e12)
    return best


def values_to_rep(values: torch.Tensor, free_mask: int) -> torch.Tensor:
    """[n, 8] value-space rows (device) -> [n, n_free] representation rows, on the device."""
    values = values.to(torch.float64).contiguous()
    n = values.shape[0]
    out = torch.empty((n, bin(free_mask).count("1")), dtype=torch.float64, device=values.device)
    check(lib().ap_values_to_rep(_ptr(values), n, int(free_mask), _ptr(out), _stream()), "ap_values_to_rep")
    return out


def damped_solve(hess: torch.Tensor, grad: torch.Tensor, L: torch.Tensor) -> torch.Tensor:
    """Batched ``LM._h`` (fit/lm.py:361-371) on the device: hess [m, p, p], grad [m, p], L [m]."""
    hess = hess.to(torch.float64).contiguous()
    grad = grad.to(torch.float64).contiguous()
    L = L.to(torch.float64).contiguous()
    m, p = grad.shape
    h = torch.empty_like(grad)
    check(lib().ap_damped_solve(m, p, _ptr(hess), _ptr(grad), _ptr(L), _ptr(h), _stream()), "ap_damped_solve")
    return h
