"""Segmentation-map helpers with the reference's interface
(``astrophot/utils/initialize/segmentation_map.py``): windows, centroids, position angles and
axis ratios of every segment, computed on the GPU (``ap_segmap_*`` in the C ABI), plus the
window arithmetic (``scale_windows``, ``filter_windows`` with GPU window fluxes,
``transfer_windows``).  Maps and images may be arrays or ``.fits`` / ``.npy`` file names.
Results are dictionaries keyed by segment id, in ``np.unique`` order, as the reference returns.
"""

from __future__ import annotations

from copy import deepcopy
from typing import Optional

import numpy as np
import torch

from . import _native as N

__all__ = ("centroids_from_segmentation_map", "PA_from_segmentation_map", "q_from_segmentation_map",
           "windows_from_segmentation_map", "scale_windows", "filter_windows", "transfer_windows",
           "segment_statistics")


def _select_img(img, hduli=0):
    """``_select_img`` (segmentation_map.py:21-30): an array, or a .fits / .npy file."""
    if isinstance(img, str):
        if img.endswith(".fits"):
            from .fits_io import read_hdus

            return read_hdus(img)[hduli][0]
        if img.endswith(".npy"):
            return np.load(img)
        raise ValueError(f"unrecognized file type, should be one of: fits, npy\n{img}")
    return img


def segment_statistics(seg_map, image=None, skip_index=(0,), north=np.pi / 2, centroids=None, PAs=None,
                       device="cuda"):
    """ids [n] (np.unique order, ``skip_index`` left out), bbox [n, 4] (xmin, xmax, ymin, ymax),
    centroid [n, 2], pa [n], q [n] of every segment, from two passes over the map on the GPU.
    ``centroids`` / ``PAs`` (dicts by id) replace the computed ones as the reference's
    arguments do."""
    lib = N.lib()
    seg = np.ascontiguousarray(np.asarray(seg_map), dtype=np.int32)
    ny, nx = seg.shape
    img = np.zeros(seg.shape, np.float32) if image is None else np.ascontiguousarray(np.asarray(image), dtype=np.float32)
    dev = torch.device(device)
    seg_d = torch.from_numpy(seg).to(dev)
    img_d = torch.from_numpy(img).to(dev)
    mm = torch.empty(2, dtype=torch.int32, device=dev)
    N.check(lib.ap_segmap_range(N._ptr(seg_d), seg.size, N._ptr(mm), N._stream()), "ap_segmap_range")
    lo, hi = (int(v) for v in mm.cpu())
    if lo < 0:
        raise ValueError("segment ids must be non-negative")
    present = torch.empty(hi + 1, dtype=torch.uint8, device=dev)
    N.check(lib.ap_segmap_present(N._ptr(seg_d), seg.size, hi, N._ptr(present), N._stream()), "ap_segmap_present")
    ids = [i for i in np.nonzero(present.cpu().numpy())[0].tolist() if i not in skip_index]
    n = len(ids)
    index = np.full(hi + 1, -1, dtype=np.int32)
    index[ids] = np.arange(n, dtype=np.int32)
    index_d = torch.from_numpy(index).to(dev)
    acc = torch.empty((max(n, 1), 5), dtype=torch.float64, device=dev)
    bbox = torch.empty((max(n, 1), 4), dtype=torch.int32, device=dev)
    cen = torch.empty((max(n, 1), 2), dtype=torch.float64, device=dev)
    pa = torch.empty(max(n, 1), dtype=torch.float64, device=dev)
    q = torch.empty(max(n, 1), dtype=torch.float64, device=dev)
    cen_in = None if centroids is None else torch.tensor([centroids[i] for i in ids], dtype=torch.float64, device=dev)
    pa_in = None if PAs is None else torch.tensor([PAs[i] for i in ids], dtype=torch.float64, device=dev)
    N.check(lib.ap_segmap_stats(N._ptr(seg_d), N._ptr(img_d), nx, ny, N._ptr(index_d), n, float(north), N._ptr(cen_in),
                                N._ptr(pa_in), N._ptr(acc), N._ptr(bbox), N._ptr(cen), N._ptr(pa), N._ptr(q),
                                N._stream()), "ap_segmap_stats")
    return dict(ids=ids, bbox=bbox[:n].cpu().numpy(), centroid=cen[:n].cpu().numpy(), pa=pa[:n].cpu().numpy(),
                q=q[:n].cpu().numpy())


def centroids_from_segmentation_map(seg_map, image, hdul_index_seg=0, hdul_index_img=0, skip_index=(0,)):
    """``centroids_from_segmentation_map`` (segmentation_map.py:33-73): flux-weighted pixel
    (x, y) of every segment."""
    st = segment_statistics(_select_img(seg_map, hdul_index_seg), _select_img(image, hdul_index_img), skip_index)
    return {i: st["centroid"][k].tolist() for k, i in enumerate(st["ids"])}


def PA_from_segmentation_map(seg_map, image, centroids=None, hdul_index_seg=0, hdul_index_img=0, skip_index=(0,),
                             north=np.pi / 2):
    """``PA_from_segmentation_map`` (segmentation_map.py:76-106): angular centre of light about
    the centroid, plus north."""
    st = segment_statistics(_select_img(seg_map, hdul_index_seg), _select_img(image, hdul_index_img), skip_index,
                            north, centroids=centroids)
    return {i: float(st["pa"][k]) for k, i in enumerate(st["ids"])}


def q_from_segmentation_map(seg_map, image, centroids=None, PAs=None, hdul_index_seg=0, hdul_index_img=0,
                            skip_index=(0,), north=np.pi / 2):
    """``q_from_segmentation_map`` (segmentation_map.py:109-143): ``axis_ratio_com`` at PA + north."""
    st = segment_statistics(_select_img(seg_map, hdul_index_seg), _select_img(image, hdul_index_img), skip_index,
                            north, centroids=centroids, PAs=PAs)
    return {i: float(st["q"][k]) for k, i in enumerate(st["ids"])}


def windows_from_segmentation_map(seg_map, hdul_index=0, skip_index=(0,)):
    """``windows_from_segmentation_map`` (segmentation_map.py:146-180): the bounding box
    [[xmin, xmax], [ymin, ymax]] of every segment."""
    st = segment_statistics(_select_img(seg_map, hdul_index), None, skip_index)
    return {i: [[int(b[0]), int(b[1])], [int(b[2]), int(b[3])]] for i, b in zip(st["ids"], st["bbox"])}


def scale_windows(windows, image_shape=None, expand_scale=1.0, expand_border=0.0):
    """``scale_windows`` (segmentation_map.py:183-214): grow each window about its centre by
    ``expand_scale`` and ``expand_border`` on every side, clipped to ``image_shape``."""
    out = {}
    for index in list(windows.keys()):
        w = deepcopy(windows[index])
        cx, cy = (w[0][0] + w[0][1]) / 2, (w[1][0] + w[1][1]) / 2
        sx, sy = w[0][1] - w[0][0], w[1][1] - w[1][0]
        w = [[int(cx - expand_scale * sx / 2 - expand_border), int(cx + expand_scale * sx / 2 + expand_border)],
             [int(cy - expand_scale * sy / 2 - expand_border), int(cy + expand_scale * sy / 2 + expand_border)]]
        if image_shape is not None:
            w = [[max(0, w[0][0]), min(image_shape[1], w[0][1])], [max(0, w[1][0]), min(image_shape[0], w[1][1])]]
        out[index] = w
    return out


def filter_windows(windows, min_size=None, max_size=None, min_area=None, max_area=None, min_flux=None,
                   max_flux=None, image=None):
    """``filter_windows`` (segmentation_map.py:217-293); window fluxes summed on the GPU."""
    keys = list(windows.keys())
    flux = {}
    if (min_flux is not None or max_flux is not None) and keys:
        img = np.ascontiguousarray(np.asarray(image), dtype=np.float32)
        ny, nx = img.shape
        wins = np.array([[windows[k][0][0], windows[k][0][1], windows[k][1][0], windows[k][1][1]] for k in keys],
                        dtype=np.int32)
        img_d = torch.from_numpy(img).cuda()
        wins_d = torch.from_numpy(wins).cuda()
        out = torch.empty(len(keys), dtype=torch.float64, device="cuda")
        N.check(N.lib().ap_window_flux(N._ptr(img_d), nx, ny, N._ptr(wins_d), len(keys), N._ptr(out), N._stream()),
                "ap_window_flux")
        flux = dict(zip(keys, out.cpu().numpy().tolist()))
    new = {}
    for w in keys:
        (x0, x1), (y0, y1) = windows[w]
        if min_size is not None and min(x1 - x0, y1 - y0) < min_size:
            continue
        if max_size is not None and max(x1 - x0, y1 - y0) > max_size:
            continue
        if min_area is not None and (x1 - x0) * (y1 - y0) < min_area:
            continue
        if max_area is not None and (x1 - x0) * (y1 - y0) > max_area:
            continue
        if min_flux is not None and flux[w] < min_flux:
            continue
        if max_flux is not None and flux[w] > max_flux:
            continue
        new[w] = windows[w]
    return new


def transfer_windows(windows, base_image, new_image):
    """``transfer_windows`` (segmentation_map.py:296-342): the windows in another image's pixel
    grid (corners through the plane, outward-rounded, clipped to the new image)."""
    out = {}
    # the reference clips at Image.shape - 1, the window's (width, height) in plane units
    # (image/window_object.py:166-178): in pixels for a unit pixel scale
    P = np.asarray(new_image.window.pixelscale, dtype=np.float64)
    nx, ny = (float(v) for v in new_image.window.pixel_shape)
    hi = np.array([np.linalg.norm(P @ [nx, 0.0]), np.linalg.norm(P @ [0.0, ny])]) - 1
    for w, win in windows.items():
        lo_c = np.floor(np.array(new_image.plane_to_pixel(*base_image.pixel_to_plane(win[0][0], win[1][0]))))
        hi_c = np.ceil(np.array(new_image.plane_to_pixel(*base_image.pixel_to_plane(win[0][1], win[1][1]))))
        lo_c = np.clip(lo_c, 0, hi)
        hi_c = np.clip(hi_c, 0, hi)
        out[w] = [[lo_c[0], hi_c[0]], [lo_c[1], hi_c[1]]]
    return out
