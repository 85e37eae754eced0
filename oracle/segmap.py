"""The reference's segmentation-map helpers restated in float64 numpy.

Test infrastructure only (the checker of the CUDA segment statistics).  Pinned by
``tests/golden/segmap_240x200.npz``, recorded from the reference's own functions
(``astrophot/utils/initialize/segmentation_map.py``).  Segment ids come in ``np.unique`` order,
ids in ``skip`` are left out; pixel coordinates are array indices (x = column, y = row).
"""

from __future__ import annotations

import numpy as np

NORTH = np.pi / 2


def segment_ids(seg, skip=(0,)):
    return [int(i) for i in np.unique(seg) if i not in skip]


def centroids(seg, image, skip=(0,)):
    """``centroids_from_segmentation_map`` (segmentation_map.py:33-73): flux-weighted (x, y)."""
    XX, YY = np.meshgrid(np.arange(seg.shape[1]), np.arange(seg.shape[0]))
    out = {}
    for i in segment_ids(seg, skip):
        N = seg == i
        out[i] = [np.sum(XX[N] * image[N]) / np.sum(image[N]), np.sum(YY[N] * image[N]) / np.sum(image[N])]
    return out


def position_angles(seg, image, cen, skip=(0,), north=NORTH):
    """``PA_from_segmentation_map`` (segmentation_map.py:76-106): the angular centre of light
    (``Angle_COM_PA``, utils/angle_operations.py:35-56) about the centroid, plus north."""
    XX, YY = np.meshgrid(np.arange(seg.shape[1]), np.arange(seg.shape[0]))
    out = {}
    for i in segment_ids(seg, skip):
        N = seg == i
        X, Y, f = XX[N] - cen[i][0], YY[N] - cen[i][1], image[N]
        theta = np.arctan2(Y, X)
        c = np.sum(f * np.cos(2 * theta)) / np.sum(f)
        s = np.sum(f * np.sin(2 * theta)) / np.sum(f)
        out[i] = np.arctan2(s, c) / 2 % np.pi + north
    return out


def axis_ratios(seg, image, cen, pas, skip=(0,), north=NORTH):
    """``q_from_segmentation_map`` (segmentation_map.py:109-143) with ``axis_ratio_com``
    (utils/operations.py:77-91) at angle PA + north: sum f sin^2 / max(sum f sin^2, sum f cos^2)."""
    XX, YY = np.meshgrid(np.arange(seg.shape[1]), np.arange(seg.shape[0]))
    out = {}
    for i in segment_ids(seg, skip):
        N = seg == i
        X, Y, f = XX[N] - cen[i][0], YY[N] - cen[i][1], image[N]
        theta = np.arctan2(Y, X) - (pas[i] + north)
        c = np.sum(f * np.cos(theta) ** 2) / np.sum(f)
        s = np.sum(f * np.sin(theta) ** 2) / np.sum(f)
        out[i] = s / max(s, c)
    return out


def windows(seg, skip=(0,)):
    """``windows_from_segmentation_map`` (segmentation_map.py:146-180): [[xmin, xmax], [ymin, ymax]]."""
    out = {}
    for i in segment_ids(seg, skip):
        Y, X = np.where(seg == i)
        out[i] = [[int(X.min()), int(X.max())], [int(Y.min()), int(Y.max())]]
    return out


def scale_windows(wins, image_shape=None, expand_scale=1.0, expand_border=0.0):
    """``scale_windows`` (segmentation_map.py:183-214)."""
    out = {}
    for i, w in wins.items():
        cx, cy = (w[0][0] + w[0][1]) / 2, (w[1][0] + w[1][1]) / 2
        sx, sy = w[0][1] - w[0][0], w[1][1] - w[1][0]
        nw = [[int(cx - expand_scale * sx / 2 - expand_border), int(cx + expand_scale * sx / 2 + expand_border)],
              [int(cy - expand_scale * sy / 2 - expand_border), int(cy + expand_scale * sy / 2 + expand_border)]]
        if image_shape is not None:
            nw = [[max(0, nw[0][0]), min(image_shape[1], nw[0][1])], [max(0, nw[1][0]), min(image_shape[0], nw[1][1])]]
        out[i] = nw
    return out


def filter_windows(wins, min_size=None, max_size=None, min_area=None, max_area=None, min_flux=None, max_flux=None,
                   image=None):
    """``filter_windows`` (segmentation_map.py:217-293)."""
    out = {}
    for i, w in wins.items():
        dx, dy = w[0][1] - w[0][0], w[1][1] - w[1][0]
        if min_size is not None and min(dx, dy) < min_size:
            continue
        if max_size is not None and max(dx, dy) > max_size:
            continue
        if min_area is not None and dx * dy < min_area:
            continue
        if max_area is not None and dx * dy > max_area:
            continue
        if min_flux is not None or max_flux is not None:
            f = np.sum(image[w[1][0]:w[1][1], w[0][0]:w[0][1]])
            if min_flux is not None and f < min_flux:
                continue
            if max_flux is not None and f > max_flux:
                continue
        out[i] = w
    return out
