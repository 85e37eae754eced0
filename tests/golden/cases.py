"""Load the golden cases written by ``make_golden.py`` into plain Python objects.

No reference import here: the golden ``.npz`` files carry every input.
"""

from __future__ import annotations

import glob
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def render_case_names():
    return sorted(os.path.basename(p)[len("render_") : -len(".npz")] for p in glob.glob(os.path.join(HERE, "render_*.npz")))


def lm_case_names():
    return sorted(os.path.basename(p)[: -len(".npz")] for p in glob.glob(os.path.join(HERE, "lm_*.npz")))


def load_render(name):
    z = np.load(os.path.join(HERE, f"render_{name}.npz"))
    d = {k: z[k] for k in z.files}
    d["spec"] = json.loads(str(d["spec"]))
    return d


def load_lm(name):
    z = np.load(os.path.join(HERE, f"{name}.npz"))
    d = {k: z[k] for k in z.files}
    d["spec"] = json.loads(str(d["spec"]))
    d["message"] = str(d["message"])
    return d


def vjp_case_names():
    return sorted(os.path.basename(p)[: -len(".npz")] for p in glob.glob(os.path.join(HERE, "vjp_*.npz")))


def load_vjp(name):
    z = np.load(os.path.join(HERE, f"{name}.npz"))
    d = {k: z[k] for k in z.files}
    d["spec"] = json.loads(str(d["spec"]))
    return d


def group_case_names():
    return sorted(os.path.basename(p)[: -len(".npz")] for p in glob.glob(os.path.join(HERE, "group_*.npz")))


def load_group(name):
    z = np.load(os.path.join(HERE, f"{name}.npz"))
    d = {k: z[k] for k in z.files}
    d["spec"] = json.loads(str(d["spec"]))
    d["message"] = str(d["message"])
    return d


def adjoint_case_names():
    return sorted(os.path.basename(p)[: -len(".npz")] for p in glob.glob(os.path.join(HERE, "adjoint_*.npz")))


def load_adjoint(name):
    z = np.load(os.path.join(HERE, f"{name}.npz"))
    d = {k: z[k] for k in z.files}
    d["spec"] = json.loads(str(d["spec"]))
    return d



def init_case_names():
    return sorted(os.path.basename(p)[: -len(".npz")] for p in glob.glob(os.path.join(HERE, "init_*.npz")))


def load_init(name):
    """A reference ``initialize()`` case: data, mask (None when absent), spec (kind, nx, ny,
    scale, given values) and the reference's values under ``value_<name>``."""
    z = np.load(os.path.join(HERE, f"{name}.npz"))
    d = {k: z[k] for k in z.files}
    d["spec"] = json.loads(str(d["spec"]))
    d["mask"] = d["mask"] if d["mask"].size else None
    return d


def iter_case_names():
    return sorted(os.path.basename(p)[: -len(".npz")] for p in glob.glob(os.path.join(HERE, "iterlm_*.npz")))


def load_iter(name):
    """An ``Iter_LM`` case: its spec (group case, chunks, method, max_iter) and the reference's
    outer loss / state histories, final state and message."""
    z = np.load(os.path.join(HERE, f"{name}.npz"))
    d = {k: z[k] for k in z.files}
    d["spec"] = json.loads(str(d["spec"]))
    d["message"] = str(d["message"])
    return d


def segmap_case_names():
    return sorted(os.path.basename(p)[: -len(".npz")] for p in glob.glob(os.path.join(HERE, "segmap_*.npz")))


def load_segmap(name):
    """A segmentation-map case: seg (int32), image, and the reference helpers' outputs per id."""
    z = np.load(os.path.join(HERE, f"{name}.npz"))
    d = {k: z[k] for k in z.files}
    d["spec"] = json.loads(str(d["spec"]))
    return d


def upscale_case_names():
    return sorted(os.path.basename(p)[: -len(".npz")] for p in glob.glob(os.path.join(HERE, "upscale_*.npz")))


def load_upscale(name):
    """A model whose PSF image has pixels ``upscale`` times finer than the image's: the inputs
    (psf at the fine scale, data, weight, truth / initial values) and the reference's model,
    representation Jacobian and LM trajectory."""
    z = np.load(os.path.join(HERE, f"{name}.npz"))
    d = {k: z[k] for k in z.files}
    d["spec"] = json.loads(str(d["spec"]))
    d["message"] = str(d["message"])
    return d
