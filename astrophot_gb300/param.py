"""Parameter objects with the reference's vector API (``astrophot/param/``).

``Parameter_Node`` keeps a value (float64 tensor), limits, a cyclic flag, a lock, an
uncertainty and links to other nodes, and exposes the flattened ``vector_*`` views the
fitter works with (``param/parameter.py:169-420``): values of the unlocked leaves in link
order, their representation (unbounded, ``transforms``), masks and identities.  Values are
checked against the limits on assignment and raise ``InvalidParameter`` outside them
(``param/parameter.py:422-450``).
"""

from __future__ import annotations

from collections import OrderedDict
from typing import Optional

import numpy as np
import torch

from . import config
from .errors import InvalidParameter
from .transforms import to_rep, to_value

__all__ = ("Parameter_Node", "Param_Unlock", "Param_SoftLimits", "Param_Mask")


def _tensor(v):
    return torch.as_tensor(v, dtype=config.ap_dtype, device="cpu").clone()


class Parameter_Node:
    """A leaf (holds a value) or a branch (links other nodes)."""

    global_unlock = False

    def __init__(self, name, value=None, limits=(None, None), cyclic=False, locked=False, units="none",
                 uncertainty=None, shape=None, **kwargs):
        if ":" in name:
            raise ValueError(f"Node names must not have ':' character. Cannot use name: {name}")
        self.name = name
        self.nodes = OrderedDict()
        self._value = None
        self._mask = None
        self.locked = False
        self.limits = limits
        self.cyclic = bool(cyclic)
        self.units = units
        self._shape = shape
        if value is not None:
            self.value = value
        self.uncertainty = uncertainty
        self.locked = bool(locked)

    # ---- structure ---------------------------------------------------------------------
    @property
    def identity(self):
        return id(self)

    @property
    def leaf(self):
        return len(self.nodes) == 0

    def link(self, *nodes):
        for node in nodes:
            for sub in node.flat(include_locked=True, include_links=True).values():
                if sub is self:
                    raise InvalidParameter("Parameter structure must be Directed Acyclic Graph!")
            self.nodes[node.name] = node

    def unlink(self, *nodes):
        for node in nodes:
            del self.nodes[node.name]

    def __getitem__(self, key):
        if key == self.name:
            return self
        if key in self.nodes:
            return self.nodes[key]
        if isinstance(key, str) and ":" in key:
            base, stem = key.split(":", 1)
            return self.nodes[base][stem]
        raise KeyError(f"Unrecognized key for '{self.name}': {key}")

    def __contains__(self, key):
        return key in self.nodes

    def __iter__(self):
        return filter(lambda n: not n.locked, self.nodes.values())

    def flat(self, include_locked=True, include_links=False):
        """Leaf nodes reachable from here, in link order (``param/base.py:170-191``)."""
        out = OrderedDict()
        if self.leaf and self.value is not None:
            if (not self.locked) or include_locked or Parameter_Node.global_unlock:
                out[self.identity] = self
        for node in self.nodes.values():
            if node.locked and not (include_locked or Parameter_Node.global_unlock):
                continue
            if node.leaf and node.value is not None:
                out[node.identity] = node
            else:
                if include_links:
                    out[node.identity] = node
                out.update(node.flat(include_locked))
        return out

    # ---- value ---------------------------------------------------------------------------
    @property
    def limits(self):
        return self._limits

    @limits.setter
    def limits(self, limits):
        lo, hi = limits
        self._limits = (None if lo is None else float(lo), None if hi is None else float(hi))

    @property
    def value(self):
        if isinstance(self._value, Parameter_Node):
            return self._value.value
        return self._value

    @value.setter
    def value(self, val):
        if self.locked and not Parameter_Node.global_unlock:
            return
        if val is None:
            self._value = None
            return
        if isinstance(val, Parameter_Node):
            self._value = val
            self.nodes = OrderedDict()
            self.link(val)
            return
        if len(self.nodes) > 0:
            self.vector_set_values(val)
            return
        self._set_val_self(val)

    def _set_val_self(self, val):
        v = _tensor(val)
        if self._shape is not None:
            v = v.reshape(self._shape)
        self._value = v
        lo, hi = self.limits
        if self.cyclic:
            self._value = lo + torch.remainder(self._value - lo, hi - lo)
            return
        if lo is not None and not torch.all(self._value > lo):
            raise InvalidParameter(f"{self.name} has lower limit {lo}")
        if hi is not None and not torch.all(self._value < hi):
            raise InvalidParameter(f"{self.name} has upper limit {hi}")

    def _soft_set_val_self(self, val):
        v = _tensor(val)
        lo, hi = self.limits
        if self.cyclic:
            self._value = lo + torch.remainder(v - lo, hi - lo)
            return
        if lo is not None:
            v = torch.maximum(v, torch.full_like(v, lo + 1e-3))
        if hi is not None:
            v = torch.minimum(v, torch.full_like(v, hi - 1e-3))
        self._value = v

    @property
    def uncertainty(self):
        return self._uncertainty

    @uncertainty.setter
    def uncertainty(self, unc):
        self._uncertainty = None if unc is None else _tensor(unc)

    @property
    def shape(self):
        v = self.value
        return None if v is None else tuple(v.shape)

    @property
    def size(self):
        if self.leaf:
            return int(self.value.numel())
        return int(self.vector_values().numel())

    def __len__(self):
        return self.size

    # ---- vector API (param/parameter.py:169-420) ----------------------------------------
    def _leaves(self):
        return list(self.flat(include_locked=False, include_links=False).values())

    @property
    def mask(self):
        if not self.leaf:
            return self.vector_mask()
        if self._mask is not None:
            return self._mask
        return torch.ones(self.value.numel(), dtype=torch.bool)

    def vector_mask(self):
        if self.leaf:
            return self.mask.flatten()
        vec = [node.vector_mask() for node in self._leaves()]
        return torch.cat(vec) if vec else torch.zeros(0, dtype=torch.bool)

    def vector_set_mask(self, mask):
        mask = torch.as_tensor(mask, dtype=torch.bool)
        if self.leaf:
            self._mask = mask.reshape(-1)
            return
        loc = 0
        for node in self._leaves():
            node.vector_set_mask(mask[loc : loc + node.size])
            loc += node.size

    def vector_values(self):
        if self.leaf:
            return self.value.flatten()[self.mask]
        vec = [node.vector_values() for node in self._leaves()]
        return torch.cat(vec) if vec else torch.zeros(0, dtype=config.ap_dtype)

    def vector_identities(self):
        if self.leaf:
            ids = np.array([f"{self.identity}:{i}" for i in range(self.value.numel())])
            return ids[self.mask.numpy()]
        vec = [node.vector_identities() for node in self._leaves()]
        return np.concatenate(vec) if vec else np.array(())

    def vector_names(self):
        if self.leaf:
            n = self.value.numel()
            names = np.array([self.name] if n == 1 else [f"{self.name}:{i}" for i in range(n)])
            return names[self.mask.numpy()]
        vec = [node.vector_names() for node in self._leaves()]
        return np.concatenate(vec) if vec else np.array(())

    def vector_uncertainty(self):
        if self.leaf:
            if self._uncertainty is None:
                self._uncertainty = torch.ones_like(self.value)
            return (self._uncertainty * torch.ones_like(self.value)).flatten()[self.mask]
        vec = [node.vector_uncertainty() for node in self._leaves()]
        return torch.cat(vec) if vec else torch.zeros(0, dtype=config.ap_dtype)

    def _split(self, vec):
        vec = _tensor(vec).flatten()
        out, loc = [], 0
        for node in self._leaves():
            k = int(node.vector_mask().sum())
            out.append((node, vec[loc : loc + k]))
            loc += k
        return out

    def vector_set_values(self, values):
        if self.leaf:
            v = self.value.clone().flatten()
            v[self.mask] = _tensor(values).flatten()
            self._set_val_self(v.reshape(self.value.shape))
            return
        for node, part in self._split(values):
            node.vector_set_values(part)

    def vector_set_uncertainty(self, unc):
        if self.leaf:
            u = (self._uncertainty if self._uncertainty is not None else torch.ones_like(self.value)).clone().flatten()
            u[self.mask] = _tensor(unc).flatten()
            self._uncertainty = u.reshape(self.value.shape)
            return
        for node, part in self._split(unc):
            node.vector_set_uncertainty(part)

    def vector_transform_val_to_rep(self, val):
        if self.leaf:
            return _tensor(to_rep(self.limits, self.cyclic, _tensor(val).numpy()))
        parts = [node.vector_transform_val_to_rep(p) for node, p in self._split(val)]
        return torch.cat(parts) if parts else torch.zeros(0, dtype=config.ap_dtype)

    def vector_transform_rep_to_val(self, rep):
        if self.leaf:
            return _tensor(to_value(self.limits, self.cyclic, _tensor(rep).numpy()))
        parts = [node.vector_transform_rep_to_val(p) for node, p in self._split(rep)]
        return torch.cat(parts) if parts else torch.zeros(0, dtype=config.ap_dtype)

    def vector_representation(self):
        return self.vector_transform_val_to_rep(self.vector_values())

    def vector_set_representation(self, rep):
        self.vector_set_values(self.vector_transform_rep_to_val(rep))

    # ---- state ---------------------------------------------------------------------------
    def get_state(self):
        state = {"name": self.name, "identity": self.identity}
        if self.locked:
            state["locked"] = True
        if self.leaf and self.value is not None:
            state["value"] = self.value.tolist()
            state["units"] = self.units
            if self.limits != (None, None):
                state["limits"] = list(self.limits)
            if self.cyclic:
                state["cyclic"] = True
            if self.uncertainty is not None:
                state["uncertainty"] = self.uncertainty.tolist()
        if self.nodes:
            state["nodes"] = [n.get_state() for n in self.nodes.values()]
        return state

    def __repr__(self):
        if self.leaf:
            return f"{self.name}: {None if self.value is None else self.value.tolist()} [{self.units}]"
        return self.name + ":\n" + "\n".join(repr(n) for n in self.nodes.values())


class Param_Unlock:
    """Temporarily unlock one parameter, or all of them (``param/param_context.py:6-31``)."""

    def __init__(self, param=None):
        self.param = param

    def __enter__(self):
        if self.param is None:
            Parameter_Node.global_unlock = True
        else:
            self.original = self.param.locked
            self.param.locked = False

    def __exit__(self, *a):
        if self.param is None:
            Parameter_Node.global_unlock = False
        else:
            self.param.locked = self.original


class Param_SoftLimits:
    """Values outside the limits are pushed 1e-3 inside instead of raising
    (``param/param_context.py:34-59``)."""

    def __init__(self, param):
        self.param = param

    def __enter__(self):
        self.original = self.param._set_val_self
        self.param._set_val_self = self.param._soft_set_val_self

    def __exit__(self, *a):
        self.param._set_val_self = self.original


class Param_Mask:
    """Temporarily hide vector elements (``param/param_context.py:62-102``)."""

    def __init__(self, param, new_mask):
        self.param = param
        self.new_mask = torch.as_tensor(new_mask, dtype=torch.bool)

    def __enter__(self):
        self.old_mask = self.param.vector_mask().clone()
        mask = self.old_mask.clone()
        mask[mask.clone()] = self.new_mask
        self.param.vector_set_mask(mask)

    def __exit__(self, *a):
        self.param.vector_set_mask(self.old_mask)
