"""
Damping parameters and damping-function markers
(``damping/functions.py``, ``damping/parameters/base.py:48-85``).

``dftd4`` uses the rational (Becke-Johnson) damping for the two-body term and
zero damping of order 9 for the ATM term; both are evaluated inside the CUDA
kernels.  The classes here only select the scheme and keep the reference's
parameter rules: ``a1`` and ``a2`` are required (``TypeError`` otherwise,
``functions.py:68-114``), a missing ``s8`` switches the dipole-quadrupole
term off (``functions.py:144-145``), ``s10`` adds the quadrupole-quadrupole
term only when present (``twobody.py:184-197``).
"""

from __future__ import annotations

from typing import Any, Dict

import torch

Param = Dict[str, Any]
"""Damping parameters: s6, s8, s9, s10, a1, a2, alp (floats or 0-d tensors)."""

S6, S8, S9, S10 = 1.0, 1.0, 1.0, 0.0
A1, A2 = 0.4, 5.0
ALP = 16.0

PARAM_ORDER = ("s6", "s8", "s10", "a1", "a2", "s9", "alp")


class Damping:
    """Base class of the damping schemes."""

    radius_type = "r4r2"

    def __eq__(self, other: Any) -> bool:
        return isinstance(other, Damping) and self.__class__ is other.__class__

    def __hash__(self) -> int:
        return hash(self.__class__)


class RationalDamping(Damping):
    """Becke-Johnson rational damping 1 / (r^n + (a1 sqrt(r4r2_ij) + a2)^n)."""

    radius_type = "r4r2"


class ZeroDamping(Damping):
    """Zero (Chai-Head-Gordon) damping; order 9 is the ATM damping."""

    radius_type = "rvdw"


def _value(v) -> float:
    if isinstance(v, torch.Tensor):
        return float(v.detach().reshape(()).item()) if v.device.type == "cpu" else float(v.detach().reshape(()).cpu().item())
    return float(v)


def resolve(param: Param) -> dict:
    """
    The numeric parameter set the kernels take, with the reference's gating.
    Raises ``TypeError`` like ``RationalDamping`` when a1/a2 are missing.
    """
    missing = [k for k in ("a1", "a2") if param.get(k) is None]
    if missing:
        raise TypeError(f"RationalDamping (order 6) requires keyword(s): {', '.join(missing)}")
    out = {
        "s6": _value(param["s6"]) if param.get("s6") is not None else S6,
        "s8": _value(param["s8"]) if param.get("s8") is not None else 0.0,
        "has_s8": param.get("s8") is not None,
        "s10": _value(param["s10"]) if param.get("s10") is not None else 0.0,
        "has_s10": param.get("s10") is not None,
        "a1": _value(param["a1"]),
        "a2": _value(param["a2"]),
        "s9": _value(param["s9"]) if param.get("s9") is not None else S9,
        "alp": _value(param["alp"]) if param.get("alp") is not None else ALP,
    }
    return out
