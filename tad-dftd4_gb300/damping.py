"""
Damping parameters and damping-function selectors
(``damping/functions.py``, ``damping/parameters/base.py:48-85``).

``dftd4`` damps the two-body term with the function passed as
``damping_function`` (rational Becke-Johnson damping by default) and the ATM
term with zero damping of order 9; both run inside the CUDA kernels.  The
classes here select the scheme and keep the reference's parameter rules:

* the orders evaluated: 6 always, 8 unless both ``s8`` and ``rs8`` are
  missing (``functions.py:141-151``), 10 only when the key ``s10`` exists
  (``twobody.py:184-197``);
* each class's required parameters per order (``REQUIRED_BY_ORDER``), a
  missing one raising ``TypeError`` with the reference's message
  (``functions.py:68-114``);
* zero, modified-zero and optimised-power damping have no order 10: an
  ``s10`` entry raises ``ValueError`` (``functions.py:352-356, 408-411,
  468-471``);
* the two-body sum scales the orders by ``s6`` and ``s8`` with defaults 1
  (``twobody.py:176-180``); the ATM radii take ``a1`` / ``a2`` with defaults
  float32(0.4) / 5 (``threebody.py:244-256``: the fallback tensor has torch's
  default dtype), ``s9`` / ``alp`` default to 1 / 16.
"""

from __future__ import annotations

from typing import Any, Dict

import torch

Param = Dict[str, Any]
"""Damping parameters: s6, s8, s9, s10, a1, a2, alp, rs6, rs8, bet (floats or 0-d tensors)."""

S6, S8, S9, S10 = 1.0, 1.0, 1.0, 0.0
A1, A2 = 0.4, 5.0
# The ATM radii's fallback when the parameters carry no a1: tad-dftd4 builds
# it as a tensor in its term object's dtype, torch's default float32
# (threebody.py:250-253), so the value is float32(0.4).
A1_ATM_FALLBACK = 0.4000000059604645
RS6, RS8, RS9 = 1.0, 1.0, 1.0
ALP = 16.0
BET = 0.0

# parameters with a gradient slot in the library's parameter gradient (in this order)
PARAM_ORDER = ("s6", "s8", "s10", "a1", "a2", "s9", "alp", "rs6", "rs8", "bet")

# parameters of the call itself, used as __call__ defaults by the reference
# (functions.py:116-131): s6 = 1, s9 = 1, rs9 = 1, alp = 16, others absent
_CALL_DEFAULTS = {"s6": S6, "s9": S9, "rs9": RS9, "alp": ALP}


class Damping:
    """Base class of the damping schemes."""

    radius_type = "r4r2"
    kind = -1  # d4_damping_kind of the library
    REQUIRED_BY_ORDER: dict = {}
    ORDERS: tuple = (6, 8, 10)

    def __eq__(self, other: Any) -> bool:
        return isinstance(other, Damping) and self.__class__ is other.__class__

    def __hash__(self) -> int:
        return hash(self.__class__)

    def _order_error(self, order: int) -> Exception:  # pragma: no cover - overridden
        return ValueError(f"{type(self).__name__} has no order {order}")


class RationalDamping(Damping):
    """Becke-Johnson rational damping 1 / (r^n + (a1 sqrt(3 r4r2_i r4r2_j) + a2)^n)."""

    radius_type = "r4r2"
    kind = 0
    REQUIRED_BY_ORDER = {6: ("a1", "a2"), 8: ("a1", "a2"), 10: ("a1", "a2")}
    ORDERS = (6, 8, 10)


class ZeroDamping(Damping):
    """Zero (Chai-Head-Gordon) damping f / r^n, f = 1 / (1 + 6 (rs r / rvdw)^alp_n);
    order 9 is the ATM damping."""

    radius_type = "rvdw"
    kind = 1
    REQUIRED_BY_ORDER = {6: ("rs6", "alp"), 8: ("rs8", "alp"), 9: ("rs9", "alp")}
    ORDERS = (6, 8, 9)

    def _order_error(self, order: int) -> Exception:
        return ValueError("Zero-damping is only implemented for order 6, 8, and 9. "
                          f"Got {order} instead.")


class MZeroDamping(Damping):
    """Modified zero damping f / r^n, f = 1 / (1 + 6 (r / (rs rvdw) + bet rvdw)^-alp_n)."""

    radius_type = "rvdw"
    kind = 2
    REQUIRED_BY_ORDER = {6: ("rs6", "alp", "bet"), 8: ("rs8", "alp", "bet")}
    ORDERS = (6, 8)

    def _order_error(self, order: int) -> Exception:
        return ValueError("Zero-damping is only implemented for order 6 and 8.")


class OptimisedPowerDamping(Damping):
    """Optimised-power damping r^bet / (r^bet r^n + R0^bet r^n) with
    R0 = a1 sqrt(3 r4r2_i r4r2_j) + a2 -- the reference's expression, whose
    second term carries r^n where the published form has R0^n."""

    radius_type = "r4r2"
    kind = 3
    REQUIRED_BY_ORDER = {6: ("a1", "a2", "bet"), 8: ("a1", "a2", "bet")}
    ORDERS = (6, 8)

    def _order_error(self, order: int) -> Exception:
        return ValueError("OP-damping is only implemented for order 6 and 8.")


def _value(v) -> float:
    if isinstance(v, torch.Tensor):
        return float(v.detach().reshape(()).cpu().item())
    return float(v)


def _given(param: Param, key: str):
    """The call's value of ``key``: the parameter dict's entry, else the
    reference's call default (None when there is none)."""
    v = param.get(key, _CALL_DEFAULTS.get(key))
    return v


def resolve(param: Param, damping: Damping | None = None) -> dict:
    """
    The numeric parameter set the kernels take, with the reference's gating
    for ``damping`` (rational when ``None``).  Raises ``TypeError`` for a
    missing required parameter and ``ValueError`` for an order the damping
    function does not have, in the order the reference evaluates them
    (order 6, 8, then 10).
    """
    damping = damping if damping is not None else RationalDamping()
    has_t8 = _given(param, "s8") is not None or _given(param, "rs8") is not None
    has_s10 = param.get("s10") is not None
    orders = [6] + ([8] if has_t8 else []) + ([10] if "s10" in param and has_s10 else [])
    name = type(damping).__name__
    for order in orders:
        if order not in damping.ORDERS:
            raise damping._order_error(order)
        missing = [k for k in damping.REQUIRED_BY_ORDER.get(order, ())
                   if _given(param, k) is None]
        if missing:
            raise TypeError(f"{name} (order {order}) requires keyword(s): {', '.join(missing)}")

    def num(key, default):
        v = param.get(key)
        return _value(v) if v is not None else default

    return {
        "damping": damping.kind,
        "s6": num("s6", S6),
        "s8": num("s8", S8) if has_t8 else 0.0,
        "has_s8": has_t8,
        "s10": num("s10", 0.0),
        "has_s10": has_s10,
        "a1": num("a1", A1_ATM_FALLBACK),
        "a2": num("a2", A2),
        "s9": num("s9", S9),
        "alp": num("alp", ALP),
        "rs6": num("rs6", RS6),
        "rs8": num("rs8", RS8),
        "bet": num("bet", BET),
    }
