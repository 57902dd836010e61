"""
Dispersion methods as classes: drop-ins for ``tad_dftd4.dispersion``'s
``Disp``, ``DispD4`` and ``DispD4Exact`` (``dispersion/base.py:104-431``,
``dispersion/d4.py:33-84``) and the term descriptors ``TwoBodyTerm``
(``dispersion/twobody.py:37-86``), ``D4ATMApprox`` and ``D4ATMExact``
(``dispersion/d4.py:44-45, 67-68``).

A method is a list of terms.  The library evaluates the terms that
``dftd4`` and the D4 method classes combine -- one two-body term at the
EEQ charges with any built-in damping function, plus at most one ATM term at
q = 0 with zero damping, approximate or exact C9 -- in one fused call, so a
method is validated against that shape when it is calculated.
"""

from __future__ import annotations

import torch

from .cutoff import Cutoff
from .damping import Damping, Param, RationalDamping, ZeroDamping
from .model import BaseModel

__all__ = ["Disp", "DispD4", "DispD4Exact", "DispTerm", "TwoBodyTerm", "ATM",
           "D4ATMApprox", "D4ATMExact"]


class DispTerm:
    """A dispersion term: its damping function and whether it uses the
    atomic charges (``dispersion/base.py:38-101``)."""

    def __init__(self, damping_fn: Damping, charge_dependent: bool):
        self.damping_fn = damping_fn
        self.charge_dependent = charge_dependent


class TwoBodyTerm(DispTerm):
    """Pairwise C6/C8 term (``dispersion/twobody.py:37-86``)."""

    def __init__(self, *, damping_fn: Damping = RationalDamping(),
                 charge_dependent: bool = True):
        super().__init__(damping_fn, charge_dependent)


class ATM(DispTerm):
    """Axilrod-Teller-Muto three-body term with Becke-Johnson radii."""

    exact_c9 = False

    def __init__(self, *, damping_fn: Damping = ZeroDamping(),
                 charge_dependent: bool = False):
        super().__init__(damping_fn, charge_dependent)


class D4ATMApprox(ATM):
    """ATM with C9 = sqrt(|C6_ij C6_ik C6_jk|) (``threebody.py:305-321``)."""


class D4ATMExact(ATM):
    """ATM with C9 by Casimir-Polder integration of three polarisabilities
    (``threebody.py:276-302``)."""

    exact_c9 = True


class Disp:
    """
    A dispersion method: a model, the D4 coordination number and a list of
    terms.  ``calculate`` has the signature of ``Disp.calculate``
    (``dispersion/base.py:285-431``) and returns atom-resolved energies that
    carry gradients (positions, damping parameters) through the library's
    adjoint.
    """

    TERMS: list = []
    _ALLOWED_MODELS = ("d3", "d4", "d4s", "d5")

    def __init__(self, model="d4", model_kwargs: dict | None = None, cn_fn=None,
                 cn_fn_kwargs: dict | None = None, *, device=None, dtype=None):
        if isinstance(model, str):
            key = model.casefold()
            if key not in self._ALLOWED_MODELS:
                raise ValueError(f"Unknown model '{key}'. "
                                 f"Please use {', '.join(self._ALLOWED_MODELS)}.")
            self._model = key
        elif isinstance(model, BaseModel):
            self._model = model
        else:
            raise TypeError(f"unsupported model object {type(model).__name__}")
        self.model_kwargs = dict(model_kwargs or {})
        self.cn_fn = cn_fn
        self.cn_fn_kwargs = dict(cn_fn_kwargs or {})
        unknown = set(self.cn_fn_kwargs) - {"counting_function"}
        if unknown:
            raise NotImplementedError(f"CN options {sorted(unknown)} are not built in")
        self.device, self.dtype = device, dtype
        self.terms: list[DispTerm] = []
        for term_cls, kw in self.TERMS:
            self.register(term_cls(**dict(kw or {})))

    def register(self, term: DispTerm) -> None:
        self.terms.append(term)

    def deregister(self, term: DispTerm) -> None:
        self.terms.remove(term)

    def get_model(self, numbers: torch.Tensor) -> BaseModel:
        from .disp import _resolve_model

        if isinstance(self._model, BaseModel):
            return self._model
        if self._model == "d4":
            from .model import D4Model

            return D4Model(numbers, **self.model_kwargs)
        if self._model == "d4s":
            from .model import D4SModel

            return D4SModel(numbers, **self.model_kwargs)
        return _resolve_model(self._model, numbers)

    def _shape(self):
        """(two-body damping, ATM term or None) of the registered terms."""
        two = [t for t in self.terms if isinstance(t, TwoBodyTerm)]
        atm = [t for t in self.terms if isinstance(t, ATM)]
        other = [t for t in self.terms if not isinstance(t, (TwoBodyTerm, ATM))]
        if len(two) != 1 or len(atm) > 1 or other:
            raise NotImplementedError(
                "the library evaluates one two-body term plus at most one ATM term")
        if not two[0].charge_dependent:
            raise NotImplementedError("the two-body term is evaluated at the EEQ charges")
        if atm:
            if atm[0].charge_dependent:
                raise NotImplementedError("the ATM term is evaluated at q = 0")
            if not isinstance(atm[0].damping_fn, ZeroDamping) and \
                    type(atm[0].damping_fn).__name__ != "ZeroDamping":
                raise NotImplementedError("the ATM term takes zero damping of order 9")
        return two[0].damping_fn, (atm[0] if atm else None)

    def calculate(self, numbers: torch.Tensor, positions: torch.Tensor, charge,
                  param: Param, *, cutoff: Cutoff | None = None, q=None, rcov=None,
                  r4r2=None, rvdw=None, precision: str | None = None) -> torch.Tensor:
        from .disp import _evaluate

        damping, atm = self._shape()
        if atm is None:  # no three-body term: the library's ATM contributes nothing
            param = {k: v for k, v in param.items() if k != "s9"}
            param["s9"] = 0.0
        return _evaluate(numbers, positions, charge, param, model=self.get_model(numbers),
                         rcov=rcov, r4r2=r4r2, rvdw=rvdw, q=q, cutoff=cutoff,
                         cn_function=self.cn_fn,
                         counting_function=self.cn_fn_kwargs.get("counting_function"),
                         damping_function=damping, precision=precision,
                         exact_c9=bool(atm is not None and atm.exact_c9))


class DispD4(Disp):
    """The standard DFT-D4 method: rational two-body term at the EEQ charges
    and ATM with approximate C9 (``dispersion/d4.py:48-61``)."""

    _ALLOWED_MODELS = ("d4", "d4s")
    TERMS = [
        (TwoBodyTerm, {"damping_fn": RationalDamping(), "charge_dependent": True}),
        (D4ATMApprox, {"damping_fn": ZeroDamping(), "charge_dependent": False}),
    ]


class DispD4Exact(Disp):
    """DFT-D4 with the exact C9 coefficients of the Casimir-Polder formula
    (``dispersion/d4.py:71-84``).  Runs on the plain FP64 kernels."""

    TERMS = [
        (TwoBodyTerm, {"damping_fn": RationalDamping(), "charge_dependent": True}),
        (D4ATMExact, {"damping_fn": ZeroDamping(), "charge_dependent": False}),
    ]
