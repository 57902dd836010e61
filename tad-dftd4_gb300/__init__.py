"""
tad-dftd4 dispersion on GB300: the ``dftd4()`` path of tad-dftd4 rebuilt as
hand-written CUDA kernels behind a C ABI (``include/tad_dftd4_gb300.h``).

Import with ``importlib.import_module("tad-dftd4_gb300")`` (the directory
name carries a hyphen).  Public API, mirroring ``tad_dftd4``:

* ``dftd4(numbers, positions, charge, param, *, model=..., cutoff=...)``
* ``Cutoff``, ``D4Model``, ``D4SModel``, ``Param``, the damping functions
  ``RationalDamping``, ``ZeroDamping``, ``MZeroDamping``,
  ``OptimisedPowerDamping``
* ``Disp``, ``DispD4``, ``DispD4Exact`` (method classes; ``DispD4Exact``
  evaluates the ATM term with exact C9) and the terms ``TwoBodyTerm``,
  ``D4ATMApprox``, ``D4ATMExact``
* ``get_properties(numbers, positions, charge=None, cutoff=None)`` -- CN,
  EEQ charges, atom-resolved C6 and static polarisabilities
* ``dispersion_energy_gradient`` -- energies and forces in one fused call
* ``hessian`` -- second derivatives of the total energy with respect to the
  positions (central differences of the fused analytic gradient)
* ``check_status()`` -- raise a pending device error of a forward call with
  gradients whose backward has not run (the backward raises it otherwise)
* ``get_params(method=..., functional=..., variant=None)`` -- damping
  parameters per density functional
"""

from __future__ import annotations

from . import _lib, tables, workloads  # noqa: F401
from .cutoff import Cutoff
from .damping import (Damping, MZeroDamping, OptimisedPowerDamping, Param, RationalDamping,
                      ZeroDamping)
from .disp import check_status, dftd4, dispersion_energy_gradient, get_properties, hessian
from .dispersion import (ATM, D4ATMApprox, D4ATMExact, Disp, DispD4, DispD4Exact, DispTerm,
                         TwoBodyTerm)
from .model import D4Model, D4SModel
from .parameters import DispersionMethod, get_params

__version__ = "0.1.0"

__all__ = [
    "Cutoff",
    "D4Model",
    "D4SModel",
    "Damping",
    "Param",
    "RationalDamping",
    "ZeroDamping",
    "MZeroDamping",
    "OptimisedPowerDamping",
    "Disp",
    "DispD4",
    "DispD4Exact",
    "DispTerm",
    "TwoBodyTerm",
    "ATM",
    "D4ATMApprox",
    "D4ATMExact",
    "dftd4",
    "dispersion_energy_gradient",
    "get_properties",
    "hessian",
    "check_status",
    "get_params",
    "DispersionMethod",
    "__version__",
]
