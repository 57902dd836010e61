"""
Dispersion model descriptors, drop-ins for ``tad_dftd4.model.D4Model`` and
``D4SModel`` (``model/base.py:107-151``, ``model/d4.py``, ``model/d4s.py``).

A model here holds the configuration that the CUDA kernels need (the kind,
the charge-scaling constants ga / gc, the weighting factor and the reference
charge set); the weights, C6 and energies are computed on the device by
``dftd4``.  Building a model does no work, unlike the reference, which
evaluates every reference C6 (N x N x 7 x 7) at construction.
"""

from __future__ import annotations

import torch

GA_DEFAULT = 3.0
GC_DEFAULT = 2.0
WF_DEFAULT = 6.0


class BaseModel:
    kind = "d4"

    def __init__(self, numbers: torch.Tensor, ga: float = GA_DEFAULT, gc: float = GC_DEFAULT,
                 wf=None, ref_charges: str = "eeq", rc6=None, device=None, dtype=None):
        if ref_charges not in ("eeq", "gfn2"):
            raise ValueError(f"Unknown reference charges: {ref_charges}")
        if rc6 is not None:
            raise NotImplementedError("custom reference C6 (rc6) is not supported")
        self.numbers = numbers
        self.ga = float(ga)
        self.gc = float(gc)
        self.ref_charges = ref_charges
        self.device = device
        self.dtype = dtype
        self.wf = self._check_wf(wf)

    def _check_wf(self, wf):
        return WF_DEFAULT if wf is None else float(wf)

    def __repr__(self) -> str:
        return (f"{self.__class__.__name__}(ga={self.ga}, gc={self.gc}, wf={self.wf}, "
                f"ref_charges={self.ref_charges})")


class D4Model(BaseModel):
    """D4: one Gaussian weighting factor (6.0) for all atoms."""

    kind = "d4"


class D4SModel(BaseModel):
    """D4S: pairwise weighting factors WFPAIR[Z_i, Z_j] (``data/wfpair.py``)."""

    kind = "d4s"

    def _check_wf(self, wf):
        if wf is not None:
            raise NotImplementedError("D4SModel takes its weighting factors from WFPAIR")
        return None
