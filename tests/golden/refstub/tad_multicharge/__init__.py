"""
Test-only stand-in for ``tad-multicharge``: EEQ charges restated from the
published EEQ model of D4.  The constraint is handled by the Schur complement
(two solves with the same matrix), deliberately different from the oracle's
augmented solve, so that the two restatements check each other.
"""

from __future__ import annotations

import math

import numpy as np
import torch

from tad_mctc.data import _table
from tad_mctc.ncoord import _pairs, cn_eeq


def get_eeq_charges(numbers, positions, charge, cutoff=25.0, **kwargs):
    dd = {"device": positions.device, "dtype": positions.dtype}
    cutoff = float(cutoff)
    real = numbers != 0
    mask, r = _pairs(numbers, positions)
    cn = cn_eeq(numbers, positions, cutoff=cutoff)
    chi, eta, kcn, rad = (
        torch.tensor(_table(k), **dd)[numbers]
        for k in ("eeq_chi", "eeq_eta", "eeq_kcn", "eeq_rad")
    )
    g = torch.rsqrt(rad[..., :, None] ** 2 + rad[..., None, :] ** 2 + (~mask).to(r.dtype))
    amat = torch.where(mask, torch.erf(g * r) / r, 0.0)
    selfterm = eta + math.sqrt(2.0 / math.pi) / torch.where(real, rad, 1.0)
    amat = amat + torch.diag_embed(torch.where(real, selfterm, 1.0))
    sq = torch.sqrt(torch.where(cn > 0, cn, 1.0)) * (cn > 0)
    x_rhs = torch.where(real, -chi + kcn * sq, 0.0)
    ones = real.to(r.dtype)
    sol = torch.linalg.solve(amat, torch.stack((x_rhs, ones), -1))
    x, y = sol[..., 0], sol[..., 1]
    charge = torch.as_tensor(charge, **dd)
    lam = ((x * ones).sum(-1) - charge) / (y * ones).sum(-1)
    return torch.where(real, x - lam.unsqueeze(-1) * y, 0.0)
