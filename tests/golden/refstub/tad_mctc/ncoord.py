"""
Coordination numbers, restated from the D4 method (Caldeweyher et al.,
J. Chem. Phys. 150, 154122 (2019)).  Written independently of the oracle so
that the two restatements check each other.
"""

from __future__ import annotations

import torch

from .batch import real_pairs
from .data import COV_D3, PAULING_EN


def erf_count(rij, r0, kcn=7.5):
    # 1/2 (1 + erf(-x)) written as 1/2 erfc(x): no cancellation for x >> 1
    return 0.5 * torch.erfc(kcn * (rij / r0 - 1.0))


def _pairs(numbers, positions):
    mask = real_pairs(numbers, mask_diagonal=True)
    diff = positions.unsqueeze(-2) - positions.unsqueeze(-3)
    d2 = (diff**2).sum(-1)
    r = torch.sqrt(torch.where(mask, d2, torch.ones_like(d2)))
    return mask, r


def cn_d4(numbers, positions, *, counting_function=erf_count, cutoff=30.0,
          kcn=7.5, k4=4.10451, k5=19.08857, k6=2 * 11.28174**2, **kwargs):
    dd = {"device": positions.device, "dtype": positions.dtype}
    mask, r = _pairs(numbers, positions)
    rc = COV_D3(**dd)[numbers]
    en = PAULING_EN(**dd)[numbers]
    r0 = rc[..., :, None] + rc[..., None, :]
    den = k4 * torch.exp(-((en[..., :, None] - en[..., None, :]).abs() + k5) ** 2 / k6)
    keep = mask & (r <= cutoff)
    return torch.sum(torch.where(keep, den * counting_function(r, r0, kcn), 0.0), dim=-1)


def cn_eeq(numbers, positions, *, cutoff=25.0, cn_max=8.0, kcn=7.5):
    dd = {"device": positions.device, "dtype": positions.dtype}
    mask, r = _pairs(numbers, positions)
    rc = COV_D3(**dd)[numbers]
    r0 = rc[..., :, None] + rc[..., None, :]
    keep = mask & (r <= cutoff)
    cn = torch.sum(torch.where(keep, erf_count(r, r0, kcn), 0.0), dim=-1)
    # smooth cap log(1 + e^max) - log(1 + e^(max - cn)), written without the
    # cancellation of the two logarithms for cn << 1
    cmax = torch.tensor(cn_max, **dd)
    return torch.log1p(torch.expm1(cn) / (1.0 + torch.exp(cn - cmax)))


def cn_d3(numbers, positions, **kwargs):  # pragma: no cover - not on this path
    raise NotImplementedError("cn_d3 is not used on the D4 path")
