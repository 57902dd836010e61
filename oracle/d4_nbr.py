"""
Float64 neighbour-list restatement of tad-dftd4's ``dftd4()`` for single
large structures (test oracle: used by ``tests/`` and as the checker of the
benchmark's 16000-atom line, never by the product).

The dense oracle (``d4_oracle``) builds the reference's (N, N, 7, 7) reference
C6 and (N, N, N) ATM tensors, which rules out thousands of atoms.  This module
computes the same quantities as the reference with

* the pair terms -- the D4 and EEQ coordination numbers, the EEQ system and
  the two-body energy -- as dense (N, N) tensors (``d4_oracle``'s
  functions, on whatever device the inputs live);
* C6 = A diag((3/pi) w) A^T from the weighted polarisabilities
  A_i(w) = sum_r gw_ir alpha_ir(w): the reference's contraction
  ``rc6[i,j,a,b] gw[i,a] gw[j,b]`` (``model/d4.py:268-289``, ``utils.py:33-94``)
  regrouped, the same sum in another order;
* the ATM energy (``dispersion/threebody.py:54-163``) over the triples its
  mask keeps -- two sides within ``disp3`` meeting at a centre atom --
  enumerated from neighbour lists and evaluated in chunks, with the
  reference's per-atom attribution (atom a of {a, b, c} receives
  e/6 [bc]([ab] + [ac]));
* the EEQ charges by a dense float64 solve of the bordered system
  (``d4_oracle.eeq_charges``'s formulation).

Gradients: every ATM chunk is differentiated on its own with respect to the
positions and C6(q = 0); the accumulated C6(q = 0) adjoint and the two-body
energy are then differentiated through C6, the weights, the CN and the EEQ
charges by autograd.  D4 model only (the large workloads use it).
"""

from __future__ import annotations

import math
from typing import Mapping

import numpy as np
import torch

from . import d4_oracle as dense

__all__ = ["device_tables", "eeq_system", "eeq_residual", "atm_triples", "dftd4_large"]


class _DeviceTables:
    """The oracle's tables as tensors on one device."""

    def __init__(self, tables: dense.OracleTables, device):
        for key in tables.raw:
            if key == "provenance":
                continue
            setattr(self, key, getattr(tables, key).to(device))


_DEV_CACHE: dict = {}


def device_tables(device, tables: dense.OracleTables | None = None) -> _DeviceTables:
    tables = tables or dense.load_tables()
    key = (str(torch.device(device)), id(tables))
    if key not in _DEV_CACHE:
        _DEV_CACHE[key] = _DeviceTables(tables, torch.device(device))
    return _DEV_CACHE[key]


def eeq_system(numbers, positions, charge, tables, cutoff: float):
    """The bordered EEQ system [[A, 1], [1^T, 0]] x = [b, Q] of one structure
    (N atoms, no padding), float64, on the inputs' device: A_ii = eta_i +
    sqrt(2/pi)/rad_i, A_ij = erf(g_ij r_ij)/r_ij, b = -chi + kcn sqrt(CN_EEQ)
    (the formulation of ``d4_oracle.eeq_charges``)."""
    dtype = positions.dtype
    dev = positions.device
    n = numbers.shape[-1]
    mask = dense._real_pairs(numbers)
    r = dense._distances(positions, mask)
    cn = dense.cn_eeq(numbers, positions, tables, cutoff=cutoff)
    chi = tables.eeq_chi.to(dtype)[numbers]
    eta = tables.eeq_eta.to(dtype)[numbers]
    kcn = tables.eeq_kcn.to(dtype)[numbers]
    rad = tables.eeq_rad.to(dtype)[numbers]
    gam = 1.0 / torch.sqrt(rad.unsqueeze(-1) ** 2 + rad.unsqueeze(-2) ** 2)
    offd = torch.where(mask, torch.erf(gam * r) / r, torch.zeros_like(r))
    amat = torch.zeros((n + 1, n + 1), dtype=dtype, device=dev)
    amat[:n, :n] = offd + torch.diag_embed(eta + math.sqrt(2.0 / math.pi) / rad)
    amat[:n, n] = 1.0
    amat[n, :n] = 1.0
    sqrt_cn = torch.where(cn > 0, torch.sqrt(torch.where(cn > 0, cn, torch.ones_like(cn))),
                          torch.zeros_like(cn))
    rhs = torch.empty(n + 1, dtype=dtype, device=dev)
    rhs[:n] = -chi + kcn * sqrt_cn
    rhs[n] = torch.as_tensor(charge, dtype=dtype, device=dev).reshape(())
    return amat, rhs


def eeq_residual(numbers, positions, charge, q, tables=None, cutoff: float = 25.0) -> float:
    """max |A q + lambda 1 - b| over the atoms for given charges q, with the
    multiplier lambda that best fits them (least squares): the residual of
    the first N rows of the EEQ system, in float64."""
    tables = tables or device_tables(positions.device)
    with torch.no_grad():
        amat, rhs = eeq_system(numbers, positions, charge, tables, cutoff)
        n = numbers.shape[-1]
        aq = amat[:n, :n] @ q.to(amat.dtype) - rhs[:n]
        lam = -aq.mean()
        return float((aq + lam).abs().max())


def atm_triples(positions: torch.Tensor, cut: float, centre_chunk: int = 64):
    """Yield (i, j, k) index tensors of the triples the reference's ATM mask
    keeps, centre atom j with neighbours i < k (r_ij, r_jk <= cut): a triple
    with r_ik beyond the cutoff has exactly one such centre; one with every
    side inside is taken at its smallest atom (j < i)."""
    n = positions.shape[0]
    x = positions.detach()
    for j0 in range(0, n, centre_chunk):
        # (no yield inside the no-grad block: the caller differentiates)
        with torch.no_grad():
            found = _centre_triples(x, j0, min(n, j0 + centre_chunk), cut * cut)
        if found is not None:
            yield found


def _centre_triples(x, j0: int, j1: int, cut2: float):
    n = x.shape[0]
    dev = x.device
    d2 = ((x[j0:j1, None, :] - x[None, :, :]) ** 2).sum(-1)  # (C, n)
    near = d2 <= cut2
    near[torch.arange(j1 - j0, device=dev), torch.arange(j0, j1, device=dev)] = False
    deg = near.sum(1)
    dmax = int(deg.max()) if deg.numel() else 0
    if dmax < 2:
        return None
    # neighbour indices in ascending order, padded with -1
    idx = torch.where(near, torch.arange(n, device=dev)[None, :],
                      torch.full_like(d2, n, dtype=torch.long))
    idx = idx.sort(dim=1).values[:, :dmax]
    idx = torch.where(idx < n, idx, torch.full_like(idx, -1))
    tu = torch.triu_indices(dmax, dmax, offset=1, device=dev)
    ii = idx[:, tu[0]]
    kk = idx[:, tu[1]]
    jj = torch.arange(j0, j1, device=dev)[:, None].expand_as(ii)
    ok = (ii >= 0) & (kk >= 0)
    ii, jj, kk = ii[ok], jj[ok], kk[ok]
    rik2 = ((x[ii] - x[kk]) ** 2).sum(-1)
    keep = (rik2 > cut2) | (jj < ii)
    return ii[keep], jj[keep], kk[keep]


def _atm_chunk(pos, c60, radii, i, j, k, s9, alp3, cut2):
    """Energies (triple total, per-atom shares) of one chunk of triples."""
    def d2(a, b):
        d = pos[a] - pos[b]
        return (d * d).sum(-1)

    r2ij, r2ik, r2jk = d2(i, j), d2(i, k), d2(j, k)
    r0 = radii[i, j] * radii[i, k] * radii[j, k]
    r2 = r2ij * r2ik * r2jk
    r1 = torch.sqrt(r2)
    r3 = r1 * r2
    r5 = r2 * r3
    fdamp = 1.0 / (1.0 + 6.0 * (r0 / r1) ** alp3)
    s = (r2ij + r2jk - r2ik) * (r2ij - r2jk + r2ik) * (-r2ij + r2jk + r2ik)
    ang = 0.375 * s / r5 + 1.0 / r3
    c9 = torch.sqrt(torch.abs(c60[i, j] * c60[i, k] * c60[j, k]))
    e = ang * fdamp * s9 * c9
    mij = (r2ij <= cut2).to(e.dtype)
    mik = (r2ik <= cut2).to(e.dtype)
    mjk = (r2jk <= cut2).to(e.dtype)
    wi = mjk * (mij + mik)
    wj = mik * (mij + mjk)
    wk = mij * (mik + mjk)
    return e, wi, wj, wk


def dftd4_large(numbers: torch.Tensor, positions: torch.Tensor, charge, param: Mapping,
                cutoff: Mapping | None = None, tables=None, triples_per_chunk: int = 20_000_000):
    """
    Atom energies (N,) and the gradient of their sum (N, 3), float64, of one
    structure without padding (numbers (N,), positions (N, 3)) on the inputs'
    device; D4 model, EEQ charges, rational two-body damping, approximate-C9
    ATM -- the ``dftd4()`` defaults.  Also returns the EEQ charges, the CN
    and the two- and three-body atom energies.
    """
    dev = positions.device
    dtype = torch.float64
    tables = tables or device_tables(dev)
    cut = dict(dense.DEFAULTS)
    if cutoff:
        cut.update(cutoff)
    numbers = numbers.to(dev)
    pos = positions.detach().to(dtype).clone().requires_grad_(True)
    n = numbers.shape[0]

    cn = dense.cn_d4(numbers, pos, tables, cutoff=cut["cn"])
    amat, rhs = eeq_system(numbers, pos, charge, tables, cut["cn_eeq"])
    q = torch.linalg.solve(amat, rhs)[:n]
    del amat, rhs
    alpha = dense.reference_alpha(tables, numbers, dtype)
    w = dense.THOPI * tables.freq_weights.to(dtype)
    gw = dense.weights_d4(numbers, cn, q, tables, dtype)
    gw0 = dense.weights_d4(numbers, cn, torch.zeros_like(q), tables, dtype)
    a = torch.einsum("nr,nrw->nw", gw, alpha)
    a0 = torch.einsum("nr,nrw->nw", gw0, alpha)
    c6 = (a * w) @ a.T
    c60 = (a0 * w) @ a0.T
    r4r2 = tables.r4r2.to(dtype)[numbers]
    e2 = dense.dispersion2(numbers[None], pos[None], param, c6[None], r4r2[None],
                           cutoff=cut["disp2"])[0]

    # ATM in chunks of triples, each differentiated on its own
    s9 = float(param.get("s9", dense.DEFAULTS["s9"]))
    alp3 = float(param.get("alp", dense.DEFAULTS["alp"])) / 3.0
    a1v = param.get("a1")
    a1 = float(a1v) if a1v is not None else float(np.float32(dense.DEFAULTS["a1"]))
    a2 = float(param.get("a2", dense.DEFAULTS["a2"]))
    cut3 = cut["disp3"]
    with torch.no_grad():
        radii = a1 * torch.sqrt(3.0 * r4r2[:, None] * r4r2[None, :]) + a2
    c60_leaf = c60.detach().requires_grad_(True)
    pos_leaf = pos.detach().requires_grad_(True)
    e3 = torch.zeros(n, dtype=dtype, device=dev)
    g_pos3 = torch.zeros_like(pos_leaf)
    g_c60 = torch.zeros_like(c60_leaf)
    pending: list = []
    count = 0

    def flush():
        nonlocal count
        if not pending:
            return
        i = torch.cat([p[0] for p in pending])
        j = torch.cat([p[1] for p in pending])
        k = torch.cat([p[2] for p in pending])
        pending.clear()
        e, wi, wj, wk = _atm_chunk(pos_leaf, c60_leaf, radii, i, j, k, s9, alp3,
                                   cut3 * cut3)
        total = (e * (wi + wj + wk)).sum() / 6.0
        gp, gc = torch.autograd.grad(total, [pos_leaf, c60_leaf])
        g_pos3.add_(gp)
        g_c60.add_(gc)
        ed = e.detach() / 6.0
        e3.index_add_(0, i, ed * wi)
        e3.index_add_(0, j, ed * wj)
        e3.index_add_(0, k, ed * wk)
        count += int(i.numel())

    size = 0
    for i, j, k in atm_triples(pos.detach(), cut3):
        pending.append((i, j, k))
        size += int(i.numel())
        if size >= triples_per_chunk:
            flush()
            size = 0
    flush()

    total2 = e2.sum() + (g_c60 * c60).sum()
    (g_pos,) = torch.autograd.grad(total2, [pos])
    grad = g_pos + g_pos3
    energy = e2.detach() + e3
    return energy, grad.detach(), {"q": q.detach(), "cn": cn.detach(), "e2": e2.detach(),
                                    "e3": e3, "triples": count}
