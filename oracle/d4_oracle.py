"""
Float64 PyTorch restatement of tad-dftd4's ``dftd4()`` (test oracle).

Every function names the reference lines it follows (paths relative to the
tad-dftd4 source package ``src/tad_dftd4``).  Dense (B, N, N) and
(B, N, N, N) tensors are used on purpose: this is the reference's own
formulation, and it keeps the oracle short and obviously equivalent.
Gradients come from torch autograd, as in the reference.
"""

from __future__ import annotations

import math
from pathlib import Path
from typing import Mapping

import numpy as np
import torch

__all__ = [
    "OracleTables",
    "load_tables",
    "erf_count",
    "cn_d4",
    "cn_eeq",
    "eeq_charges",
    "zeta",
    "reference_alpha",
    "weights_d4",
    "weights_d4s",
    "c6_d4",
    "c6_d4s",
    "dispersion2",
    "weighted_pols",
    "c9_exact",
    "atm_dispersion",
    "dftd4",
    "dftd4_energy_and_grad",
    "DEFAULTS",
]

TABLES_PATH = (
    Path(__file__).resolve().parents[1] / "tad-dftd4_gb300" / "data" / "d4_tables.npz"
)

# defaults.py:26-93, cutoff.py:60-90, model/base.py:57-59
DEFAULTS = {
    "disp2": 60.0,
    "disp3": 40.0,
    "cn": 30.0,
    "cn_eeq": 25.0,
    "cn_eeq_max": 8.0,
    "kcn": 7.5,
    "k4": 4.10451,
    "k5": 19.08857,
    "k6": 2 * 11.28174**2,
    "s6": 1.0,
    "s8": 1.0,
    "s9": 1.0,
    "a1": 0.4,
    "a2": 5.0,
    "alp": 16.0,
    "ga": 3.0,
    "gc": 2.0,
    "wf": 6.0,
}

THOPI = 3.0 / 3.141592653589793238462643383279502884197  # utils.py:50


class OracleTables:
    """Element tables as float64 / int64 CPU tensors."""

    def __init__(self, arrays: Mapping[str, np.ndarray]):
        self.raw = dict(arrays)
        for key, val in arrays.items():
            if key == "provenance":
                continue
            setattr(self, key, torch.from_numpy(np.array(val)))


_TABLE_CACHE: dict[str, OracleTables] = {}


def load_tables(path: str | Path | None = None) -> OracleTables:
    key = str(path or TABLES_PATH)
    if key not in _TABLE_CACHE:
        with np.load(key) as npz:
            _TABLE_CACHE[key] = OracleTables({k: npz[k] for k in npz.files})
    return _TABLE_CACHE[key]


# --------------------------------------------------------------------------
# masks and distances (tad_mctc.batch.real_* and storch.cdist semantics)
# --------------------------------------------------------------------------


def _real_atoms(numbers: torch.Tensor) -> torch.Tensor:
    return numbers != 0


def _real_pairs(numbers: torch.Tensor) -> torch.Tensor:
    ra = _real_atoms(numbers)
    n = numbers.shape[-1]
    eye = torch.eye(n, dtype=torch.bool, device=numbers.device)
    return ra.unsqueeze(-1) & ra.unsqueeze(-2) & ~eye


def _real_triples(numbers: torch.Tensor) -> torch.Tensor:
    rp = _real_pairs(numbers)
    return rp.unsqueeze(-1) & rp.unsqueeze(-2) & rp.unsqueeze(-3)


def _distances(positions: torch.Tensor, mask: torch.Tensor) -> torch.Tensor:
    """Pair distances on ``mask``; 1.0 elsewhere (safe for autograd)."""
    diff = positions.unsqueeze(-2) - positions.unsqueeze(-3)
    d2 = torch.sum(diff * diff, dim=-1)
    return torch.sqrt(torch.where(mask, d2, torch.ones_like(d2)))


# --------------------------------------------------------------------------
# coordination numbers and EEQ charges (restated; tad-mctc / tad-multicharge)
# --------------------------------------------------------------------------


def erf_count(r: torch.Tensor, r0: torch.Tensor, kcn: float) -> torch.Tensor:
    """Error-function counting function 1/2 (1 + erf(-k (r/r0 - 1))),
    evaluated as 1/2 erfc(k (r/r0 - 1)): the same function without the
    cancellation of 1 + erf(-x) for the far pairs (x >> 1) that make up the
    coordination number of a nearly isolated atom."""
    return 0.5 * torch.erfc(kcn * (r / r0 - 1.0))


def cn_d4(
    numbers: torch.Tensor,
    positions: torch.Tensor,
    tables: OracleTables,
    cutoff: float = DEFAULTS["cn"],
    kcn: float = DEFAULTS["kcn"],
    k4: float = DEFAULTS["k4"],
    k5: float = DEFAULTS["k5"],
    k6: float = DEFAULTS["k6"],
) -> torch.Tensor:
    """
    D4 coordination number with electronegativity weighting.

    Called at ``dispersion/base.py:390`` (``tad_mctc.ncoord.cn_d4`` with
    ``erf_count``), constants from ``defaults.py:41-50``.  The pair radius is
    the sum of the D3 covalent radii; the electronegativity factor is
    k4 exp(-(|EN_i - EN_j| + k5)^2 / k6).
    """
    dtype = positions.dtype
    mask = _real_pairs(numbers)
    r = _distances(positions, mask)
    rcov = tables.cov_d3.to(dtype)[numbers]
    en = tables.en.to(dtype)[numbers]
    r0 = rcov.unsqueeze(-1) + rcov.unsqueeze(-2)
    den = k4 * torch.exp(
        -((torch.abs(en.unsqueeze(-1) - en.unsqueeze(-2)) + k5) ** 2) / k6
    )
    cf = erf_count(r, r0, kcn)
    val = torch.where(mask & (r <= cutoff), den * cf, torch.zeros_like(r))
    return val.sum(-1)


def cn_eeq(
    numbers: torch.Tensor,
    positions: torch.Tensor,
    tables: OracleTables,
    cutoff: float = DEFAULTS["cn_eeq"],
    cn_max: float = DEFAULTS["cn_eeq_max"],
    kcn: float = DEFAULTS["kcn"],
) -> torch.Tensor:
    """
    EEQ coordination number: plain erf counting within ``cutoff``
    (``Cutoff.cn_eeq``, ``dispersion/base.py:401-407``), then the smooth cap
    log(1 + e^max) - log(1 + e^(max - cn)) at ``defaults.py:32``, evaluated
    as log1p(expm1(cn) / (1 + e^(cn - max))): the same function without the
    cancellation of the two logarithms for cn << 1 (nearly isolated atoms,
    whose sqrt(cn) enters the EEQ right-hand side).
    """
    dtype = positions.dtype
    mask = _real_pairs(numbers)
    r = _distances(positions, mask)
    rcov = tables.cov_d3.to(dtype)[numbers]
    r0 = rcov.unsqueeze(-1) + rcov.unsqueeze(-2)
    cf = erf_count(r, r0, kcn)
    cn = torch.where(mask & (r <= cutoff), cf, torch.zeros_like(r)).sum(-1)
    return torch.log1p(torch.expm1(cn) / (1.0 + torch.exp(cn - cn_max)))


def eeq_charges(
    numbers: torch.Tensor,
    positions: torch.Tensor,
    charge: torch.Tensor,
    tables: OracleTables,
    cutoff: float = DEFAULTS["cn_eeq"],
) -> torch.Tensor:
    """
    Electronegativity-equilibration charges (``tad_multicharge.get_eeq_charges``
    at ``dispersion/base.py:401-407``).

    Solves [[A, 1], [1^T, 0]] [q, l] = [-chi + kcn sqrt(cn), Q] with
    A_ii = eta_i + sqrt(2/pi)/rad_i and A_ij = erf(g_ij r_ij)/r_ij,
    g_ij = 1/sqrt(rad_i^2 + rad_j^2).  Padding atoms get an identity row.
    """
    dtype = positions.dtype
    real = _real_atoms(numbers)
    mask = _real_pairs(numbers)
    r = _distances(positions, mask)
    cn = cn_eeq(numbers, positions, tables, cutoff=cutoff)

    chi = tables.eeq_chi.to(dtype)[numbers]
    eta = tables.eeq_eta.to(dtype)[numbers]
    kcn = tables.eeq_kcn.to(dtype)[numbers]
    rad = tables.eeq_rad.to(dtype)[numbers]

    gam = 1.0 / torch.sqrt(rad.unsqueeze(-1) ** 2 + rad.unsqueeze(-2) ** 2)
    offd = torch.where(mask, torch.erf(gam * r) / r, torch.zeros_like(r))
    diag = torch.where(
        real, eta + math.sqrt(2.0 / math.pi) / torch.where(real, rad, 1.0), 1.0
    )
    amat_n = offd + torch.diag_embed(diag)

    safe_cn = torch.where(cn > 0, cn, torch.ones_like(cn))
    sqrt_cn = torch.where(cn > 0, torch.sqrt(safe_cn), torch.zeros_like(cn))
    rhs_n = torch.where(real, -chi + kcn * sqrt_cn, torch.zeros_like(cn))

    shape = numbers.shape
    n = shape[-1]
    one = real.to(dtype)
    amat = torch.zeros((*shape[:-1], n + 1, n + 1), dtype=dtype)
    amat[..., :n, :n] = amat_n
    amat[..., :n, n] = one
    amat[..., n, :n] = one
    rhs = torch.zeros((*shape[:-1], n + 1), dtype=dtype)
    rhs[..., :n] = rhs_n
    rhs[..., n] = charge.to(dtype).expand(shape[:-1]) if charge.dim() else charge.to(dtype)
    sol = torch.linalg.solve(amat, rhs.unsqueeze(-1)).squeeze(-1)
    return torch.where(real, sol[..., :n], torch.zeros_like(sol[..., :n]))


# --------------------------------------------------------------------------
# model: charge scaling, reference polarisabilities, weights, C6
# --------------------------------------------------------------------------


def zeta(gam, qref, qmod, ga: float, eps: float):
    """Charge scaling ``model/base.py:308-335``."""
    scale = torch.exp(gam * (1.0 - qref / (qmod - eps)))
    return torch.where(
        qmod > 0.0,
        torch.exp(ga * (1.0 - scale)),
        torch.full_like(qmod, math.exp(ga)),
    )


def _ref_charges(tables: OracleTables, ref_charges: str):
    if ref_charges == "eeq":
        return tables.clsq, tables.clsh
    if ref_charges == "gfn2":
        return tables.refq_gfn2, tables.refh_gfn2
    raise ValueError(f"Unknown reference charges: {ref_charges}")


def reference_alpha(
    tables: OracleTables,
    numbers: torch.Tensor,
    dtype: torch.dtype = torch.float64,
    ga: float = DEFAULTS["ga"],
    gc: float = DEFAULTS["gc"],
    ref_charges: str = "eeq",
) -> torch.Tensor:
    """Reference polarisabilities alpha(i w) per atom, ``model/base.py:367-418``."""
    _, refh = _ref_charges(tables, ref_charges)
    eps = torch.finfo(dtype).eps
    refsys = tables.refsys[numbers]
    refascale = tables.refascale.to(dtype)[numbers]
    refalpha = tables.refalpha.to(dtype)[numbers]
    refscount = tables.refscount.to(dtype)[numbers]
    secscale = tables.secscale.to(dtype)
    secalpha = tables.secalpha.to(dtype)
    refsq = refh.to(dtype)[numbers]
    zeff = tables.zeff[refsys].to(dtype)
    gam = tables.gam.to(dtype)[refsys] * gc
    z = torch.where(refsys > 0, zeta(gam, zeff, refsq + zeff, ga, eps), 0.0)
    aiw = secscale[refsys].unsqueeze(-1) * secalpha[refsys] * z.unsqueeze(-1)
    alpha = refascale.unsqueeze(-1) * (refalpha - refscount.unsqueeze(-1) * aiw)
    return torch.where(alpha > 0.0, alpha, torch.zeros_like(alpha))


def weights_d4(
    numbers: torch.Tensor,
    cn: torch.Tensor,
    q: torch.Tensor | None,
    tables: OracleTables,
    dtype: torch.dtype = torch.float64,
    ga: float = DEFAULTS["ga"],
    gc: float = DEFAULTS["gc"],
    wf: float = DEFAULTS["wf"],
    ref_charges: str = "eeq",
) -> torch.Tensor:
    """Charge-scaled Gaussian reference weights, ``model/d4.py:137-228``."""
    if q is None:
        q = torch.zeros(numbers.shape, dtype=dtype)
    refq, _ = _ref_charges(tables, ref_charges)
    eps = torch.finfo(dtype).eps
    refc = tables.refc[numbers]
    mask = refc > 0
    refcn = tables.refcovcn.to(torch.float64)[numbers]
    dcn = cn.unsqueeze(-1).to(torch.float64) - refcn
    tmp = torch.exp(-dcn * dcn)
    p1 = torch.pow(tmp, wf)
    p3 = p1 + torch.pow(tmp, 2 * wf) + torch.pow(tmp, 3 * wf)
    expw = torch.where(refc == 3, p3, torch.where(refc == 1, p1, tmp))
    expw = torch.where(mask, expw, torch.zeros_like(expw))
    norm = torch.where(mask, expw.sum(-1, keepdim=True), torch.full_like(expw, 1e-300))
    exceptional = ~torch.isfinite(expw / norm) | (
        (expw / norm).to(dtype) > torch.finfo(dtype).max
    )
    safe_norm = torch.where(exceptional, torch.ones_like(norm), norm)
    gw_tmp = (expw / safe_norm).to(dtype)
    maxcn = refcn.max(-1, keepdim=True)[0]
    fallback = torch.where(refcn == maxcn, 1.0, 0.0).to(dtype)
    gw = torch.where(exceptional, fallback, gw_tmp)
    zeff = tables.zeff[numbers].to(dtype).unsqueeze(-1)
    gam = tables.gam.to(dtype)[numbers].unsqueeze(-1) * gc
    qref = refq.to(dtype)[numbers]
    z = torch.where(mask, zeta(gam, qref + zeff, q.unsqueeze(-1) + zeff, ga, eps), 0.0)
    return z * gw


def weights_d4s(
    numbers: torch.Tensor,
    cn: torch.Tensor,
    q: torch.Tensor | None,
    tables: OracleTables,
    dtype: torch.dtype = torch.float64,
    ga: float = DEFAULTS["ga"],
    gc: float = DEFAULTS["gc"],
    ref_charges: str = "eeq",
) -> torch.Tensor:
    """
    Pairwise D4S weights gw[..., m, n, r] (weights of atom n's references with
    the WFPAIR exponent for partner m), ``model/d4s.py:143-248``.
    """
    if q is None:
        q = torch.zeros(numbers.shape, dtype=dtype)
    refq, _ = _ref_charges(tables, ref_charges)
    eps = torch.finfo(dtype).eps
    wfp = tables.wfpair.to(dtype)[numbers.unsqueeze(-1), numbers.unsqueeze(-2)]
    shp = (*numbers.shape[:-1], numbers.shape[-1], numbers.shape[-1], 7)
    refc = tables.refc[numbers].unsqueeze(-3).expand(shp)
    mask = refc > 0
    refcn = tables.refcovcn.to(torch.float64)[numbers].unsqueeze(-3).expand(shp)
    dcn = cn.to(torch.float64).unsqueeze(-1).unsqueeze(-3) - refcn
    # wf[n, m] multiplies entry [m, n, r]
    arg = -dcn * dcn * wfp.transpose(-1, -2).unsqueeze(-1).to(torch.float64)
    tmp = torch.where(mask, torch.exp(arg), torch.zeros_like(arg))
    p1 = tmp
    p3 = tmp + torch.pow(tmp, 2) + torch.pow(tmp, 3)
    expw = torch.where(refc == 3, p3, torch.where(refc == 1, p1, tmp))
    expw = torch.where(mask, expw, torch.zeros_like(expw))
    norm = torch.where(mask, expw.sum(-1, keepdim=True), torch.full_like(expw, 1e-300))
    exceptional = ~torch.isfinite(expw / norm) | (
        (expw / norm).to(dtype) > torch.finfo(dtype).max
    )
    safe_norm = torch.where(exceptional, torch.ones_like(norm), norm)
    gw_tmp = (expw / safe_norm).to(dtype)
    maxcn = refcn.max(-1, keepdim=True)[0]
    fallback = torch.where(refcn == maxcn, 1.0, 0.0).to(dtype)
    gw = torch.where(exceptional, fallback, gw_tmp)
    zeff = tables.zeff[numbers].to(dtype).unsqueeze(-1)
    gam = tables.gam.to(dtype)[numbers].unsqueeze(-1) * gc
    qref = refq.to(dtype)[numbers]
    z = zeta(gam, qref + zeff, q.unsqueeze(-1) + zeff, ga, eps).unsqueeze(-3)
    z = torch.where(mask, z.expand_as(gw), torch.zeros_like(gw))
    return z * gw


def _rc6(alpha: torch.Tensor, tables: OracleTables) -> torch.Tensor:
    """Reference C6 by Casimir-Polder quadrature, ``utils.py:33-94``."""
    w = tables.freq_weights.to(alpha.dtype)
    return THOPI * torch.einsum("w,...iaw,...jbw->...ijab", w, alpha, alpha)


def c6_d4(gw: torch.Tensor, alpha: torch.Tensor, tables: OracleTables) -> torch.Tensor:
    """Atomic C6, ``model/d4.py:268-289``."""
    return torch.einsum("...ijab,...ia,...jb->...ij", _rc6(alpha, tables), gw, gw)


def c6_d4s(gw: torch.Tensor, alpha: torch.Tensor, tables: OracleTables) -> torch.Tensor:
    """Atomic C6 with pairwise weights, ``model/d4s.py:268-290``."""
    return torch.einsum("...ijab,...jia,...ijb->...ij", _rc6(alpha, tables), gw, gw)


# --------------------------------------------------------------------------
# energies
# --------------------------------------------------------------------------


def _param(param: Mapping, key: str, dtype) -> torch.Tensor:
    val = param.get(key, DEFAULTS[key])
    return torch.as_tensor(val, dtype=dtype)


def _damp_d3(kind: str, order: int, r, rvdw, radius_r4r2, param, dtype):
    """D3-family two-body damping t_n = f_n / r^n, ``damping/functions.py``:
    zero 329-378 (argument rs * r / rvdw, exponent alp, alp + 2 for n = 8),
    modified zero 381-434 (r / (rs rvdw) + bet rvdw, exponent -alp_n),
    optimised power 437-484 (r^bet / (r^bet r^n + R0^bet r^n), as written
    there)."""
    alp = _param(param, "alp", dtype)
    if kind == "zero":
        rs = torch.as_tensor(param["rs6" if order == 6 else "rs8"], dtype=dtype)
        alp_n = alp if order == 6 else alp + 2.0
        t = rs * r / rvdw
        return (1.0 / (1.0 + 6.0 * t**alp_n)) / r**order
    if kind == "mzero":
        rs = torch.as_tensor(param["rs6" if order == 6 else "rs8"], dtype=dtype)
        bet = torch.as_tensor(param["bet"], dtype=dtype)
        alp_n = alp if order == 6 else alp + 2.0
        t = r / (rs * rvdw) + bet * rvdw
        return (1.0 / (1.0 + 6.0 * t ** (-alp_n))) / r**order
    if kind == "op":
        bet = torch.as_tensor(param["bet"], dtype=dtype)
        ab = radius_r4r2**bet
        rb = r**bet
        return rb / (rb * r**order + ab * r**order)
    raise ValueError(kind)


def dispersion2(
    numbers: torch.Tensor,
    positions: torch.Tensor,
    param: Mapping,
    c6: torch.Tensor,
    r4r2: torch.Tensor,
    cutoff: float = DEFAULTS["disp2"],
    damping: str = "rational",
    rvdw: torch.Tensor | None = None,
) -> torch.Tensor:
    """Damped two-body energy, ``dispersion/twobody.py:89-201`` with
    ``damping/functions.py:116-169`` (gating) and the damping function:
    rational 262-305 (default) or the D3 family (``_damp_d3``).  The
    dipole-quadrupole order is evaluated unless both s8 and rs8 are missing
    and is scaled by s8 (default 1)."""
    dtype = positions.dtype
    if damping in ("rational", "op"):
        for key in ("a1", "a2"):
            if param.get(key) is None:
                raise TypeError(f"RationalDamping (order 6) requires keyword(s): {key}")
    mask = _real_pairs(numbers)
    r = _distances(positions, mask)
    qq = 3.0 * r4r2.unsqueeze(-1) * r4r2.unsqueeze(-2)
    radius = None
    if damping in ("rational", "op"):
        a1 = torch.as_tensor(param["a1"], dtype=dtype)
        a2 = torch.as_tensor(param["a2"], dtype=dtype)
        radius = a1 * torch.sqrt(qq) + a2
    rv = None
    if damping in ("zero", "mzero"):
        rv = torch.where(mask, rvdw.to(dtype), torch.ones_like(r))
    inside = mask & (r <= cutoff)
    zero = torch.zeros_like(r)

    def damp(order):
        if damping == "rational":
            return torch.where(inside, 1.0 / (r**order + radius**order), zero)
        return torch.where(inside, _damp_d3(damping, order, r, rv, radius, param, dtype), zero)

    s6 = _param(param, "s6", dtype)
    e6 = torch.sum(c6 * damp(6), dim=-1)
    edisp = s6 * e6
    if param.get("s8") is not None or param.get("rs8") is not None:
        s8 = _param(param, "s8", dtype)
        edisp = edisp + s8 * torch.sum(c6 * qq * damp(8), dim=-1)
    if "s10" in param:
        if damping != "rational":
            raise ValueError(f"{damping} damping has no order 10")
        c10 = c6 * qq * qq * 49.0 / 40.0
        if param["s10"] is not None:
            edisp = edisp + torch.as_tensor(param["s10"], dtype=dtype) * torch.sum(
                c10 * damp(10), dim=-1
            )
    return -0.5 * edisp


def weighted_pols(numbers: torch.Tensor, gw: torch.Tensor, alpha: torch.Tensor,
                  model: str) -> torch.Tensor:
    """Weighted polarisabilities a_i(w): D4 ``model/d4.py:291-307``
    (sum_r gw_ir alpha_irw); D4S ``model/d4s.py:292-316`` (the pair weights
    gw[m, n, r] contracted with alpha[n, r, w] over n and r, divided by the
    number of real atoms)."""
    if model == "d4":
        return torch.einsum("...nr,...nrw->...nw", gw, alpha)
    # per structure: the reference divides by a (B, 1) count, which only
    # broadcasts for a single structure; (B, 1, 1) gives every structure its own
    nat = _real_atoms(numbers).sum(-1, keepdim=True).unsqueeze(-1).to(alpha.dtype)
    return torch.einsum("...mnr,...nrw->...mw", gw, alpha) / nat


def c9_exact(aiw: torch.Tensor, tables: OracleTables) -> torch.Tensor:
    """C9_ijk = (3/pi) sum_w w_w a_i a_j a_k (``threebody.py:276-302`` with
    ``utils.py:155-205``)."""
    w = tables.freq_weights.to(aiw.dtype)
    return THOPI * torch.einsum("...iw,...jw,...kw,w->...ijk", aiw, aiw, aiw, w)


def atm_dispersion(
    numbers: torch.Tensor,
    positions: torch.Tensor,
    param: Mapping,
    c6_0: torch.Tensor,
    r4r2: torch.Tensor,
    cutoff: float = DEFAULTS["disp3"],
    c9: torch.Tensor | None = None,
    absolute: bool = False,
) -> torch.Tensor:
    """
    ATM three-body energy with C9 = sqrt|C6 C6 C6| (or the given exact
    ``c9``) and BJ radii, ``dispersion/threebody.py:54-163, 210-256,
    311-321``; zero damping of order 9 with the (r0, r1) argument order of
    ``threebody.py:133-145``.  ``absolute``: sum the magnitudes of the
    triple terms instead (the scale of each atom's rounding error).
    """
    dtype = positions.dtype
    s9 = _param(param, "s9", dtype)
    # threebody.py:93-94 converts alp to the positions' dtype before /3.
    alp_third = _param(param, "alp", dtype) / 3.0
    # RadiiBJMixin (threebody.py:250-253) falls back to torch.tensor(A1) in
    # the term's own dtype, which is torch's default (float32): a missing a1
    # is float32(0.4) = 0.4000000059604645 (a2 = 5 is exact either way)
    a1 = torch.as_tensor(param["a1"] if param.get("a1") is not None
                         else float(np.float32(DEFAULTS["a1"])), dtype=dtype)
    a2 = _param(param, "a2", dtype)
    mask_p = _real_pairs(numbers)
    mask_t = _real_triples(numbers)

    radii = a1 * torch.sqrt(3.0 * r4r2.unsqueeze(-1) * r4r2.unsqueeze(-2)) + a2
    r0 = radii.unsqueeze(-1) * radii.unsqueeze(-2) * radii.unsqueeze(-3)

    r = _distances(positions, mask_p)
    d2 = torch.where(mask_p, r * r, torch.zeros_like(r))
    r2ij = d2.unsqueeze(-1)
    r2ik = d2.unsqueeze(-2)
    r2jk = d2.unsqueeze(-3)
    r2 = r2ij * r2ik * r2jk
    one = torch.ones_like(r2)
    r2s = torch.where(mask_t, r2, one)
    r1 = torch.sqrt(r2s)
    r3 = r1 * r2s
    r5 = r2s * r3

    fdamp = 1.0 / (1.0 + 6.0 * (r0 / r1) ** alp_third)
    s = (r2ij + r2jk - r2ik) * (r2ij - r2jk + r2ik) * (-r2ij + r2jk + r2ik)
    cut2 = cutoff * cutoff
    inside = mask_t & (r2ij <= cut2) & (r2jk <= cut2)
    ang = torch.where(inside, 0.375 * s / r5 + 1.0 / r3, torch.zeros_like(r2))

    if c9 is None:
        prod = c6_0.unsqueeze(-1) * c6_0.unsqueeze(-2) * c6_0.unsqueeze(-3)
        prod = torch.abs(prod)
        c9 = torch.where(mask_t & (prod > 0), torch.sqrt(torch.where(prod > 0, prod, one)),
                         0.0)
    else:
        c9 = torch.where(mask_t, c9, torch.zeros_like(c9))
    energy = ang * fdamp * s9 * c9
    if absolute:
        energy = energy.abs()
    return torch.sum(energy, dim=(-2, -1)) / 6.0


def dftd4(
    numbers: torch.Tensor,
    positions: torch.Tensor,
    charge,
    param: Mapping,
    *,
    model: str = "d4",
    tables: OracleTables | None = None,
    q: torch.Tensor | None = None,
    cutoff: Mapping | None = None,
    ref_charges: str = "eeq",
    return_parts: bool = False,
    damping: str = "rational",
    rvdw: torch.Tensor | None = None,
    exact_c9: bool = False,
):
    """
    Atom-resolved D4 energy, the whole ``disp.py:44-146`` path:
    CN -> EEQ -> weights -> C6 -> two-body (``damping``: rational, zero,
    mzero or op; ``rvdw`` the pair radii of the zero family) + ATM(q = 0),
    with the exact C9 of ``DispD4Exact`` when ``exact_c9``.
    """
    tables = tables or load_tables()
    dtype = positions.dtype
    cut = dict(DEFAULTS)
    if cutoff:
        cut.update(cutoff)
    charge = torch.as_tensor(charge, dtype=dtype)
    cn = cn_d4(numbers, positions, tables, cutoff=cut["cn"])
    if q is None:
        q = eeq_charges(numbers, positions, charge, tables, cutoff=cut["cn_eeq"])
    alpha = reference_alpha(tables, numbers, dtype, ref_charges=ref_charges)
    r4r2 = tables.r4r2.to(dtype)[numbers]
    if model == "d4":
        gw = weights_d4(numbers, cn, q, tables, dtype, ref_charges=ref_charges)
        gw0 = weights_d4(numbers, cn, None, tables, dtype, ref_charges=ref_charges)
        c6 = c6_d4(gw, alpha, tables)
        c6_0 = c6_d4(gw0, alpha, tables)
    elif model == "d4s":
        gw = weights_d4s(numbers, cn, q, tables, dtype, ref_charges=ref_charges)
        gw0 = weights_d4s(numbers, cn, None, tables, dtype, ref_charges=ref_charges)
        c6 = c6_d4s(gw, alpha, tables)
        c6_0 = c6_d4s(gw0, alpha, tables)
    else:
        raise ValueError(f"Unknown model '{model}'")
    e2 = dispersion2(numbers, positions, param, c6, r4r2, cutoff=cut["disp2"],
                     damping=damping, rvdw=rvdw)
    c9 = c9_exact(weighted_pols(numbers, gw0, alpha, model), tables) if exact_c9 else None
    e3 = atm_dispersion(numbers, positions, param, c6_0, r4r2, cutoff=cut["disp3"], c9=c9)
    energy = e2 + e3
    if return_parts:
        with torch.no_grad():
            e3_abs = atm_dispersion(numbers, positions, param, c6_0, r4r2, cutoff=cut["disp3"],
                                    c9=c9, absolute=True)
        return energy, {"cn": cn, "q": q, "c6": c6, "c6_0": c6_0, "e2": e2, "e3": e3,
                        "scale": e2.detach().abs() + e3_abs}
    return energy


def dftd4_energy_and_grad(numbers, positions, charge, param, **kw):
    """Energies (B, N) and dE_total/dR (B, N, 3) by autograd."""
    pos = positions.detach().clone().requires_grad_(True)
    energy = dftd4(numbers, pos, charge, param, **kw)
    (grad,) = torch.autograd.grad(energy.sum(), pos)
    return energy.detach(), grad
