"""
Pin the CPU oracle against outputs of tad-dftd4's own code (``golden.npz``).

The fixtures hold the reference's energies, autograd gradients and
intermediates (weights, C6, two-body and ATM energies) for the reference's
example geometries and for seeded structures, D4 and D4S.  Tolerance: 1e-12
relative with a 1e-15 absolute floor (energies in Eh, gradients in Eh/Bohr);
the reference's own tests use sqrt(eps)*10 ~ 1.5e-7 for energies.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

import oracle
from conftest import assert_close, golden_cases, golden_variant_cases

CASES = golden_cases()
RTOL, ATOL = 1e-12, 1e-15


def _inputs(arrays, meta):
    numbers = torch.from_numpy(arrays["numbers"])
    positions = torch.from_numpy(arrays["positions"])
    charge = torch.from_numpy(arrays["charge"])
    return numbers, positions, charge, meta["param"], meta["cutoff"] or None


@pytest.mark.parametrize("tag,arrays,meta", CASES, ids=[c[0] for c in CASES])
def test_intermediates(tag, arrays, meta):
    tables = oracle.load_tables()
    numbers, positions, charge, param, cutoff = _inputs(arrays, meta)
    energy, parts = oracle.dftd4(numbers, positions, charge, param, model=meta["model"],
                                 cutoff=cutoff, ref_charges=meta["ref_charges"],
                                 return_parts=True)
    assert_close(parts["cn"], arrays["cn"], RTOL, ATOL, "cn")
    assert_close(parts["q"], arrays["q"], 1e-10, 1e-13, "q")
    assert_close(parts["c6"], arrays["c6"], RTOL, ATOL, "c6")
    assert_close(parts["c6_0"], arrays["c6_0"], RTOL, ATOL, "c6_0")
    assert_close(parts["e2"], arrays["e2"], RTOL, ATOL, "e2")
    assert_close(parts["e3"], arrays["e3"], RTOL, ATOL, "e3")
    assert_close(energy, arrays["energy"], RTOL, ATOL, "energy")
    alpha = oracle.reference_alpha(tables, numbers, ref_charges=meta["ref_charges"])
    assert_close(alpha, arrays["alpha"], RTOL, ATOL, "alpha")


@pytest.mark.parametrize("tag,arrays,meta", CASES, ids=[c[0] for c in CASES])
def test_weights(tag, arrays, meta):
    tables = oracle.load_tables()
    numbers = torch.from_numpy(arrays["numbers"])
    cn = torch.from_numpy(arrays["cn"])
    q = torch.from_numpy(arrays["q"])
    fn = oracle.weights_d4 if meta["model"] == "d4" else oracle.weights_d4s
    gw = fn(numbers, cn, q, tables, ref_charges=meta["ref_charges"])
    assert_close(gw, arrays["gw"], RTOL, ATOL, "gw")


@pytest.mark.parametrize("tag,arrays,meta",
                         [c for c in CASES if not c[2]["energy_only"]],
                         ids=[c[0] for c in CASES if not c[2]["energy_only"]])
def test_gradients(tag, arrays, meta):
    numbers, positions, charge, param, cutoff = _inputs(arrays, meta)
    pos = positions.clone().requires_grad_(True)
    keys = sorted(param)
    ptens = {k: torch.tensor(v, dtype=torch.float64, requires_grad=True)
             for k, v in param.items()}
    energy = oracle.dftd4(numbers, pos, charge, ptens, model=meta["model"],
                          cutoff=cutoff, ref_charges=meta["ref_charges"])
    grads = torch.autograd.grad(energy.sum(), [pos] + [ptens[k] for k in keys])
    assert_close(grads[0], arrays["grad"], 1e-10, 1e-14, "grad")
    assert_close(np.array([g.item() for g in grads[1:]]), arrays["param_grad"],
                 1e-10, 1e-14, "param_grad")


def test_exceptional_case_is_exceptional():
    """The dense cluster really drives some weights through the fallback."""
    tables = oracle.load_tables()
    (tag, arrays, meta), = [c for c in CASES if c[0] == "dense_exceptional/d4"]
    numbers = torch.from_numpy(arrays["numbers"])
    cn = torch.from_numpy(arrays["cn"])
    refcn = tables.refcovcn[numbers]
    dcn = (cn.unsqueeze(-1) - refcn).abs().min(-1)[0]
    assert (dcn > 11.0).any(), dcn


VARIANTS = golden_variant_cases()


def _variant_kwargs(arrays, meta):
    kw = {"model": meta["model"], "damping": meta["damping"], "exact_c9": meta["exact_c9"]}
    if "rvdw" in arrays:
        kw["rvdw"] = torch.from_numpy(arrays["rvdw"])
    return kw


@pytest.mark.parametrize("tag,arrays,meta", VARIANTS, ids=[c[0] for c in VARIANTS])
def test_damping_variants_and_exact_c9(tag, arrays, meta):
    """The oracle's D3-family damping and exact C9 against the reference's
    ZeroDamping / MZeroDamping / OptimisedPowerDamping and DispD4Exact:
    energies 1e-12, position and parameter gradients 1e-10."""
    numbers, positions, charge, param, cutoff = _inputs(arrays, meta)
    pos = positions.clone().requires_grad_(True)
    keys = sorted(param)
    ptens = {k: torch.tensor(v, dtype=torch.float64, requires_grad=True)
             for k, v in param.items()}
    energy = oracle.dftd4(numbers, pos, charge, ptens, cutoff=cutoff,
                          **_variant_kwargs(arrays, meta))
    assert_close(energy.detach(), arrays["energy"], RTOL, ATOL, "energy")
    grads = torch.autograd.grad(energy.sum(), [pos] + [ptens[k] for k in keys])
    assert_close(grads[0], arrays["grad"], 1e-10, 1e-14, "grad")
    assert_close(np.array([g.item() for g in grads[1:]]), arrays["param_grad"],
                 1e-10, 1e-14, "param_grad")
