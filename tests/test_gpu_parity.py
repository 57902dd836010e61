"""
Parity of the CUDA path with tad-dftd4's own outputs and with the oracle.

Tolerances (float64, plain method): atom energies 1e-12 relative with a
1e-15 Eh absolute floor; gradients 1e-10 relative with a 1e-13 Eh/Bohr
floor; charges and CN 1e-10 relative.  The golden fixtures are the
reference's own values (``tests/golden/golden.npz``).
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

import oracle
from conftest import assert_close, golden_cases, package

pytestmark = pytest.mark.gpu

CASES = golden_cases()
E_RTOL, E_ATOL = 1e-12, 1e-15
G_RTOL, G_ATOL = 1e-10, 1e-13


@pytest.fixture(scope="module")
def d4():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return package()


def _model(d4, meta, numbers):
    cls = d4.D4Model if meta["model"] == "d4" else d4.D4SModel
    return cls(numbers, ref_charges=meta["ref_charges"])


def _run(d4, arrays, meta, grad=True, param_grad=False):
    dev = torch.device("cuda")
    numbers = torch.from_numpy(arrays["numbers"]).to(dev)
    positions = torch.from_numpy(arrays["positions"]).to(dev)
    charge = torch.from_numpy(arrays["charge"]).to(dev)
    cutoff = d4.Cutoff(**meta["cutoff"]) if meta["cutoff"] else None
    keys = sorted(meta["param"])
    param = {k: torch.tensor(v, dtype=torch.float64, device=dev, requires_grad=param_grad)
             for k, v in meta["param"].items()}
    pos = positions.clone().requires_grad_(grad)
    energy = d4.dftd4(numbers, pos, charge, param, model=_model(d4, meta, numbers),
                      cutoff=cutoff)
    out = {"energy": energy.detach().cpu().numpy()}
    if grad or param_grad:
        wrt = ([pos] if grad else []) + ([param[k] for k in keys] if param_grad else [])
        gs = torch.autograd.grad(energy.sum(), wrt)
        if grad:
            out["grad"] = gs[0].cpu().numpy()
        if param_grad:
            out["param_grad"] = np.array([g.item() for g in gs[-len(keys):]])
    return out


@pytest.mark.parametrize("tag,arrays,meta", CASES, ids=[c[0] for c in CASES])
def test_energy_matches_reference(d4, tag, arrays, meta):
    out = _run(d4, arrays, meta, grad=False)
    assert_close(out["energy"], arrays["energy"], E_RTOL, E_ATOL, "energy")


@pytest.mark.parametrize("tag,arrays,meta",
                         [c for c in CASES if not c[2]["energy_only"]],
                         ids=[c[0] for c in CASES if not c[2]["energy_only"]])
def test_gradient_matches_reference(d4, tag, arrays, meta):
    out = _run(d4, arrays, meta, grad=True)
    assert_close(out["energy"], arrays["energy"], E_RTOL, E_ATOL, "energy")
    assert_close(out["grad"], arrays["grad"], G_RTOL, G_ATOL, "grad")


@pytest.mark.parametrize("tag,arrays,meta",
                         [c for c in CASES if not c[2]["energy_only"]],
                         ids=[c[0] for c in CASES if not c[2]["energy_only"]])
def test_param_gradient_matches_reference(d4, tag, arrays, meta):
    out = _run(d4, arrays, meta, grad=False, param_grad=True)
    assert_close(out["param_grad"], arrays["param_grad"], G_RTOL, G_ATOL, "param_grad")


@pytest.mark.parametrize("tag,arrays,meta", CASES, ids=[c[0] for c in CASES])
def test_charges_and_cn(d4, tag, arrays, meta):
    from importlib import import_module
    disp = import_module("tad-dftd4_gb300.disp")
    dev = torch.device("cuda")
    numbers = torch.from_numpy(arrays["numbers"]).to(dev)
    positions = torch.from_numpy(arrays["positions"]).to(dev)
    charge = torch.from_numpy(arrays["charge"]).to(dev)
    cutoff = d4.Cutoff(**meta["cutoff"]) if meta["cutoff"] else None
    runner, _, _ = disp._prepare(numbers, positions, charge, meta["param"],
                                 _model(d4, meta, numbers), None, None, None, None, cutoff,
                                 None, None, None)
    _, _, _, q, cn = runner.run(positions, charges_out=True, cn_out=True)
    assert_close(cn.cpu().numpy(), arrays["cn"], 1e-12, 1e-15, "cn")
    assert_close(q.cpu().numpy(), arrays["q"], 1e-10, 1e-13, "q")


def _batch(seed, nstruct, nmin, nmax, charged=True):
    wl = package().workloads
    return wl.batch_uniform(seed, nstruct, nmin, nmax, wl.ELEMENTS_12, charged, "t", nmax)


@pytest.mark.parametrize("model", ["d4", "d4s"])
def test_random_batch_vs_oracle(d4, model):
    b = _batch(101, 6, 5, 60)
    param = {"s6": 1.0, "s8": 1.2, "a1": 0.4, "a2": 5.0, "s9": 1.0}
    numbers = torch.from_numpy(b.numbers)
    positions = torch.from_numpy(b.positions)
    charge = torch.from_numpy(b.charge)
    e_ref, g_ref = oracle.dftd4_energy_and_grad(numbers, positions, charge, param, model=model)
    dev = torch.device("cuda")
    e, g = d4.dispersion_energy_gradient(numbers.to(dev), positions.to(dev), charge.to(dev),
                                         param, model=model)
    assert_close(e.cpu().numpy(), e_ref.numpy(), E_RTOL, E_ATOL, "energy")
    assert_close(g.cpu().numpy(), g_ref.numpy(), G_RTOL, G_ATOL, "grad")


def test_nonuniform_backward_weights(d4):
    """autograd with per-atom weights (not a plain sum) re-runs the adjoint."""
    b = _batch(102, 3, 4, 20)
    param = {"s6": 1.0, "s8": 1.2, "a1": 0.4, "a2": 5.0, "s9": 1.0}
    numbers = torch.from_numpy(b.numbers)
    positions = torch.from_numpy(b.positions)
    charge = torch.from_numpy(b.charge)
    wts = torch.linspace(0.2, 1.7, numbers.numel(), dtype=torch.float64).reshape(numbers.shape)
    pos_ref = positions.clone().requires_grad_(True)
    e_ref = oracle.dftd4(numbers, pos_ref, charge, param)
    (g_ref,) = torch.autograd.grad((e_ref * wts).sum(), pos_ref)
    dev = torch.device("cuda")
    pos = positions.to(dev).requires_grad_(True)
    e = d4.dftd4(numbers.to(dev), pos, charge.to(dev), param)
    (g,) = torch.autograd.grad((e * wts.to(dev)).sum(), pos)
    assert_close(g.cpu().numpy(), g_ref.numpy(), G_RTOL, G_ATOL, "weighted grad")


def test_padding_in_the_middle_and_empty_structure(d4):
    b = _batch(103, 3, 6, 12)
    numbers = b.numbers.copy()
    positions = b.positions.copy()
    numbers[0, 2] = 0  # a hole inside structure 0
    numbers[2, :] = 0  # an all-padding structure
    param = {"s6": 1.0, "s8": 1.2, "a1": 0.4, "a2": 5.0, "s9": 1.0}
    nt, pt, ct = map(torch.from_numpy, (numbers, positions, b.charge * 0))
    # the oracle's dense EEQ system is singular for an all-padding structure,
    # so it sees only the first two
    e_ref, g_ref = oracle.dftd4_energy_and_grad(nt[:2], pt[:2], ct[:2], param)
    dev = torch.device("cuda")
    e, g = d4.dispersion_energy_gradient(nt.to(dev), pt.to(dev), ct.to(dev), param)
    assert_close(e.cpu().numpy()[:2], e_ref.numpy(), E_RTOL, E_ATOL, "energy")
    assert_close(g.cpu().numpy()[:2], g_ref.numpy(), G_RTOL, G_ATOL, "grad")
    assert (e.cpu().numpy()[2] == 0).all() and (g.cpu().numpy()[2] == 0).all()


def test_single_and_two_atoms(d4):
    dev = torch.device("cuda")
    param = {"s6": 1.0, "s8": 1.2, "a1": 0.4, "a2": 5.0, "s9": 1.0}
    for z, r in (([6], [[0.0, 0.0, 0.0]]), ([1, 8], [[0.0, 0.0, 0.0], [0.0, 0.0, 1.8]])):
        nt = torch.tensor(z)
        pt = torch.tensor(r, dtype=torch.float64)
        e_ref, g_ref = oracle.dftd4_energy_and_grad(nt, pt, torch.tensor(0.0), param)
        e, g = d4.dispersion_energy_gradient(nt.to(dev), pt.to(dev), 0.0, param)
        assert e.shape == nt.shape
        assert_close(e.cpu().numpy(), e_ref.numpy(), E_RTOL, E_ATOL, "energy")
        assert_close(g.cpu().numpy(), g_ref.numpy(), G_RTOL, G_ATOL, "grad")


def test_given_charges_and_r4r2(d4):
    b = _batch(104, 2, 8, 16, charged=False)
    param = {"s6": 1.0, "s8": 1.2, "a1": 0.4, "a2": 5.0, "s9": 1.0}
    nt, pt, ct = map(torch.from_numpy, (b.numbers, b.positions, b.charge))
    q = torch.linspace(-0.3, 0.3, nt.numel(), dtype=torch.float64).reshape(nt.shape)
    q = torch.where(nt != 0, q, torch.zeros_like(q))
    e_ref = oracle.dftd4(nt, pt, ct, param, q=q)
    dev = torch.device("cuda")
    e = d4.dftd4(nt.to(dev), pt.to(dev), ct.to(dev), param, q=q.to(dev))
    assert_close(e.cpu().numpy(), e_ref.numpy(), E_RTOL, E_ATOL, "energy with q")


def test_float32_positions_follow_dtype(d4):
    b = _batch(105, 2, 8, 16)
    param = {"s6": 1.0, "s8": 1.2, "a1": 0.4, "a2": 5.0, "s9": 1.0}
    dev = torch.device("cuda")
    pos = torch.from_numpy(b.positions).to(dev, torch.float32)
    e = d4.dftd4(torch.from_numpy(b.numbers).to(dev), pos, torch.from_numpy(b.charge).to(dev),
                 param)
    assert e.dtype == torch.float32 and e.device == pos.device


def test_bad_element_raises(d4):
    dev = torch.device("cuda")
    nt = torch.tensor([1, 104], device=dev)
    pt = torch.tensor([[0.0, 0, 0], [0, 0, 2.0]], dtype=torch.float64, device=dev)
    with pytest.raises(ValueError):
        d4.dftd4(nt, pt, 0.0, {"a1": 0.4, "a2": 5.0})


def test_bad_element_with_gradient_raises_at_backward(d4):
    """With positions that require gradients the forward call leaves its
    device status word pending: the error surfaces from autograd.grad when
    the forward has finished by then, else from the next library call or
    check_status() -- exactly once either way."""
    dev = torch.device("cuda")
    nt = torch.tensor([1, 104], device=dev)
    pt = torch.tensor([[0.0, 0, 0], [0, 0, 2.0]], dtype=torch.float64, device=dev,
                      requires_grad=True)
    e = d4.dftd4(nt, pt, 0.0, {"a1": 0.4, "a2": 5.0})
    raised = 0
    try:
        torch.autograd.grad(e.sum(), pt)
    except ValueError:
        raised += 1
    try:
        d4.check_status()
    except ValueError:
        raised += 1
    assert raised == 1
    d4.dftd4(nt, pt, 0.0, {"a1": 0.4, "a2": 5.0})
    with pytest.raises(ValueError):
        d4.check_status()
    d4.check_status()  # nothing pending any more
    good = torch.tensor([1, 8], device=dev)
    e = d4.dftd4(good, pt, 0.0, {"a1": 0.4, "a2": 5.0})
    (g,) = torch.autograd.grad(e.sum(), pt)
    assert torch.isfinite(g).all()


def test_nonfinite_positions_raise(d4):
    dev = torch.device("cuda")
    nt = torch.tensor([1, 1], device=dev)
    pt = torch.tensor([[0.0, 0, 0], [0, 0, float("nan")]], dtype=torch.float64, device=dev)
    with pytest.raises(ValueError):
        d4.dftd4(nt, pt, 0.0, {"a1": 0.4, "a2": 5.0})


@pytest.mark.parametrize("tag,arrays,meta",
                         [c for c in CASES if c[2]["model"] == "d4"
                          and c[2]["ref_charges"] == "eeq"],
                         ids=[c[0] for c in CASES if c[2]["model"] == "d4"
                              and c[2]["ref_charges"] == "eeq"])
def test_get_properties_matches_reference(d4, tag, arrays, meta):
    """get_properties (disp.py:149-197): CN, EEQ charges, C6 at the charges
    and static polarisabilities sum_r w_r alpha_r(0), against the values the
    reference's own model code produced (1e-12 relative)."""
    dev = torch.device("cuda")
    numbers = torch.from_numpy(arrays["numbers"]).to(dev)
    positions = torch.from_numpy(arrays["positions"]).to(dev)
    charge = torch.from_numpy(arrays["charge"]).to(dev)
    cutoff = d4.Cutoff(**meta["cutoff"]) if meta["cutoff"] else None
    cn, q, c6, alpha = d4.get_properties(numbers, positions, charge, cutoff=cutoff)
    assert c6.shape == numbers.shape + numbers.shape[-1:]
    assert_close(cn.cpu(), arrays["cn"], 1e-12, 1e-14, "cn")
    assert_close(q.cpu(), arrays["q"], 1e-12, 1e-13, "q")
    assert_close(c6.cpu(), arrays["c6"], 1e-12, 1e-12, "c6")
    alpha_ref = np.einsum("...r,...r->...", arrays["gw"], arrays["alpha"][..., 0])
    assert_close(alpha.cpu(), alpha_ref, 1e-12, 1e-13, "alpha")


# ---------------------------------------------------------------- damping
# variants and exact C9 (reference fixtures golden_variants.npz)

from conftest import golden_variant_cases  # noqa: E402

VARIANTS = golden_variant_cases()


def _run_variant(d4, arrays, meta):
    dev = torch.device("cuda")
    numbers = torch.from_numpy(arrays["numbers"]).to(dev)
    pos = torch.from_numpy(arrays["positions"]).to(dev).requires_grad_(True)
    charge = torch.from_numpy(arrays["charge"]).to(dev)
    cutoff = d4.Cutoff(**meta["cutoff"]) if meta["cutoff"] else None
    keys = sorted(meta["param"])
    param = {k: torch.tensor(v, dtype=torch.float64, device=dev, requires_grad=True)
             for k, v in meta["param"].items()}
    model = _model(d4, meta, numbers)
    if meta["exact_c9"]:
        energy = d4.DispD4Exact(model=model).calculate(numbers, pos, charge, param,
                                                       cutoff=cutoff)
    else:
        damping = {"zero": d4.ZeroDamping, "mzero": d4.MZeroDamping,
                   "op": d4.OptimisedPowerDamping}[meta["damping"]]()
        rvdw = torch.from_numpy(arrays["rvdw"]).to(dev) if "rvdw" in arrays else None
        energy = d4.dftd4(numbers, pos, charge, param, model=model, cutoff=cutoff,
                          rvdw=rvdw, damping_function=damping)
    gs = torch.autograd.grad(energy.sum(), [pos] + [param[k] for k in keys])
    return (energy.detach().cpu().numpy(), gs[0].cpu().numpy(),
            np.array([g.item() for g in gs[1:]]))


@pytest.mark.parametrize("tag,arrays,meta", VARIANTS, ids=[c[0] for c in VARIANTS])
def test_damping_variants_and_exact_c9_match_reference(d4, tag, arrays, meta):
    """Zero / modified-zero / optimised-power two-body damping and the exact
    C9 of DispD4Exact, plain FP64 kernels, against the reference's own
    classes: energies 1e-12, position and parameter gradients 1e-10."""
    e, g, pg = _run_variant(d4, arrays, meta)
    assert_close(e, arrays["energy"], E_RTOL, E_ATOL, "energy")
    assert_close(g, arrays["grad"], G_RTOL, G_ATOL, "grad")
    assert_close(pg, arrays["param_grad"], G_RTOL, G_ATOL, "param_grad")


@pytest.mark.parametrize("model", ["d4", "d4s"])
def test_exact_c9_batch_vs_oracle(d4, model):
    """Exact C9 on a padded, charged batch (the reference's D4S variant has
    no batched result; the oracle divides per structure)."""
    b = _batch(102, 5, 4, 40)
    param = {"s6": 1.0, "s8": 1.2, "a1": 0.4, "a2": 5.0, "s9": 1.0}
    numbers = torch.from_numpy(b.numbers)
    positions = torch.from_numpy(b.positions)
    charge = torch.from_numpy(b.charge)
    e_ref, g_ref = oracle.dftd4_energy_and_grad(numbers, positions, charge, param,
                                                model=model, exact_c9=True,
                                                cutoff={"disp3": 12.0})
    dev = torch.device("cuda")
    e, g = d4.dispersion_energy_gradient(numbers.to(dev), positions.to(dev), charge.to(dev),
                                         param, model=model, exact_c9=True,
                                         cutoff=d4.Cutoff(disp3=12.0))
    assert_close(e.cpu().numpy(), e_ref.numpy(), E_RTOL, E_ATOL, "energy")
    assert_close(g.cpu().numpy(), g_ref.numpy(), G_RTOL, G_ATOL, "grad")


def test_variant_argument_errors(d4):
    """The reference's errors for the damping family: missing parameters
    (TypeError), order 10 without it (ValueError), no pair radii, and the
    precision form refusing what it does not run."""
    dev = torch.device("cuda")
    b = _batch(103, 1, 6, 10)
    numbers = torch.from_numpy(b.numbers).to(dev)
    positions = torch.from_numpy(b.positions).to(dev)
    rv = torch.full((1, numbers.shape[1], numbers.shape[1]), 4.0, dtype=torch.float64,
                    device=dev)
    with pytest.raises(TypeError, match=r"ZeroDamping \(order 8\) requires keyword\(s\): rs8"):
        d4.dftd4(numbers, positions, 0.0, {"rs6": 1.0, "s8": 1.0}, rvdw=rv,
                 damping_function=d4.ZeroDamping())
    with pytest.raises(ValueError, match="OP-damping is only implemented"):
        d4.dftd4(numbers, positions, 0.0, {"a1": 0.4, "a2": 5.0, "bet": 1.0, "s10": 1.0},
                 damping_function=d4.OptimisedPowerDamping())
    with pytest.raises(ValueError, match="rvdw"):
        d4.dftd4(numbers, positions, 0.0, {"rs6": 1.0}, damping_function=d4.ZeroDamping())
    with pytest.raises(ValueError, match="precision form"):
        d4.dftd4(numbers, positions, 0.0, {"rs6": 1.0}, rvdw=rv,
                 damping_function=d4.ZeroDamping(), precision="mixed")


# ---------------------------------------------------------------- the plain
# FP64 method at the benchmarked sizes (the batch512 workload draws N from
# [8, 200]): the oracle per structure, unpadded, against the padded batch

def _oracle_with_scale(numbers, positions, charge, param, model="d4"):
    """Oracle energies, gradients and the per-atom error scale: each atom
    energy is a float64 sum of ~N two-body and ~N^2/2 three-body terms of
    both signs, so two summation orders differ by up to ~1e-16 sqrt(terms)
    times the sum of the terms' magnitudes, not times the net value.  The
    scale is |E2_i| + sum |ATM shares of i|."""
    pos = positions.clone().requires_grad_(True)
    e, parts = oracle.dftd4(numbers, pos, charge, param, model=model, return_parts=True)
    (g,) = torch.autograd.grad(e.sum(), pos)
    return e.detach().numpy(), g.numpy(), parts["scale"].detach().numpy()


@pytest.mark.parametrize("model", ["d4", "d4s"])
def test_plain_fp64_at_batch512_sizes_vs_oracle(d4, model):
    """8 charged structures with N in [150, 200], padded to 200, 12
    elements at density 0.01 / Bohr^3 (the batch512 generator).  Energies:
    1e-12 relative to the magnitude of each atom's summed contributions
    (|E2_i| + sum of |ATM shares|; a few atoms' net energies cancel to 1e-3
    of that, where the plain relative error of two float64 summation orders
    reaches ~4e-11); gradients 1e-10 relative with a 1e-13 Eh/Bohr floor."""
    wl = package().workloads
    b = wl.batch_uniform(7, 8, 150, 200, wl.ELEMENTS_12, True, "plain8", 200)
    param = dict(wl.BJ_PARAMS)
    dev = torch.device("cuda")
    e, g = d4.dispersion_energy_gradient(torch.from_numpy(b.numbers).to(dev),
                                         torch.from_numpy(b.positions).to(dev),
                                         torch.from_numpy(b.charge).to(dev), param,
                                         model=model, precision="fp64")
    e, g = e.cpu().numpy(), g.cpu().numpy()
    for k in range(len(b.numbers)):
        n = int((b.numbers[k] != 0).sum())
        assert 150 <= n <= 200
        e_ref, g_ref, scale = _oracle_with_scale(
            torch.from_numpy(b.numbers[k:k + 1, :n]), torch.from_numpy(b.positions[k:k + 1, :n]),
            torch.from_numpy(b.charge[k:k + 1]), param, model=model)
        err = np.abs(e[k, :n] - e_ref[0])
        assert (err <= E_RTOL * scale[0] + E_ATOL).all(), (k, (err / scale[0]).max())
        assert_close(g[k, :n], g_ref[0], G_RTOL, G_ATOL, f"grad {k}")
        assert (e[k, n:] == 0).all() and (g[k, n:] == 0).all()


def test_plain_fp64_global_memory_eeq_vs_oracle(d4):
    """One 280-atom structure: its packed Cholesky factor exceeds shared
    memory, so the FP64 EEQ solve and its adjoint run from global memory
    (the path every 400-1100-atom precision-form test compares against)."""
    wl = package().workloads
    z, r = wl.structure(4280, 280)
    numbers, positions = z[None], r[None]
    charge = np.array([1.0])
    param = dict(wl.BJ_PARAMS)
    dev = torch.device("cuda")
    e, g = d4.dispersion_energy_gradient(torch.from_numpy(numbers).to(dev),
                                         torch.from_numpy(positions).to(dev),
                                         torch.from_numpy(charge).to(dev), param,
                                         precision="fp64")
    e_ref, g_ref, scale = _oracle_with_scale(torch.from_numpy(numbers),
                                             torch.from_numpy(positions),
                                             torch.from_numpy(charge), param)
    err = np.abs(e.cpu().numpy() - e_ref)
    assert (err <= E_RTOL * scale + E_ATOL).all(), (err / scale).max()
    assert_close(g.cpu().numpy(), g_ref, G_RTOL, G_ATOL, "grad")
