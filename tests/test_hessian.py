"""
Hessian of the total dispersion energy (``hessian``): finite differences of
the analytic gradient -- the scheme of the Fortran dftd4 program behind the
reference's golden Hessians (``test/test_grad/test_hessian.py:20-28``) --
with Richardson extrapolation.  The golden values themselves need the
element tables this build lacks (see the parity notes), so the bar is the
oracle's exact second derivatives (autograd through the float64
restatement): the reference test's tolerance, 1e-7 (``test_hessian.py:47``),
on small structures, and 1e-10 Eh/Bohr^2 on 30-atom structures, D4 and D4S.
"""

from __future__ import annotations

from importlib import import_module

import pytest
import torch

import oracle
from conftest import package

TOL = 1e-7
PARAM = {"s6": 1.0, "s8": 1.62438102, "s9": 1.0, "a1": 0.40329022, "a2": 4.80537871}


def _batch(seed=305, nmin=4, nmax=7):
    wl = package().workloads
    b = wl.batch_uniform(seed, 2, nmin, nmax, wl.ELEMENTS_12, True, "t", nmax)
    return tuple(torch.from_numpy(x) for x in (b.numbers, b.positions, b.charge))


def _oracle_hessian(nt, pt, ct, model="d4"):
    out = []
    for k in range(nt.shape[0]):
        def energy(p, k=k):
            return oracle.dftd4(nt[k:k + 1], p[None], ct[k:k + 1], PARAM, model=model).sum()
        out.append(torch.autograd.functional.hessian(energy, pt[k].clone()))
    return torch.stack(out)


@pytest.mark.parametrize("order", [2, 4])
def test_fd_hessian_of_a_quadratic_is_exact(order):
    """E = 1/2 x^T A x per structure: central differences of A x, and their
    Richardson combination, give A."""
    disp = import_module("tad-dftd4_gb300.disp")
    B, N = 3, 4
    g = torch.Generator().manual_seed(11)
    a = torch.randn(B, 3 * N, 3 * N, generator=g, dtype=torch.float64)
    a = a + a.transpose(1, 2)
    nums = (torch.arange(B) + 1)[:, None].expand(B, N)  # numbers tag the structure
    pos = torch.randn(B, N, 3, generator=g, dtype=torch.float64)

    calls = []

    def grad_fn(n, p, c, src):
        k = n[:, 0] - 1  # structure of each geometry
        assert torch.equal(k, src)
        calls.append(len(n))
        return torch.einsum("mij,mj->mi", a[k], p.reshape(-1, 3 * N)).reshape(-1, N, 3)

    h = disp._fd_hessian(grad_fn, nums, pos, torch.zeros(B), 1e-3, max_structs=40,
                         order=order)
    assert torch.allclose(h.reshape(B, 3 * N, 3 * N), a, atol=1e-9, rtol=0)
    assert max(calls) <= 40 and sum(calls) == B * order * 3 * N


@pytest.mark.parametrize("order", [2, 4])
def test_fd_hessian_splits_a_structure_beyond_the_call_limit(order):
    """2 x 3N (4 x 3N) displaced geometries above max_structs: the
    coordinates of one structure are split over several calls, none larger
    than the limit."""
    disp = import_module("tad-dftd4_gb300.disp")
    B, N = 2, 5  # 30 geometries per structure
    g = torch.Generator().manual_seed(12)
    a = torch.randn(B, 3 * N, 3 * N, generator=g, dtype=torch.float64)
    a = a + a.transpose(1, 2)
    nums = (torch.arange(B) + 1)[:, None].expand(B, N)
    pos = torch.randn(B, N, 3, generator=g, dtype=torch.float64)
    calls = []

    def grad_fn(n, p, c, src):
        calls.append(len(n))
        return torch.einsum("mij,mj->mi", a[src], p.reshape(-1, 3 * N)).reshape(-1, N, 3)

    h = disp._fd_hessian(grad_fn, nums, pos, torch.zeros(B), 1e-3, max_structs=8,
                         order=order)
    assert torch.allclose(h.reshape(B, 3 * N, 3 * N), a, atol=1e-9, rtol=0)
    assert max(calls) <= 8 and sum(calls) == B * order * 3 * N


def test_fd_hessian_of_the_oracle_gradient_matches_autograd():
    """The scheme at its default step on the oracle's own gradient against
    its exact second derivatives: central differences reach ~1e-7 on
    30-atom structures with close contacts, the Richardson combination
    ~1e-12."""
    disp = import_module("tad-dftd4_gb300.disp")
    nt, pt, ct = _batch(306, 24, 30)

    def grad_fn(n, p, c, src):
        return oracle.dftd4_energy_and_grad(n, p, c, PARAM)[1]

    ref = _oracle_hessian(nt, pt, ct)
    h = disp._fd_hessian(grad_fn, nt, pt, ct, 1.25e-4, order=4)
    assert (h - ref).abs().max().item() < 1e-10
    h2 = disp._fd_hessian(grad_fn, nt, pt, ct, 1e-4, order=2)
    assert (h2 - ref).abs().max().item() > 1e-9  # what the extrapolation removes


@pytest.mark.gpu
def test_hessian_matches_oracle_second_derivatives():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    d4 = package()
    nt, pt, ct = _batch()
    dev = torch.device("cuda")
    ref = _oracle_hessian(nt, pt, ct)
    h = d4.hessian(nt.to(dev), pt.to(dev), ct.to(dev), PARAM).cpu()
    assert h.shape == (2, 7, 3, 7, 3)
    assert torch.allclose(h, ref, atol=TOL, rtol=TOL)
    h1 = d4.hessian(nt[0].to(dev), pt[0].to(dev), ct[0].to(dev), PARAM).cpu()
    assert h1.shape == (7, 3, 7, 3)
    assert torch.allclose(h1, ref[0], atol=TOL, rtol=TOL)
    real = nt != 0
    assert (h[~real] == 0).all()


@pytest.mark.gpu
@pytest.mark.parametrize("model", ["d4", "d4s"])
def test_hessian_of_30_atom_structures_matches_oracle(model):
    """Two charged 24-30-atom structures (one padded): the GPU Hessian
    against the oracle's autograd Hessian at 1e-10 Eh/Bohr^2, D4 and D4S."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    d4 = package()
    nt, pt, ct = _batch(306, 24, 30)
    dev = torch.device("cuda")
    ref = _oracle_hessian(nt, pt, ct, model)
    h = d4.hessian(nt.to(dev), pt.to(dev), ct.to(dev), PARAM, model=model).cpu()
    assert (h - ref).abs().max().item() < 1e-10
