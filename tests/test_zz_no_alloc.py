"""
The allocation-free entry point ``d4_dispersion_noalloc`` (for callers that
cannot call cudaMalloc, e.g. code inside a host callback, a real-time loop
with a fixed memory budget, or a plugin that must not use its host's
allocator).  Called through the C ABI with ctypes, two calls in a row on
different inputs, each compared with ``d4_dispersion`` on a caller-provided
workspace.  This file is collected last on purpose.
"""

from __future__ import annotations

import importlib

import numpy as np
import pytest
import torch

from conftest import assert_close, package

pytestmark = pytest.mark.gpu

E_RTOL, E_ATOL = 1e-12, 1e-15
G_RTOL, G_ATOL = 1e-10, 1e-13


def _call(lib, m, runner, positions, noalloc: bool):
    """One call through the C ABI; returns (status, energy, gradient)."""
    B, N = runner.numbers.shape
    dev = positions.device
    flags = m.FLAG_GRADIENT
    energy = torch.full((B, N), float("nan"), dtype=torch.float64, device=dev)
    grad = torch.full((B, N, 3), float("nan"), dtype=torch.float64, device=dev)
    p = runner.params
    params = m.Params(s6=p["s6"], s8=p["s8"], s10=p["s10"], a1=p["a1"], a2=p["a2"],
                      s9=p["s9"], alp=p["alp"], has_s8=int(p["has_s8"]),
                      has_s10=int(p["has_s10"]), cut_disp2=runner.cut["disp2"],
                      cut_disp3=runner.cut["disp3"], cut_cn=runner.cut["cn"],
                      cut_cn_eeq=runner.cut["cn_eeq"], cn_eeq_max=8.0, kcn=7.5,
                      k4=4.10451, k5=19.08857, k6=2 * 11.28174**2)
    batch = m.Batch(n_struct=B, n_pad=N, d_numbers=runner.numbers.data_ptr(),
                    d_positions=positions.data_ptr(), d_charge=runner.charge.data_ptr())
    outs = m.Outputs(d_energy=energy.data_ptr(), d_gradient=grad.data_ptr())
    cfg = m.ModelCfg(kind=m.MODEL_D4, ga=3.0, gc=2.0, wf=6.0)
    stream = torch.cuda.current_stream(dev).cuda_stream
    if noalloc:
        status = lib.d4_dispersion_noalloc(runner.tables.struct, cfg, batch, params, flags, 1,
                                           outs, 1, stream)
    else:
        size = lib.d4_workspace_size(B, N, 1, flags)
        work = torch.empty(size, dtype=torch.uint8, device=dev)
        status = lib.d4_dispersion(runner.tables.struct, cfg, batch, params, flags, 1,
                                   work.data_ptr(), size, outs, stream)
        if status == 0:
            status = lib.d4_read_status(work.data_ptr(), stream)
    torch.cuda.synchronize(dev)
    return status, energy.cpu().numpy(), grad.cpu().numpy()


def _runner(seed, nstruct, nmax):
    pkg = package()
    disp = importlib.import_module("tad-dftd4_gb300.disp")
    wl = pkg.workloads
    b = wl.batch_uniform(seed, nstruct, 4, nmax, wl.ELEMENTS_12, True, "noalloc", nmax)
    dev = torch.device("cuda")
    numbers = torch.from_numpy(b.numbers).to(dev)
    positions = torch.from_numpy(b.positions).to(dev)
    charge = torch.from_numpy(b.charge).to(dev)
    runner, _, _ = disp._prepare(numbers, positions, charge, dict(wl.BJ_PARAMS), "d4", None,
                                 None, None, None, None, None, None, None)
    return runner, positions


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return package()._lib.load()


def test_noalloc_matches_workspace_entry_point_twice(lib):
    m = package()._lib
    # two different problems in a row: the second call must not see the first
    for seed, nstruct, nmax in ((201, 6, 48), (202, 3, 90)):
        runner, positions = _runner(seed, nstruct, nmax)
        s_ref, e_ref, g_ref = _call(lib, m, runner, positions, noalloc=False)
        s_new, e_new, g_new = _call(lib, m, runner, positions, noalloc=True)
        assert s_ref == 0 and s_new == 0, (s_ref, s_new)
        assert np.isfinite(e_new).all() and np.isfinite(g_new).all()
        assert_close(e_new, e_ref, E_RTOL, E_ATOL, "energy")
        assert_close(g_new, g_ref, G_RTOL, G_ATOL, "gradient")


def test_noalloc_rejects_problems_beyond_its_scratch(lib):
    m = package()._lib
    runner, positions = _runner(203, 2, 16)
    big_b, big_n = 64, 256
    assert lib.d4_workspace_size(big_b, big_n, 1, m.FLAG_GRADIENT) > 32 * 1024 * 1024
    batch = m.Batch(n_struct=big_b, n_pad=big_n, d_numbers=runner.numbers.data_ptr(),
                    d_positions=positions.data_ptr(), d_charge=runner.charge.data_ptr())
    outs = m.Outputs(d_energy=positions.data_ptr())
    status = lib.d4_dispersion_noalloc(runner.tables.struct, m.ModelCfg(kind=0, ga=3.0,
                                       gc=2.0, wf=6.0), batch, m.Params(), m.FLAG_GRADIENT,
                                       1, outs, 1, torch.cuda.current_stream().cuda_stream)
    assert status == 2  # D4_ERR_WORKSPACE, nothing queued
