"""
Bounded waits on the GPU (failure detection without a GPU fault).

Every wait of the tensor-core kernels is bounded by the GPU's global timer
and reports ``D4_ERR_DEVICE_TIMEOUT`` through the status word instead of
hanging.  ``d4_selftest_wait`` runs that wait loop on an mbarrier nothing
ever arrives on, with a 2 ms limit: it must give up and report the timeout.
``D4_FLAG_TEST_TIMEOUT`` makes the tensor-core pair kernel treat its first
MMA wait as timed out: the call must report status 8 (raised on the host),
and the next normal call must be unaffected (tensor memory released, no
leftover state) -- checked against the oracle at the precision form's bar.
"""

from __future__ import annotations

import ctypes
import time
from importlib import import_module

import numpy as np
import pytest
import torch

import oracle
from conftest import package

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def d4():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return package()


def test_bounded_wait_gives_up_and_reports(d4):
    lib = d4._lib.load()
    res = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    assert lib.d4_selftest_wait(ctypes.c_void_p(res.data_ptr()), 2_000_000, stream) == 0
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    assert int(res.item()) == 8  # D4_ERR_DEVICE_TIMEOUT
    assert dt >= 2e-3
    assert lib.d4_selftest_wait(None, 1000, stream) == 1  # argument check, nothing launched


def test_timed_out_mma_wait_reports_and_the_next_call_is_clean(d4):
    disp = import_module("tad-dftd4_gb300.disp")
    wl = d4.workloads
    b = wl.batch_uniform(31, 6, 20, 80, wl.ELEMENTS_12, True, "timeout", 80)
    param = dict(wl.BJ_PARAMS)
    dev = torch.device("cuda")
    nt, pt, ct = (torch.from_numpy(x).to(dev) for x in (b.numbers, b.positions, b.charge))
    runner, _, _ = disp._prepare(nt, pt, ct, param, "d4", None, None, None, None, None,
                                 None, None, None, "mixed")
    with pytest.raises(d4._lib.LibraryError, match="D4_ERR_DEVICE_TIMEOUT"):
        runner.run(pt, gradient=True, extra_flags=d4._lib.FLAG_TEST_TIMEOUT)
    e, g, _, _, _ = runner.run(pt, gradient=True)
    e_ref, g_ref = oracle.dftd4_energy_and_grad(torch.from_numpy(b.numbers),
                                                torch.from_numpy(b.positions),
                                                torch.from_numpy(b.charge), param)
    de = np.abs(e.sum(-1).cpu().numpy() - e_ref.sum(-1).numpy()).max()
    dg = np.abs(g.cpu().numpy() - g_ref.numpy()).max()
    assert de <= 1e-7 and dg <= 1e-6, (de, dg)
