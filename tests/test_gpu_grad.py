"""
The hand-written adjoint against central finite differences (the
differentiation form: structures of 20-150 atoms over 12 elements, damping
parameters drawn per structure, D4 and D4S).  Forces: central differences
with h = 1e-4 Bohr on a sample of coordinates; parameter gradients
dE/d(s6, s8, a1, a2, s9): central differences in the parameter.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import package

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def d4():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return package()


def _structures(count=3):
    batch, params = package().workloads.diff256(3, 6)
    out = []
    for k in range(count):
        n = int((batch.numbers[k] != 0).sum())
        out.append((batch.numbers[k, :n], batch.positions[k, :n], params[k]))
    return out


def _energy(d4, z, r, param, model, precision):
    dev = torch.device("cuda")
    nt = torch.from_numpy(z).to(dev)
    pt = torch.from_numpy(r).to(dev)
    return float(d4.dftd4(nt, pt, 0.0, param, model=model, precision=precision).sum())


@pytest.mark.parametrize("model", ["d4", "d4s"])
@pytest.mark.parametrize("precision,atol,rtol", [("fp64", 1e-8, 1e-6), ("mixed", 1e-6, 0.0)])
def test_forces_match_central_differences(d4, model, precision, atol, rtol):
    """Central differences of the FP64 energy (h = 1e-4 Bohr) against the
    analytic gradient of each method: the FP64 adjoint to 1e-8 Eh/Bohr, the
    precision form's within its force bar (1e-6 Eh/Bohr).  (Differences of
    the precision form's own energy would measure its ~1e-9 Eh FP32
    rounding noise divided by 2h, not its gradient.)"""
    dev = torch.device("cuda")
    h = 1e-4
    rng = np.random.default_rng(11)
    for z, r, param in _structures():
        nt = torch.from_numpy(z).to(dev)
        pt = torch.from_numpy(r).to(dev)
        _, g = d4.dispersion_energy_gradient(nt, pt, 0.0, param, model=model,
                                             precision=precision)
        g = g.cpu().numpy()
        for _ in range(6):
            a, x = int(rng.integers(len(z))), int(rng.integers(3))
            rp, rm = r.copy(), r.copy()
            rp[a, x] += h
            rm[a, x] -= h
            fd = (_energy(d4, z, rp, param, model, "fp64") -
                  _energy(d4, z, rm, param, model, "fp64")) / (2 * h)
            assert abs(fd - g[a, x]) <= atol + rtol * abs(fd), (a, x, fd, g[a, x])


@pytest.mark.parametrize("model", ["d4", "d4s"])
def test_parameter_gradients_match_central_differences(d4, model):
    dev = torch.device("cuda")
    keys = ["s6", "s8", "a1", "a2", "s9"]
    for z, r, param in _structures(2):
        nt = torch.from_numpy(z).to(dev)
        pt = torch.from_numpy(r).to(dev)
        pd = {k: torch.tensor(param[k], dtype=torch.float64, device=dev, requires_grad=True)
              for k in keys}
        e = d4.dftd4(nt, pt, 0.0, pd, model=model)
        grads = torch.autograd.grad(e.sum(), [pd[k] for k in keys])
        for k, g in zip(keys, grads):
            h = 1e-5 * max(1.0, abs(param[k]))
            pp, pm = dict(param), dict(param)
            pp[k] += h
            pm[k] -= h
            fd = (_energy(d4, z, r, pp, model, "fp64") - _energy(d4, z, r, pm, model, "fp64")) / (2 * h)
            assert abs(fd - g.item()) <= 1e-9 + 1e-6 * abs(fd), (k, fd, g.item())
