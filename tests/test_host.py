"""
Host-side behaviour of the drop-in ``dftd4()`` that needs no GPU: the
reference's argument checks and error types (``dispersion/base.py:354-414``,
``damping/functions.py:68-114``) and the refusal to compute on the CPU.
"""

from __future__ import annotations

import pytest
import torch

from conftest import package

PARAM = {"s6": 1.0, "s8": 1.0, "a1": 0.4, "a2": 5.0}


@pytest.fixture
def d4():
    return package()


def test_shape_errors(d4):
    numbers = torch.tensor([1, 1])
    positions = torch.tensor([[0.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
    with pytest.raises(ValueError):
        d4.dftd4(numbers, positions, 0.0, PARAM, rcov=torch.tensor([1.0]))
    with pytest.raises(ValueError):
        d4.dftd4(numbers, positions, 0.0, PARAM, r4r2=torch.tensor([1.0]))
    with pytest.raises(ValueError):
        d4.dftd4(numbers, positions, 0.0, PARAM, rvdw=torch.tensor([1.0]))
    with pytest.raises(ValueError):
        d4.dftd4(numbers, positions, 0.0, PARAM, q=torch.tensor([1.0]))
    with pytest.raises(ValueError):
        d4.dftd4(torch.tensor([1]), positions, 0.0, PARAM, q=torch.tensor([0.5, -0.5]))


def test_missing_damping_parameters_raise_type_error(d4):
    numbers = torch.tensor([1, 1])
    positions = torch.tensor([[0.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
    with pytest.raises(TypeError):
        d4.dftd4(numbers, positions, 0.0, {"s6": 1.0})


def test_unknown_model(d4):
    numbers = torch.tensor([1, 1])
    positions = torch.tensor([[0.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
    with pytest.raises(ValueError):
        d4.dftd4(numbers, positions, 0.0, PARAM, model="d9")


def test_cpu_inputs_are_refused(d4):
    numbers = torch.tensor([1, 1])
    positions = torch.tensor([[0.0, 0.0, 0.0], [0.0, 0.0, 1.0]], dtype=torch.float64)
    with pytest.raises(RuntimeError, match="CUDA"):
        d4.dftd4(numbers, positions, 0.0, PARAM)


def test_param_resolution_follows_reference_gating(d4):
    from importlib import import_module
    damping = import_module("tad-dftd4_gb300.damping")
    r = damping.resolve({"a1": 0.5, "a2": 4.0})
    assert r["s6"] == 1.0 and not r["has_s8"] and not r["has_s10"]
    assert r["s9"] == 1.0 and r["alp"] == 16.0
    r = damping.resolve({"a1": torch.tensor(0.5), "a2": 4.0, "s8": 2.0, "s10": 0.0})
    assert r["has_s8"] and r["s8"] == 2.0 and r["has_s10"]


def test_cutoff_defaults(d4):
    c = d4.Cutoff()
    assert float(c.disp2) == 60.0 and float(c.disp3) == 40.0
    assert float(c.cn) == 30.0 and float(c.cn_eeq) == 25.0


def test_model_descriptors(d4):
    z = torch.tensor([6, 1])
    assert d4.D4Model(z).wf == 6.0
    with pytest.raises(ValueError):
        d4.D4Model(z, ref_charges="xyz")
    with pytest.raises(NotImplementedError):
        d4.D4SModel(z, wf=3.0)


class _FakeEvent:
    """Stands in for torch.cuda.Event: completed or not, synchronize() marks
    it completed."""

    def __init__(self, done):
        self.done = done
        self.waited = False

    def query(self):
        return self.done

    def synchronize(self):
        self.waited = True
        self.done = True


def _token(status, done):
    return (torch.tensor([status], dtype=torch.int32), _FakeEvent(done), "test call")


def test_deferred_status_words():
    """The status words that forward calls with gradients leave pending:
    a completed word is read by the next call's drain (raising its error),
    an incomplete one stays until check_status() waits for it; errors map
    to the same exceptions as the synchronous check."""
    from importlib import import_module
    disp = import_module("tad-dftd4_gb300.disp")
    disp._PENDING.clear()
    try:
        ok_done, bad_busy = _token(0, True), _token(4, False)
        disp._PENDING.extend([ok_done, bad_busy])
        disp._drain_pending()  # reads the completed word, keeps the busy one
        assert len(disp._PENDING) == 1 and disp._PENDING[0] is bad_busy
        assert not bad_busy[1].waited
        with pytest.raises(ValueError, match="element tables"):
            disp.check_status()
        assert bad_busy[1].waited and not disp._PENDING
        disp._PENDING.append(_token(6, True))
        with pytest.raises(ValueError, match="non-finite"):
            disp._drain_pending()
        # more pending words than the cap: the oldest are waited for
        toks = [_token(0, False) for _ in range(disp._PENDING_MAX + 3)]
        disp._PENDING.extend(toks)
        disp._drain_pending()
        assert len(disp._PENDING) == disp._PENDING_MAX
        assert all(t[1].waited for t in toks[:3])
    finally:
        disp._PENDING.clear()


def test_configuration_cache_keys():
    """Plain configurations (D4 by name, parameters as numbers) get a
    hashable cache key; parameter tensors, other models and custom cutoff
    objects do not (they take the full preparation on every call)."""
    from importlib import import_module
    disp = import_module("tad-dftd4_gb300.disp")
    Cutoff = package().Cutoff
    dev, dt = torch.device("cuda", 0), torch.float64
    p = {"s6": 1.0, "s8": 1.2, "a1": 0.4, "a2": 5.0}
    k1 = disp._config_key(p, "d4", None, "mixed", dev, dt)
    k2 = disp._config_key(dict(p), "D4", None, "mixed", dev, dt)
    assert k1 is not None and k1 == k2 and hash(k1) == hash(k2)
    assert disp._config_key(dict(p, a1=0.41), "d4", None, "mixed", dev, dt) != k1
    assert disp._config_key(p, "d4", None, "fp64", dev, dt) != k1
    assert disp._config_key(p, "d4", Cutoff(disp3=25.0), "mixed", dev, dt) != k1
    assert disp._config_key(dict(p, s8=torch.tensor(1.2)), "d4", None, "mixed", dev, dt) is None
    assert disp._config_key(p, "d4s", None, "mixed", dev, dt) is None
    assert disp._config_key(p, object(), None, "mixed", dev, dt) is None
