"""
The serving loop (``tad-dftd4_gb300/serving.py``): scheduling policy on the
CPU with stand-in slots (bucketing, batch-size choice, max-wait dispatch,
admission by memory), and on the GPU the property the serving form promises:
every result is the same alone and in a mixed stream.
"""

from __future__ import annotations

import importlib

import numpy as np
import pytest
import torch

from conftest import package

PARAM = {"s6": 1.0, "s8": 1.2, "a1": 0.4, "a2": 5.0, "s9": 1.0}


def serving():
    return importlib.import_module("tad-dftd4_gb300.serving")


class FakeSlot:
    """Completes after ``delay`` polls; energy = request id."""

    def __init__(self, N, B, nbytes, delay=1):
        self.N, self.B, self.bytes, self.delay = N, B, nbytes, delay
        self.reqs, self.left = None, 0
        self.launches = []

    def launch(self, reqs, now):
        self.reqs, self.left = reqs, self.delay
        self.launches.append(len(reqs))

    def ready(self):
        self.left -= 1
        return self.left < 0

    def collect(self, now):
        sv = serving()
        out = [sv.Result(r.rid, float(r.rid), np.zeros(len(r.numbers)),
                         np.zeros((len(r.numbers), 3)), 0, r.arrival, now) for r in self.reqs]
        self.reqs = None
        return out


def _batcher(budget=1e12, max_wait=1e-3, per_shape=2, delay=1):
    sv = serving()
    buckets = (16, 64)
    sizes = {N: sv.batch_sizes_for(N, 256) for N in buckets}  # 16: (1, 4, 16); 64: (1, 4)
    made = []

    def make(N, B):
        s = FakeSlot(N, B, N * B, delay)
        made.append(s)
        return s

    b = sv.Batcher(buckets, sizes, max_wait, budget, per_shape, make, lambda N, B: N * B)
    return b, made


def _req(rid, n, t):
    sv = serving()
    return sv.Request(rid, np.full(n, 6), np.zeros((n, 3)), 0.0, t)


def test_batch_sizes_and_buckets():
    sv = serving()
    assert sv.batch_sizes_for(16, 256) == (1, 4, 16)
    assert sv.batch_sizes_for(64, 256) == (1, 4)
    assert sv.batch_sizes_for(4096) == (1, 2)
    b, _ = _batcher()
    assert b.bucket_of(5) == 16 and b.bucket_of(16) == 16 and b.bucket_of(17) == 64
    with pytest.raises(ValueError):
        b.bucket_of(65)


def test_full_batch_goes_at_once_partial_waits():
    b, made = _batcher(max_wait=1.0)
    for k in range(16):
        b.submit(_req(k, 10, 0.0))
    b.submit(_req(99, 40, 0.0))
    b.dispatch(0.0)
    assert len(b.busy) == 1 and b.busy[0].B == 16 and made[0].launches == [16]
    assert len(b.queues[64]) == 1  # alone in its bucket: waits for max_wait
    b.dispatch(1.5)
    assert len(b.busy) == 2 and b.busy[1].N == 64 and b.busy[1].B == 1


def test_batch_size_is_the_smallest_that_holds_the_queue():
    b, _ = _batcher(max_wait=0.0)
    for k in range(5):
        b.submit(_req(k, 8, 0.0))
    b.dispatch(0.0)
    assert [s.B for s in b.busy] == [16]


def test_admission_by_memory_and_slot_reuse():
    # budget for one 16 x 16 slot only: the second batch waits for the first
    b, made = _batcher(budget=16 * 16, max_wait=0.0, delay=2)
    for k in range(32):
        b.submit(_req(k, 12, 0.0))
    done = []
    for step in range(20):
        b.dispatch(float(step))
        done.extend(b.poll(float(step)))
        if len(done) == 32:
            break
    assert sorted(r.rid for r in done) == list(range(32))
    assert len(made) == 1 and made[0].launches == [16, 16]
    assert b.stats["admission_waits"] > 0 and b.bytes <= 16 * 16


@pytest.fixture(scope="module")
def gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return package()


def _stream(seed, count, nmax):
    sv = serving()
    wl = package().workloads
    rng = np.random.default_rng(seed)
    sizes = np.clip(np.round(rng.lognormal(np.log(40), 0.8, count)), 3, nmax).astype(int)
    reqs = []
    for k, n in enumerate(sizes):
        z, r = wl.structure(seed * 1000 + k, int(n))
        reqs.append(sv.Request(k, z, r, float(rng.integers(-1, 2)), 1e-4 * k))
    return reqs


@pytest.mark.gpu
@pytest.mark.parametrize("precision,e_tol,f_tol", [("mixed", 1e-8, 1e-7), ("fp64", 1e-12, 1e-12)])
def test_results_same_alone_and_in_the_mix(gpu, precision, e_tol, f_tol):
    """A stream of uneven sizes (several buckets, partial and full batches,
    overlapping on several streams) gives each structure the result it gets
    alone in a batch of one, and the result of the direct ``dftd4`` call."""
    sv = serving()
    reqs = _stream(41, 40, 300)
    srv = sv.Server(PARAM, precision=precision, max_wait=2e-3, buckets=(16, 64, 128, 512))
    mixed, stats = sv.serve_stream(srv, reqs, realtime=False)
    assert stats["failed"] == 0 and stats["batches"] < len(reqs)
    for r in reqs[:12]:
        srv.submit(sv.Request(r.rid, r.numbers, r.positions, r.charge, 0.0))
        alone = []
        while not alone:
            srv.dispatch(1e9)
            alone = srv.poll(0.0)
        a, m = alone[0], mixed[r.rid]
        assert a.status == 0
        assert abs(a.energy - m.energy) <= e_tol, (r.rid, a.energy, m.energy)
        assert np.abs(a.gradient - m.gradient).max() <= f_tol
    dev = torch.device("cuda")
    for r in reqs[12:16]:
        e, g = gpu.dispersion_energy_gradient(
            torch.from_numpy(r.numbers).to(dev), torch.from_numpy(r.positions).to(dev),
            r.charge, PARAM, precision=precision)
        m = mixed[r.rid]
        assert abs(e.sum().item() - m.energy) <= max(e_tol, 1e-7 if precision == "mixed" else 0)
        assert np.abs(g.cpu().numpy() - m.gradient).max() <= max(f_tol, 1e-6 if precision ==
                                                                     "mixed" else 0)
