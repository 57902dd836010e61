"""
Energy + force serving: continuous batching of independent structures onto
the CUDA library, one captured CUDA graph per (size bucket, batch size).

A request is one structure (atomic numbers, positions in Bohr, total
charge).  It waits in the queue of the smallest size bucket N >= n (padded
with atomic number 0, the batch convention of ``dftd4``).  A bucket is
dispatched when it holds a full batch or its oldest request has waited
``max_wait`` seconds; the batch size is the smallest captured size that
holds the queue (up to the bucket's largest).  Each (N, B) shape owns
"slots": pinned host buffers, device buffers, a workspace and the graph that
copies the inputs in, runs the whole energy + gradient call and copies the
results and the device status word out, replayed on the slot's own stream.
Batches of different shapes (and several of the same shape) are therefore
in flight together and overlap on the device; a finished slot is recycled
as soon as its event completes.  Slots are created on demand while their
memory fits the HBM budget; when it does not, requests wait until a slot is
free (admission by memory).  Charges, coordination numbers and the pair
tables of a batch stay in the slot's workspace on the device; only inputs
and results cross PCIe / C2C.

The result of a request does not depend on its batch: structures are
independent in every kernel (padding atoms and padded structures contribute
nothing), so a structure alone and in a mixed batch agree within the
precision of the method (tests/test_serving.py checks it).
"""

from __future__ import annotations

import collections
import time
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .cutoff import D4_CN_EEQ_MAX, D4_K4, D4_K5, D4_K6, D4_KCN
from .disp import _prepare

__all__ = ["Request", "Result", "Batcher", "Server", "serve_stream", "DEFAULT_BUCKETS"]

DEFAULT_BUCKETS = (16, 32, 64, 128, 256, 512, 1024, 2048, 4096)


@dataclass
class Request:
    """One structure to evaluate (no padding)."""

    rid: int
    numbers: np.ndarray  # (n,) atomic numbers
    positions: np.ndarray  # (n, 3) Bohr
    charge: float = 0.0
    arrival: float = 0.0  # server clock, seconds


@dataclass
class Result:
    rid: int
    energy: float  # total dispersion energy, Eh
    atom_energies: np.ndarray  # (n,)
    gradient: np.ndarray  # (n, 3) dE/dR, Eh/Bohr
    status: int  # d4_status of the batch (0: ok)
    arrival: float
    done: float

    @property
    def latency(self) -> float:
        return self.done - self.arrival


def batch_sizes_for(n_pad: int, atoms_per_batch: int = 8192, max_batch: int = 256):
    """Captured batch sizes of a bucket: 1, 4, 16, ... up to about
    ``atoms_per_batch`` padded atoms."""
    top = max(1, min(max_batch, atoms_per_batch // n_pad))
    sizes, b = [], 1
    while b < top:
        sizes.append(b)
        b *= 4
    sizes.append(top)
    return tuple(sorted(set(sizes)))


class _Slot:
    """Buffers, workspace, stream and captured graph of one (N, B) shape."""

    def __init__(self, srv: "Server", n_pad: int, batch: int):
        lib = _lib.load()
        dev = srv.device
        self.N, self.B = n_pad, batch
        B, N = batch, n_pad
        pin = dict(pin_memory=True)
        self.h_num = torch.zeros((B, N), dtype=torch.int64, **pin)
        self.h_pos = torch.zeros((B, N, 3), dtype=torch.float64, **pin)
        self.h_chg = torch.zeros((B,), dtype=torch.float64, **pin)
        self.h_en = torch.zeros((B, N), dtype=torch.float64, **pin)
        self.h_gr = torch.zeros((B, N, 3), dtype=torch.float64, **pin)
        self.h_st = torch.zeros((4,), dtype=torch.int32, **pin)
        self.d_num = torch.zeros((B, N), dtype=torch.int64, device=dev)
        self.d_pos = torch.zeros((B, N, 3), dtype=torch.float64, device=dev)
        self.d_chg = torch.zeros((B,), dtype=torch.float64, device=dev)
        self.d_en = torch.zeros((B, N), dtype=torch.float64, device=dev)
        self.d_gr = torch.zeros((B, N, 3), dtype=torch.float64, device=dev)
        self.flags = _lib.FLAG_GRADIENT | (_lib.FLAG_MIXED if srv.mixed else 0)
        self.ws = lib.d4_workspace_size(B, N, srv.n_slots, self.flags)
        self.work = torch.zeros(self.ws, dtype=torch.uint8, device=dev)
        self.bytes = self.ws + 2 * (B * N * (8 + 24 + 8 + 24) + 8 * B)
        self.batch = _lib.Batch(n_struct=B, n_pad=N, d_numbers=self.d_num.data_ptr(),
                                d_positions=self.d_pos.data_ptr(),
                                d_charge=self.d_chg.data_ptr())
        self.outs = _lib.Outputs(d_energy=self.d_en.data_ptr(), d_gradient=self.d_gr.data_ptr())
        self.srv = srv
        self.stream = torch.cuda.Stream(dev)
        self.event = torch.cuda.Event()
        self.reqs: list[Request] | None = None
        self.t_launch = 0.0
        with torch.cuda.device(dev):
            with torch.cuda.stream(self.stream):  # one plain call first (attributes, tables)
                self._enqueue()
            self.stream.synchronize()
            self.graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self.graph, stream=self.stream, capture_error_mode="relaxed"):
                self._enqueue()
            self.stream.synchronize()

    def _enqueue(self):
        lib = _lib.load()
        srv = self.srv
        stream = torch.cuda.current_stream(srv.device)
        self.d_num.copy_(self.h_num, non_blocking=True)
        self.d_pos.copy_(self.h_pos, non_blocking=True)
        self.d_chg.copy_(self.h_chg, non_blocking=True)
        _lib.check(lib.d4_dispersion(srv.tables.struct, srv.cfg, self.batch, srv.params,
                                     self.flags, srv.n_slots, self.work.data_ptr(), self.ws,
                                     self.outs, stream.cuda_stream), "d4_dispersion")
        self.h_en.copy_(self.d_en, non_blocking=True)
        self.h_gr.copy_(self.d_gr, non_blocking=True)
        status = self.work[_lib.STATUS_OFFSET:_lib.STATUS_OFFSET + 16].view(torch.int32)
        self.h_st.copy_(status, non_blocking=True)

    def launch(self, reqs: list[Request], now: float):
        self.h_num.zero_()
        num, pos, chg = self.h_num.numpy(), self.h_pos.numpy(), self.h_chg.numpy()
        for k, r in enumerate(reqs):
            n = len(r.numbers)
            num[k, :n] = r.numbers
            pos[k, :n] = r.positions
            chg[k] = r.charge
        chg[len(reqs):] = 0.0
        with torch.cuda.stream(self.stream):
            self.graph.replay()
            self.event.record(self.stream)
        self.reqs = reqs
        self.t_launch = now

    def ready(self) -> bool:
        return self.event.query()

    def collect(self, now: float) -> list[Result]:
        en, gr = self.h_en.numpy(), self.h_gr.numpy()
        status = int(self.h_st[0])
        out = []
        for k, r in enumerate(self.reqs):
            n = len(r.numbers)
            e = en[k, :n].copy()
            out.append(Result(r.rid, float(e.sum()), e, gr[k, :n].copy(), status,
                              r.arrival, now))
        self.reqs = None
        return out


class Batcher:
    """
    The scheduling policy of the server, independent of CUDA: per-bucket
    queues, dispatch (full batch or ``max_wait`` reached), the choice of the
    captured batch size, slot reuse and admission by memory.  ``make_slot``
    (N, B) builds a slot (``launch``, ``ready``, ``collect``, ``bytes``) and
    ``slot_bytes`` (N, B) predicts its memory.
    """

    def __init__(self, buckets, sizes, max_wait, hbm_budget, slots_per_shape, make_slot,
                 slot_bytes):
        self.buckets = tuple(sorted(buckets))
        self.sizes = sizes
        self.max_wait = max_wait
        self.hbm_budget = hbm_budget
        self.slots_per_shape = slots_per_shape
        self.make_slot = make_slot
        self.slot_bytes = slot_bytes
        self.queues = {N: collections.deque() for N in self.buckets}
        self.free: dict[tuple, list] = collections.defaultdict(list)
        self.count: dict[tuple, int] = collections.defaultdict(int)
        self.busy: list = []
        self.bytes = 0
        self.stats = collections.Counter()

    def bucket_of(self, n: int) -> int:
        for N in self.buckets:
            if n <= N:
                return N
        raise ValueError(f"structure of {n} atoms exceeds the largest bucket {self.buckets[-1]}")

    def _slot(self, N: int, B: int):
        key = (N, B)
        if self.free[key]:
            return self.free[key].pop()
        if self.count[key] >= self.slots_per_shape:
            return None
        if self.bytes + self.slot_bytes(N, B) > self.hbm_budget:
            self.stats["admission_waits"] += 1
            return None
        slot = self.make_slot(N, B)
        self.bytes += slot.bytes
        self.count[key] += 1
        self.stats["slots"] += 1
        return slot

    def warmup(self, shapes=None):
        """Create one slot per shape ahead of time (within the budget)."""
        shapes = shapes or [(N, B) for N in self.buckets for B in self.sizes[N]]
        for N, B in shapes:
            s = self._slot(N, B)
            if s is not None:
                self.free[(N, B)].append(s)

    def submit(self, req: Request):
        self.queues[self.bucket_of(len(req.numbers))].append(req)

    def dispatch(self, now: float):
        """Launch every bucket that is full or whose oldest request waited
        ``max_wait``, as long as slots (memory) allow."""
        for N in self.buckets:
            q = self.queues[N]
            while q:
                top = self.sizes[N][-1]
                if len(q) < top and now - q[0].arrival < self.max_wait:
                    break
                B = next(b for b in self.sizes[N] if b >= min(len(q), top))
                slot = self._slot(N, B)
                for smaller in reversed([b for b in self.sizes[N] if b < B]):
                    if slot is not None:
                        break
                    slot = self._slot(N, smaller)  # all slots of size B busy: a smaller one
                    B = smaller
                if slot is None:
                    break  # memory or slots exhausted: wait for a batch to finish
                take = [q.popleft() for _ in range(min(B, len(q)))]
                slot.launch(take, now)
                self.busy.append(slot)
                self.stats["batches"] += 1

    def poll(self, now: float) -> list[Result]:
        out, still = [], []
        for s in self.busy:
            if s.ready():
                out.extend(s.collect(now))
                self.free[(s.N, s.B)].append(s)
            else:
                still.append(s)
        self.busy = still
        return out


class Server(Batcher):
    """
    Continuous-batching request loop on one GPU (see the module docstring).

    ``param`` are the damping parameters of ``dftd4``; ``precision`` "mixed"
    (the precision form) or "fp64" (the plain method); ``hbm_budget`` bounds
    the bytes of all slots (workspaces + buffers).
    """

    def __init__(self, param, *, device="cuda", model="d4", precision="mixed", cutoff=None,
                 buckets=DEFAULT_BUCKETS, max_wait: float = 1e-3, hbm_budget: float = 40e9,
                 slots_per_shape: int = 2, atoms_per_batch: int = 8192, n_slots: int = 1):
        self.device = torch.device(device)
        numbers = torch.tensor([[6, 1]], device=self.device)
        positions = torch.tensor([[[0.0, 0.0, 0.0], [0.0, 0.0, 2.0]]], dtype=torch.float64,
                                 device=self.device)
        runner, _, _ = _prepare(numbers, positions, 0.0, param, model, None, None, None, None,
                                cutoff, None, None, None, precision)
        if runner.model.kind == "d4s" and n_slots < 2:
            raise ValueError("D4S serving needs n_slots >= the distinct elements of a batch")
        self.mixed = runner.mixed
        self.tables = runner.tables
        self.n_slots = n_slots if runner.model.kind == "d4s" else 1
        p, cut = runner.params, runner.cut
        self.params = _lib.Params(
            s6=p["s6"], s8=p["s8"], s10=p["s10"], a1=p["a1"], a2=p["a2"], s9=p["s9"],
            alp=p["alp"], has_s8=int(p["has_s8"]), has_s10=int(p["has_s10"]),
            cut_disp2=cut["disp2"], cut_disp3=cut["disp3"], cut_cn=cut["cn"],
            cut_cn_eeq=cut["cn_eeq"], cn_eeq_max=D4_CN_EEQ_MAX, kcn=D4_KCN, k4=D4_K4,
            k5=D4_K5, k6=D4_K6)
        m = runner.model
        self.cfg = _lib.ModelCfg(kind=_lib.MODEL_D4S if m.kind == "d4s" else _lib.MODEL_D4,
                                 ga=m.ga, gc=m.gc, wf=m.wf if m.wf is not None else 6.0)
        flags = _lib.FLAG_GRADIENT | (_lib.FLAG_MIXED if self.mixed else 0)
        lib = _lib.load()
        buckets = tuple(sorted(buckets))
        super().__init__(
            buckets, {N: batch_sizes_for(N, atoms_per_batch) for N in buckets}, max_wait,
            hbm_budget, slots_per_shape, lambda N, B: _Slot(self, N, B),
            lambda N, B: lib.d4_workspace_size(B, N, self.n_slots, flags) + 2 * B * N * 64)

    def pending(self) -> int:
        return sum(len(q) for q in self.queues.values()) + sum(len(s.reqs) for s in self.busy)


def serve_stream(server: Server, requests: list[Request], realtime: bool = True,
                 clock=time.perf_counter) -> tuple[list[Result], dict]:
    """
    Replay ``requests`` (sorted by arrival, seconds from 0) through the
    server in real time and return the results with throughput and latency
    percentiles.
    """
    t0 = clock()
    i, results = 0, []
    nreq = len(requests)
    while len(results) < nreq:
        now = clock() - t0
        while i < nreq and (requests[i].arrival <= now or not realtime):
            server.submit(requests[i])
            i += 1
        server.dispatch(now)
        results.extend(server.poll(clock() - t0))
    lat = np.array([r.latency for r in results])
    first = min(r.arrival for r in requests)
    last = max(r.done for r in results)
    stats = {
        "requests": nreq,
        "structures_per_s": nreq / max(last - first, 1e-9),
        "atoms_per_s": sum(len(r.numbers) for r in requests) / max(last - first, 1e-9),
        "p50_ms": float(np.percentile(lat, 50) * 1e3),
        "p99_ms": float(np.percentile(lat, 99) * 1e3),
        "max_ms": float(lat.max() * 1e3),
        "batches": server.stats["batches"],
        "slots": server.stats["slots"],
        "slot_bytes": server.bytes,
        "admission_waits": server.stats["admission_waits"],
        "failed": sum(1 for r in results if r.status != 0),
    }
    return sorted(results, key=lambda r: r.rid), stats
