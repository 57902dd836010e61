"""
Drop-in ``dftd4()`` (``tad_dftd4/disp.py:44-146``) on the CUDA library.

The signature, the zero-padded batch convention (atomic number 0 marks
padding), the result's shape, dtype and device, and the errors follow the
reference.  Every number is computed by the compiled kernels through the C
ABI; this module only validates, packs pointers and wires autograd.

Gradients: when ``positions`` (or a damping parameter) requires grad, the
forward call also runs the hand-written adjoint and keeps dE_b/dR per
structure.  ``backward`` scales it by the incoming gradient when that is
uniform within each structure (the case of ``energy.sum()`` or per-structure
sums); any other weighting re-runs the adjoint with those per-atom weights.
"""

from __future__ import annotations

import contextlib
import ctypes
from dataclasses import dataclass

import torch

from . import _lib, tables as _tables
from .cutoff import (D4_CN_CUTOFF, D4_CN_EEQ_MAX, D4_K4, D4_K5, D4_K6, D4_KCN, Cutoff)
from .damping import (PARAM_ORDER, Damping, MZeroDamping, OptimisedPowerDamping, Param,
                      RationalDamping, ZeroDamping, resolve)
from .model import BaseModel, D4Model, D4SModel

__all__ = ["dftd4", "dispersion_energy_gradient", "get_properties", "hessian", "check_status",
           "Runner"]

_ALLOWED_MODELS = ("d3", "d4", "d4s", "d5")
CHECK_STATUS = True

# Device status words not read yet: (pinned copy, event after the copy,
# label).  A forward call whose result feeds autograd leaves its status here
# and its backward reads it, so the host is not held up between the forward
# launches and the backward bookkeeping; every public call first reads the
# words of the calls that have completed, and check_status() waits for all.
_PENDING: list = []
_PENDING_MAX = 64


def _raise_status(status: int, what: str, origin: str = "") -> None:
    if status == 4:
        raise ValueError("atomic number outside the element tables" + origin)
    if status == 6:
        raise ValueError("non-finite positions or charges" + origin)
    _lib.check(status, what + origin)


def _read_token(token) -> None:
    word, ev, what = token
    ev.synchronize()
    _raise_status(int(word[0]), "d4_dispersion (device status)", f" [raised for {what}]")


_CALLS = [0]  # public calls with deferred status so far (labels their errors)
_WS_BYTES: dict = {}  # (B, N, slots, flags) -> workspace bytes


def _on_device(device: torch.device):
    """``torch.cuda.device(device)`` unless it is the current device already
    (the library launches on the current device)."""
    if device.index is None or device.index == torch.cuda.current_device():
        return contextlib.nullcontext()
    return torch.cuda.device(device)


def check_status() -> None:
    """Wait for every call whose device status word has not been read (a
    forward call with gradients leaves it to its backward) and raise the
    first error among them (``ValueError`` for elements outside the tables
    or non-finite input)."""
    pending = list(_PENDING)
    _PENDING.clear()
    for token in pending:
        _read_token(token)


def _drain_pending() -> None:
    """Read the status words of the pending calls that have completed (and
    of the oldest ones beyond _PENDING_MAX), raising the first error."""
    while _PENDING and (_PENDING[0][1].query() or len(_PENDING) > _PENDING_MAX):
        _read_token(_PENDING.pop(0))


def _as_tensor(x, device, dtype):
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=dtype)
    return torch.tensor(x, device=device, dtype=dtype)


def _resolve_model(model, numbers) -> BaseModel:
    if isinstance(model, str):
        key = model.casefold()
        if key not in _ALLOWED_MODELS:
            raise ValueError(
                f"Unknown model '{key}'. Please use {', '.join(_ALLOWED_MODELS)}."
            )
        if key == "d4":
            return D4Model(numbers)
        if key == "d4s":
            return D4SModel(numbers)
        raise NotImplementedError(f"model '{key}' has no dispersion model in tad-dftd4")
    if isinstance(model, BaseModel):
        return model
    raise TypeError(f"unsupported model object {type(model).__name__}")


@dataclass
class Runner:
    """One configured call of the library on a padded batch (B, N)."""

    numbers: torch.Tensor  # (B, N) int64, device
    charge: torch.Tensor  # (B,) float64, device
    tables: _tables.DeviceTables
    model: BaseModel
    params: dict
    cut: dict
    q: torch.Tensor | None = None
    r4r2: torch.Tensor | None = None
    n_slots: int = 1
    mixed: bool = False
    rvdw: torch.Tensor | None = None  # (B, N, N) pair radii of rvdw-type damping
    exact_c9: bool = False            # ATM with the exact C9 (DispD4Exact)
    last_work: torch.Tensor | None = None  # workspace of the last call (residuals)
    ct_params: object = None  # ctypes parameter / model blocks shared by calls of one
    ct_cfg: object = None     # configuration (built on first use)

    def run_blocks(self) -> None:
        """Build the ctypes parameter and model blocks of this configuration
        (once; calls of the same configuration share them)."""
        if self.ct_params is None:
            p = self.params
            self.ct_params = _lib.Params(
                s6=p["s6"], s8=p["s8"], s10=p["s10"], a1=p["a1"], a2=p["a2"], s9=p["s9"],
                alp=p["alp"], has_s8=int(p["has_s8"]), has_s10=int(p["has_s10"]),
                cut_disp2=self.cut["disp2"], cut_disp3=self.cut["disp3"],
                cut_cn=self.cut["cn"], cut_cn_eeq=self.cut["cn_eeq"],
                cn_eeq_max=D4_CN_EEQ_MAX, kcn=D4_KCN, k4=D4_K4, k5=D4_K5, k6=D4_K6,
                damping=p["damping"], rs6=p["rs6"], rs8=p["rs8"], bet=p["bet"],
            )
        if self.ct_cfg is None:
            self.ct_cfg = _lib.ModelCfg(
                kind=_lib.MODEL_D4S if self.model.kind == "d4s" else _lib.MODEL_D4,
                ga=self.model.ga, gc=self.model.gc,
                wf=self.model.wf if self.model.wf is not None else 6.0)

    def run(self, positions: torch.Tensor, gradient: bool = False, param_grad: bool = False,
            weights: torch.Tensor | None = None, charges_out: bool = False,
            cn_out: bool = False, cn_eeq_out: bool = False, defer_status: bool = False,
            extra_flags: int = 0):
        lib = _lib.load()
        device = positions.device
        B, N = self.numbers.shape
        pos = positions.detach().to(torch.float64).contiguous()
        flags = 0
        if gradient or param_grad:
            flags |= _lib.FLAG_GRADIENT
        if param_grad:
            flags |= _lib.FLAG_PARAM_GRAD
        if self.q is not None:
            flags |= _lib.FLAG_CHARGES_IN
        if self.mixed:
            flags |= _lib.FLAG_MIXED
        if self.exact_c9:
            flags |= _lib.FLAG_EXACT_C9
        flags |= extra_flags
        energy = torch.empty((B, N), dtype=torch.float64, device=device)
        grad = (torch.empty((B, N, 3), dtype=torch.float64, device=device)
                if flags & _lib.FLAG_GRADIENT else None)
        pgrad = (torch.empty((B, _lib.PARAM_GRAD_STRIDE), dtype=torch.float64, device=device)
                 if param_grad else None)
        qout = torch.empty((B, N), dtype=torch.float64, device=device) if charges_out else None
        cnout = torch.empty((B, N), dtype=torch.float64, device=device) if cn_out else None
        cnqout = (torch.empty((B, N), dtype=torch.float64, device=device)
                  if cn_eeq_out else None)
        w = None if weights is None else weights.to(torch.float64).contiguous()
        wkey = (B, N, self.n_slots, flags)
        ws_bytes = _WS_BYTES.get(wkey)
        if ws_bytes is None:
            ws_bytes = lib.d4_workspace_size(B, N, self.n_slots, flags)
            if len(_WS_BYTES) > 256:
                _WS_BYTES.clear()
            _WS_BYTES[wkey] = ws_bytes
        self.last_work = None
        work = torch.empty(ws_bytes, dtype=torch.uint8, device=device)
        self.last_work = work
        self.run_blocks()
        params, cfg = self.ct_params, self.ct_cfg
        batch = _lib.Batch(
            n_struct=B, n_pad=N, d_numbers=self.numbers.data_ptr(), d_positions=pos.data_ptr(),
            d_charge=self.charge.data_ptr(),
            d_charges_in=self.q.data_ptr() if self.q is not None else None,
            d_r4r2_in=self.r4r2.data_ptr() if self.r4r2 is not None else None,
            d_energy_weights=w.data_ptr() if w is not None else None,
            d_rvdw_in=self.rvdw.data_ptr() if self.rvdw is not None else None,
        )
        outs = _lib.Outputs(
            d_energy=energy.data_ptr(),
            d_gradient=grad.data_ptr() if grad is not None else None,
            d_charges=qout.data_ptr() if qout is not None else None,
            d_cn=cnout.data_ptr() if cnout is not None else None,
            d_param_grad=pgrad.data_ptr() if pgrad is not None else None,
            d_cn_eeq=cnqout.data_ptr() if cnqout is not None else None,
        )
        cur = torch.cuda.current_stream(device)
        stream = cur.cuda_stream
        with _on_device(device):
            _lib.check(lib.d4_dispersion(self.tables.struct, cfg, batch, params, flags,
                                         self.n_slots, work.data_ptr(), ws_bytes, outs, stream),
                       "d4_dispersion")
            self.token = None
            if CHECK_STATUS and defer_status:  # the status word stays in the stream
                word = torch.empty(1, dtype=torch.int32, pin_memory=True)
                _lib.check(lib.d4_status_async(work.data_ptr(), word.data_ptr(), stream),
                           "d4_status_async")
                ev = torch.cuda.Event()
                ev.record(cur)
                _CALLS[0] += 1
                self.token = (word, ev, f"forward call #{_CALLS[0]} with gradients "
                                        f"({B} structures x {N} atoms)")
                _PENDING.append(self.token)
            elif CHECK_STATUS:
                _raise_status(lib.d4_read_status(work.data_ptr(), stream),
                              "d4_dispersion (device status)")
        if cn_eeq_out:
            return energy, grad, pgrad, qout, cnout, cnqout
        return energy, grad, pgrad, qout, cnout


    def eeq_residuals(self) -> torch.Tensor:
        """(B, 2) final EEQ refinement residuals max |A x - b| of the last
        call (forward charges, adjoint solve) of the precision form; zeros
        where no refinement ran.  Waits for the call to finish."""
        if self.last_work is None:
            raise RuntimeError("no call has run yet")
        B = self.numbers.shape[0]
        out = torch.empty((B, 2), dtype=torch.float32, pin_memory=True)
        stream = torch.cuda.current_stream(self.last_work.device).cuda_stream
        with torch.cuda.device(self.last_work.device):
            _lib.check(_lib.load().d4_eeq_residuals(self.last_work.data_ptr(), B,
                                                    out.data_ptr(), stream),
                       "d4_eeq_residuals")
        return out.clone()


class _D4Function(torch.autograd.Function):
    @staticmethod
    def forward(ctx, positions, pvec, runner: Runner):
        need_pos = ctx.needs_input_grad[0]
        need_par = ctx.needs_input_grad[1]
        energy, grad, pgrad, _, _ = runner.run(positions, gradient=need_pos or need_par,
                                               param_grad=need_par,
                                               defer_status=need_pos or need_par)
        ctx.token = runner.token
        ctx.runner = runner
        ctx.positions = positions.detach()
        ctx.save_for_backward(grad if grad is not None else torch.empty(0),
                              pgrad if pgrad is not None else torch.empty(0))
        return energy.to(positions.dtype)

    @staticmethod
    def backward(ctx, go):
        grad, pgrad = ctx.saved_tensors
        runner: Runner = ctx.runner
        if go.numel() > 0 and all(st == 0 for st in go.stride()):
            # one value broadcast over all atoms (the gradient of energy.sum()):
            # uniform, no need to look at it on the host
            w0 = go.reshape(-1)[:1].to(torch.float64).reshape(1, 1)
            uniform = True
        else:
            go = go.to(torch.float64)
            real = runner.numbers != 0
            first = torch.argmax(real.to(torch.int8), dim=-1, keepdim=True)
            w0 = torch.gather(go, -1, first)  # (B, 1)
            uniform = bool((((go - w0) * real).abs().amax() == 0).item())
        if not uniform:
            _, grad, pgrad, _, _ = runner.run(ctx.positions, gradient=True,
                                              param_grad=ctx.needs_input_grad[1],
                                              weights=go * real)
            w0 = torch.ones_like(w0)
        gpos = gpar = None
        if ctx.needs_input_grad[0]:
            gpos = (w0.unsqueeze(-1) * grad).to(ctx.positions.dtype)
        if ctx.needs_input_grad[1]:
            gpar = (w0 * pgrad).sum(0)[: len(PARAM_ORDER)]
        # the forward's status word: read here if the forward has finished,
        # else left to the next library call or check_status() -- the host
        # does not wait for the GPU in the backward (whatever the caller
        # queues next, e.g. the copies of the results, follows the kernels
        # directly), the way CUDA reports asynchronous errors
        for idx, token in enumerate(_PENDING):
            if token is ctx.token:
                if token[1].query():
                    del _PENDING[idx]
                    _read_token(token)
                break
        return gpos, gpar, None


def _named(fn, name: str) -> bool:
    """True for ``None`` (the default) or a function called ``name``: the
    reference's defaults ``tad_mctc.ncoord.cn_d4`` / ``erf_count`` passed
    explicitly select the built-in D4 coordination number."""
    return fn is None or getattr(fn, "__name__", None) == name


PRECISIONS = ("fp64", "mixed")
_PVEC: dict = {}


_DAMPING_BY_NAME = {cls.__name__: cls for cls in
                    (RationalDamping, ZeroDamping, MZeroDamping, OptimisedPowerDamping)}


def _damping(fn) -> Damping:
    """The two-body damping selected by ``damping_function``: this package's
    classes, or tad-dftd4's own instances matched by class name."""
    if fn is None:
        return RationalDamping()
    if isinstance(fn, Damping) and fn.kind >= 0:
        return fn
    cls = _DAMPING_BY_NAME.get(type(fn).__name__)
    if cls is None:
        raise NotImplementedError(
            f"damping function {type(fn).__name__} is not built in (rational, zero, "
            "modified-zero and optimised-power damping are)")
    return cls()


# Configurations of plain calls (D4 model given by name, parameters as plain
# numbers, default CN / damping, no per-atom overrides), so that a repeated
# call skips the parameter resolution, the model and table look-ups and the
# ctypes parameter blocks: key -> (model, resolved, tables, cutoffs, pvec,
# precision, ctypes params, ctypes model block).
_CONFIGS: dict = {}
_CONFIGS_MAX = 64


def _config_key(param, model, cutoff, precision, device, dtype):
    if type(model) is not str or model.casefold() != "d4":
        return None
    if cutoff is not None and not isinstance(cutoff, Cutoff):
        return None
    items = []
    for k, v in param.items():
        if type(v) is not float and type(v) is not int:
            return None
        items.append((k, v))
    ck = None if cutoff is None else tuple(sorted(cutoff.host_values().items()))
    return (device, dtype, ck, precision, tuple(items))


def _prepare(numbers, positions, charge, param, model, rcov, r4r2, rvdw, q, cutoff,
             cn_function, counting_function, damping_function, precision=None,
             exact_c9: bool = False):
    _drain_pending()
    device = positions.device
    dtype = positions.dtype
    ckey = None
    if (rcov is None and r4r2 is None and rvdw is None and q is None and cn_function is None
            and counting_function is None and damping_function is None and not exact_c9):
        ckey = _config_key(param, model, cutoff, precision, device, dtype)
        hit = _CONFIGS.get(ckey) if ckey is not None else None
        if hit is not None:
            mdl, resolved, tab, cut, pvec, prec, ct_params, ct_cfg = hit
            if numbers.shape != positions.shape[:-1]:
                raise ValueError(
                    f"Shape of positions ({positions.shape}) is not consistent with atomic "
                    f"numbers ({numbers.shape})."
                )
            shape = numbers.shape
            N = shape[-1]
            nums = numbers.reshape(-1, N).to(device=device, dtype=torch.int64).contiguous()
            B = nums.shape[0]
            charge = _as_tensor(charge, device, dtype)
            if charge.dim() == 0:
                chg = charge.to(torch.float64).expand(B).contiguous()
            else:
                chg = charge.reshape(-1).to(torch.float64).contiguous()
                if chg.numel() != B:
                    raise ValueError(f"charge of shape {tuple(charge.shape)} for {B} structures")
            runner = Runner(numbers=nums, charge=chg, tables=tab, model=mdl, params=resolved,
                            cut=cut, mixed=prec == "mixed", ct_params=ct_params, ct_cfg=ct_cfg)
            return runner, pvec, shape
    charge = _as_tensor(charge, device, dtype)
    if numbers.shape != positions.shape[:-1]:
        raise ValueError(
            f"Shape of positions ({positions.shape}) is not consistent with atomic "
            f"numbers ({numbers.shape})."
        )
    cut_host = (Cutoff.DEFAULTS if cutoff is None else
                cutoff.host_values() if isinstance(cutoff, Cutoff) else
                {k: float(getattr(cutoff, k)) for k in ("disp2", "disp3", "cn", "cn_eeq")})
    mdl = _resolve_model(model, numbers)
    if rcov is not None and numbers.shape != rcov.shape:
        raise ValueError(f"Shape of covalent radii ({rcov.shape}) is not consistent with "
                         f"atomic numbers ({numbers.shape}).")
    if r4r2 is not None and numbers.shape != r4r2.shape:
        raise ValueError(f"Shape of expectation values r4r2 ({r4r2.shape}) is not "
                         f"consistent with atomic numbers ({numbers.shape}).")
    if rvdw is not None and numbers.shape != rvdw.shape[:-1]:
        raise ValueError(f"Shape of van der Waals radii ({rvdw.shape}) is not consistent "
                         f"with atomic numbers ({numbers.shape}).")
    if q is not None and numbers.shape != q.shape:
        raise ValueError(f"Shape of atomic charges ({q.shape}) is not consistent with "
                         f"atomic numbers ({numbers.shape}).")
    if not (_named(cn_function, "cn_d4") and _named(counting_function, "erf_count")):
        raise NotImplementedError(
            "only the default D4 coordination number (cn_d4 with erf_count) is built in")
    damp = _damping(damping_function)
    resolved = resolve(param, damp)
    plain_only = damp.kind != RationalDamping.kind or exact_c9
    if precision is None:
        precision = "mixed" if dtype == torch.float32 and not plain_only else "fp64"
    if precision not in PRECISIONS:
        raise ValueError(f"precision must be one of {PRECISIONS}, got {precision!r}")
    if precision == "mixed" and plain_only:
        raise ValueError("the precision form runs the rational damping with the approximate "
                         "C9; other damping functions and the exact C9 use precision='fp64'")
    if device.type != "cuda":
        raise RuntimeError("tad-dftd4_gb300 runs on CUDA devices; move the inputs to a GPU")

    shape = numbers.shape
    N = shape[-1]
    nums = numbers.reshape(-1, N).to(device=device, dtype=torch.int64).contiguous()
    B = nums.shape[0]
    if charge.dim() == 0:
        chg = charge.to(torch.float64).expand(B).contiguous()
    else:
        chg = charge.reshape(-1).to(torch.float64).contiguous()
        if chg.numel() != B:
            raise ValueError(f"charge of shape {tuple(charge.shape)} for {B} structures")
    tab = _tables.device_tables(device, mdl.ref_charges, mdl.ga, mdl.gc)
    n_slots = 1
    if mdl.kind == "d4s":
        present = torch.zeros((B, 128), dtype=torch.int32, device=device)
        present.scatter_(1, nums.clamp(0, 127), 1)
        present[:, 0] = 0
        n_slots = max(1, int(present.sum(1).max().item()))
    cut = {
        "disp2": cut_host["disp2"], "disp3": cut_host["disp3"],
        "cn": D4_CN_CUTOFF, "cn_eeq": cut_host["cn_eeq"],
    }
    rv = None
    if damp.radius_type == "rvdw":
        if rvdw is None:
            rvdw = _tables.vdw_pairwise(device, nums)
        if rvdw is None:
            raise ValueError(
                "`rvdw` must be provided for `rvdw` radius type: the pairwise van der Waals "
                "radii (tad-mctc's VDW_PAIRWISE) are not in the element table file")
        rv = rvdw.reshape(B, N, N).to(device=device, dtype=torch.float64).contiguous()
    runner = Runner(
        numbers=nums, charge=chg, tables=tab, model=mdl, params=resolved, cut=cut,
        q=None if q is None else q.reshape(-1, N).to(torch.float64).contiguous(),
        r4r2=None if r4r2 is None else r4r2.reshape(-1, N).to(torch.float64).contiguous(),
        n_slots=n_slots, mixed=precision == "mixed", rvdw=rv, exact_c9=exact_c9,
    )
    if any(isinstance(param.get(k), torch.Tensor) for k in PARAM_ORDER):
        pvec = []
        for key in PARAM_ORDER:
            v = param.get(key)
            if isinstance(v, torch.Tensor):
                pvec.append(v.reshape(()).to(device=device, dtype=torch.float64))
            else:
                pvec.append(torch.tensor(resolved[key], dtype=torch.float64, device=device))
        pvec = torch.stack(pvec)
    else:  # plain numbers: a cached constant vector (no copy per call)
        key = (device, tuple(float(resolved[k]) for k in PARAM_ORDER))
        pvec = _PVEC.get(key)
        if pvec is None:
            pvec = torch.tensor(key[1], dtype=torch.float64, device=device)
            if len(_PVEC) > 64:
                _PVEC.clear()
            _PVEC[key] = pvec
    if ckey is not None:  # a plain configuration: remember it for the next call
        runner.run_blocks()
        if len(_CONFIGS) >= _CONFIGS_MAX:
            _CONFIGS.clear()
        _CONFIGS[ckey] = (mdl, resolved, tab, cut, pvec, precision, runner.ct_params,
                          runner.ct_cfg)
    return runner, pvec, shape


def dftd4(numbers: torch.Tensor, positions: torch.Tensor, charge, param: Param, *,
          model="d4", rcov=None, r4r2=None, rvdw=None, q=None, cutoff: Cutoff | None = None,
          cn_function=None, counting_function=None,
          damping_function: Damping | None = None, precision: str | None = None
          ) -> torch.Tensor:
    """
    Atom-resolved DFT-D4 dispersion energy of a structure or a padded batch.

    Same arguments and result as ``tad_dftd4.dftd4``: ``numbers`` (..., N)
    with 0 for padding, ``positions`` (..., N, 3) in Bohr on a CUDA device,
    total ``charge`` (scalar or per structure), damping parameters ``param``.
    Returns (..., N) energies in Hartree with the dtype of ``positions``.
    ``cn_function`` / ``counting_function`` accept the defaults (the D4 CN
    with erf counting, given as ``None`` or as tad-mctc's ``cn_d4`` /
    ``erf_count``).  ``damping_function`` selects the two-body damping:
    ``RationalDamping`` (default), ``ZeroDamping``, ``MZeroDamping`` or
    ``OptimisedPowerDamping`` (this package's classes or tad-dftd4's own
    instances); the zero-damping family takes the pairwise radii ``rvdw``
    (..., N, N), which must be passed unless the table file carries them.
    The damping functions other than the rational one run on the plain FP64
    kernels whatever the dtype.

    ``precision`` (an addition to the reference signature): ``"fp64"`` runs
    the plain method in double precision (default for float64 positions);
    ``"mixed"`` the precision form -- FP32 pair and triple arithmetic with
    compensated sums, FP32 EEQ factorisation refined in FP64, FP64 CN,
    weights and final reductions (default for float32 positions).
    """
    return _evaluate(numbers, positions, charge, param, model=model, rcov=rcov, r4r2=r4r2,
                     rvdw=rvdw, q=q, cutoff=cutoff, cn_function=cn_function,
                     counting_function=counting_function, damping_function=damping_function,
                     precision=precision)


def _evaluate(numbers, positions, charge, param, *, model, rcov, r4r2, rvdw, q, cutoff,
              cn_function, counting_function, damping_function, precision,
              exact_c9: bool = False) -> torch.Tensor:
    """The library call behind ``dftd4`` and the ``Disp`` classes: energies
    with gradients through the hand-written adjoint."""
    runner, pvec, shape = _prepare(numbers, positions, charge, param, model, rcov, r4r2,
                                   rvdw, q, cutoff, cn_function, counting_function,
                                   damping_function, precision, exact_c9)
    pos = positions.reshape(-1, shape[-1], 3)
    energy = _D4Function.apply(pos, pvec, runner)
    return energy.reshape(shape)


def dispersion_energy_gradient(numbers, positions, charge, param, **kw):
    """
    Energies (..., N) and the gradient d(sum E)/dR (..., N, 3) in one fused
    call, without autograd bookkeeping.  Same arguments as ``dftd4``.
    """
    runner, _, shape = _prepare(numbers, positions, charge, param, kw.pop("model", "d4"),
                                kw.pop("rcov", None), kw.pop("r4r2", None),
                                kw.pop("rvdw", None), kw.pop("q", None),
                                kw.pop("cutoff", None), kw.pop("cn_function", None),
                                kw.pop("counting_function", None),
                                kw.pop("damping_function", None),
                                kw.pop("precision", None), kw.pop("exact_c9", False))
    if kw:
        raise TypeError(f"unexpected arguments {sorted(kw)}")
    pos = positions.reshape(-1, shape[-1], 3)
    energy, grad, _, _, _ = runner.run(pos, gradient=True)
    return (energy.reshape(shape).to(positions.dtype),
            grad.reshape(*shape, 3).to(positions.dtype))


def _fd_hessian(grad_fn, numbers: torch.Tensor, positions: torch.Tensor,
                charge: torch.Tensor, step: float, max_structs: int = 4096,
                order: int = 4) -> torch.Tensor:
    """Finite differences of a batched gradient: ``grad_fn(numbers (M, N),
    positions (M, N, 3), charge (M,), source (M,))`` -> (M, N, 3), where
    ``source`` holds the index of the structure each geometry displaces.

    ``order`` 2: central differences D(h) = (g(x + h) - g(x - h)) / 2h,
    error O(h^2), two displaced geometries per coordinate.  ``order`` 4:
    Richardson's combination (4 D(h) - D(2h)) / 3, which cancels the h^2
    term (error O(h^4)), four geometries per coordinate.  A call takes at
    most ``max_structs`` geometries -- several structures' sets at once when
    they fit, else consecutive slices of one structure's coordinates.
    Returns the symmetrised (B, N, 3, N, 3) second derivatives in float64."""
    if order not in (2, 4):
        raise ValueError(f"order must be 2 or 4, got {order}")
    B, N = numbers.shape
    dt = torch.float64
    dev = positions.device
    pos = positions.detach().to(dt)
    m = 3 * N
    offsets = (1.0, -1.0) if order == 2 else (1.0, -1.0, 2.0, -2.0)
    G = len(offsets)
    out = torch.empty((B, m, N, 3), dtype=dt, device=dev)
    cap = max(G, int(max_structs))
    # (structure range, coordinate range) per call
    if G * m <= cap:
        per = cap // (G * m)
        plan = [((b0, min(B, b0 + per)), (0, m)) for b0 in range(0, B, per)]
    else:
        rows = cap // G
        plan = [((b, b + 1), (k0, min(m, k0 + rows))) for b in range(B)
                for k0 in range(0, m, rows)]
    for (b0, b1), (k0, k1) in plan:
        nb, nk = b1 - b0, k1 - k0
        unit = torch.zeros((nk, m), dtype=dt, device=dev)
        unit[torch.arange(nk, device=dev), torch.arange(k0, k1, device=dev)] = step
        unit = unit.reshape(nk, N, 3)
        p = pos[b0:b1, None]
        geo = torch.cat([p + o * unit for o in offsets], dim=1).reshape(nb * G * nk, N, 3)
        nums = numbers[b0:b1, None].expand(nb, G * nk, N).reshape(-1, N)
        chg = charge[b0:b1, None].to(dt).expand(nb, G * nk).reshape(-1)
        src = torch.arange(b0, b1, device=dev)[:, None].expand(nb, G * nk).reshape(-1)
        g = grad_fn(nums, geo, chg, src).to(dt).reshape(nb, G, nk, N, 3)
        d1 = (g[:, 0] - g[:, 1]) / (2.0 * step)
        if order == 4:
            d2 = (g[:, 2] - g[:, 3]) / (4.0 * step)
            d1 = (4.0 * d1 - d2) / 3.0
        out[b0:b1, k0:k1] = d1
    h = out.reshape(B, N, 3, N, 3)
    return 0.5 * (h + h.permute(0, 3, 4, 1, 2))


def hessian(numbers: torch.Tensor, positions: torch.Tensor, charge, param: Param, *,
            step: float = 1.25e-4, order: int = 4, **kw) -> torch.Tensor:
    """
    Hessian of each structure's total dispersion energy with respect to the
    positions, shape (..., N, 3, N, 3): the quantity the reference obtains
    with ``tad_mctc.autograd.hessian`` of ``dftd4(...).sum(-1)``
    (``test/test_grad/test_hessian.py:73-104``).  Computed from the
    analytic gradient, as the Fortran dftd4 program computes the
    reference's golden Hessians (``test_hessian.py:20-28``): the fused
    energy + gradient kernels (the plain FP64 method unless ``precision``
    says otherwise) at displaced geometries, all of a structure's
    displacements in one batched call, differenced and symmetrised.
    ``order`` 4 (default) combines the central differences at ``step`` and
    2 ``step`` Bohr by Richardson extrapolation (truncation error O(step^4):
    a few 1e-12 Eh/Bohr^2 at the default step on 30-atom structures, against
    ~1e-7 for central differences alone); ``order`` 2 takes plain central
    differences.  Other keyword arguments as for ``dftd4``.  Padding atoms
    have zero rows and columns.
    """
    shape = numbers.shape
    N = shape[-1]
    nums = numbers.reshape(-1, N)
    B = nums.shape[0]
    pos = positions.reshape(-1, N, 3)
    chg = _as_tensor(charge, positions.device, torch.float64)
    chg = chg.expand(B) if chg.dim() == 0 else chg.reshape(-1)
    if chg.numel() != B:
        raise ValueError(f"charge of shape {tuple(chg.shape)} for {B} structures")
    kw.setdefault("precision", "fp64")
    max_structs = kw.pop("max_structs", 4096)
    # per-atom (and per-pair) inputs follow their structure's displaced copies
    per_atom = {}
    for key in ("q", "rcov", "r4r2", "rvdw"):
        v = kw.pop(key, None)
        if v is None:
            continue
        if tuple(v.shape[:len(shape)]) != tuple(shape):
            raise ValueError(f"Shape of {key} ({tuple(v.shape)}) is not consistent with "
                             f"atomic numbers ({tuple(shape)}).")
        per_atom[key] = v.reshape(B, *v.shape[len(shape):])

    def grad_fn(n, p, c, src):
        extra = {k: v.index_select(0, src.to(v.device)) for k, v in per_atom.items()}
        return dispersion_energy_gradient(n, p, c, param, **kw, **extra)[1]

    h = _fd_hessian(grad_fn, nums, pos, chg, step, max_structs, order)
    return h.reshape(*shape, 3, N, 3).to(positions.dtype)


def get_properties(numbers: torch.Tensor, positions: torch.Tensor, charge=None,
                   cutoff: Cutoff | None = None):
    """
    Properties of the D4 model, the drop-in for ``tad_dftd4.get_properties``
    (``disp.py:149-197``): D4 coordination numbers (..., N), EEQ charges
    (..., N), atom-resolved C6 coefficients at those charges (..., N, N) and
    static polarisabilities (..., N), in the dtype of ``positions``.  Plain
    FP64 kernels; padding atoms (atomic number 0) get zeros.
    """
    if numbers.shape != positions.shape[:-1]:
        raise ValueError(
            f"Shape of positions ({positions.shape}) is not consistent with atomic "
            f"numbers ({numbers.shape})."
        )
    device, dtype = positions.device, positions.dtype
    if device.type != "cuda":
        raise RuntimeError("tad-dftd4_gb300 runs on CUDA devices; move the inputs to a GPU")
    cut_host = (Cutoff.DEFAULTS if cutoff is None else
                cutoff.host_values() if isinstance(cutoff, Cutoff) else
                {k: float(getattr(cutoff, k)) for k in ("disp2", "disp3", "cn", "cn_eeq")})
    shape = numbers.shape
    N = shape[-1]
    nums = numbers.reshape(-1, N).to(device=device, dtype=torch.int64).contiguous()
    B = nums.shape[0]
    pos = positions.reshape(-1, N, 3).detach().to(torch.float64).contiguous()
    charge = 0.0 if charge is None else charge
    chg = _as_tensor(charge, device, torch.float64)
    chg = (chg.expand(B) if chg.dim() == 0 else chg.reshape(-1)).contiguous()
    if chg.numel() != B:
        raise ValueError(f"charge of shape {tuple(chg.shape)} for {B} structures")
    mdl = D4Model(nums)
    tab = _tables.device_tables(device, mdl.ref_charges, mdl.ga, mdl.gc)
    lib = _lib.load()
    cn = torch.empty((B, N), dtype=torch.float64, device=device)
    q = torch.empty((B, N), dtype=torch.float64, device=device)
    c6 = torch.empty((B, N, N), dtype=torch.float64, device=device)
    alpha = torch.empty((B, N), dtype=torch.float64, device=device)
    ws_bytes = lib.d4_workspace_size(B, N, 1, 0)
    work = torch.empty(ws_bytes, dtype=torch.uint8, device=device)
    params = _lib.Params(
        s6=1.0, s8=1.0, s10=0.0, a1=0.4, a2=5.0, s9=1.0, alp=16.0, has_s8=1, has_s10=0,
        cut_disp2=cut_host["disp2"], cut_disp3=cut_host["disp3"], cut_cn=D4_CN_CUTOFF,
        cut_cn_eeq=cut_host["cn_eeq"], cn_eeq_max=D4_CN_EEQ_MAX, kcn=D4_KCN, k4=D4_K4, k5=D4_K5,
        k6=D4_K6)
    batch = _lib.Batch(n_struct=B, n_pad=N, d_numbers=nums.data_ptr(), d_positions=pos.data_ptr(),
                       d_charge=chg.data_ptr())
    props = _lib.Properties(d_cn=cn.data_ptr(), d_charges=q.data_ptr(), d_c6=c6.data_ptr(),
                            d_alpha=alpha.data_ptr())
    cfg = _lib.ModelCfg(kind=_lib.MODEL_D4, ga=mdl.ga, gc=mdl.gc, wf=mdl.wf)
    stream = torch.cuda.current_stream(device).cuda_stream
    with torch.cuda.device(device):
        _lib.check(lib.d4_properties(tab.struct, cfg, batch, params, work.data_ptr(), ws_bytes,
                                     props, stream), "d4_properties")
        status = lib.d4_read_status(work.data_ptr(), stream)
        if status == 4:
            raise ValueError("atomic number outside the element tables")
        if status == 6:
            raise ValueError("non-finite positions or charges")
        _lib.check(status, "d4_properties (device status)")
    return (cn.reshape(shape).to(dtype), q.reshape(shape).to(dtype),
            c6.reshape(*shape, N).to(dtype), alpha.reshape(shape).to(dtype))
