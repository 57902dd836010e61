"""
Generate ``golden.npz``: outputs of tad-dftd4's own code on seeded inputs.

tad-dftd4 itself cannot be installed here (its dependencies ``tad-mctc`` and
``tad-multicharge`` are absent), so this script imports the reference package
straight from its source tree with the test-only stand-ins in ``refstub/`` on
``sys.path``.  Everything tad-dftd4 computes itself (reference
polarisabilities, charge scaling, D4 / D4S weights, C6, BJ two-body, ATM,
autograd gradients) is therefore the reference's own code.  CN and EEQ come
from the stand-ins (an independent restatement of the published method).

Run from the repository root (needs the reference source tree)::

    python tests/golden/make_golden.py --src <reference>/src

Cases: the geometries of the reference's examples (``examples/single.py``,
``examples/batch.py``) and NaN test (``test/test_grad/test_nan.py``), read from
those files, plus seeded structures from ``workloads.py``.
"""

from __future__ import annotations

import argparse
import importlib
import json
import re
import sys
import tomllib
from pathlib import Path

import numpy as np
import torch

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
OUT = HERE / "golden.npz"
OUT_VARIANTS = HERE / "golden_variants.npz"


def _setup(src: Path):
    sys.path.insert(0, str(HERE / "refstub"))
    sys.path.insert(0, str(src))
    sys.modules.setdefault("tomli", tomllib)
    d4 = importlib.import_module("tad_dftd4")
    workloads = importlib.import_module("tad-dftd4_gb300.workloads")
    return d4, workloads


def _tensor_block(text: str, anchor: str) -> np.ndarray:
    """Numbers of the first ``[...]`` list of 3-vectors after ``anchor``."""
    rows = re.findall(
        r"\[\s*([-+]?\d+\.\d+),\s*([-+]?\d+\.\d+),\s*([-+]?\d+\.\d+)\s*\]",
        text.split(anchor, 1)[1],
    )
    return np.array([[float(x) for x in row] for row in rows])


def _symbols(text: str) -> list[list[str]]:
    return [s.split() for s in re.findall(r'"([A-Z][A-Za-z ]+)"\.split\(\)', text)]


SYM = {"H": 1, "B": 5, "C": 6, "N": 7, "O": 8, "F": 9, "Si": 14, "P": 15,
       "S": 16, "Cl": 17, "Br": 35, "I": 53}


def reference_cases(ref_root: Path) -> list[dict]:
    cases = []
    single = (ref_root / "examples/single.py").read_text()
    (syms,) = _symbols(single)
    pos = _tensor_block(single, "positions = torch.tensor(")
    cases.append({"name": "example_single", "numbers": np.array([[SYM[s] for s in syms]]),
                  "positions": pos[None], "charge": np.zeros(1)})

    batch = (ref_root / "examples/batch.py").read_text()
    syms2 = _symbols(batch)
    rows = _tensor_block(batch, "positions = mctc.batch.pack(")
    n1, n2 = len(syms2[0]), len(syms2[1])
    numbers = np.zeros((2, n1), dtype=np.int64)
    positions = np.zeros((2, n1, 3))
    numbers[0] = [SYM[s] for s in syms2[0]]
    numbers[1, :n2] = [SYM[s] for s in syms2[1]]
    positions[0] = rows[:n1]
    positions[1, :n2] = rows[n1:n1 + n2]
    cases.append({"name": "example_batch", "numbers": numbers, "positions": positions,
                  "charge": np.zeros(2)})

    nan = (ref_root / "test/test_grad/test_nan.py").read_text()
    znan = re.findall(r"numbers = torch.tensor\(\[([\d, ]+)\]\)", nan)[0]
    pos = _tensor_block(nan, "positions = torch.tensor(")
    cases.append({"name": "close17", "numbers": np.array([[int(x) for x in znan.split(",")]]),
                  "positions": pos[None], "charge": np.zeros(1)})
    return cases


def seeded_cases(workloads) -> list[dict]:
    cases = []
    b = workloads.single32(0)
    cases.append({"name": "single32", "numbers": b.numbers, "positions": b.positions,
                  "charge": b.charge})
    b = workloads.batch_uniform(11, 4, 8, 30, workloads.ELEMENTS_12, True, "small4", 30)
    cases.append({"name": "batch4_charged", "numbers": b.numbers, "positions": b.positions,
                  "charge": b.charge})
    b = workloads.single32(5)
    cases.append({"name": "short_cutoffs", "numbers": b.numbers, "positions": b.positions,
                  "charge": b.charge, "cutoff": {"disp2": 9.0, "disp3": 6.0}})
    b = workloads.single32(6)
    cases.append({"name": "param_variants", "numbers": b.numbers, "positions": b.positions,
                  "charge": np.array([1.0]),
                  "param": {"s6": 0.9, "s10": 0.7, "a1": 0.5, "a2": 4.0, "s9": 1.3,
                            "alp": 14.0}})
    rng = np.random.default_rng(21)
    z = np.ones(22, dtype=np.int64)
    z[:4] = 6
    pos = workloads.cube_positions(rng, 22, 2.6, dmin=0.45)
    cases.append({"name": "dense_exceptional", "numbers": z[None], "positions": pos[None],
                  "charge": np.zeros(1), "energy_only": True})
    b = workloads.single32(7)
    cases.append({"name": "gfn2_refcharges", "numbers": b.numbers, "positions": b.positions,
                  "charge": b.charge, "ref_charges": "gfn2", "models": ("d4",)})
    b = workloads.batch_uniform(12, 3, 2, 6, workloads.ELEMENTS_12, False, "tiny3", 6)
    cases.append({"name": "tiny_batch", "numbers": b.numbers, "positions": b.positions,
                  "charge": b.charge})
    return cases


DEFAULT_PARAM = {"s6": 1.0, "s8": 1.2, "s9": 1.0, "a1": 0.40, "a2": 5.0}


def pair_radii(numbers: np.ndarray) -> np.ndarray:
    """Deterministic pairwise radii for the zero-damping family (the
    reference's VDW_PAIRWISE table lives in tad-mctc, absent here, so the
    fixtures pass ``rvdw`` explicitly): 2.8 + 0.35 (sqrt Z_i + sqrt Z_j)
    Bohr, symmetric, positive also for padding."""
    z = np.sqrt(numbers.astype(np.float64))
    return 2.8 + 0.35 * (z[..., :, None] + z[..., None, :])


def variant_cases(workloads) -> list[dict]:
    """D3-family two-body damping (damping/functions.py:308-484) and the
    exact-C9 method DispD4Exact (dispersion/d4.py:71-84)."""
    cases = []
    b = workloads.single32(8)
    cases.append({"name": "zero_damping", "numbers": b.numbers, "positions": b.positions,
                  "charge": b.charge, "damping": "zero", "rvdw": pair_radii(b.numbers),
                  "param": {"s6": 1.0, "s8": 0.9, "rs6": 1.2, "rs8": 1.0, "alp": 14.0,
                            "s9": 1.0}})
    b = workloads.batch_uniform(13, 3, 8, 24, workloads.ELEMENTS_12, True, "v3", 24)
    cases.append({"name": "mzero_damping_batch", "numbers": b.numbers,
                  "positions": b.positions, "charge": b.charge, "damping": "mzero",
                  "rvdw": pair_radii(b.numbers),
                  "param": {"s6": 1.0, "s8": 0.8, "rs6": 1.1, "rs8": 1.0, "alp": 14.0,
                            "bet": 0.3, "a1": 0.45, "a2": 4.5, "s9": 1.0}})
    b = workloads.single32(9)
    cases.append({"name": "op_damping", "numbers": b.numbers, "positions": b.positions,
                  "charge": np.array([-1.0]), "damping": "op",
                  "param": {"s6": 1.0, "s8": 0.7, "a1": 0.5, "a2": 3.0, "bet": 2.0,
                            "s9": 1.0}})
    b = workloads.single32(10)
    cases.append({"name": "zero_damping_short_cutoffs", "numbers": b.numbers,
                  "positions": b.positions, "charge": b.charge, "damping": "zero",
                  "rvdw": pair_radii(b.numbers), "cutoff": {"disp2": 9.0, "disp3": 6.0},
                  "param": {"s6": 0.9, "rs6": 1.3, "rs8": 1.1, "alp": 16.0, "s9": 1.0}})
    b = workloads.single32(11)
    cases.append({"name": "exact_c9", "numbers": b.numbers, "positions": b.positions,
                  "charge": b.charge, "exact_c9": True})
    b = workloads.batch_uniform(14, 3, 6, 20, workloads.ELEMENTS_12, True, "x3", 20)
    # D4S is left out here: the reference's D4S get_weighted_pols divides a
    # (B, N, 23) tensor by a (B, 1) atom count (model/d4s.py:313-316), which
    # does not broadcast for batches, so it has no batched D4S result
    cases.append({"name": "exact_c9_batch_short_cutoff", "numbers": b.numbers,
                  "positions": b.positions, "charge": b.charge, "exact_c9": True,
                  "cutoff": {"disp3": 7.0}, "models": ("d4",),
                  "param": {"s6": 1.0, "s8": 1.1, "a1": 0.42, "a2": 4.8, "s9": 1.2,
                            "alp": 15.0}})
    return cases


def run_variant(d4, case: dict, model_key: str) -> dict[str, np.ndarray]:
    from tad_dftd4.damping import (MZeroDamping, OptimisedPowerDamping, RationalDamping,
                                   ZeroDamping)
    from tad_dftd4.dispersion.d4 import DispD4Exact

    dd = {"device": torch.device("cpu"), "dtype": torch.float64}
    numbers = torch.tensor(case["numbers"])
    positions = torch.tensor(case["positions"], **dd)
    charge = torch.tensor(case["charge"], **dd)
    pdict = case.get("param", DEFAULT_PARAM)
    param = {k: torch.tensor(v, **dd, requires_grad=True) for k, v in pdict.items()}
    cutoff = d4.Cutoff(**case.get("cutoff", {}), **dd)
    cls = d4.D4Model if model_key == "d4" else d4.D4SModel
    model = cls(numbers, **dd)
    pos = positions.clone().requires_grad_(True)
    if case.get("exact_c9"):
        disp = DispD4Exact(model=model, **dd)
        energy = disp.calculate(numbers, pos, charge, param, cutoff=cutoff)
    else:
        damping = {"zero": ZeroDamping, "mzero": MZeroDamping, "op": OptimisedPowerDamping,
                   "rational": RationalDamping}[case["damping"]]()
        rvdw = torch.tensor(case["rvdw"], **dd) if "rvdw" in case else None
        energy = d4.dftd4(numbers, pos, charge, param, model=model, cutoff=cutoff,
                          rvdw=rvdw, damping_function=damping)
    keys = sorted(param)
    grads = torch.autograd.grad(energy.sum(), [pos] + [param[k] for k in keys])
    return {"energy": energy.detach().numpy(), "grad": grads[0].numpy(),
            "param_grad": np.array([g.item() for g in grads[1:]]),
            "param_grad_keys": np.array(json.dumps(keys))}


def run_case(d4, case: dict, model_key: str) -> dict[str, np.ndarray]:
    from tad_dftd4.damping import RationalDamping, ZeroDamping
    from tad_dftd4.dispersion.d4 import D4ATMApprox
    from tad_dftd4.dispersion.twobody import dispersion2
    from tad_mctc.ncoord import cn_d4
    from tad_multicharge import get_eeq_charges

    dd = {"device": torch.device("cpu"), "dtype": torch.float64}
    numbers = torch.tensor(case["numbers"])
    positions = torch.tensor(case["positions"], **dd)
    charge = torch.tensor(case["charge"], **dd)
    pdict = case.get("param", DEFAULT_PARAM)
    param = {k: torch.tensor(v, **dd, requires_grad=True) for k, v in pdict.items()}
    cutoff = d4.Cutoff(**case.get("cutoff", {}), **dd)
    ref_charges = case.get("ref_charges", "eeq")

    def make_model():
        cls = d4.D4Model if model_key == "d4" else d4.D4SModel
        return cls(numbers, ref_charges=ref_charges, **dd)

    pos = positions.clone().requires_grad_(True)
    energy = d4.dftd4(numbers, pos, charge, param, model=make_model(), cutoff=cutoff)
    out = {"energy": energy.detach().numpy()}
    if not case.get("energy_only"):
        keys = sorted(param)
        grads = torch.autograd.grad(energy.sum(), [pos] + [param[k] for k in keys])
        out["grad"] = grads[0].numpy()
        out["param_grad"] = np.array([g.item() for g in grads[1:]])
        out["param_grad_keys"] = np.array(json.dumps(keys))

    with torch.no_grad():
        model = make_model()
        cn = cn_d4(numbers, positions)
        q = get_eeq_charges(numbers, positions, charge, cutoff=cutoff.cn_eeq)
        gw = model.weight_references(cn, q)
        gw0 = model.weight_references(cn, None)
        c6 = model.get_atomic_c6(gw)
        c6_0 = model.get_atomic_c6(gw0)
        r4r2 = d4.data.R4R2(**dd)[numbers]
        pplain = {k: v.detach() for k, v in param.items()}
        e2 = dispersion2(numbers, positions, pplain, c6, r4r2, None, RationalDamping(),
                         cutoff.disp2)
        atm = D4ATMApprox(damping_fn=ZeroDamping(), charge_dependent=False)
        e3 = atm.calculate(numbers, positions, pplain, cn, model, None, r4r2, None, cutoff)
        alpha = model._get_alpha()
    out.update({"cn": cn.numpy(), "q": q.numpy(), "gw": gw.numpy(), "c6": c6.numpy(),
                "c6_0": c6_0.numpy(), "e2": e2.numpy(), "e3": e3.numpy(),
                "alpha": alpha.numpy()})
    return out


def write_variants(d4, workloads, out: Path) -> None:
    arrays: dict[str, np.ndarray] = {}
    index = []
    for case in variant_cases(workloads):
        for model_key in case.get("models", ("d4", "d4s")):
            tag = f"{case['name']}/{model_key}"
            res = run_variant(d4, case, model_key)
            meta = {"name": case["name"], "model": model_key,
                    "param": case.get("param", DEFAULT_PARAM),
                    "cutoff": case.get("cutoff", {}), "ref_charges": "eeq",
                    "energy_only": False, "damping": case.get("damping", "rational"),
                    "exact_c9": bool(case.get("exact_c9", False))}
            arrays[f"{tag}/numbers"] = np.asarray(case["numbers"], dtype=np.int64)
            arrays[f"{tag}/positions"] = np.asarray(case["positions"], dtype=np.float64)
            arrays[f"{tag}/charge"] = np.asarray(case["charge"], dtype=np.float64)
            if "rvdw" in case:
                arrays[f"{tag}/rvdw"] = np.asarray(case["rvdw"], dtype=np.float64)
            arrays[f"{tag}/meta"] = np.array(json.dumps(meta))
            for k, v in res.items():
                arrays[f"{tag}/{k}"] = v
            index.append(tag)
            print(tag, "E =", float(res["energy"].sum()))
    arrays["index"] = np.array(json.dumps(index))
    np.savez_compressed(out, **arrays)
    print("wrote", out)


def main():
    parser = argparse.ArgumentParser()
    parser.add_argument("--src", type=Path, required=True, help="reference src/ directory")
    parser.add_argument("--out", type=Path, default=OUT)
    parser.add_argument("--variants-out", type=Path, default=OUT_VARIANTS)
    parser.add_argument("--only-variants", action="store_true",
                        help="write only the damping-variant / exact-C9 fixtures")
    args = parser.parse_args()
    sys.path.insert(0, str(REPO))
    d4, workloads = _setup(args.src)
    write_variants(d4, workloads, args.variants_out)
    if args.only_variants:
        return
    cases = reference_cases(args.src.parent) + seeded_cases(workloads)
    arrays: dict[str, np.ndarray] = {}
    index = []
    for case in cases:
        for model_key in case.get("models", ("d4", "d4s")):
            tag = f"{case['name']}/{model_key}"
            res = run_case(d4, case, model_key)
            meta = {"name": case["name"], "model": model_key,
                    "param": case.get("param", DEFAULT_PARAM),
                    "cutoff": case.get("cutoff", {}),
                    "ref_charges": case.get("ref_charges", "eeq"),
                    "energy_only": bool(case.get("energy_only", False))}
            arrays[f"{tag}/numbers"] = np.asarray(case["numbers"], dtype=np.int64)
            arrays[f"{tag}/positions"] = np.asarray(case["positions"], dtype=np.float64)
            arrays[f"{tag}/charge"] = np.asarray(case["charge"], dtype=np.float64)
            arrays[f"{tag}/meta"] = np.array(json.dumps(meta))
            for k, v in res.items():
                arrays[f"{tag}/{k}"] = v
            index.append(tag)
            print(tag, "E =", float(res["energy"].sum()))
    arrays["index"] = np.array(json.dumps(index))
    np.savez_compressed(args.out, **arrays)
    print("wrote", args.out)


if __name__ == "__main__":
    main()
