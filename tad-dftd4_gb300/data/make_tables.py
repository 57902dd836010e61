"""
Build ``d4_tables.npz``, the element tables every kernel takes as input.

The DFT-D4 model is defined by element-indexed tables.  The kernels never bake
them in: they are uploaded once per device from this file.  Two groups exist.

1. Tables that ship inside tad-dftd4 itself.  They are read from the
   reference's Python sources and stored unchanged (same values, same index
   convention: row 0 is the dummy element).

   ==============  ==========================================================
   refcovcn        ``reference/d4/params.py:40-979``   (104, 7)  reference CN
   refalpha        ``reference/d4/params.py:1142-19553`` (104, 7, 23)
   refascale       ``reference/d4/params.py:19556-20495`` (104, 7)
   refscount       ``reference/d4/params.py:20498-21437`` (104, 7)
   refsys          ``reference/d4/params.py:21440-21547`` (104, 7) int
   refc            ``reference/d4/params.py:21550-21657`` (104, 7) int
   secscale        ``reference/d4/params.py:21659-21680`` (18,)
   secalpha        ``reference/d4/params.py:21683-22136`` (18, 23)
   clsq, clsh      ``reference/d4/charge_eeq.py:29-1910`` (104, 7)
   refq_gfn2,
   refh_gfn2       ``reference/d4/charge_gfn2.py:29-1605`` (87, 7)
   r4r2            ``data/r4r2.py:34-88``  (119,) already transformed to
                   sqrt(0.5 * r4r2 * sqrt(Z)) in float64
   wfpair          ``data/wfpair.py:36-3735`` (119, 119)
   freq_weights    ``utils.py:52-80`` (23,) Casimir-Polder quadrature weights
   ==============  ==========================================================

2. Tables that tad-dftd4 imports from ``tad-mctc==0.7.0`` and
   ``tad-multicharge==0.5.0``: chemical hardness ``gam``, effective nuclear
   charge ``zeff``, D3 covalent radii ``cov_d3``, Pauling electronegativity
   ``en`` and the EEQ parameters ``eeq_chi``, ``eeq_eta``, ``eeq_kcn``,
   ``eeq_rad``.  Those packages are not part of the reference source tree.
   Pass ``--external FILE.npz`` holding these eight arrays (length >= 104,
   row 0 = dummy) dumped from an installation of those packages to get the
   physical values (the file may also hold ``vdw_pairwise`` (>= 104 x 104),
   tad-mctc's pairwise van der Waals radii, which the zero-damping family of
   two-body damping functions takes; without it those callers pass ``rvdw``).
   Without it, deterministic PLACEHOLDER values are written
   and ``provenance`` says so for each of them.  Placeholders make every
   kernel and every parity test meaningful (GPU and oracle see the same
   inputs), but energies then differ from a real tad-dftd4 installation.

Usage::

    python make_tables.py --src <tad_dftd4 source dir> [--external ext.npz]
"""

from __future__ import annotations

import argparse
import importlib.util
import json
import re
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
OUT = HERE / "d4_tables.npz"

N_ELEM = 119  # dummy + Z = 1..118, the extent of r4r2 / wfpair
EXTERNAL_KEYS = (
    "gam", "zeff", "cov_d3", "en", "eeq_chi", "eeq_eta", "eeq_kcn", "eeq_rad"
)


def _load_module(name: str, path: Path) -> types.ModuleType:
    spec = importlib.util.spec_from_file_location(name, path)
    assert spec is not None and spec.loader is not None
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _reference_tables(src: Path) -> dict[str, np.ndarray]:
    """Read the in-tree tables of tad-dftd4 (torch tensors) as numpy arrays."""
    import torch

    # data/wfpair.py imports a type alias from tad_mctc; nothing else is used.
    if "tad_mctc.typing" not in sys.modules:
        pkg = types.ModuleType("tad_mctc")
        typ = types.ModuleType("tad_mctc.typing")
        typ.Tensor = torch.Tensor  # type: ignore[attr-defined]
        pkg.typing = typ  # type: ignore[attr-defined]
        sys.modules.setdefault("tad_mctc", pkg)
        sys.modules["tad_mctc.typing"] = typ

    params = _load_module("_d4_params", src / "reference/d4/params.py")
    ceeq = _load_module("_d4_charge_eeq", src / "reference/d4/charge_eeq.py")
    cgfn = _load_module("_d4_charge_gfn2", src / "reference/d4/charge_gfn2.py")
    r4r2 = _load_module("_d4_r4r2", src / "data/r4r2.py")
    wfp = _load_module("_d4_wfpair", src / "data/wfpair.py")

    t: dict[str, np.ndarray] = {}
    for key in ("refcovcn", "refalpha", "refascale", "refscount"):
        t[key] = getattr(params, key).to(torch.float64).numpy()
    t["refsys"] = params.refsys.to(torch.int64).numpy()
    t["refc"] = params.refc.to(torch.int64).numpy()
    t["secscale"] = params.secscale.to(torch.float64).numpy().reshape(-1)
    t["secalpha"] = params.secalpha.to(torch.float64).numpy()
    t["clsq"] = ceeq.clsq.to(torch.float64).numpy()
    t["clsh"] = ceeq.clsh.to(torch.float64).numpy()
    t["refq_gfn2"] = cgfn.refq.to(torch.float64).numpy()
    t["refh_gfn2"] = cgfn.refh.to(torch.float64).numpy()
    t["r4r2"] = r4r2.R4R2(dtype=torch.float64).numpy()
    t["wfpair"] = wfp.WFPAIR(dtype=torch.float64).numpy()

    # The 23 quadrature weights are a literal list inside ``trapzd``.
    text = (src / "utils.py").read_text()
    block = text.split("def trapzd(", 1)[1].split("weights = torch.tensor(", 1)[1]
    block = block.split("]", 1)[0]
    weights = [float(x) for x in re.findall(r"[-+]?\d+\.\d+(?:e[-+]?\d+)?", block)]
    assert len(weights) == 23, weights
    t["freq_weights"] = np.asarray(weights, dtype=np.float64)
    return t


def _placeholder_tables() -> dict[str, np.ndarray]:
    """
    Deterministic stand-ins for the tad-mctc / tad-multicharge tables.

    They are smooth functions of Z with physically plausible magnitudes
    (positive hardness and radii, EEQ hardness > 0 so that the EEQ matrix is
    positive definite).  They are NOT the published values.
    """
    z = np.arange(N_ELEM, dtype=np.float64)
    out = {
        "gam": 0.25 + 0.35 * np.exp(-z / 30.0),
        "zeff": np.arange(N_ELEM, dtype=np.int64),
        "cov_d3": 0.8 + 2.4 * (1.0 - np.exp(-z / 15.0)),
        "en": 2.2 + 0.8 * np.sin(0.7 * z),
        "eeq_chi": 1.0 + 0.3 * np.cos(0.9 * z),
        "eeq_eta": 0.6 + 0.4 * np.exp(-z / 25.0),
        "eeq_kcn": 0.05 + 0.05 * np.sin(z),
        "eeq_rad": 1.0 + 1.5 * (1.0 - np.exp(-z / 20.0)),
    }
    for key in out:
        out[key][0] = 0
    return out


def build(src: Path, external: Path | None = None) -> dict[str, np.ndarray]:
    tables = _reference_tables(src)
    prov = {k: "tad-dftd4 source" for k in tables}
    if external is not None:
        ext = np.load(external)
        if "vdw_pairwise" in ext.files:  # optional: the zero-damping family's radii
            vdw = np.asarray(ext["vdw_pairwise"], dtype=np.float64)
            full = np.zeros((N_ELEM, N_ELEM))
            m = min(vdw.shape[0], N_ELEM)
            full[:m, :m] = vdw[:m, :m]
            tables["vdw_pairwise"] = full
            prov["vdw_pairwise"] = f"external: {external.name}"
        for key in EXTERNAL_KEYS:
            arr = np.asarray(ext[key])
            full = np.zeros(N_ELEM, dtype=np.int64 if key == "zeff" else np.float64)
            full[: min(len(arr), N_ELEM)] = arr[:N_ELEM]
            tables[key] = full
            prov[key] = f"external: {external.name}"
    else:
        for key, arr in _placeholder_tables().items():
            tables[key] = arr
            prov[key] = "PLACEHOLDER (tad-mctc / tad-multicharge not available)"
    tables["provenance"] = np.asarray(json.dumps(prov, sort_keys=True))
    return tables


def main() -> None:
    parser = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    parser.add_argument("--src", type=Path, required=True,
                        help="tad_dftd4 package source directory")
    parser.add_argument("--external", type=Path, default=None)
    parser.add_argument("--out", type=Path, default=OUT)
    args = parser.parse_args()
    tables = build(args.src, args.external)
    np.savez_compressed(args.out, **tables)
    print(f"wrote {args.out}")


if __name__ == "__main__":
    main()
