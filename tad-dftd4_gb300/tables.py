"""
Element tables on the device.

The tables are read once from ``data/d4_tables.npz`` (see
``data/make_tables.py`` for their provenance) and uploaded once per device
and model configuration.  The reference copies every table to the device on
every call (``model/base.py:381-386``, ``model/d4.py:154-172``); here they
stay resident.  The reference polarisabilities alpha(i w) depend only on
the element, so they are computed once per configuration by a CUDA kernel
(``d4_prepare_alpha``), not per call.
"""

from __future__ import annotations

import json
import os
import warnings
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np
import torch

from . import _lib

DEFAULT_PATH = Path(__file__).resolve().parent / "data" / "d4_tables.npz"
ENV_PATH = "TAD_DFTD4_GB300_TABLES"

_HOST: dict[str, dict[str, np.ndarray]] = {}
_DEVICE: dict[tuple, "DeviceTables"] = {}
_WARNED = False


def tables_path() -> Path:
    return Path(os.environ.get(ENV_PATH, DEFAULT_PATH))


def host_tables(path: str | Path | None = None) -> dict[str, np.ndarray]:
    key = str(path or tables_path())
    if key not in _HOST:
        with np.load(key) as npz:
            _HOST[key] = {k: np.array(npz[k]) for k in npz.files}
    return _HOST[key]


def provenance(path: str | Path | None = None) -> dict[str, str]:
    return json.loads(str(host_tables(path)["provenance"]))


def _warn_placeholders(path: str | Path | None) -> None:
    global _WARNED
    if _WARNED:
        return
    prov = provenance(path)
    missing = sorted(k for k, v in prov.items() if v.startswith("PLACEHOLDER"))
    if missing:
        warnings.warn(
            "tad-dftd4_gb300 runs with placeholder values for the tables "
            f"{', '.join(missing)} (they come from tad-mctc / tad-multicharge, "
            "which were not available when the table file was built); energies "
            "differ from tad-dftd4 until the file is rebuilt with "
            "data/make_tables.py --external.",
            RuntimeWarning,
            stacklevel=3,
        )
    _WARNED = True


def _pad_rows(arr: np.ndarray, rows: int) -> np.ndarray:
    if arr.shape[0] >= rows:
        return arr[:rows]
    out = np.zeros((rows, *arr.shape[1:]), dtype=arr.dtype)
    out[: arr.shape[0]] = arr
    return out


@dataclass
class DeviceTables:
    """Tables of one (device, reference charges, ga, gc) configuration."""

    device: torch.device
    ref_charges: str
    ga: float
    gc: float
    tensors: dict[str, torch.Tensor] = field(default_factory=dict)
    struct: _lib.Tables | None = None
    max_z: int = 0

    @property
    def n_ref_elem(self) -> int:
        return int(self.tensors["refcovcn"].shape[0])


def device_tables(device: torch.device, ref_charges: str = "eeq", ga: float = 3.0,
                  gc: float = 2.0, path: str | Path | None = None) -> DeviceTables:
    """Upload (once) and return the tables for this configuration."""
    if ref_charges not in ("eeq", "gfn2"):
        raise ValueError(f"Unknown reference charges: {ref_charges}")
    device = torch.device(device)
    if device.type != "cuda":
        raise ValueError("tad-dftd4_gb300 computes on CUDA devices only")
    if device.index is None:
        device = torch.device("cuda", torch.cuda.current_device())
    key = (device.index, ref_charges, float(ga), float(gc), str(path or tables_path()))
    if key in _DEVICE:
        return _DEVICE[key]
    _warn_placeholders(path)
    lib = _lib.load()
    host = host_tables(path)
    n_ref = host["refcovcn"].shape[0]
    n_elem = host["r4r2"].shape[0]

    def dev(arr, dtype=torch.float64):
        return torch.from_numpy(np.ascontiguousarray(arr)).to(device=device, dtype=dtype)

    if ref_charges == "eeq":
        refq, refh = host["clsq"], host["clsh"]
        max_z = n_ref - 1
    else:
        refq = _pad_rows(host["refq_gfn2"], n_ref)
        refh = _pad_rows(host["refh_gfn2"], n_ref)
        max_z = host["refq_gfn2"].shape[0] - 1
    t = {
        "refcovcn": dev(host["refcovcn"]),
        "refc": dev(host["refc"], torch.int64),
        "refq": dev(refq),
        "gam": dev(host["gam"]),
        "zeff": dev(host["zeff"], torch.int64),
        "r4r2": dev(host["r4r2"]),
        "cov_d3": dev(host["cov_d3"]),
        "en": dev(host["en"]),
        "eeq_chi": dev(host["eeq_chi"]),
        "eeq_eta": dev(host["eeq_eta"]),
        "eeq_kcn": dev(host["eeq_kcn"]),
        "eeq_rad": dev(host["eeq_rad"]),
        "wfpair": dev(host["wfpair"]),
        "freq_weights": dev(host["freq_weights"]),
        "alpha": torch.empty((n_ref, _lib.NREF, _lib.NFREQ), dtype=torch.float64,
                             device=device),
    }
    st = _lib.Tables(
        n_ref_elem=n_ref,
        n_elem=n_elem,
        **{name: t[name].data_ptr() for name in
           ("alpha", "refcovcn", "refc", "refq", "gam", "zeff", "r4r2", "cov_d3", "en",
            "eeq_chi", "eeq_eta", "eeq_kcn", "eeq_rad", "wfpair", "freq_weights")},
    )
    raw = {
        "refalpha": dev(host["refalpha"]),
        "refascale": dev(host["refascale"]),
        "refscount": dev(host["refscount"]),
        "refsys": dev(host["refsys"], torch.int64),
        "secscale": dev(host["secscale"]),
        "secalpha": dev(host["secalpha"]),
        "refh": dev(refh),
    }
    cfg = _lib.ModelCfg(kind=_lib.MODEL_D4, ga=ga, gc=gc, wf=6.0)
    stream = torch.cuda.current_stream(device).cuda_stream
    with torch.cuda.device(device):
        _lib.check(
            lib.d4_prepare_alpha(
                st, cfg, raw["refalpha"].data_ptr(), raw["refascale"].data_ptr(),
                raw["refscount"].data_ptr(), raw["refsys"].data_ptr(),
                raw["secscale"].data_ptr(), raw["secalpha"].data_ptr(),
                int(raw["secscale"].shape[0]), raw["refh"].data_ptr(),
                t["alpha"].data_ptr(), stream),
            "d4_prepare_alpha",
        )
        torch.cuda.current_stream(device).synchronize()
    tab = DeviceTables(device, ref_charges, float(ga), float(gc), t, st, max_z)
    _DEVICE[key] = tab
    return tab


_VDW: dict = {}


def vdw_pairwise(device: torch.device, numbers: torch.Tensor,
                 path: str | Path | None = None) -> torch.Tensor | None:
    """
    Pairwise van der Waals radii rvdw[b, i, j] = VDW_PAIRWISE[Z_i, Z_j] of a
    padded batch (the radii the zero-damping family takes, tad-dftd4
    ``dispersion/base.py:275-281``), or ``None`` when the table file holds no
    ``vdw_pairwise`` table (that table belongs to tad-mctc; a file built by
    ``data/make_tables.py --external`` from an installation carries it).
    """
    host = host_tables(path)
    if "vdw_pairwise" not in host:
        return None
    device = torch.device(device)
    key = (str(device), str(path or tables_path()))
    tab = _VDW.get(key)
    if tab is None:
        tab = torch.from_numpy(np.ascontiguousarray(host["vdw_pairwise"])).to(
            device=device, dtype=torch.float64)
        _VDW[key] = tab
    z = numbers.to(device=device, dtype=torch.int64).clamp(0, tab.shape[0] - 1)
    return tab[z.unsqueeze(-1), z.unsqueeze(-2)]
