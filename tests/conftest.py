"""Shared test setup: import paths, the ``gpu`` marker, fixture loading."""

from __future__ import annotations

import importlib
import json
import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))

GOLDEN = REPO / "tests" / "golden" / "golden.npz"
GOLDEN_VARIANTS = REPO / "tests" / "golden" / "golden_variants.npz"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def package():
    """The product package (its directory name has a hyphen)."""
    return importlib.import_module("tad-dftd4_gb300")


def golden_cases(path=GOLDEN):
    """List of (tag, dict of arrays, meta) from a golden fixture file."""
    with np.load(path) as npz:
        index = json.loads(str(npz["index"]))
        out = []
        for tag in index:
            arrays = {k.split("/", 2)[2]: np.array(npz[k]) for k in npz.files
                      if k.startswith(tag + "/")}
            meta = json.loads(str(arrays.pop("meta")))
            out.append((tag, arrays, meta))
    return out


def assert_close(actual, expected, rtol, atol, what=""):
    actual = np.asarray(actual, dtype=np.float64)
    expected = np.asarray(expected, dtype=np.float64)
    assert actual.shape == expected.shape, (what, actual.shape, expected.shape)
    err = np.abs(actual - expected)
    lim = atol + rtol * np.abs(expected)
    bad = err > lim
    assert not bad.any(), (
        f"{what}: {bad.sum()} of {bad.size} off; max abs err {err.max():.3e}, "
        f"max rel err {(err / np.maximum(np.abs(expected), 1e-300)).max():.3e}"
    )


def golden_variant_cases():
    """Cases of the damping-variant / exact-C9 fixture file."""
    return golden_cases(GOLDEN_VARIANTS)
