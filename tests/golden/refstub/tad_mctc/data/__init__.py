"""Element tables, served from the product's table file."""

from __future__ import annotations

from pathlib import Path

import numpy as np
import torch

from .zeff import ZEFF  # noqa: F401

_TABLES = Path(__file__).resolve().parents[5] / "tad-dftd4_gb300" / "data" / "d4_tables.npz"


def _table(key):
    with np.load(_TABLES) as npz:
        return np.array(npz[key])


def GAM(device=None, dtype=None):
    return torch.tensor(_table("gam"), device=device, dtype=dtype or torch.get_default_dtype())


def COV_D3(device=None, dtype=None):
    return torch.tensor(_table("cov_d3"), device=device, dtype=dtype or torch.get_default_dtype())


def PAULING_EN(device=None, dtype=None):
    return torch.tensor(_table("en"), device=device, dtype=dtype or torch.get_default_dtype())


def VDW_PAIRWISE(device=None, dtype=None):
    # only its shape is used on the dftd4() path
    return torch.zeros((119, 119), device=device, dtype=dtype or torch.get_default_dtype())
