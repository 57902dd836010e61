"""Effective nuclear charges, served from the product's table file."""

from __future__ import annotations

from pathlib import Path

import numpy as np
import torch

_TABLES = Path(__file__).resolve().parents[5] / "tad-dftd4_gb300" / "data" / "d4_tables.npz"


def ZEFF(device=None, dtype=torch.long):
    with np.load(_TABLES) as npz:
        return torch.tensor(np.array(npz["zeff"]), device=device, dtype=dtype)
