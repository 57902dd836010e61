"""Padding masks and packing; atomic number 0 marks padding."""

from __future__ import annotations

import torch

from .mask import real_atoms, real_pairs, real_triples  # noqa: F401


def pack(tensors, value=0):
    n = max(t.shape[0] for t in tensors)
    out = tensors[0].new_full((len(tensors), n, *tensors[0].shape[1:]), value)
    for i, t in enumerate(tensors):
        out[i, : t.shape[0]] = t
    return out
