"""einsum wrapper (the ``optimize`` hint is ignored)."""

from __future__ import annotations

import torch


def einsum(equation, *operands, optimize=None):
    return torch.einsum(equation, *operands)
