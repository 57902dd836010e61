"""Autograd-safe elementary functions (finite gradients at zero)."""

from __future__ import annotations

import torch


def _eps(x):
    return torch.finfo(x.dtype).eps


def sqrt(x):
    return torch.sqrt(torch.clamp(x, min=_eps(x)))


def divide(x, y):
    y = torch.as_tensor(y, dtype=x.dtype, device=x.device)
    return x / torch.where(y == 0, torch.full_like(y, _eps(x)), y)


def cdist(x, y=None, p=2):
    assert p == 2
    y = x if y is None else y
    diff = x.unsqueeze(-2) - y.unsqueeze(-3)
    return torch.sqrt(torch.clamp(torch.sum(diff * diff, -1), min=_eps(x)))
