"""Masks of real atoms, pairs and triples."""

from __future__ import annotations

import torch


def real_atoms(numbers):
    return numbers != 0


def real_pairs(numbers, mask_diagonal=True):
    ra = real_atoms(numbers)
    mask = ra.unsqueeze(-1) & ra.unsqueeze(-2)
    if mask_diagonal:
        n = numbers.shape[-1]
        mask = mask & ~torch.eye(n, dtype=torch.bool, device=numbers.device)
    return mask


def real_triples(numbers, mask_diagonal=True, mask_self=True):
    ra = real_atoms(numbers)
    mask = ra.unsqueeze(-1).unsqueeze(-1) & ra.unsqueeze(-2).unsqueeze(-1) & ra.unsqueeze(-2).unsqueeze(-2)
    n = numbers.shape[-1]
    eye = torch.eye(n, dtype=torch.bool, device=numbers.device)
    if mask_diagonal:
        mask = mask & ~eye.unsqueeze(-3)
    if mask_self:
        mask = mask & ~eye.unsqueeze(-1) & ~eye.unsqueeze(-2)
    return mask
