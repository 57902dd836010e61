"""
The neighbour-list float64 restatement (``oracle/d4_nbr.py``, the checker of
the 16000-atom benchmark line) against the dense oracle, which follows the
reference's own tensors: energies 1e-12 relative, gradients 1e-10.  Short
cutoffs give partial neighbourhoods (triples with one side beyond disp3,
taken at their unique centre); a long cutoff puts every side inside (each
triple taken once, at its smallest atom).
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import d4_nbr, d4_oracle
from conftest import assert_close, package

PARAM = {"s6": 1.0, "s8": 1.2, "a1": 0.4, "a2": 5.0, "s9": 1.0}


@pytest.mark.parametrize("n,cutoff,charge", [
    (150, {"disp2": 20.0, "disp3": 8.0}, 0.0),
    (90, {"disp2": 60.0, "disp3": 40.0}, 1.0),
    (120, {"disp2": 15.0, "disp3": 11.0, "cn_eeq": 9.0}, -1.0),
])
def test_neighbour_list_oracle_matches_dense_oracle(n, cutoff, charge):
    wl = package().workloads
    z, r = wl.structure(900 + n, n)
    numbers = torch.from_numpy(z)
    positions = torch.from_numpy(r)
    e_d, g_d = d4_oracle.dftd4_energy_and_grad(numbers[None], positions[None],
                                               torch.tensor([charge]), PARAM, cutoff=cutoff)
    e, g, extra = d4_nbr.dftd4_large(numbers, positions, charge, PARAM, cutoff=cutoff,
                                     triples_per_chunk=50_000)
    assert extra["triples"] > 0
    assert_close(e.numpy(), e_d.numpy()[0], 1e-12, 1e-15, "energy")
    assert_close(g.numpy(), g_d.numpy()[0], 1e-10, 1e-14, "grad")


def test_triple_enumeration_counts_each_kept_triple_once():
    wl = package().workloads
    _, r = wl.structure(77, 60)
    pos = torch.from_numpy(r)
    cut = 9.0
    seen = []
    for i, j, k in d4_nbr.atm_triples(pos, cut, centre_chunk=7):
        seen.append(torch.sort(torch.stack([i, j, k]), dim=0).values.T)
    got = torch.cat(seen).numpy()
    assert len({tuple(t) for t in got}) == len(got)
    d = np.sqrt(((r[:, None] - r[None]) ** 2).sum(-1))
    m = (d <= cut).astype(int)
    want = 0
    for a in range(60):
        for b in range(a + 1, 60):
            for c in range(b + 1, 60):
                want += (m[a, b] + m[a, c] + m[b, c]) >= 2
    assert len(got) == want


def test_eeq_residual_of_the_exact_solution_is_tiny():
    wl = package().workloads
    z, r = wl.structure(55, 40)
    numbers, positions = torch.from_numpy(z), torch.from_numpy(r)
    tables = d4_nbr.device_tables("cpu")
    q = d4_oracle.eeq_charges(numbers, positions, torch.tensor(0.0), d4_oracle.load_tables())
    assert d4_nbr.eeq_residual(numbers, positions, 0.0, q, tables) < 1e-12
    q2 = q.clone()
    q2[0] += 1e-6
    assert d4_nbr.eeq_residual(numbers, positions, 0.0, q2, tables) > 1e-7
