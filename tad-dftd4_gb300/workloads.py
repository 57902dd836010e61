"""
Seeded synthetic structures for the dispersion workloads.

No public dataset backs these workloads; each generator draws elements from a
fixed distribution and places atoms uniformly in a cube, rejecting any atom
closer than ``dmin`` Bohr to an earlier one.  All randomness comes from
``numpy.random.default_rng(seed)``, so every workload is reproducible.

=========  ==================================================================
single32   N = 32, H/C/N/O (0.5/0.3/0.1/0.1), 12 Bohr cube, neutral
batch512   512 structures, N ~ U[8, 200] padded to 200, 12 elements (H 0.45,
           C 0.30, the other ten 0.025 each), cube side (N / 0.01)^(1/3),
           total charge ~ U{-1, 0, +1}
large16k   N = 16 000, H/C/N/O/S (0.45/0.3/0.1/0.1/0.05), density 0.01
diff256    256 structures, N ~ U[20, 150], 12 elements, random BJ params
stream20k  log-normal sizes (median 60, sigma 1.0) clipped to [5, 4000],
           Poisson arrival times at a target rate
=========  ==================================================================
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

# atomic numbers
H, B, C, N, O, F, SI, P, S, CL, BR, I = 1, 5, 6, 7, 8, 9, 14, 15, 16, 17, 35, 53

ELEMENTS_HCNO = ((H, 0.5), (C, 0.3), (N, 0.1), (O, 0.1))
ELEMENTS_12 = ((H, 0.45), (C, 0.30)) + tuple(
    (z, 0.025) for z in (B, N, O, F, SI, P, S, CL, BR, I)
)
ELEMENTS_HCNOS = ((H, 0.45), (C, 0.30), (N, 0.10), (O, 0.10), (S, 0.05))

BJ_PARAMS = {"s6": 1.0, "s8": 1.2, "a1": 0.40, "a2": 5.0, "s9": 1.0}
DENSITY = 0.01  # atoms / Bohr^3
DMIN = 1.8  # Bohr


@dataclass
class Batch:
    """Zero-padded batch in the reference's layout."""

    numbers: np.ndarray  # (B, N) int64, 0 = padding
    positions: np.ndarray  # (B, N, 3) float64, Bohr
    charge: np.ndarray  # (B,) float64
    seed: int
    name: str

    @property
    def natoms(self) -> np.ndarray:
        return (self.numbers != 0).sum(-1)


def draw_elements(rng: np.random.Generator, n: int, table) -> np.ndarray:
    z = np.array([e for e, _ in table], dtype=np.int64)
    p = np.array([w for _, w in table], dtype=np.float64)
    return rng.choice(z, size=n, p=p / p.sum())


def cube_positions(rng: np.random.Generator, n: int, side: float,
                   dmin: float = DMIN, max_tries: int = 100000) -> np.ndarray:
    """Uniform points in [0, side)^3 with pairwise distance >= dmin."""
    out = np.empty((n, 3), dtype=np.float64)
    cell = max(dmin, 1e-9)
    grid: dict[tuple[int, int, int], list[int]] = {}
    d2min = dmin * dmin
    for i in range(n):
        for _ in range(max_tries):
            p = rng.uniform(0.0, side, size=3)
            c = tuple((p // cell).astype(int))
            ok = True
            for dx in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    for dz in (-1, 0, 1):
                        for j in grid.get((c[0] + dx, c[1] + dy, c[2] + dz), ()):
                            d = out[j] - p
                            if d @ d < d2min:
                                ok = False
                                break
                        if not ok:
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if ok:
                out[i] = p
                grid.setdefault(c, []).append(i)
                break
        else:  # pragma: no cover
            raise RuntimeError("could not place atom; density too high")
    return out


def pad(structures, nmax: int | None = None):
    """Pack a list of (numbers, positions) into the zero-padded layout."""
    nmax = nmax or max(len(z) for z, _ in structures)
    b = len(structures)
    numbers = np.zeros((b, nmax), dtype=np.int64)
    positions = np.zeros((b, nmax, 3), dtype=np.float64)
    for k, (z, r) in enumerate(structures):
        numbers[k, : len(z)] = z
        positions[k, : len(z)] = r
    return numbers, positions


def single32(seed: int = 0) -> Batch:
    rng = np.random.default_rng(seed)
    z = draw_elements(rng, 32, ELEMENTS_HCNO)
    r = cube_positions(rng, 32, 12.0)
    return Batch(z[None], r[None], np.zeros(1), seed, "single32")


def batch_uniform(seed: int, nstruct: int, nmin: int, nmax: int, table,
                  charged: bool, name: str, pad_to: int | None = None) -> Batch:
    rng = np.random.default_rng(seed)
    sizes = rng.integers(nmin, nmax + 1, size=nstruct)
    structs = []
    for n in sizes:
        z = draw_elements(rng, int(n), table)
        side = (n / DENSITY) ** (1.0 / 3.0)
        structs.append((z, cube_positions(rng, int(n), side)))
    charge = (rng.integers(-1, 2, size=nstruct).astype(np.float64)
              if charged else np.zeros(nstruct))
    numbers, positions = pad(structs, pad_to or nmax)
    return Batch(numbers, positions, charge, seed, name)


def batch512(seed: int = 1, nstruct: int = 512) -> Batch:
    return batch_uniform(seed, nstruct, 8, 200, ELEMENTS_12, True, "batch512", 200)


def diff256(seed: int = 3, nstruct: int = 256) -> tuple[Batch, list[dict]]:
    batch = batch_uniform(seed, nstruct, 20, 150, ELEMENTS_12, False, "diff256", 150)
    rng = np.random.default_rng(seed + 1000)
    params = [
        {"s6": 1.0, "s9": 1.0, "s8": float(rng.uniform(0.5, 2.0)),
         "a1": float(rng.uniform(0.3, 0.6)), "a2": float(rng.uniform(3.0, 6.0))}
        for _ in range(nstruct)
    ]
    return batch, params


def large16k(seed: int = 2, natoms: int = 16000) -> Batch:
    rng = np.random.default_rng(seed)
    z = draw_elements(rng, natoms, ELEMENTS_HCNOS)
    side = (natoms / DENSITY) ** (1.0 / 3.0)
    r = cube_positions(rng, natoms, side)
    return Batch(z[None], r[None], np.zeros(1), seed, "large16k")


def stream_sizes(seed: int = 4, nreq: int = 20000, median: float = 60.0,
                 sigma: float = 1.0, nmin: int = 5, nmax: int = 4000,
                 rate: float = 2000.0):
    """Request sizes and Poisson arrival times (seconds)."""
    rng = np.random.default_rng(seed)
    sizes = np.clip(np.round(rng.lognormal(np.log(median), sigma, nreq)), nmin, nmax)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, nreq))
    return sizes.astype(np.int64), arrivals


def structure(seed: int, n: int, table=ELEMENTS_12, density: float = DENSITY):
    """One structure of ``n`` atoms at the given density."""
    rng = np.random.default_rng(seed)
    z = draw_elements(rng, n, table)
    side = (n / density) ** (1.0 / 3.0)
    return z, cube_positions(rng, n, side)
