"""
The precision form (``precision="mixed"``) against the FP64 oracle and the
reference's own outputs.  Bar (the precision form's contract): per-structure
energy error <= 1e-7 Eh and force error <= 1e-6 Eh/Bohr; charges from the
FP32 factorisation refined in FP64 agree with the FP64 solve to 1e-10.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

import oracle
from conftest import golden_cases, package

pytestmark = pytest.mark.gpu

CASES = golden_cases()
E_TOL = 1e-7   # Eh per structure
F_TOL = 1e-6   # Eh/Bohr per component
PARAM = {"s6": 1.0, "s8": 1.2, "a1": 0.4, "a2": 5.0, "s9": 1.0}


@pytest.fixture(scope="module")
def d4():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return package()


def _check(e, g, e_ref, g_ref):
    e = np.asarray(e).reshape(-1, np.asarray(e).shape[-1])
    e_ref = np.asarray(e_ref).reshape(e.shape)
    de = np.abs(e.sum(-1) - e_ref.sum(-1)).max()
    df = np.abs(np.asarray(g) - np.asarray(g_ref)).max()
    assert de <= E_TOL, f"max per-structure |dE| = {de:.3e} Eh"
    assert df <= F_TOL, f"max |dF| = {df:.3e} Eh/Bohr"
    return de, df


@pytest.mark.parametrize("tag,arrays,meta",
                         [c for c in CASES if not c[2]["energy_only"]],
                         ids=[c[0] for c in CASES if not c[2]["energy_only"]])
def test_golden_within_precision_bar(d4, tag, arrays, meta):
    dev = torch.device("cuda")
    numbers = torch.from_numpy(arrays["numbers"]).to(dev)
    positions = torch.from_numpy(arrays["positions"]).to(dev)
    charge = torch.from_numpy(arrays["charge"]).to(dev)
    cutoff = d4.Cutoff(**meta["cutoff"]) if meta["cutoff"] else None
    cls = d4.D4Model if meta["model"] == "d4" else d4.D4SModel
    e, g = d4.dispersion_energy_gradient(numbers, positions, charge, meta["param"],
                                         model=cls(numbers, ref_charges=meta["ref_charges"]),
                                         cutoff=cutoff, precision="mixed")
    _check(e.cpu().numpy(), g.cpu().numpy(), arrays["energy"], arrays["grad"])


@pytest.mark.parametrize("model", ["d4", "d4s"])
def test_random_batch_within_precision_bar(d4, model):
    wl = package().workloads
    b = wl.batch_uniform(301, 8, 5, 120, wl.ELEMENTS_12, True, "t", 120)
    nt, pt, ct = map(torch.from_numpy, (b.numbers, b.positions, b.charge))
    e_ref, g_ref = oracle.dftd4_energy_and_grad(nt, pt, ct, PARAM, model=model)
    dev = torch.device("cuda")
    e, g = d4.dispersion_energy_gradient(nt.to(dev), pt.to(dev), ct.to(dev), PARAM,
                                         model=model, precision="mixed")
    _check(e.cpu().numpy(), g.cpu().numpy(), e_ref.numpy(), g_ref.numpy())


def _eeq_fp64(numbers, positions, charge, cnq, tables):
    """FP64 solve of the EEQ system for given (capped) EEQ CN values."""
    import math
    real = numbers != 0
    n = int(real.sum())
    z = numbers[:n]
    r = positions[:n]
    rad = tables.eeq_rad[z]
    d = torch.cdist(r, r)
    g = 1.0 / torch.sqrt(rad[:, None] ** 2 + rad[None, :] ** 2)
    a = torch.where(torch.eye(n, dtype=torch.bool), 0.0, torch.erf(g * d) / torch.where(
        d > 0, d, 1.0))
    a = a + torch.diag(tables.eeq_eta[z] + math.sqrt(2.0 / math.pi) / rad)
    m = torch.zeros((n + 1, n + 1), dtype=torch.float64)
    m[:n, :n] = a
    m[:n, n] = 1.0
    m[n, :n] = 1.0
    rhs = torch.zeros(n + 1, dtype=torch.float64)
    c = cnq[:n]
    rhs[:n] = -tables.eeq_chi[z] + tables.eeq_kcn[z] * torch.sqrt(torch.clamp(c, min=0.0))
    rhs[n] = charge
    return torch.linalg.solve(m, rhs)[:n]


def test_charges_refined_to_fp64(d4):
    """The FP32 factorisation refined in FP64 solves the FP64 EEQ system
    (for the precision form's own coordination numbers): residual below
    1e-10, charges within 1e-9 of an FP64 solve."""
    from importlib import import_module
    disp = import_module("tad-dftd4_gb300.disp")
    wl = package().workloads
    b = wl.batch_uniform(302, 4, 20, 150, wl.ELEMENTS_12, True, "t", 150)
    dev = torch.device("cuda")
    nt, pt, ct = (torch.from_numpy(x).to(dev) for x in (b.numbers, b.positions, b.charge))
    runner, _, _ = disp._prepare(nt, pt, ct, PARAM, "d4", None, None, None, None, None,
                                 None, None, None, "mixed")
    out = runner.run(pt, charges_out=True, cn_eeq_out=True)
    q, cnq = out[3].cpu(), out[5].cpu()
    res = runner.eeq_residuals()  # the refinement's own final residuals
    assert (res[:, 0] < 1e-10).all() and res[:, 0].max() > 0, res
    assert (res[:, 1] == 0).all()  # no adjoint solve in an energy-only call
    tables = oracle.load_tables()
    for k in range(len(b.numbers)):
        q_ref = _eeq_fp64(torch.from_numpy(b.numbers[k]), torch.from_numpy(b.positions[k]),
                          float(b.charge[k]), cnq[k], tables)
        n = len(q_ref)
        assert (q[k, :n] - q_ref).abs().max().item() < 1e-9


def test_multi_cta_eeq_of_3700_atoms_refined_to_fp64(d4):
    """3700 atoms (eight 512-row blocks: the refinement's later iterations
    are launched only after the host has read the residuals): forward and
    adjoint residuals below 1e-10, charges within 1e-9 of an FP64 solve of
    the same EEQ system."""
    from importlib import import_module
    disp = import_module("tad-dftd4_gb300.disp")
    wl = package().workloads
    b = wl.large16k(5, 3700)
    dev = torch.device("cuda")
    nt, pt, ct = (torch.from_numpy(x).to(dev) for x in (b.numbers, b.positions, b.charge))
    runner, _, _ = disp._prepare(nt, pt, ct, PARAM, "d4", None, None, None, None, None,
                                 None, None, None, "mixed")
    out = runner.run(pt, gradient=True, charges_out=True, cn_eeq_out=True)
    q, cnq = out[3].cpu(), out[5].cpu()
    res = runner.eeq_residuals()
    assert (res < 1e-10).all() and (res > 0).all(), res
    tables = oracle.load_tables()
    q_ref = _eeq_fp64(torch.from_numpy(b.numbers[0]), torch.from_numpy(b.positions[0]),
                      float(b.charge[0]), cnq[0], tables)
    assert (q[0] - q_ref).abs().max().item() < 1e-9
    # without the host's residual read every iteration is launched and the
    # converged structure skips the later ones on the device: the same
    # charges and charge residual (the adjoint's right-hand side carries the
    # order-dependent last bits of FP32 atomics, so only its bar is checked)
    lib = import_module("tad-dftd4_gb300._lib")
    out2 = runner.run(pt, gradient=True, charges_out=True, extra_flags=lib.FLAG_NO_HOST_WAIT)
    assert torch.equal(out2[3].cpu(), q)
    res2 = runner.eeq_residuals()
    assert res2[0, 0] == res[0, 0] and 0 < res2[0, 1] < 1e-10


def test_large_structure_global_accumulation(d4):
    """n > 234 switches the ATM kernel to global accumulation."""
    wl = package().workloads
    z, r = wl.structure(303, 240)
    nt, pt = torch.from_numpy(z), torch.from_numpy(r)
    e_ref, g_ref = oracle.dftd4_energy_and_grad(nt, pt, torch.tensor(0.0), PARAM)
    dev = torch.device("cuda")
    e, g = d4.dispersion_energy_gradient(nt.to(dev), pt.to(dev), 0.0, PARAM, precision="mixed")
    _check(e.cpu().numpy()[None], g.cpu().numpy(), e_ref.numpy()[None], g_ref.numpy())


def test_param_gradients_mixed(d4):
    wl = package().workloads
    b = wl.batch_uniform(304, 3, 10, 40, wl.ELEMENTS_12, False, "t", 40)
    dev = torch.device("cuda")
    nt, pt, ct = map(torch.from_numpy, (b.numbers, b.positions, b.charge))
    keys = ["s6", "s8", "a1", "a2", "s9"]
    pref = {k: torch.tensor(PARAM[k], dtype=torch.float64, requires_grad=True) for k in keys}
    e_ref = oracle.dftd4(nt, pt, ct, pref)
    g_ref = torch.autograd.grad(e_ref.sum(), [pref[k] for k in keys])
    pd = {k: torch.tensor(PARAM[k], dtype=torch.float64, device=dev, requires_grad=True)
          for k in keys}
    e = d4.dftd4(nt.to(dev), pt.to(dev), ct.to(dev), pd, precision="mixed")
    g = torch.autograd.grad(e.sum(), [pd[k] for k in keys])
    for k, a, r in zip(keys, g, g_ref):
        assert abs(a.item() - r.item()) <= 1e-6 * max(1.0, abs(r.item())), (k, a.item(), r.item())


def test_float32_inputs_use_precision_form(d4):
    wl = package().workloads
    b = wl.batch_uniform(305, 2, 8, 30, wl.ELEMENTS_12, False, "t", 30)
    dev = torch.device("cuda")
    nt, pt, ct = map(torch.from_numpy, (b.numbers, b.positions, b.charge))
    e_ref = oracle.dftd4(nt, pt, ct, PARAM)
    e = d4.dftd4(nt.to(dev), pt.to(dev, torch.float32), ct.to(dev), PARAM)
    assert e.dtype == torch.float32
    assert np.abs(e.double().cpu().numpy().sum(-1) - e_ref.numpy().sum(-1)).max() <= 1e-6


def _runner(nt, pt, ct, precision):
    from importlib import import_module
    disp = import_module("tad-dftd4_gb300.disp")
    runner, _, _ = disp._prepare(nt, pt, ct, PARAM, "d4", None, None, None, None, None,
                                 None, None, None, precision)
    return runner


@pytest.mark.parametrize("sizes,pad", [((330, 380), 400), ((700,), 700), ((299,), 301)],
                         ids=["two-structures-N400", "one-structure-N700",
                              "odd-row-stride-N301"])
def test_multi_cta_eeq_and_atm_match_fp64_path(d4, sizes, pad):
    """Structures padded beyond the one-CTA EEQ limit (N > 290) take the
    multi-CTA factorisation (128-column panels, SYRK trailing updates, block
    sweeps) and the task-parallel global ATM; charges, energies and forces
    match the plain FP64 path within the precision bar, and the charges
    match an FP64 solve of the same EEQ system (the precision form's own
    coordination numbers) to 1e-9."""
    wl = package().workloads
    structs = [wl.structure(310 + k, n) for k, n in enumerate(sizes)]
    B = len(sizes)
    numbers = np.zeros((B, pad), dtype=np.int64)
    positions = np.zeros((B, pad, 3))
    for k, (z, r) in enumerate(structs):
        numbers[k, :len(z)] = z
        positions[k, :len(z)] = r
    charge = np.array([1.0, -1.0][:B])
    dev = torch.device("cuda")
    nt, pt, ct = (torch.from_numpy(x).to(dev) for x in (numbers, positions, charge))
    mixed_runner = _runner(nt, pt, ct, "mixed")
    mixed = mixed_runner.run(pt, gradient=True, charges_out=True, cn_eeq_out=True)
    res = mixed_runner.eeq_residuals()  # forward and adjoint refinements converged
    assert (res < 1e-10).all() and res.max() > 0, res
    plain = _runner(nt, pt, ct, "fp64").run(pt, gradient=True, charges_out=True)
    e, g, q, cnq = mixed[0], mixed[1], mixed[3].cpu(), mixed[5].cpu()
    _check(e.cpu().numpy(), g.cpu().numpy(), plain[0].cpu().numpy(), plain[1].cpu().numpy())
    # the precision form's FP32 coordination numbers move q by ~1e-7
    assert (q - plain[3].cpu()).abs().max().item() < 1e-6
    tables = oracle.load_tables()
    for k in range(B):
        q_ref = _eeq_fp64(torch.from_numpy(numbers[k]), torch.from_numpy(positions[k]),
                          float(charge[k]), cnq[k], tables)
        n = len(q_ref)
        assert (q[k, :n] - q_ref).abs().max().item() < 1e-9


def _sparse_counts(z, r, cut3):
    """Centre-pair visits and largest neighbour count of the neighbour-triple ATM."""
    d2 = ((r[:, None, :] - r[None, :, :]) ** 2).sum(-1)
    np.fill_diagonal(d2, np.inf)
    deg = (d2 <= cut3 * cut3).sum(1).astype(np.int64)
    return int((deg * (deg - 1) // 2).sum()), int(deg.max())


def test_neighbour_triple_atm_matches_dense_fp64_path(d4):
    """Structures whose disp3 sphere holds few of their atoms take the
    neighbour-triple ATM (centre-atom enumeration; each triple once, with the
    reference's per-atom attribution); a smaller, denser structure in the same
    batch keeps the all-triples kernel.  Energies, forces, parameter gradients
    and a non-uniform energy weighting match the plain FP64 path (all
    triples, FP64) within the precision bar."""
    from importlib import import_module
    disp = import_module("tad-dftd4_gb300.disp")
    wl = package().workloads
    cut3 = 15.0
    structs = [wl.structure(320, 1100), wl.structure(321, 300, density=0.03)]
    sparse = []
    for z, r in structs:
        n = len(z)
        visits, dmax = _sparse_counts(z, r, cut3)
        sparse.append(dmax <= 2048 and 2 * visits < n * (n - 1) * (n - 2) // 6)
    assert sparse == [True, False]
    pad = 1100
    B = len(structs)
    numbers = np.zeros((B, pad), dtype=np.int64)
    positions = np.zeros((B, pad, 3))
    for k, (z, r) in enumerate(structs):
        numbers[k, :len(z)] = z
        positions[k, :len(z)] = r
    charge = np.array([0.0, 1.0])
    dev = torch.device("cuda")
    nt, pt, ct = (torch.from_numpy(x).to(dev) for x in (numbers, positions, charge))
    cutoff = d4.Cutoff(disp2=50.0, disp3=cut3)
    param = dict(PARAM, alp=14.0)

    def run(precision, **kw):
        runner, _, _ = disp._prepare(nt, pt, ct, param, "d4", None, None, None, None, cutoff,
                                     None, None, None, precision)
        return runner.run(pt, **kw)

    mixed = run("mixed", gradient=True, param_grad=True)
    plain = run("fp64", gradient=True, param_grad=True)
    _check(mixed[0].cpu().numpy(), mixed[1].cpu().numpy(), plain[0].cpu().numpy(),
           plain[1].cpu().numpy())
    pm, pp = mixed[2].cpu().numpy(), plain[2].cpu().numpy()
    assert np.abs(pm - pp).max() <= 1e-6 * max(1.0, np.abs(pp).max()), (pm, pp)
    w = torch.rand(nt.shape, dtype=torch.float64, generator=torch.Generator().manual_seed(7))
    w = (w * (nt.cpu() != 0)).to(dev)
    gm = run("mixed", gradient=True, weights=w)[1]
    gp = run("fp64", gradient=True, weights=w)[1]
    assert (gm - gp).abs().max().item() <= F_TOL


@pytest.mark.parametrize("cut3", [40.0, 20.0, 12.0])
@pytest.mark.parametrize("gradient", [True, False])
def test_atm_tiles_and_per_triple_fallback_match_fp64(d4, cut3, gradient):
    """The shared-memory ATM evaluates gapless structures with register tiles
    of eight middle atoms: plain steps (unit attribution weights, atom
    energies from the pair sums) where no atom of the step has a pair beyond
    disp3, masked steps (weights 1, 1/3, 0 and the energy corrections of the
    1/3 triples) where one has; structures with padding below their last
    atom take the per-triple masks in the same kernel.  disp3 = 40 Bohr: a
    few far atoms in the largest structures; 20 Bohr: plain and masked steps
    mixed; 12 Bohr: nearly every step masked.  Energies (per structure and
    per atom) and forces match the plain FP64 path within the precision bar,
    with and without gradients."""
    from importlib import import_module
    disp = import_module("tad-dftd4_gb300.disp")
    wl = package().workloads
    b = wl.batch_uniform(303, 12, 5, 200, wl.ELEMENTS_12, True, "t", 200)
    numbers = b.numbers.copy()
    numbers[1, 2] = 0   # padding below the last real atom
    numbers[4, 0] = 0
    dev = torch.device("cuda")
    nt, pt, ct = (torch.from_numpy(x).to(dev) for x in (numbers, b.positions, b.charge))
    cutoff = d4.Cutoff(disp3=cut3)

    def run(precision):
        runner, _, _ = disp._prepare(nt, pt, ct, PARAM, "d4", None, None, None, None, cutoff,
                                     None, None, None, precision)
        return runner.run(pt, gradient=gradient)

    mixed, plain = run("mixed"), run("fp64")
    em, ep = mixed[0].cpu().numpy(), plain[0].cpu().numpy()
    assert np.abs(em - ep).max() <= E_TOL
    assert np.abs(em.sum(-1) - ep.sum(-1)).max() <= E_TOL
    if gradient:
        assert (mixed[1] - plain[1]).abs().max().item() <= F_TOL


def test_many_small_structures_padded_wide(d4):
    """A batch with more tiles of 128 atoms than the GPU has SMs x 4 (one CTA
    per tile, no partner split), small structures (tiles of <= 32 and <= 64
    atoms hold every atom in 4 and 2 rows of the tensor-core tile) padded to
    N = 230 (tiles of padding only): energies per atom, padding included,
    and forces match the plain FP64 path."""
    from importlib import import_module
    disp = import_module("tad-dftd4_gb300.disp")
    wl = package().workloads
    b = wl.batch_uniform(304, 700, 3, 100, wl.ELEMENTS_12, True, "t", 230)
    dev = torch.device("cuda")
    nt, pt, ct = (torch.from_numpy(x).to(dev) for x in (b.numbers, b.positions, b.charge))

    def run(precision):
        runner, _, _ = disp._prepare(nt, pt, ct, PARAM, "d4", None, None, None, None, None,
                                     None, None, None, precision)
        return runner.run(pt, gradient=True)

    mixed, plain = run("mixed"), run("fp64")
    em, ep = mixed[0].cpu().numpy(), plain[0].cpu().numpy()
    assert np.abs(em - ep).max() <= E_TOL
    assert np.all(em[b.numbers == 0] == 0.0)
    assert (mixed[1] - plain[1]).abs().max().item() <= F_TOL


def test_large_structure_call_replays_from_a_cuda_graph(d4):
    """A call on a structure large enough for the multi-CTA EEQ (its look-ahead
    runs on a second stream, ordered by events) captured into a CUDA graph:
    the replay gives the eager call's energies and forces."""
    from importlib import import_module
    disp = import_module("tad-dftd4_gb300.disp")
    wl = package().workloads
    z, r = wl.structure(331, 420)
    N = 423  # odd padding: the factor's row stride is rounded up
    numbers = np.zeros((1, N), dtype=np.int64)
    positions = np.zeros((1, N, 3))
    numbers[0, :len(z)] = z
    positions[0, :len(z)] = r
    dev = torch.device("cuda")
    nt, pt = torch.from_numpy(numbers).to(dev), torch.from_numpy(positions).to(dev)
    ct = torch.zeros(1, dtype=torch.float64, device=dev)
    runner = _runner(nt, pt, ct, "mixed")
    e0, g0 = (x.clone() for x in runner.run(pt, gradient=True)[:2])
    torch.cuda.synchronize()
    check = disp.CHECK_STATUS
    disp.CHECK_STATUS = False  # no host synchronisation inside a capture
    try:
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=side, capture_error_mode="relaxed"):
            out = runner.run(pt, gradient=True)
        graph.replay()
        torch.cuda.synchronize()
    finally:
        disp.CHECK_STATUS = check
    # (FP32 atomics of the partner-split kernels make the last bits order-dependent)
    assert abs(out[0].sum().item() - e0.sum().item()) <= 1e-9
    assert (out[1] - g0).abs().max().item() <= 1e-8
    res = runner.eeq_residuals()
    assert res[0, 0] < 1e-10 and res[0, 1] < 1e-10
