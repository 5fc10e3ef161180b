"""nxm_pme_reciprocal_noalloc (the PME reciprocal step with every
intermediate in a fixed device array) against the engine's own PME step.

The comparison system has no bonds and no two atoms (or periodic images)
within the cutoff, so the engine's nonbonded force (nxm_compute_forces +
nxm_get_forces) is the reciprocal-space force alone and nxm_get_energies'
`recip` is the reciprocal energy.  Both entry points are called through the
C ABI; the new one gets device buffers made by torch (the test allocates,
the entry point does not).  Two calls in a row with different grids, then
the first grid again, check that no state left in the shared array leaks
into the next call: the repeated call must give the first call's numbers
bit for bit (the fixed-point charge grid makes each call deterministic).
The same calls are also checked against the FP64 oracle's reciprocal force
and energy (the reference's PME restated, NonbondedForce.cpp:51-461).

This file sorts last so that it also runs after every other test; it passes
alone in a fresh process as well.
"""
import ctypes as C
import types

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MIXED_FORCE_TOL = 1e-5     # force rel-RMS bound of every mixed-precision parity test
MIXED_ENERGY_TOL = 1e-5


def _lattice_system(seed=3, box=4.0, per_axis=7, n=300, cutoff=0.5):
    """Charged atoms on a jittered periodic lattice: nearest distance >= box/per_axis - 0.04 > cutoff."""
    rng = np.random.default_rng(seed)
    h = box / per_axis
    sites = np.stack(np.meshgrid(*[np.arange(per_axis)] * 3, indexing="ij"), -1).reshape(-1, 3)
    pick = rng.choice(len(sites), n, replace=False)
    pos = (sites[pick] + 0.5) * h + rng.uniform(-0.02, 0.02, (n, 3))
    q = rng.uniform(-1.0, 1.0, n)
    e2 = np.zeros((0, 2), np.int32)
    return types.SimpleNamespace(
        n=n, pos=pos, mass=np.ones(n), charge=q, sigma=np.full(n, 0.3), epsilon=np.zeros(n),
        bonds=e2, bond_prm=np.zeros((0, 2)), angles=np.zeros((0, 3), np.int32), angle_prm=np.zeros((0, 2)),
        torsions=np.zeros((0, 4), np.int32), torsion_prm=np.zeros((0, 2)), torsion_n=np.zeros(0, np.int32),
        cutoff=cutoff, ewald_tol=5e-4, box=np.full(3, box), grid=(0, 0, 0))


def _engine_reciprocal(s, grid):
    from nexusmd_gb300 import engine as E
    eng = E.Engine(s, precision=E.PRECISION_MIXED, force_mask=E.FORCE_NONBONDED, box="explicit", grid=grid)
    try:
        F = eng.compute_forces()
        en = eng.energies()
        alpha = eng.alpha()
    finally:
        eng.close()
    # the construction leaves no pair inside the cutoff and no exclusion
    assert en["coulomb"] == 0.0 and en["vdw"] == 0.0 and en["exclusion"] == 0.0
    return F, en["recip"], alpha


def _bind():
    from nexusmd_gb300.engine import load_library
    L = load_library()
    f = L.nxm_pme_reciprocal_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double),
                  C.POINTER(C.c_int32), C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return L, f


def _noalloc(f, xyz_d, q_d, box, grid, alpha, torch):
    n = xyz_d.shape[0]
    F = torch.full((n, 3), float("nan"), dtype=torch.float64, device=xyz_d.device)
    e = torch.full((1,), float("nan"), dtype=torch.float64, device=xyz_d.device)
    lb = (C.c_double * 3)(0.0, 0.0, 0.0)
    ub = (C.c_double * 3)(*map(float, box))
    g = (C.c_int32 * 3)(*map(int, grid))
    st = torch.cuda.current_stream(xyz_d.device).cuda_stream
    rc = f(xyz_d.data_ptr(), q_d.data_ptr(), n, lb, ub, g, float(alpha), F.data_ptr(), e.data_ptr(), st)
    torch.cuda.synchronize(xyz_d.device)
    return rc, F.cpu().numpy(), float(e.cpu().numpy()[0])


def _rel_rms(a, b):
    return float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))


def test_noalloc_pme_matches_engine_on_consecutive_calls(oracle):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    s = _lattice_system()
    L, f = _bind()
    dev = torch.device("cuda", 0)
    xyz_d = torch.tensor(s.pos, dtype=torch.float64, device=dev).contiguous()
    q_d = torch.tensor(s.charge, dtype=torch.float64, device=dev).contiguous()
    box = oracle.box_explicit([0.0, 0.0, 0.0], list(s.box))
    results = []
    for grid in ((40, 36, 30), (32, 32, 32), (40, 36, 30)):
        F_ref, E_ref, alpha = _engine_reciprocal(s, grid)
        rc, F, E = _noalloc(f, xyz_d, q_d, s.box, grid, alpha, torch)
        assert rc == 0, L.nxm_last_error().decode()
        err = _rel_rms(F, F_ref)
        E_o, F_o = oracle.pme(s.pos, s.charge, box, alpha, np.array(grid, np.int32))
        err_o = _rel_rms(F, F_o)
        print("grid", grid, "force rel-RMS vs engine", err, "vs oracle", err_o, "energy", E, "engine", E_ref,
              "oracle", E_o)
        assert np.isfinite(F).all()
        assert err <= MIXED_FORCE_TOL, (grid, err)
        assert abs(E - E_ref) <= MIXED_ENERGY_TOL * abs(E_ref), (grid, E, E_ref)
        assert err_o <= MIXED_FORCE_TOL, (grid, err_o)
        assert abs(E - E_o) <= MIXED_ENERGY_TOL * abs(E_o), (grid, E, E_o)
        results.append((F, E))
    # the second grid differs, so its result must too; the third call repeats
    # the first grid after the second left its contents in the shared array,
    # and must reproduce the first call exactly
    assert results[0][1] != results[1][1]
    assert np.array_equal(results[2][0], results[0][0])
    assert results[2][1] == results[0][1]


def test_noalloc_pme_no_atoms_after_charged_call():
    """A call with no atoms, right after a charged one, finds nothing stale:
    its energy is exactly zero."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    s = _lattice_system(n=50)
    L, f = _bind()
    dev = torch.device("cuda", 0)
    xyz_d = torch.tensor(s.pos, dtype=torch.float64, device=dev).contiguous()
    q_d = torch.tensor(s.charge, dtype=torch.float64, device=dev).contiguous()
    rc, _, E = _noalloc(f, xyz_d, q_d, s.box, (32, 32, 32), 5.0, torch)
    assert rc == 0 and E != 0.0
    rc, _, E0 = _noalloc(f, xyz_d[:0], q_d[:0], s.box, (32, 32, 32), 5.0, torch)
    assert rc == 0, L.nxm_last_error().decode()
    assert E0 == 0.0


def test_noalloc_pme_rejects_grid_above_limit():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    L, f = _bind()
    s = _lattice_system(n=20)
    dev = torch.device("cuda", 0)
    xyz_d = torch.tensor(s.pos, dtype=torch.float64, device=dev)
    q_d = torch.tensor(s.charge, dtype=torch.float64, device=dev)
    rc, _, _ = _noalloc(f, xyz_d, q_d, s.box, (72, 32, 32), 5.0, torch)
    assert rc == -3  # NXM_ERR_CAPACITY
    assert "limit of 64" in L.nxm_last_error().decode()
