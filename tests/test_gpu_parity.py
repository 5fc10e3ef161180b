"""CUDA engine vs the FP64 oracle on the same inputs (GPU required).

Each case runs the reference's algorithm twice -- once in the oracle (a C
restatement of the reference, pinned to the compiled reference by
test_oracle_pins.py) and once through the engine's C ABI -- and compares
forces, every energy term and the neighbour pair set.

Tolerances:
* FP64 engine: forces and energies within 1e-9 relative (summation order
  differs from the reference's serial loops).
* mixed engine: force rel-RMS <= 1e-5 (the stated target), each energy term
  within 2e-5 relative of the largest nonbonded term.
* neighbour pair set: identical.
"""
import numpy as np
import pytest

from nexusmd_gb300 import synthetic as sy

pytestmark = pytest.mark.gpu


def _engine(s, **kw):
    from nexusmd_gb300.engine import Engine
    return Engine(s, **kw)


def _oracle_forces(oracle, s, force_mask=15, grid=None, box_mode=0, lb=None, ub=None):
    if box_mode == 0:
        box = oracle.box_from_positions(s.pos)
    else:
        box = oracle.box_explicit(lb, ub)
    eoff, el = oracle.exclusions(s.n, s.bonds)
    d = oracle.describe(s, force_mask=force_mask, grid=grid, box_mode=box_mode, lb=lb, ub=ub)
    F, E = oracle.forces(d, s.pos, box, eoff, el)
    return F, E, box, eoff, el


def rel_rms(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


TERMS = ("bond", "angle", "torsion", "recip", "self", "coulomb", "vdw", "exclusion")


@pytest.mark.parametrize("grid", [(0, 0, 0), (32, 32, 32)])
def test_fp64_forces_energies_c1(oracle, c1_compat, grid):
    s = c1_compat
    F0, E0, box, _, _ = _oracle_forces(oracle, s, grid=grid)
    eng = _engine(s, precision=0, skin=0.0, rebuild_interval=1, grid=grid)
    lb, ub = eng.box()
    assert np.array_equal(lb, np.array(box.lb)) and np.array_equal(ub, np.array(box.ub))
    if grid == (0, 0, 0):
        assert eng.grid() == oracle.pow2_grid(box)
    F = eng.compute_forces()
    E = eng.energies()
    assert rel_rms(F, F0) < 1e-9, rel_rms(F, F0)
    scale = max(abs(E0[k]) for k in TERMS)
    for k in TERMS:
        assert abs(E[k] - E0[k]) <= 1e-9 * scale + 1e-6, (k, E[k], E0[k])
    assert abs(E["reported_potential"] - E0["reported_pe"]) <= 1e-9 * scale


def test_mixed_forces_energies_c1(oracle, c1_compat):
    s = c1_compat
    F0, E0, _, _, _ = _oracle_forces(oracle, s)
    eng = _engine(s, precision=1, skin=0.0, rebuild_interval=1, grid=(0, 0, 0))
    F = eng.compute_forces()
    E = eng.energies()
    err = rel_rms(F, F0)
    print("mixed rel-RMS force error", err, "max atom", np.abs(F - F0).max())
    assert err <= 1e-5, err
    scale = max(abs(E0[k]) for k in TERMS)
    for k in TERMS:
        assert abs(E[k] - E0[k]) <= 2e-5 * scale, (k, E[k], E0[k])


@pytest.mark.parametrize("precision", [0, 1])
def test_neighbor_set_bit_exact(oracle, c1_compat, precision):
    s = c1_compat
    box = oracle.box_from_positions(s.pos)
    eoff, el = oracle.exclusions(s.n, s.bonds)
    ref = oracle.neighbor_pairs(s.pos, box, eoff, el, s.cutoff)
    ref = ref[np.lexsort((ref[:, 1], ref[:, 0]))]
    eng = _engine(s, precision=precision, skin=0.0, rebuild_interval=1)
    eng.compute_forces()
    got = eng.pairs()
    assert got.shape == ref.shape
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("mask", [1, 2, 4, 8, 3, 15])
def test_force_masks_fp64(oracle, small_compat, mask):
    s = small_compat
    F0, E0, _, _, _ = _oracle_forces(oracle, s, force_mask=mask)
    eng = _engine(s, precision=0, skin=0.0, rebuild_interval=1, force_mask=mask)
    F = eng.compute_forces()
    assert rel_rms(F, F0) < 1e-9
    E = eng.energies()
    assert abs(E["reported_potential"] - E0["reported_pe"]) <= 1e-9 * max(1.0, abs(E0["reported_pe"]))


def test_trajectory_fp64_matches_oracle(oracle, small_compat):
    """10 leapfrog steps from v = 0 (the reference's Simulate path)."""
    s = small_compat
    d = oracle.describe(s)
    p, v, F, rep, box = oracle.run(d, s.pos, np.zeros_like(s.pos), 0.0005, 10, interval=1)
    eng = _engine(s, precision=0, skin=0.0, rebuild_interval=1)
    kes, pes = [], []
    for k in range(10):
        eng.step(1, 0.0005)
        e = eng.energies()
        kes.append(e["kinetic"])
        pes.append(e["reported_potential"])
    x, vel = eng.state()
    assert np.abs(x - p).max() < 1e-9
    assert np.abs(vel - v).max() < 1e-6 * max(1.0, np.abs(v).max())
    assert np.allclose(kes, rep[:, 1], rtol=1e-8, atol=1e-8)
    assert np.allclose(pes, rep[:, 2], rtol=1e-9, atol=1e-6)


def test_mixed_trajectory_tracks_fp64(small_compat):
    s = small_compat
    a = _engine(s, precision=0, skin=0.0, rebuild_interval=1)
    b = _engine(s, precision=1, skin=0.1, rebuild_interval=10)
    a.step(20, 0.0005)
    b.step(20, 0.0005)
    xa, _ = a.state()
    xb, _ = b.state()
    assert np.abs(xa - xb).max() < 1e-5
    ea, eb = a.energies(), b.energies()
    assert abs(ea["kinetic"] - eb["kinetic"]) <= 1e-4 * abs(ea["kinetic"]) + 1e-3


def test_mixed_bit_reproducible(c1_compat):
    s = c1_compat
    outs = []
    for _ in range(2):
        e = _engine(s, precision=1, skin=0.1, rebuild_interval=5)
        e.step(7, 0.0005)
        outs.append((e.forces(), e.state()[0]))
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])


def test_explicit_box_skin_list(oracle):
    """Physics-mode system: periodic box [0, L), list with skin rebuilt on a schedule."""
    s = sy.config_system(1)
    lb, ub = np.zeros(3), s.box.copy()
    F0, E0, _, _, _ = _oracle_forces(oracle, s, box_mode=1, lb=lb, ub=ub)
    for prec, tol in ((0, 1e-9), (1, 1e-5)):
        eng = _engine(s, precision=prec, skin=0.1, rebuild_interval=10, box="explicit")
        F = eng.compute_forces()
        assert rel_rms(F, F0) <= tol, (prec, rel_rms(F, F0))


def _sparse_gas(seed=8, n_mol=150, box=5.0):
    """Diatomic molecules scattered in a large box: most cells are empty, so
    many cell groups start with an empty cell (the tile is then anchored at
    the group's first non-empty cell)."""
    import types
    rng = np.random.default_rng(seed)
    pos = []
    while len(pos) < 2 * n_mol:
        a = rng.uniform(0, box, 3)
        d = rng.normal(size=3)
        b = a + 0.12 * d / np.linalg.norm(d)
        ok = True
        for p in pos:
            for c in (a, b):
                r = c - p
                r -= box * np.round(r / box)
                if (r * r).sum() < 0.3 ** 2:
                    ok = False
        if ok:
            pos += [a, np.mod(b, box)]
    n = len(pos)
    q = rng.uniform(-0.8, 0.8, n)
    bonds = np.arange(n, dtype=np.int32).reshape(-1, 2)
    return types.SimpleNamespace(
        n=n, pos=np.array(pos), mass=np.full(n, 12.0), charge=q, sigma=rng.uniform(0.2, 0.3, n),
        epsilon=rng.uniform(0.1, 0.5, n), bonds=bonds, bond_prm=np.tile([0.12, 3.0e5], (n // 2, 1)),
        angles=np.zeros((0, 3), np.int32), angle_prm=np.zeros((0, 2)), torsions=np.zeros((0, 4), np.int32),
        torsion_prm=np.zeros((0, 2)), torsion_n=np.zeros(0, np.int32), cutoff=0.9, ewald_tol=5e-4,
        box=np.full(3, box), grid=(50, 50, 50))


def test_sparse_system_empty_cells(oracle):
    s = _sparse_gas()
    lb, ub = np.zeros(3), s.box.copy()
    F0, E0, box, eoff, el = _oracle_forces(oracle, s, grid=s.grid, box_mode=1, lb=lb, ub=ub)
    ref = oracle.neighbor_pairs(s.pos, box, eoff, el, s.cutoff)
    ref = ref[np.lexsort((ref[:, 1], ref[:, 0]))]
    assert len(ref) > 50
    for prec, tol in ((0, 1e-9), (1, 1e-5)):
        eng = _engine(s, precision=prec, skin=0.1, rebuild_interval=10, box="explicit", grid=s.grid)
        F = eng.compute_forces()
        assert np.isfinite(F).all()
        assert rel_rms(F, F0) <= tol, (prec, rel_rms(F, F0))
        assert np.array_equal(eng.pairs(), ref)
        eng.close()


@pytest.mark.parametrize("depth", [3, 2, 60])
def test_exceptions_physics_mode(oracle, depth):
    """Scaled 1-4 exceptions (OpenMM semantics) vs the oracle.  With depth 2
    the 1-4 pairs are excluded only because they are exceptions, so the
    engine's union of bonded exclusions and exception pairs is exercised.
    The exclusion sets are built on the device; with depth 60 the chain
    atoms' sets (well over 96 atoms) exceed the device search and the host
    builds them instead."""
    s = sy.with_exceptions(sy.config_system(1))
    lb, ub = np.zeros(3), s.box.copy()
    box = oracle.box_explicit(lb, ub)
    off, lst = oracle.exclusions(s.n, s.bonds, depth=depth)
    off, lst = oracle.union_exclusions(off, lst, s.exc_idx)
    d = oracle.describe(s, box_mode=1, lb=lb, ub=ub, exclusion_depth=depth, exceptions=(s.exc_idx, s.exc_prm))
    F0, E0 = oracle.forces(d, s.pos, box, off, lst)
    assert E0["exception"] != 0.0
    scale = max(abs(E0[k]) for k in TERMS)
    for prec, tol in ((0, 1e-9), (1, 1e-5)):
        eng = _engine(s, precision=prec, skin=0.1, rebuild_interval=10, box="explicit", exclusion_depth=depth,
                      exceptions=True)
        F = eng.compute_forces()
        E = eng.energies()
        assert rel_rms(F, F0) <= tol, (prec, depth, rel_rms(F, F0))
        etol = 1e-9 if prec == 0 else 2e-5
        for k in TERMS + ("exception",):
            assert abs(E[k] - E0[k]) <= etol * scale + 1e-6, (prec, k, E[k], E0[k])
        assert abs(E["potential"] - (E0["bond"] + E0["angle"] + E0["torsion"] + E0["recip"] + E0["self"]
                                     + E0["coulomb"] + E0["vdw"] - E0["exclusion"] + E0["exception"])) \
            <= etol * scale + 1e-6
        eng.close()


def test_batched_uneven_systems_match_per_system_oracle(oracle):
    """Several independent systems of uneven size (lambda-scaled chain
    charges, own boxes and PME grids) in one context: each system's forces,
    energies and pair set equal the oracle's for that system alone."""
    systems = [sy.with_exceptions(x) for x in sy.batch_systems(count=4, seed=77, lo=2000, hi=6000)]
    sizes = [x.n for x in systems]
    assert len(set(sizes)) == len(sizes)
    for prec, tol in ((0, 1e-9), (1, 1e-5)):
        eng = _engine(systems, precision=prec, skin=0.1, rebuild_interval=10, box="explicit", exceptions=True)
        F = eng.compute_forces()
        off = 0
        for k, s in enumerate(systems):
            lb, ub = np.zeros(3), s.box.copy()
            box = oracle.box_explicit(lb, ub)
            eo, el = oracle.exclusions(s.n, s.bonds)
            eo, el = oracle.union_exclusions(eo, el, s.exc_idx)
            d = oracle.describe(s, box_mode=1, lb=lb, ub=ub, exceptions=(s.exc_idx, s.exc_prm))
            F0, E0 = oracle.forces(d, s.pos, box, eo, el)
            assert rel_rms(F[off:off + s.n], F0) <= tol, (prec, k, rel_rms(F[off:off + s.n], F0))
            E = eng.energies(k)
            scale = max(abs(E0[t]) for t in TERMS)
            etol = 1e-9 if prec == 0 else 2e-5
            for t in TERMS + ("exception",):
                assert abs(E[t] - E0[t]) <= etol * scale + 1e-6, (prec, k, t, E[t], E0[t])
            if prec == 1:
                ref = oracle.neighbor_pairs(s.pos, box, eo, el, s.cutoff)
                ref = ref[np.lexsort((ref[:, 1], ref[:, 0]))]
                assert np.array_equal(eng.pairs(k), ref)
            off += s.n
        eng.close()


def test_batch_with_per_system_force_masks_matches_oracle(oracle):
    """Systems of one batch with different force masks: each kind's terms
    are taken in for the systems whose mask has it (the bonds of every
    system still define its exclusions), so the per-system term offsets
    have empty ranges between full ones; each system's FP64 forces and
    energies equal the oracle's with that system's mask."""
    systems = [sy.with_exceptions(x) for x in sy.batch_systems(count=4, seed=91, lo=2000, hi=5000)]
    masks = [15, 8, 13, 3]  # all; nonbonded only; no angles; bonds + angles only
    eng = _engine(systems, precision=0, skin=0.1, rebuild_interval=10, box="explicit", exceptions=True,
                  force_mask=masks)
    F = eng.compute_forces()
    off = 0
    for k, (s, m) in enumerate(zip(systems, masks)):
        lb, ub = np.zeros(3), s.box.copy()
        box = oracle.box_explicit(lb, ub)
        eo, el = oracle.exclusions(s.n, s.bonds)
        xc = (s.exc_idx, s.exc_prm) if m & 8 else None
        if xc is not None:
            eo, el = oracle.union_exclusions(eo, el, s.exc_idx)
        d = oracle.describe(s, force_mask=m, box_mode=1, lb=lb, ub=ub, exceptions=xc)
        F0, E0 = oracle.forces(d, s.pos, box, eo, el)
        assert rel_rms(F[off:off + s.n], F0) <= 1e-9, (k, m, rel_rms(F[off:off + s.n], F0))
        E = eng.energies(k)
        scale = max(abs(E0[t]) for t in TERMS) or 1.0
        for t in TERMS:
            assert abs(E[t] - E0[t]) <= 1e-9 * scale + 1e-6, (k, m, t, E[t], E0[t])
        off += s.n
    eng.close()


def test_contexts_of_different_sizes_coexist():
    """Per-kernel launch limits are process-wide: a context created after a
    larger one must not make the larger one's launches fail."""
    big = sy.with_exceptions(sy.config_system(2))
    small = sy.with_exceptions(sy.config_system(1))
    e1 = _engine(big, precision=1, skin=0.1, rebuild_interval=10, box="explicit", exceptions=True)
    F1 = e1.compute_forces()
    e2 = _engine(small, precision=1, skin=0.1, rebuild_interval=10, box="explicit", exceptions=True, grid=(16, 16, 16))
    e2.compute_forces()
    F1b = e1.compute_forces()
    assert np.array_equal(F1, F1b)
    e1.close()
    e2.close()


def test_exceptions_bit_reproducible():
    s = sy.with_exceptions(sy.config_system(1))
    outs = []
    for _ in range(2):
        eng = _engine(s, precision=1, skin=0.1, rebuild_interval=10, box="explicit", exceptions=True)
        eng.step(5, 0.0005)
        outs.append(eng.forces())
        eng.close()
    assert np.array_equal(outs[0], outs[1])
