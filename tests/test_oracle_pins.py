"""The C oracle pinned to the reference (CPU only).

Two anchors: (1) the committed golden fixtures in tests/golden/, made by
tests/golden/make_golden.py from the reference compiled from its own sources
(oracle/_ref); (2) where the reference tree is present, the compiled
reference itself, phase by phase, on freshly generated systems.
"""
import hashlib
import os

import numpy as np
import pytest

from nexusmd_gb300 import synthetic as sy

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _load(name):
    z = np.load(os.path.join(GOLD, name + ".npz"))
    return {k: z[k] for k in z.files}


def _sys_from_golden(g):
    return sy.System(pos=g["pos"], mass=g["mass"], charge=g["q"], sigma=g["sig"], epsilon=g["eps"],
                     bonds=g["bonds"], bond_prm=g["bond_prm"], angles=g["angles"],
                     angle_prm=g["angle_prm"], torsions=g["torsions"], torsion_prm=g["torsion_prm"],
                     torsion_n=g["torsion_n"], box=np.ones(3), cutoff=float(g["cutoff"]),
                     ewald_tol=float(g["tol"]), grid=tuple(int(x) for x in g["grid"]))


GOLDEN_CASES = sorted(f[:-4] for f in os.listdir(GOLD) if f.endswith(".npz")) if os.path.isdir(GOLD) else []


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_oracle_matches_golden(oracle, case):
    g = _load(case)
    s = _sys_from_golden(g)
    box = oracle.box_from_positions(s.pos)
    assert np.array_equal(box.as9(), g["box9"])
    eoff, el = oracle.exclusions(s.n, s.bonds)
    assert np.array_equal(eoff, g["excl_off"]) and np.array_equal(el, g["excl_lst"])
    pairs = oracle.neighbor_pairs(s.pos, box, eoff, el, s.cutoff)
    assert len(pairs) == int(g["n_pairs"])
    digest = hashlib.sha256(np.ascontiguousarray(pairs, np.int32).tobytes()).digest()
    assert digest == g["pairs_sha256"].tobytes()
    for kind in ("bonds", "angles"):
        prm = g["bond_prm"] if kind == "bonds" else g["angle_prm"]
        E, F = getattr(oracle, kind)(s.pos, getattr(s, kind), prm, box)
        assert np.allclose(F, g["F_" + kind], rtol=0, atol=1e-12 * max(1, np.abs(g["F_" + kind]).max()))
        assert abs(E - float(g["E_" + kind])) <= 1e-12 * max(1, abs(float(g["E_" + kind])))
    E, F = oracle.torsions(s.pos, s.torsions, s.torsion_prm, s.torsion_n, box)
    assert np.allclose(F, g["F_torsions"], rtol=0, atol=1e-12 * max(1, np.abs(g["F_torsions"]).max()))
    d = oracle.describe(s, force_mask=8, grid=tuple(int(x) for x in g["grid"]))
    F, En = oracle.forces(d, s.pos, box, eoff, el)
    scale = np.abs(g["F_nonbonded"]).max()
    assert np.allclose(F, g["F_nonbonded"], rtol=0, atol=1e-11 * scale)
    ref = g["E_nonbonded"]  # recip, self, direct, -exclusion (reference accumulators)
    got = [En["recip"], En["self"], En["coulomb"] + En["vdw"], -En["exclusion"]]
    for a, b in zip(got, ref):
        assert abs(a - b) <= 1e-10 * max(1.0, abs(b))
    # leapfrog + kinetic energy of one step
    p1, v1 = oracle.leapfrog(s.pos, g["v0"], g["F_total"], s.mass, 0.0005, box)
    assert np.array_equal(p1, g["pos1"]) and np.array_equal(v1, g["vel1"])
    ke = oracle.kinetic(g["v0"], s.mass, g["F_total"], 0.0005)
    assert ke == float(g["ke"])


def test_fft_against_numpy(oracle):
    rng = np.random.default_rng(3)
    for shape in [(8, 12, 10), (32, 32, 32), (6, 25, 18), (16, 9, 30)]:
        a = rng.normal(size=shape) + 1j * rng.normal(size=shape)
        f = oracle.fft3d(a, -1)
        assert np.abs(f - np.fft.fftn(a)).max() < 1e-11 * np.abs(f).max()
        b = oracle.fft3d(a, +1)
        assert np.abs(b - np.fft.ifftn(a) * a.size).max() < 1e-11 * np.abs(b).max()


def test_exclusion_depth_semantics(oracle):
    # chain 0-1-2-3-4-5 plus a branch 2-6: partners within 3 bonds
    bonds = np.array([[0, 1], [1, 2], [2, 3], [3, 4], [4, 5], [2, 6]], np.int32)
    off, lst = oracle.exclusions(7, bonds, depth=3)
    got = {i: set(lst[off[i]:off[i + 1]].tolist()) for i in range(7)}
    assert got[0] == {1, 2, 3, 6}
    assert got[5] == {2, 3, 4}
    assert got[6] == {0, 1, 2, 3, 4}
    with pytest.raises(ValueError):
        oracle.exclusions(3, np.array([[0, 5]], np.int32))


def test_oracle_vs_reference_live(oracle, reference):
    """Phase-by-phase equality with the compiled reference on a fresh system."""
    s = sy.compat_system(sy.make_system(1, 12, 200, 2.3, seed=4242, grid=(0, 0, 0)))
    box = oracle.box_from_positions(s.pos)
    b9 = reference.box(s.pos)
    assert np.array_equal(box.as9(), b9)
    eoff, el = oracle.exclusions(s.n, s.bonds)
    roff, rl = reference.exclusions(s.n, s.bonds)
    assert np.array_equal(eoff, roff) and np.array_equal(el, rl)
    assert np.array_equal(oracle.neighbor_pairs(s.pos, box, eoff, el, s.cutoff),
                          reference.neighbor_pairs(s.pos, b9, eoff, el, s.cutoff))
    for kind, prm in (("bonds", s.bond_prm), ("angles", s.angle_prm)):
        Eo, Fo = getattr(oracle, kind)(s.pos, getattr(s, kind), prm, box)
        Er, Fr = getattr(reference, kind)(s.pos, getattr(s, kind), prm, b9)
        assert Eo == Er and np.array_equal(Fo, Fr)
    Eo, Fo = oracle.torsions(s.pos, s.torsions, s.torsion_prm, s.torsion_n, box)
    Er, Fr = reference.torsions(s.pos, s.torsions, s.torsion_prm, s.torsion_n, b9)
    assert Eo == Er and np.array_equal(Fo, Fr)
    for grid in [(0, 0, 0), (24, 25, 27)]:
        Fr, Er = reference.nonbonded(s, s.pos, b9, eoff, el, grid=grid)
        Fo, Eo = oracle.forces(oracle.describe(s, force_mask=8, grid=grid), s.pos, box, eoff, el)
        assert np.array_equal(Fo, Fr)
        assert Eo["recip"] == Er["recip"] and Eo["self"] == Er["self"]
        assert Eo["coulomb"] + Eo["vdw"] == Er["direct"]
        assert -Eo["exclusion"] == Er["exclusion_signed"]
    v = np.random.default_rng(1).normal(size=s.pos.shape)
    F = np.random.default_rng(2).normal(size=s.pos.shape) * 100
    po, vo = oracle.leapfrog(s.pos, v, F, s.mass, 0.0005, box)
    pr, vr = reference.leapfrog(s.pos, v, F, s.mass, 0.0005, b9)
    assert np.array_equal(po, pr) and np.array_equal(vo, vr)
    assert oracle.kinetic(v, s.mass, F, 0.0005) == reference.kinetic(v, s.mass, F, 0.0005)
