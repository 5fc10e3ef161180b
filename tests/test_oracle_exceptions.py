"""The oracle's exception term (OpenMM NonbondedForce semantics).

The reference parses <Exceptions> (core/common/src/SystemXMLParser.cpp:182-191)
but never applies them, so there is no reference output to pin against: the
C restatement is checked against an independent numpy evaluation of the
same formula, and its bookkeeping (union with the bonded exclusions, energy
total) against the reference-pinned terms it is built from.
"""
import numpy as np

from nexusmd_gb300 import synthetic as sy

KE = 138.93545764446428693393


def _numpy_exceptions(s):
    i, j = s.exc_idx[:, 0], s.exc_idx[:, 1]
    d = s.pos[i] - s.pos[j]
    d -= s.box * np.round(d / s.box)
    r = np.linalg.norm(d, axis=1)
    qq, sg, ep = s.exc_prm.T
    e = KE * qq / r + 4 * ep * ((sg / r) ** 12 - (sg / r) ** 6)
    dEdR = (KE * qq / r + 4 * ep * (12 * (sg / r) ** 12 - 6 * (sg / r) ** 6)) / r ** 2
    F = np.zeros_like(s.pos)
    np.add.at(F, i, d * dEdR[:, None])
    np.add.at(F, j, -d * dEdR[:, None])
    return e.sum(), F


def test_exception_term_matches_numpy(oracle):
    s = sy.with_exceptions(sy.config_system(1))
    assert len(s.exc_idx) > 400
    box = oracle.box_explicit(np.zeros(3), s.box)
    E, F = oracle.exceptions(s.pos, s.exc_idx, s.exc_prm, box)
    E2, F2 = _numpy_exceptions(s)
    assert abs(E - E2) <= 1e-12 * abs(E2)
    assert np.abs(F - F2).max() <= 1e-9 * np.abs(F2).max()


def test_exception_parameters_follow_openmm_scaling():
    s = sy.with_exceptions(sy.config_system(1))
    i, j = s.exc_idx[:, 0], s.exc_idx[:, 1]
    assert np.allclose(s.exc_prm[:, 0], sy.COULOMB14 * s.charge[i] * s.charge[j])
    assert np.allclose(s.exc_prm[:, 1], 0.5 * (s.sigma[i] + s.sigma[j]))
    assert np.allclose(s.exc_prm[:, 2], sy.LJ14 * np.sqrt(s.epsilon[i] * s.epsilon[j]))
    # exactly the torsion end pairs, each once
    ends = {tuple(sorted(t)) for t in s.torsions[:, [0, 3]].tolist()}
    assert {tuple(p) for p in s.exc_idx.tolist()} == ends


def test_physics_mode_total_is_compat_plus_exceptions(oracle):
    """Depth-3 exclusions already hold every 1-4 pair, so the exception
    term adds to the reference-pinned terms and changes nothing else."""
    s = sy.with_exceptions(sy.config_system(1))
    lb, ub = np.zeros(3), s.box.copy()
    box = oracle.box_explicit(lb, ub)
    off, lst = oracle.exclusions(s.n, s.bonds)
    off2, lst2 = oracle.union_exclusions(off, lst, s.exc_idx)
    assert np.array_equal(off, off2) and np.array_equal(lst, lst2)
    F0, E0 = oracle.forces(oracle.describe(s, box_mode=1, lb=lb, ub=ub), s.pos, box, off, lst)
    d = oracle.describe(s, box_mode=1, lb=lb, ub=ub, exceptions=(s.exc_idx, s.exc_prm))
    F1, E1 = oracle.forces(d, s.pos, box, off2, lst2)
    Ex, Fx = oracle.exceptions(s.pos, s.exc_idx, s.exc_prm, box)
    assert E1["exception"] == Ex and E0["exception"] == 0.0
    for k in ("recip", "self", "coulomb", "vdw", "exclusion"):
        assert E1[k] == E0[k]
    assert abs(E1["reported_pe"] - (E0["reported_pe"] + Ex)) <= 1e-9 * abs(E0["reported_pe"])
    assert np.allclose(F1, F0 + Fx, rtol=0, atol=1e-9 * np.abs(F0).max())


def test_union_adds_exception_pairs_outside_the_bond_depth(oracle):
    s = sy.with_exceptions(sy.config_system(1))
    off, lst = oracle.exclusions(s.n, s.bonds, depth=2)
    off2, lst2 = oracle.union_exclusions(off, lst, s.exc_idx)
    assert len(lst2) == len(lst) + 2 * len(s.exc_idx)
    for a, b in s.exc_idx[:50]:
        assert b in lst2[off2[a]:off2[a + 1]] and a in lst2[off2[b]:off2[b + 1]]
        seg = lst2[off2[a]:off2[a + 1]]
        assert np.all(np.diff(seg) > 0)
