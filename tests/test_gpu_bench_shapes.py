"""CUDA engine vs the FP64 oracle at the benchmarked shapes (GPU required).

The configurations the bench times, each compared with the oracle on the
same positions, in the physics mode the bench runs (1-2/1-3 exclusions, 1-4
pairs as exceptions scaled 0.8333/0.5, explicit periodic box):

* config 2 in full: 23,800 atoms, 6.2 nm box, PME 64^3, rc 1.0 nm;
* a config-5-shaped system: config 5's density, composition, cutoff
  (1.2 nm), Ewald tolerance (1e-5) and PME grid (180^3, FFT passes of
  radix 10, 9 and 2) in a 6.72 nm box, which gives config 5's cell edge
  (0.672 nm) and so its tile shape (one-cell neighbourhoods too dense for
  two blocks per SM: one 32-warp block per SM, groups of 4 cells); both FFT
  launch shapes, the plane path in chunks of lines as at 180^3;
* config 4 in full: all 32 uneven lambda-window systems in one context.

Each checks the neighbour pair set (array-equal to the oracle's, which is
the reference's voxel list, NeighborList.cpp:129-154), the forces and every
energy term.  Tolerances as in test_gpu_parity.py: FP64 1e-9 relative; mixed
force rel-RMS <= 1e-5 and each energy term within 2e-5 of the largest term.
"""
import numpy as np
import pytest

from nexusmd_gb300 import synthetic as sy

pytestmark = pytest.mark.gpu

TERMS = ("bond", "angle", "torsion", "recip", "self", "coulomb", "vdw", "exclusion", "exception")


def _engine(s, **kw):
    from nexusmd_gb300.engine import Engine
    return Engine(s, skin=0.1, rebuild_interval=10, box="explicit", exceptions=True, **kw)


def _oracle(oracle, s):
    """Forces, energies and sorted pair set of one physics-mode system."""
    lb, ub = np.zeros(3), s.box.copy()
    box = oracle.box_explicit(lb, ub)
    off, lst = oracle.exclusions(s.n, s.bonds)
    off, lst = oracle.union_exclusions(off, lst, s.exc_idx)
    d = oracle.describe(s, box_mode=1, lb=lb, ub=ub, exceptions=(s.exc_idx, s.exc_prm))
    F0, E0 = oracle.forces(d, s.pos, box, off, lst)
    ref = oracle.neighbor_pairs(s.pos, box, off, lst, s.cutoff)
    return F0, E0, ref[np.lexsort((ref[:, 1], ref[:, 0]))]


def rel_rms(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


def _check(F, E, F0, E0, prec, what):
    tol = 1e-9 if prec == 0 else 1e-5
    err = rel_rms(F, F0)
    print("%s precision %d: force rel-RMS %.3e, max atom %.3e" % (what, prec, err,
                                                                   np.sqrt(((F - F0) ** 2).sum(1)).max()))
    assert err <= tol, (what, prec, err)
    scale = max(abs(E0[k]) for k in TERMS)
    etol = 1e-9 if prec == 0 else 2e-5
    for k in TERMS:
        assert abs(E[k] - E0[k]) <= etol * scale + 1e-6, (what, prec, k, E[k], E0[k])


@pytest.fixture(scope="module")
def c2():
    return sy.with_exceptions(sy.config_system(2))


@pytest.mark.parametrize("prec", [0, 1])
def test_config2_full(oracle, c2, prec):
    s = c2
    F0, E0, ref = _oracle(oracle, s)
    eng = _engine(s, precision=prec)
    F = eng.compute_forces()
    _check(F, eng.energies(), F0, E0, prec, "config 2")
    got = eng.pairs()
    assert got.shape == ref.shape and np.array_equal(got, ref)
    eng.close()


def config5_shaped():
    """Config 5's recipe (8% chain particles, flexible water, ~100 atoms/nm^3,
    rc 1.2 nm, tol 1e-5, grid 180^3) in a 6.72 nm box: 30,300 atoms."""
    return sy.with_exceptions(sy.make_system(1, 300, 9300, 6.72, 1105, cutoff=1.2, ewald_tol=1e-5,
                                             grid=(180, 180, 180)))


@pytest.fixture(scope="module")
def c5s():
    return config5_shaped()


@pytest.mark.parametrize("prec,fft_path", [(1, 1), (1, 2), (0, 1)])
def test_config5_shape(oracle, c5s, prec, fft_path):
    s = c5s
    F0, E0, ref = _oracle(oracle, s)
    eng = _engine(s, precision=prec, fft_path=fft_path)
    lay = eng.layout()
    # config 5's list and FFT geometry: 0.672 nm cells whose one-cell
    # neighbourhoods need one tile block per SM, groups of 4 cells (10 cells
    # as 4 + 4 + 2), 180 = 10 x 9 x 2 per axis, and on the plane path
    # x-planes larger than the shared-memory scratch
    assert lay["cells_per_group"] == 4 and lay["hood_capacity"] > 4400, lay
    assert lay["cells_x"] == lay["cells_y"] == lay["cells_z"] == 10, lay
    assert lay["fft_radices"] == ((10, 9, 2),) * 3, lay
    assert lay["fft_path"] == fft_path, lay
    if fft_path == 2:
        assert lay["fft_plane_chunked"] == 1, lay
    F = eng.compute_forces()
    _check(F, eng.energies(), F0, E0, prec, "config-5 shape fft_path %d" % fft_path)
    got = eng.pairs()
    assert got.shape == ref.shape and np.array_equal(got, ref)
    eng.close()


@pytest.fixture(scope="module")
def c4(oracle):
    systems = [sy.with_exceptions(x) for x in sy.batch_systems()]
    return systems, [_oracle(oracle, s) for s in systems]


@pytest.mark.parametrize("prec", [1, 0])
def test_config4_all_32_systems(c4, prec):
    systems, refs = c4
    assert len(systems) == 32
    eng = _engine(systems, precision=prec)
    F = eng.compute_forces()
    off = 0
    for k, s in enumerate(systems):
        F0, E0, ref = refs[k]
        _check(F[off:off + s.n], eng.energies(k), F0, E0, prec, "config 4 system %d (%d atoms)" % (k, s.n))
        got = eng.pairs(k)
        assert got.shape == ref.shape and np.array_equal(got, ref), k
        off += s.n
    eng.close()
