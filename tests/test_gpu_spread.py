"""The mixed engine's PME charge grid against the oracle's spread (GPU required).

The mixed engine sums the charge grid as int32 fixed point (units of 2^-24 e;
FP32 B-spline weights, k_spread_warp).  The grid after a force evaluation
(nxm_get_pme_grids) is compared with the oracle's FP64 spread of the same
positions (gridSpreadCharge_Reference, NonbondedForce.cpp:220-260):

* config 1 (3.0 nm box, 32^3) and config 3 (9.8 nm box, 100^3);
* a config-5-shaped box (6.72 nm, 180^3: radix 10 x 9 x 2 axes);
* config 1 with a 0.5 nm skin, 300 steps after the list build: cell-relative
  offsets that have drifted far past their cells (the grid coordinate is the
  cell corner's plus the offset, so drift must not matter).

Tolerance: each point within 4e-6 e of the oracle (FP32 weights, 2^-25
rounding per contribution) and grid rel-RMS <= 1e-5.
"""
import numpy as np
import pytest

from nexusmd_gb300 import synthetic as sy

pytestmark = pytest.mark.gpu


def _charge_grid_check(oracle, eng, s, pos, evaluate=True):
    if evaluate:
        eng.compute_forces()
    q, _, _ = eng.pme_grids()
    lb, ub = np.zeros(3), s.box.copy()
    ref = oracle.spread(pos, s.charge, oracle.box_explicit(lb, ub), list(q.shape))[..., 0]
    err = np.abs(q - ref)
    rel = float(np.sqrt((err ** 2).sum() / (ref ** 2).sum()))
    print("grid", q.shape, "max abs", err.max(), "rel-RMS", rel, "charge sum", q.sum(), ref.sum())
    assert err.max() <= 4e-6, err.max()
    assert rel <= 1e-5, rel


def _engine(s, **kw):
    from nexusmd_gb300.engine import Engine
    return Engine(s, precision=1, box="explicit", **kw)


@pytest.mark.parametrize("cfg", [1, 3])
def test_charge_grid_matches_oracle(oracle, cfg):
    s = sy.config_system(cfg)
    eng = _engine(s, skin=0.1, rebuild_interval=10)
    _charge_grid_check(oracle, eng, s, s.pos)
    eng.close()


def test_charge_grid_direct_route(oracle):
    s = sy.make_system(1, 300, 9300, 6.72, 1105, cutoff=1.2, ewald_tol=1e-5, grid=(180, 180, 180))
    eng = _engine(s, skin=0.1, rebuild_interval=10)
    _charge_grid_check(oracle, eng, s, s.pos)
    eng.close()


def test_charge_grid_after_drift(oracle):
    s = sy.config_system(1)
    eng = _engine(s, skin=0.5, rebuild_interval=100000)
    eng.set_velocities(sy.maxwell_boltzmann(s.mass, 300.0, seed=7))
    eng.step(299, 0.0005)
    pos, _ = eng.state()
    # the next step's forces are evaluated at these positions, from the
    # cells of the last rebuild (compute_forces would rebuild first)
    eng.step(1, 0.0005)
    print("list rebuilds", eng.rebuilds())
    _charge_grid_check(oracle, eng, s, pos, evaluate=False)
    eng.close()
