"""Pipelined stepping (nxm_step_async / nxm_frame_wait) against the
synchronous calls (GPU required).

The pipelined loop double-buffers each frame on the device and copies it to
pinned host memory on a second stream while the next step runs; the frames
must be the ones the synchronous loop (nxm_step(1) + nxm_get_positions +
nxm_get_energies) reads, bit for bit: the same steps in the same order, the
mixed engine being deterministic.  The reference's loop is
Engine::RunSimulation with Report every step (Engine.cpp:162-188).
"""
import numpy as np
import pytest

from nexusmd_gb300 import synthetic as sy

pytestmark = pytest.mark.gpu

DT = 0.0005
KW = dict(precision=1, skin=0.1, rebuild_interval=10, box="explicit", exceptions=True)


@pytest.fixture(scope="module")
def system():
    s = sy.with_exceptions(sy.config_system(1))
    return s, sy.maxwell_boltzmann(s.mass, 300.0, seed=5)


def test_pipelined_frames_match_synchronous_steps(system):
    from nexusmd_gb300.engine import Engine
    s, v0 = system
    steps = 25  # crosses the 10-step rebuild interval twice
    a = Engine(s, **KW)
    a.set_velocities(v0)
    ref = []
    for _ in range(steps):
        a.step(1, DT)
        ref.append((a.snapshot_positions(), a.energies()))
    a.close()
    b = Engine(s, **KW)
    b.set_velocities(v0)
    got = []
    b.step_async(1, DT)
    for _ in range(steps - 1):
        b.step_async(1, DT)
        got.append(b.frame_wait())
    got.append(b.frame_wait())
    for k, ((xa, ea), (xb, eb)) in enumerate(zip(ref, got)):
        assert np.array_equal(xa, xb), k
        for t in ("kinetic", "potential", "coulomb", "vdw", "recip", "bond", "exception"):
            assert ea[t] == eb[t], (k, t, ea[t], eb[t])
    # synchronous calls still work after pipelined ones, from the same state
    b.step(1, DT)
    assert np.isfinite(b.snapshot_positions()).all()
    b.close()


def test_frame_ring_full_is_refused(system):
    from nexusmd_gb300.engine import Engine, NxmError
    s, v0 = system
    e = Engine(s, **KW)
    e.set_velocities(v0)
    e.step_async(1, DT)
    e.step_async(1, DT)  # the default ring holds two frames
    with pytest.raises(NxmError, match="ring full"):
        e.step_async(1, DT)
    e.frame_wait()
    e.frame_wait()
    with pytest.raises(NxmError, match="no frame pending"):
        e.frame_wait()
    e.close()
