"""TaskDispatcher.Simulate through the C ABI vs the reference's own Simulate.

tests/golden/simulate_small holds the inputs and the three report files the
reference wrote for them (made by tests/golden/make_golden.py).  The FP64
engine must reproduce every line: formats byte-for-byte (headers, widths,
record layout, model numbering), numbers to round-off.
"""
import gzip
import os
import re

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "simulate_small")
NUM = re.compile(r"-?\d+\.\d+(?:e[+-]\d+)?|-?\d+(?:e[+-]\d+)?")


def _gold(name):
    with gzip.open(os.path.join(GOLD, name + ".gz"), "rt") as f:
        return f.read().splitlines()


def _lines_match(got, ref, rtol, atol):
    """Same text, or the same text with numbers equal within tolerance."""
    if got == ref:
        return True
    if NUM.sub("#", got) != NUM.sub("#", ref):
        return False
    a = [float(x) for x in NUM.findall(got)]
    b = [float(x) for x in NUM.findall(ref)]
    return len(a) == len(b) and np.allclose(a, b, rtol=rtol, atol=atol)


def _run(tmp_path, precision, steps, interval, idx, state=None, **opts):
    import NexusMD
    d = NexusMD.TaskDispatcher.CreateDispatcher("GPU")
    d.EnableHarmonicBondForce()
    d.EnableHarmonicAngleForce()
    d.EnablePeriodicTorsionForce()
    d.EnableNonbondedForce()
    d.SetOptions(precision=precision, skin=0.1, rebuild_interval=10, **opts)
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        out = "out%d.pdb" % idx
        d.Simulate(os.path.join(GOLD, "system_small.xml"), state or os.path.join(GOLD, "state_small.xml"),
                   os.path.join(GOLD, "small.pdb"), out, 0.0005, steps, interval)
        return {f: open(os.path.join(tmp_path, f)).read().splitlines()
                for f in (out, "PVFReport" + out, "TotalEnergy" + out)}
    finally:
        os.chdir(cwd)


@pytest.mark.parametrize("steps,interval,idx", [(10, 1, 0), (7, 3, 1)])
def test_simulate_fp64_matches_reference_files(tmp_path, steps, interval, idx):
    got = _run(tmp_path, "fp64", steps, interval, idx)
    for name, lines in got.items():
        ref = _gold(name)
        assert len(lines) == len(ref), name
        for k, (a, b) in enumerate(zip(lines, ref)):
            if a.startswith("REMARK   Generated by"):
                assert b.startswith("REMARK   Generated by")
                continue
            # positions/velocities to 1e-9, forces and energies to 1e-8 relative
            assert _lines_match(a, b, rtol=1e-8, atol=2e-9), (name, k, a, b)


def test_simulate_mixed_precision_tracks_reference(tmp_path):
    got = _run(tmp_path, "mixed", 10, 1, 0)
    ref = _gold("TotalEnergyout0.pdb")
    te = got["TotalEnergyout0.pdb"]
    assert te[0] == ref[0] and len(te) == len(ref)
    a = np.array([[float(x) for x in l.split()] for l in te[1:]])
    b = np.array([[float(x) for x in l.split()] for l in ref[1:]])
    assert np.allclose(a[:, 1:], b[:, 1:], rtol=2e-4, atol=0.05)
    pvf, rpvf = got["PVFReportout0.pdb"], _gold("PVFReportout0.pdb")
    assert len(pvf) == len(rpvf)
    assert all(NUM.sub("#", x) == NUM.sub("#", y) for x, y in zip(pvf, rpvf))


def test_simulate_applies_xml_exceptions_on_request(tmp_path, oracle):
    """SetOptions(exceptions=True): the system XML's <Exceptions> (scaled
    1-4 pairs) enter the run; the step-0 potential in TotalEnergy equals the
    oracle's in the same mode, and without the option the file is the
    reference's (exceptions ignored)."""
    import NexusMD
    from nexusmd_gb300 import synthetic as sy
    s = sy.with_exceptions(sy.compat_system(sy.make_system(1, 4, 100, 2.8, seed=21)))
    sp, st, pdb = sy.write_inputs(s, str(tmp_path), "exc")
    pe = {}
    for use in (False, True):
        d = NexusMD.TaskDispatcher.CreateDispatcher("GPU")
        d.EnableHarmonicBondForce()
        d.EnableHarmonicAngleForce()
        d.EnablePeriodicTorsionForce()
        d.EnableNonbondedForce()
        d.SetOptions(precision="fp64", exceptions=use)
        cwd = os.getcwd()
        os.chdir(tmp_path)
        try:
            d.Simulate(sp, st, pdb, "o%d.pdb" % use, 0.0005, 1, 1)
            line = open(os.path.join(tmp_path, "TotalEnergyo%d.pdb" % use)).read().splitlines()[1]
        finally:
            os.chdir(cwd)
        pe[use] = float(line.split()[2])
    box = oracle.box_from_positions(s.pos)
    off, lst = oracle.exclusions(s.n, s.bonds)
    off, lst = oracle.union_exclusions(off, lst, s.exc_idx)
    ref_off = oracle.describe(s)
    _, E0 = oracle.forces(ref_off, s.pos, box, off, lst)
    _, E1 = oracle.forces(oracle.describe(s, exceptions=(s.exc_idx, s.exc_prm)), s.pos, box, off, lst)
    assert E1["exception"] != 0.0
    assert abs(pe[False] - E0["reported_pe"]) <= 1e-8 * abs(E0["reported_pe"]) + 1e-6
    assert abs(pe[True] - E1["reported_pe"]) <= 1e-8 * abs(E1["reported_pe"]) + 1e-6


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_async_reporter_writes_the_synchronous_files(tmp_path, precision):
    """report_threads > 0 (pinned double-buffered snapshot copies, files
    written on a host thread while the GPU steps on) gives the same bytes as
    writing each report before the next step.  The mixed engine is
    bit-reproducible (fixed-point force sums), so its files must be equal
    byte for byte; the FP64 engine sums forces with floating-point atomics,
    whose order varies between runs (the reciprocal energy's charge grid
    included), so there the numbers agree to ~1e-11 relative, not bit for
    bit."""
    sync = _run(tmp_path, precision, 23, 2, 0, report_threads=0)
    asyn = _run(tmp_path, precision, 23, 2, 1, report_threads=3)
    for name, lines in sync.items():
        other = asyn[name.replace("out0", "out1")]
        assert len(other) == len(lines), name
        for a, b in zip(lines, other):
            if a.startswith("REMARK   Generated by"):
                continue
            if precision == "mixed":
                assert a == b, (name, a, b)
            else:
                assert _lines_match(a, b, rtol=1e-9, atol=2e-10), (name, a, b)


def test_simulate_starts_from_state_velocities_on_request(tmp_path):
    """state_velocities=True takes v0 from the state file's <Velocities>: the
    step-0 PVF velocity column is those velocities (10 decimals); without the
    option it is zero, as the reference."""
    import NexusMD
    src = os.path.join(GOLD, "state_small.xml")
    pos = NexusMD.StateXMLParser.parseStateXML(src)
    rng = np.random.default_rng(11)
    vel = rng.normal(0.0, 0.5, (len(pos), 3))
    st = str(tmp_path / "state_v.xml")
    NexusMD.StateXMLParser.writeStateXML(st, pos, [tuple(r) for r in vel])
    for use, idx in ((True, 0), (False, 1)):
        got = _run(tmp_path, "fp64", 1, 1, idx, state=st, state_velocities=use)
        rows = got["PVFReportout%d.pdb" % idx][2:2 + len(pos)]
        v = np.array([[float(x) for x in NUM.findall(r.split("\t")[2])] for r in rows])
        assert np.allclose(v, vel if use else 0.0, rtol=0, atol=6e-11)


def test_checkpoint_round_trip_through_engine(tmp_path):
    """Engine.save_state writes the context's current positions and
    velocities; reading the file back gives the same doubles."""
    import NexusMD
    from nexusmd_gb300 import synthetic as sy
    from nexusmd_gb300.engine import Engine
    s = sy.compat_system(sy.make_system(1, 4, 120, 2.9, seed=31))
    e = Engine(s)
    e.set_velocities(sy.maxwell_boltzmann(np.asarray(s.mass), 300.0, seed=2))
    e.step(37, 0.0005)
    x, v = e.state()
    path = str(tmp_path / "ck.xml")
    e.save_state(path, step=37, time=37 * 0.0005)
    px = np.array([p.data for p in NexusMD.StateXMLParser.parseStateXML(path)])
    pv = np.array([p.data for p in NexusMD.StateXMLParser.parseStateVelocities(path)])
    assert np.array_equal(px, x) and np.array_equal(pv, v)
