"""The C ABI library and the host-side parsers, without a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from nexusmd_gb300 import synthetic as sy

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in ("include/nxm.h",):
        txt = open(os.path.join(ROOT, h)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names |= set(re.findall(r"\b(nxm_[a-z0-9_]+)\s*\(", txt))
    return names


def test_library_exports_every_declared_symbol():
    from nexusmd_gb300.engine import load_library
    L = load_library()
    missing = [n for n in sorted(declared_symbols()) if not hasattr(L, n)]
    assert not missing, missing
    assert b"sm_103a" in L.nxm_version()


def test_create_without_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from nexusmd_gb300.engine import Engine, NxmError
    s = sy.make_system(1, 2, 20, 2.2, seed=1)
    with pytest.raises(NxmError, match="no CUDA device"):
        Engine(s)


def test_parsers_round_trip(tmp_path):
    import NexusMD
    s = sy.make_system(1, 5, 30, 2.3, seed=9)
    sp, st, pdb = sy.write_inputs(s, str(tmp_path), "t")
    assert NexusMD.SystemXMLParser.MassesParser(sp) == list(s.mass)
    b = NexusMD.SystemXMLParser.HBondParser(sp)
    assert [(x.p1, x.p2, x.d, x.k) for x in b] == [(int(i), int(j), d, k) for (i, j), (d, k) in zip(s.bonds, s.bond_prm)]
    a = NexusMD.SystemXMLParser.HAngleParser(sp)
    assert [(x.p1, x.p2, x.p3, x.a, x.k) for x in a] == [
        (int(i), int(j), int(k), th, kk) for (i, j, k), (th, kk) in zip(s.angles, s.angle_prm)]
    t = NexusMD.SystemXMLParser.PTorsionParser(sp)
    assert [(x.p1, x.p4, x.k, x.phase, x.periodicity) for x in t] == [
        (int(q[0]), int(q[3]), p[0], p[1], int(n)) for q, p, n in zip(s.torsions, s.torsion_prm, s.torsion_n)]
    nb = NexusMD.SystemXMLParser.NonBondedParser(sp)
    assert nb.cutoff == s.cutoff and nb.ewaldTolerance == s.ewald_tol
    assert [(p.q, p.sig, p.eps) for p in nb.particles] == list(zip(s.charge, s.sigma, s.epsilon))
    pos = NexusMD.StateXMLParser.parseStateXML(st)
    assert np.array_equal(np.array([p.data for p in pos]), s.pos)


def test_parser_conventions(tmp_path, capfd):
    """Missing attributes read as 0; an unreadable file prints the reference's
    message and yields empty results (SystemXMLParser.cpp:22-25)."""
    import NexusMD
    p = tmp_path / "s.xml"
    p.write_text('<?xml version="1.0"?>\n<!-- c --><System><Particles><Particle mass="1.5"/><Particle/>'
                 '</Particles><Forces><Force type="HarmonicBondForce"><Bonds><Bond p1="0" p2="1" d="0.1"/>'
                 '</Bonds></Force><Force type="HarmonicBondForce"><Bonds><Bond p1=\'1\' p2="2" k="5"/>'
                 '</Bonds></Force></Forces></System>')
    assert NexusMD.SystemXMLParser.MassesParser(str(p)) == [1.5, 0.0]
    b = NexusMD.SystemXMLParser.HBondParser(str(p))
    assert [(x.p1, x.p2, x.d, x.k) for x in b] == [(0, 1, 0.1, 0.0), (1, 2, 0.0, 5.0)]
    nb = NexusMD.SystemXMLParser.NonBondedParser(str(p))
    assert nb.particles == [] and "No NonbondedForce found in the XML." in capfd.readouterr().err
    bad = tmp_path / "bad.xml"
    bad.write_text("<System><Particles></System>")
    assert NexusMD.SystemXMLParser.MassesParser(str(bad)) == []
    assert "parsed with errors" in capfd.readouterr().err
    assert NexusMD.SystemXMLParser.MassesParser(str(tmp_path / "missing.xml")) == []


def test_dispatcher_factory_messages(capfd):
    import NexusMD
    NexusMD.TaskDispatcher.CreateDispatcher("GPU")
    assert capfd.readouterr().err == ""
    NexusMD.TaskDispatcher.CreateDispatcher("CPU")
    assert "Invalid processor type" in capfd.readouterr().err


def test_state_checkpoint_round_trip(tmp_path):
    """nxm_write_state_xml writes OpenMM's state format with 17 significant
    digits; the reader gives back the same doubles, positions and velocities."""
    import NexusMD
    rng = np.random.default_rng(5)
    n = 257
    x = rng.normal(0, 3.0, (n, 3)) * 10.0 ** rng.integers(-6, 3, (n, 3))
    v = rng.normal(0, 1.0, (n, 3))
    x[0] = [0.0, -0.0, 1e-300]
    v[1] = [np.nextafter(1.0, 2.0), -np.pi, 6.02214076e23]
    path = str(tmp_path / "ckpt.xml")
    NexusMD.StateXMLParser.writeStateXML(path, [tuple(r) for r in x], [tuple(r) for r in v],
                                         box=(3.1, 3.2, 3.3), step=1234, time=0.617)
    px = np.array([p.data for p in NexusMD.StateXMLParser.parseStateXML(path)])
    pv = np.array([p.data for p in NexusMD.StateXMLParser.parseStateVelocities(path)])
    assert np.array_equal(px, x) and np.array_equal(pv, v)
    txt = open(path).read()
    assert '<State stepCount="1234"' in txt and '<A x="3.1000000000000001" y="0" z="0"/>' in txt


def test_state_without_velocities(tmp_path):
    """A state file with positions only (the reference's inputs) has no velocities."""
    import NexusMD
    s = sy.make_system(1, 3, 10, 2.2, seed=4)
    sp, st, pdb = sy.write_inputs(s, str(tmp_path), "nv")
    assert NexusMD.StateXMLParser.parseStateVelocities(st) == []
    path = str(tmp_path / "pos_only.xml")
    NexusMD.StateXMLParser.writeStateXML(path, [tuple(r) for r in s.pos])
    assert "<Velocities>" not in open(path).read()
    assert np.array_equal(np.array([p.data for p in NexusMD.StateXMLParser.parseStateXML(path)]), s.pos)


def _fmt(L, x, prec, width):
    buf = ctypes.create_string_buffer(512)
    n = L.nxm_format_fixed(ctypes.c_double(x), prec, width, buf, 512)
    assert n >= 0
    return buf.value.decode()


def test_report_number_formatter_matches_printf():
    """The PVF / PDB number formatter prints what printf("%*.*f") prints:
    random magnitudes, exact decimal ties (k / 2^11 at 10 decimals), negative
    zero and tiny negatives, subnormals and values past the fast range."""
    from nexusmd_gb300.engine import load_library
    L = load_library()
    L.nxm_format_fixed.argtypes = [ctypes.c_double, ctypes.c_int32, ctypes.c_int32, ctypes.c_char_p,
                                   ctypes.c_int32]
    rng = np.random.default_rng(17)
    xs = list(rng.normal(0, 1, 4000) * 10.0 ** rng.integers(-14, 13, 4000))
    xs += [k / 2048.0 for k in range(-3000, 3000, 7)]            # ties at 10 decimals
    xs += [(2 * k + 1) / 2000.0 for k in range(-500, 500)]        # ties at 3 decimals, as doubles
    xs += [0.0, -0.0, -1e-12, 1e-12, 5e-324, -5e-324, 2.0 ** 40 - 1, 2.0 ** 40, -2.0 ** 41 + 0.5,
           1e300, -1e300, 0.5, 1.5, 2.5, -2.5, 123456.789012345678, float("inf"), float("-inf"), float("nan")]
    for prec, width in ((10, 10), (3, 8), (2, 6), (0, 5), (17, 0)):
        for x in xs:
            assert _fmt(L, x, prec, width) == "%*.*f" % (width, prec, x), (x, prec, width)
