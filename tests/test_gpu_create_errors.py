"""Context creation rejects terms with atom indices outside their system.

The engine checks the indices on the device while it ingests the terms
(k_terms_ingest) and reports them when it reads the exclusion build's
totals; an invalid term is replaced by the system's first atom before any
other set-up kernel reads it, so the failed creation touches nothing out of
range and the next context on the device works.  Messages as the host
checks gave them (bonds: Exclusions.cpp's createExclusions message).
"""
import copy

import numpy as np
import pytest

from nexusmd_gb300 import synthetic as sy

pytestmark = pytest.mark.gpu


def _engine(s, **kw):
    from nexusmd_gb300.engine import Engine
    return Engine(s, box="explicit", **kw)


def _broken(kind, value):
    s = copy.deepcopy(sy.config_system(1))
    arr = np.array(getattr(s, kind), dtype=np.int32).copy()
    arr.reshape(-1)[7] = value
    setattr(s, kind, arr)
    return s


@pytest.mark.parametrize("kind,value,msg", [
    ("bonds", 10 ** 6, "Illegal particle index in list of bonds"),
    ("bonds", -1, "Illegal particle index in list of bonds"),
    ("angles", -3, "angle atom index out of range"),
    ("torsions", 10 ** 7, "torsion atom index out of range"),
])
def test_invalid_term_index_fails_creation(kind, value, msg):
    from nexusmd_gb300.engine import NxmError
    with pytest.raises(NxmError, match=msg):
        _engine(_broken(kind, value))


def test_batch_reports_invalid_index_of_second_system():
    from nexusmd_gb300.engine import NxmError
    a = sy.config_system(1)
    b = _broken("angles", a.n)  # one past the second system's atoms
    with pytest.raises(NxmError, match="angle atom index out of range"):
        _engine([a, b])


def test_device_usable_after_failed_creation():
    from nexusmd_gb300.engine import NxmError
    with pytest.raises(NxmError):
        _engine(_broken("torsions", -2))
    s = sy.config_system(1)
    eng = _engine(s)
    F = eng.compute_forces()
    assert np.isfinite(F).all() and np.abs(F).max() > 0
    eng.close()


def test_disabled_kind_is_not_checked():
    """A kind switched off by the force mask is not taken in, so its indices
    are not read (bonds still are: they define the exclusions)."""
    s = _broken("angles", -5)
    eng = _engine(s, force_mask=1 | 4 | 8)  # bonds, torsions, nonbonded
    F = eng.compute_forces()
    assert np.isfinite(F).all()
    eng.close()
