"""The two launch shapes of the PME FFT against each other and the oracle.

The plane path (one block per x-plane for the z and y transforms; 3 FFT
launches) and the line path (5 launches over tiles of lines) run the same
Stockham passes on the same lines.  With an even K1 the z transforms also
pair the same real lines, so the mixed engine's results (fixed-point force
sums) must be equal bit for bit; with an odd K1 the line path pairs lines
across x-planes and only the rounding differs.  Every case is also checked
against the FP64 oracle on the same grid: FP64 engine within 1e-9, mixed
within the 1e-5 force rel-RMS target.

(8, 200, 216) does not fit one x-plane's scratch in shared memory, so the
plane kernels transform it in chunks of lines; in FP64 the plane itself does
not fit and the engine takes the line path on its own.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TERMS = ("recip", "self", "coulomb", "vdw", "exclusion")


def _run(s, grid, precision, fft_path):
    from nexusmd_gb300.engine import Engine
    eng = Engine(s, precision=precision, skin=0.0, rebuild_interval=1, grid=grid, fft_path=fft_path)
    try:
        tune = eng.tuning() + (eng.fft_plane_threads(),)
        return eng.compute_forces(), eng.energies(), tune
    finally:
        eng.close()


def _rel_rms(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


@pytest.mark.parametrize("grid", [(24, 30, 20), (20, 27, 24), (8, 200, 216)])
def test_plane_and_line_paths_agree_with_oracle(oracle, c1_compat, grid):
    s = c1_compat
    box = oracle.box_from_positions(s.pos)
    eoff, el = oracle.exclusions(s.n, s.bonds)
    F0, E0 = oracle.forces(oracle.describe(s, grid=grid), s.pos, box, eoff, el)
    scale = max(abs(E0[k]) for k in TERMS)
    for precision, ftol, etol in ((1, 1e-5, 2e-5), (0, 1e-9, 1e-9)):
        Fp, Ep, tp = _run(s, grid, precision, 2)
        Fl, El, tl = _run(s, grid, precision, 1)
        assert tl[0] > 0 and tl[3] == 0  # the line path reports its z blocking
        if precision == 1:
            # every mixed case here fits the plane path
            assert tp[0] == 0 and tp[3] in (256, 512, 1024)
        for F, E in ((Fp, Ep), (Fl, El)):
            assert _rel_rms(F, F0) <= ftol, (grid, precision, _rel_rms(F, F0))
            for k in TERMS:
                assert abs(E[k] - E0[k]) <= etol * scale + 1e-6, (grid, precision, k, E[k], E0[k])
        if precision == 1 and grid[1] % 2 == 0:
            assert np.array_equal(Fp, Fl), (grid, np.abs(Fp - Fl).max())
            assert Ep["recip"] == El["recip"]
        else:
            assert _rel_rms(Fp, Fl) <= (1e-6 if precision == 1 else 1e-12), (grid, _rel_rms(Fp, Fl))


def test_autotuned_path_gives_the_line_path_numbers(c1_compat):
    """fft_path 0 lets the autotuner pick either path only where both give
    the same bits (K1 even), so the pick cannot change results."""
    grid = (24, 30, 20)
    Fa, Ea, _ = _run(c1_compat, grid, 1, 0)
    Fl, El, _ = _run(c1_compat, grid, 1, 1)
    assert np.array_equal(Fa, Fl) and Ea["recip"] == El["recip"]


def test_bad_fft_path_is_rejected(c1_compat):
    from nexusmd_gb300.engine import Engine, NxmError
    with pytest.raises(NxmError, match="fft_path"):
        Engine(c1_compat, precision=1, grid=(24, 30, 20), fft_path=3)
