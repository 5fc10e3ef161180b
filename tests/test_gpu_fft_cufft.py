"""The hand-written PME FFT against cuFFT on the device (GPU required).

After a force evaluation the engine's charge grid, influence function and
convolved real grid are read back (nxm_get_pme_grids); the same convolution
is then done with cuFFT through torch.fft in FP64 on the GPU:
    potential = irfftn(rfftn(Q) * eterm), both transforms unnormalised,
which is the reference's forward c2c FFT, multiply, backward c2c FFT on a
real grid (NonbondedForce.cpp:264-290, 323-388).  The reciprocal energy
0.5 * sum over the full spectrum of eterm |Q^|^2 is checked too.

Grids: the configurations' 32^3, 64^3, 100^3 and 180^3 (passes of radix
8, 10, 9, 6, 4, 2), and a mixed 40 x 36 x 30.  Tolerances: FP32 engine
rel-RMS 1e-5 on the grid and 1e-5 relative on the energy; FP64 engine 1e-11
on the grid and 1e-9 on the energy, which the engine sums per spectrum
element as fixed point in units of 2^-28 kJ/mol (order-free, ~5e5 roundings
at 100^3), as every FP64 energy parity test allows.
"""
import numpy as np
import pytest

from nexusmd_gb300 import synthetic as sy

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def system():
    return sy.config_system(1)


def _cufft_reference(q, eterm):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    Q = torch.tensor(q, dtype=torch.float64, device=dev)
    E = torch.tensor(eterm, dtype=torch.float64, device=dev)
    F = torch.fft.rfftn(Q)  # unnormalised forward (cuFFT)
    pot = torch.fft.irfftn(F * E, s=q.shape, norm="forward")  # unnormalised inverse
    K2 = q.shape[2]
    w = torch.full((K2 // 2 + 1,), 2.0, dtype=torch.float64, device=dev)
    w[0] = 1.0
    if K2 % 2 == 0:
        w[-1] = 1.0
    energy = 0.5 * float((w * E * (F.real ** 2 + F.imag ** 2)).sum())
    return pot.cpu().numpy(), energy


@pytest.mark.parametrize("grid", [(32, 32, 32), (64, 64, 64), (100, 100, 100), (180, 180, 180), (40, 36, 30)])
@pytest.mark.parametrize("prec,fft_path", [(1, 1), (1, 2), (0, 1)])
def test_fft_convolution_matches_cufft(system, grid, prec, fft_path):
    from nexusmd_gb300.engine import Engine, FORCE_NONBONDED
    eng = Engine(system, precision=prec, force_mask=FORCE_NONBONDED, box="explicit", grid=grid, skin=0.0,
                 rebuild_interval=1, fft_path=fft_path)
    if fft_path == 2 and eng.layout()["fft_path"] != 2:
        eng.close()
        pytest.skip("plane path not available for this grid")
    eng.compute_forces()
    q, eterm, pot = eng.pme_grids()
    e_recip = eng.energies()["recip"]
    eng.close()
    assert np.abs(q).sum() > 0
    ref, e_ref = _cufft_reference(q, eterm)
    err = float(np.sqrt(((pot - ref) ** 2).sum() / (ref ** 2).sum()))
    tol, etol = (1e-5, 1e-5) if prec == 1 else (1e-11, 1e-9)
    print("grid", grid, "precision", prec, "path", fft_path, "grid rel-RMS vs cuFFT", err,
          "energy", e_recip, "cuFFT", e_ref)
    assert err <= tol, (grid, prec, err)
    assert abs(e_recip - e_ref) <= etol * abs(e_ref), (grid, prec, e_recip, e_ref)
