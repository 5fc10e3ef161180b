"""Generates tests/golden/*.npz from the reference compiled from its own
sources (oracle/_ref/libnxm_ref.so, built by oracle/Makefile where the
reference tree exists).  Every array in a fixture is the reference's own
output for the seeded synthetic input stored beside it.

    python tests/golden/make_golden.py
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from nexusmd_gb300 import synthetic as sy  # noqa: E402
from oracle import nxo  # noqa: E402

CASES = {
    # name: (system factory, PME grid for the nonbonded phase)
    "chain_water_800": (lambda: sy.compat_system(sy.make_system(1, 20, 240, 2.4, seed=77)), (24, 24, 24)),
    "chain_water_800_pow2": (lambda: sy.compat_system(sy.make_system(1, 20, 240, 2.4, seed=77)), (0, 0, 0)),
    "two_chains_600": (lambda: sy.compat_system(sy.make_system(2, 12, 140, 2.3, seed=5, jitter=0.006)), (20, 25, 27)),
}


def main():
    nxo.build(ref=True)
    r = nxo.Reference()
    for name, (make, grid) in CASES.items():
        s = make()
        b9 = r.box(s.pos)
        off, lst = r.exclusions(s.n, s.bonds)
        pairs = r.neighbor_pairs(s.pos, b9, off, lst, s.cutoff)
        Eb, Fb = r.bonds(s.pos, s.bonds, s.bond_prm, b9)
        Ea, Fa = r.angles(s.pos, s.angles, s.angle_prm, b9)
        Et, Ft = r.torsions(s.pos, s.torsions, s.torsion_prm, s.torsion_n, b9)
        Fn, En = r.nonbonded(s, s.pos, b9, off, lst, grid=grid)
        Ftot = Fb + Fa + Ft + Fn
        v0 = np.random.default_rng(11).normal(0, 0.5, size=s.pos.shape)
        p1, v1 = r.leapfrog(s.pos, v0, Ftot, s.mass, 0.0005, b9)
        ke = r.kinetic(v0, s.mass, Ftot, 0.0005)
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"), pos=s.pos, mass=s.mass, q=s.charge, sig=s.sigma,
            eps=s.epsilon, bonds=s.bonds, bond_prm=s.bond_prm, angles=s.angles,
            angle_prm=s.angle_prm, torsions=s.torsions, torsion_prm=s.torsion_prm,
            torsion_n=s.torsion_n, cutoff=s.cutoff, tol=s.ewald_tol, grid=np.array(grid),
            box9=b9, excl_off=off, excl_lst=lst, n_pairs=len(pairs),
            pairs_sha256=np.frombuffer(hashlib.sha256(np.ascontiguousarray(pairs, np.int32).tobytes()).digest(), np.uint8), E_bonds=Eb, F_bonds=Fb,
            E_angles=Ea, F_angles=Fa, E_torsions=Et, F_torsions=Ft, F_nonbonded=Fn,
            E_nonbonded=np.array([En["recip"], En["self"], En["direct"], En["exclusion_signed"]]),
            F_total=Ftot, v0=v0, pos1=p1, vel1=v1, ke=ke)
        print(name, s.n, "atoms,", len(pairs), "pairs")
    simulate_case(r)


def simulate_case(r):
    """The reference's own Simulate on a small system: inputs and the three
    report files it writes (PVFReport<out>, TotalEnergy<out>, <out>)."""
    import gzip
    import shutil
    import tempfile
    d = os.path.join(HERE, "simulate_small")
    os.makedirs(d, exist_ok=True)
    s = sy.compat_system(sy.make_system(1, 4, 100, 2.8, seed=21))
    sy.write_inputs(s, d, "small")
    with tempfile.TemporaryDirectory() as tmp:
        cwd = os.getcwd()
        os.chdir(tmp)
        try:
            for i, (steps, interval) in enumerate(((10, 1), (7, 3))):
                out = "out%d.pdb" % i
                rc = r.simulate(os.path.join(d, "system_small.xml"), os.path.join(d, "state_small.xml"),
                                os.path.join(d, "small.pdb"), out, 0.0005, steps, interval)
                assert rc == 0
                for f in (out, "PVFReport" + out, "TotalEnergy" + out):
                    with open(f, "rb") as src, gzip.open(os.path.join(d, f + ".gz"), "wb") as dst:
                        shutil.copyfileobj(src, dst)
        finally:
            os.chdir(cwd)
    print("simulate_small", s.n, "atoms")


if __name__ == "__main__":
    main()
