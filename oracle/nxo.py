"""ctypes view of the CPU oracle -- TEST INFRASTRUCTURE.

``Oracle`` wraps liboracle.so (the C restatement in oracle.c); ``Reference``
wraps _ref/libnxm_ref.so (the reference's own sources, compiled in place by
oracle/Makefile where the reference tree exists).  Only tests, the smoke
check and the CPU-baseline leg of bench.py import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference's source tree (its NexusMD/ directory's parent), named by the
# build recipe through NXM_REFERENCE_TREE; without it only a reference library
# built earlier (_ref/libnxm_ref.so) can be used.
REF_TREE = os.environ.get("NXM_REFERENCE_TREE") or None
REF_LIB = os.path.join(HERE, "_ref", "libnxm_ref.so")


def reference_tree_present() -> bool:
    return bool(REF_TREE) and os.path.isdir(os.path.join(REF_TREE, "NexusMD", "core"))


def reference_available() -> bool:
    """The reference library exists or can be built from its tree."""
    return reference_tree_present() or os.path.exists(REF_LIB)

_dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


def build(ref: bool | None = None) -> None:
    """Compile liboracle.so (and the reference library when its tree exists)."""
    targets = ["oracle"]
    if ref is None or (ref and not reference_tree_present()):
        # without the tree a reference library built earlier is used as it is
        ref = reference_tree_present()
    if ref:
        targets.append("ref")
    cmd = ["make", "-s", "-j8", "-C", HERE] + (["REF=" + REF_TREE] if ref else []) + targets
    subprocess.run(cmd, check=True)


class Box(C.Structure):
    _fields_ = [("lb", C.c_double * 3), ("ub", C.c_double * 3), ("size", C.c_double * 3)]

    def as9(self):
        return np.array(list(self.lb) + list(self.ub) + list(self.size), np.float64)

    @classmethod
    def from9(cls, a):
        b = cls()
        for d in range(3):
            b.lb[d], b.ub[d], b.size[d] = a[d], a[3 + d], a[6 + d]
        return b


class Energy(C.Structure):
    _fields_ = [(k, C.c_double) for k in
                ("bond", "angle", "torsion", "recip", "self", "coulomb", "vdw", "exclusion",
                 "reported_pe", "exception")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class SystemDesc(C.Structure):
    _fields_ = [("n", C.c_int), ("mass", C.c_void_p), ("q", C.c_void_p), ("sig", C.c_void_p),
                ("eps", C.c_void_p), ("nb", C.c_int), ("bonds", C.c_void_p),
                ("bond_prm", C.c_void_p), ("na", C.c_int), ("angles", C.c_void_p),
                ("angle_prm", C.c_void_p), ("nt", C.c_int), ("torsions", C.c_void_p),
                ("torsion_prm", C.c_void_p), ("torsion_per", C.c_void_p),
                ("cutoff", C.c_double), ("ewald_tol", C.c_double), ("use_switch", C.c_int),
                ("switch_dist", C.c_double), ("switch_quirk", C.c_int), ("grid", C.c_int * 3),
                ("box_mode", C.c_int), ("lb", C.c_double * 3), ("ub", C.c_double * 3),
                ("force_mask", C.c_int), ("exclusion_depth", C.c_int), ("nexc", C.c_int),
                ("exc_idx", C.c_void_p), ("exc_prm", C.c_void_p)]


class Timing(C.Structure):
    _fields_ = [(k, C.c_double) for k in
                ("nlist", "direct", "recip", "bonded", "exclusion", "integrate")]


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


class Oracle:
    """The C restatement (liboracle.so)."""

    def __init__(self, path: str | None = None):
        path = path or os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build(ref=False)
        L = self.lib = C.CDLL(path)
        L.nxo_box_from_positions.argtypes = [C.c_int, _dp, C.POINTER(Box)]
        L.nxo_bonds.argtypes = [_dp, C.c_int, _ip, _dp, C.POINTER(Box), _dp]
        L.nxo_bonds.restype = C.c_double
        L.nxo_angles.argtypes = [_dp, C.c_int, _ip, _dp, C.POINTER(Box), _dp]
        L.nxo_angles.restype = C.c_double
        L.nxo_torsions.argtypes = [_dp, C.c_int, _ip, _dp, _ip, C.POINTER(Box), _dp]
        L.nxo_torsions.restype = C.c_double
        L.nxo_exclusions.argtypes = [C.c_int, C.c_int, _ip, C.c_int, _ip, _ip, C.c_long]
        L.nxo_exclusions.restype = C.c_long
        L.nxo_pow2_grid.argtypes = [C.POINTER(Box), _ip]
        L.nxo_alpha.argtypes = [C.c_double, C.c_double]
        L.nxo_alpha.restype = C.c_double
        L.nxo_neighbor_pairs.argtypes = [C.c_int, _dp, C.POINTER(Box), _ip, _ip, C.c_double, _ip,
                                         C.c_long]
        L.nxo_neighbor_pairs.restype = C.c_long
        L.nxo_pme.argtypes = [C.c_int, _dp, _dp, C.POINTER(Box), C.c_double, _ip, _dp]
        L.nxo_pme.restype = C.c_double
        L.nxo_bspline_moduli.argtypes = [C.c_int, _dp]
        L.nxo_spread.argtypes = [C.c_int, _dp, _dp, C.POINTER(Box), _ip, _dp]
        L.nxo_forces.argtypes = [C.POINTER(SystemDesc), _dp, C.POINTER(Box), _ip, _ip, _dp,
                                 C.POINTER(Energy)]
        L.nxo_leapfrog.argtypes = [C.c_int, _dp, _dp, _dp, _dp, C.c_double, C.POINTER(Box)]
        L.nxo_kinetic.argtypes = [C.c_int, _dp, _dp, _dp, C.c_double]
        L.nxo_kinetic.restype = C.c_double
        L.nxo_run.argtypes = [C.POINTER(SystemDesc), _dp, _dp, _dp, C.c_double, C.c_int, C.c_int,
                              _dp, C.POINTER(Box)]
        L.nxo_run_timed.argtypes = [C.POINTER(SystemDesc), _dp, _dp, C.c_double, C.c_int,
                                    C.POINTER(Timing)]
        L.nxo_fft3d.argtypes = [_dp, C.c_int, C.c_int, C.c_int, C.c_int]
        L.nxo_exceptions.argtypes = [_dp, C.c_int, _ip, _dp, C.POINTER(Box), _dp]
        L.nxo_exceptions.restype = C.c_double

    # -- geometry
    def box_from_positions(self, pos) -> Box:
        b = Box()
        p = _c(pos, np.float64)
        self.lib.nxo_box_from_positions(len(p), p, C.byref(b))
        return b

    @staticmethod
    def box_explicit(lb, ub) -> Box:
        b = Box()
        for d in range(3):
            b.lb[d], b.ub[d], b.size[d] = lb[d], ub[d], abs(ub[d] - lb[d])
        return b

    def pow2_grid(self, box: Box):
        g = np.zeros(3, np.int32)
        self.lib.nxo_pow2_grid(C.byref(box), g)
        return tuple(int(x) for x in g)

    def alpha(self, cutoff, tol):
        return self.lib.nxo_alpha(cutoff, tol)

    # -- bonded
    def bonds(self, pos, idx, prm, box):
        F = np.zeros((len(pos), 3))
        E = self.lib.nxo_bonds(_c(pos, np.float64), len(idx), _c(idx, np.int32), _c(prm, np.float64),
                               C.byref(box), F)
        return E, F

    def angles(self, pos, idx, prm, box):
        F = np.zeros((len(pos), 3))
        E = self.lib.nxo_angles(_c(pos, np.float64), len(idx), _c(idx, np.int32),
                                _c(prm, np.float64), C.byref(box), F)
        return E, F

    def torsions(self, pos, idx, prm, per, box):
        F = np.zeros((len(pos), 3))
        E = self.lib.nxo_torsions(_c(pos, np.float64), len(idx), _c(idx, np.int32),
                                  _c(prm, np.float64), _c(per, np.int32), C.byref(box), F)
        return E, F

    # -- topology and pairs
    def exclusions(self, n, bonds, depth=3):
        b = _c(bonds, np.int32).reshape(-1)
        off = np.zeros(n + 1, np.int32)
        cap = 8 * n + 16
        while True:
            lst = np.zeros(cap, np.int32)
            ne = self.lib.nxo_exclusions(n, len(b) // 2, b, depth, off, lst, cap)
            if ne == -1 and len(b):
                raise ValueError("createExclusions: Illegal particle index in list of bonds")
            if ne >= 0:
                return off, lst[:ne].copy()
            cap = -ne

    @staticmethod
    def union_exclusions(off, lst, exc_idx):
        """Exclusion CSR united with exception pairs (both directions),
        partners ascending and unique."""
        n = len(off) - 1
        parts = [set(lst[off[i]:off[i + 1]].tolist()) for i in range(n)]
        for a, b in np.asarray(exc_idx, np.int64).reshape(-1, 2):
            parts[a].add(int(b))
            parts[b].add(int(a))
        noff = np.zeros(n + 1, np.int32)
        out = []
        for i in range(n):
            p = sorted(parts[i])
            out.extend(p)
            noff[i + 1] = noff[i] + len(p)
        return noff, np.array(out, np.int32)

    def exceptions(self, pos, idx, prm, box):
        """Exception pairs in OpenMM semantics: (energy, forces)."""
        F = np.zeros((len(pos), 3))
        E = self.lib.nxo_exceptions(_c(pos, np.float64), len(idx), _c(idx, np.int32), _c(prm, np.float64),
                                    C.byref(box), F)
        return E, F

    def neighbor_pairs(self, pos, box, eoff, elst, cutoff):
        p = _c(pos, np.float64)
        # first capacity from the density: pairs ~ (2/3) pi rc^3 n^2 / V, plus a margin
        vol = float(np.prod(np.asarray(list(box.size))))
        est = 2.0 / 3.0 * np.pi * cutoff ** 3 * len(p) * len(p) / vol if vol > 0 else 300.0 * len(p)
        cap = int(1.25 * est) + 1024
        while True:
            out = np.zeros(2 * cap, np.int32)
            np_ = self.lib.nxo_neighbor_pairs(len(p), p, C.byref(box), _c(eoff, np.int32),
                                              _c(elst, np.int32), cutoff, out, cap)
            if np_ >= 0:
                return out[:2 * np_].reshape(-1, 2).copy()
            cap = -np_

    # -- PME
    def bspline_moduli(self, K):
        m = np.zeros(K)
        self.lib.nxo_bspline_moduli(K, m)
        return m

    def spread(self, pos, q, box, grid):
        g = np.zeros(int(np.prod(grid)) * 2)
        self.lib.nxo_spread(len(pos), _c(pos, np.float64), _c(q, np.float64), C.byref(box),
                            _c(grid, np.int32), g)
        return g.reshape(tuple(grid) + (2,))

    def pme(self, pos, q, box, alpha, grid):
        F = np.zeros((len(pos), 3))
        E = self.lib.nxo_pme(len(pos), _c(pos, np.float64), _c(q, np.float64), C.byref(box), alpha,
                             _c(grid, np.int32), F)
        return E, F

    def fft3d(self, data_c, sign):
        a = np.ascontiguousarray(np.stack([data_c.real, data_c.imag], -1), np.float64)
        self.lib.nxo_fft3d(a.reshape(-1), *data_c.shape, sign)
        return a[..., 0] + 1j * a[..., 1]

    # -- whole system
    def describe(self, s, force_mask=15, box_mode=0, lb=None, ub=None, grid=None,
                 use_switch=0, switch_dist=0.0, switch_quirk=1, exclusion_depth=3, exceptions=None):
        """SystemDesc for a synthetic.System (keeps the arrays alive on the desc).
        exceptions: None, or (idx m x 2, prm m x 3: chargeProd, sigma, epsilon)."""
        keep = dict(mass=_c(s.mass, np.float64), q=_c(s.charge, np.float64),
                    sig=_c(s.sigma, np.float64), eps=_c(s.epsilon, np.float64),
                    bonds=_c(s.bonds, np.int32), bond_prm=_c(s.bond_prm, np.float64),
                    angles=_c(s.angles, np.int32), angle_prm=_c(s.angle_prm, np.float64),
                    torsions=_c(s.torsions, np.int32), torsion_prm=_c(s.torsion_prm, np.float64),
                    torsion_per=_c(s.torsion_n, np.int32))
        d = SystemDesc()
        d.n = s.n
        for k, v in keep.items():
            setattr(d, k, v.ctypes.data)
        d.nb, d.na, d.nt = len(s.bonds), len(s.angles), len(s.torsions)
        d.cutoff, d.ewald_tol = s.cutoff, s.ewald_tol
        d.use_switch, d.switch_dist, d.switch_quirk = use_switch, switch_dist, switch_quirk
        g = s.grid if grid is None else grid
        for k in range(3):
            d.grid[k] = int(g[k])
        d.box_mode = box_mode
        if box_mode:
            for k in range(3):
                d.lb[k], d.ub[k] = lb[k], ub[k]
        d.force_mask = force_mask
        d.exclusion_depth = exclusion_depth
        if exceptions is not None and len(exceptions[0]):
            keep["exc_idx"] = _c(exceptions[0], np.int32)
            keep["exc_prm"] = _c(exceptions[1], np.float64)
            d.nexc = len(keep["exc_idx"])
            d.exc_idx, d.exc_prm = keep["exc_idx"].ctypes.data, keep["exc_prm"].ctypes.data
        d._keep = keep
        return d

    def forces(self, desc, pos, box, eoff, elst):
        F = np.zeros((desc.n, 3))
        E = Energy()
        self.lib.nxo_forces(C.byref(desc), _c(pos, np.float64), C.byref(box), _c(eoff, np.int32),
                            _c(elst, np.int32), F, C.byref(E))
        return F, E.as_dict()

    def leapfrog(self, pos, vel, F, mass, dt, box):
        p = _c(pos, np.float64).copy()
        v = _c(vel, np.float64).copy()
        invm = np.where(mass == 0, 0.0, 1.0 / np.where(mass == 0, 1.0, mass))
        self.lib.nxo_leapfrog(len(p), p, v, _c(F, np.float64), _c(invm, np.float64), dt,
                              C.byref(box))
        return p, v

    def kinetic(self, vel, mass, F, dt):
        return self.lib.nxo_kinetic(len(vel), _c(vel, np.float64), _c(mass, np.float64),
                                    _c(F, np.float64), dt)

    def run(self, desc, pos, vel, dt, steps, interval=1):
        p = _c(pos, np.float64).copy()
        v = _c(vel, np.float64).copy()
        F = np.zeros_like(p)
        rep = np.zeros((steps + 1) * 4)
        box = Box()
        nrep = self.lib.nxo_run(C.byref(desc), p, v, F, dt, steps, interval, rep, C.byref(box))
        if nrep < 0:
            raise ValueError("oracle run failed (bad bond index?)")
        return p, v, F, rep[:4 * nrep].reshape(-1, 4), box

    def run_timed(self, desc, pos, vel, dt, steps):
        p = _c(pos, np.float64).copy()
        v = _c(vel, np.float64).copy()
        t = Timing()
        self.lib.nxo_run_timed(C.byref(desc), p, v, dt, steps, C.byref(t))
        return {k: getattr(t, k) for k, _ in t._fields_}


class Reference:
    """The reference's own sources compiled in place (oracle/_ref/libnxm_ref.so)."""

    def __init__(self, path: str | None = None):
        path = path or os.path.join(HERE, "_ref", "libnxm_ref.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = self.lib = C.CDLL(path)
        L.ref_box.argtypes = [C.c_int, _dp, _dp]
        for name, extra in (("ref_bonds", []), ("ref_angles", [])):
            f = getattr(L, name)
            f.argtypes = [C.c_int, _dp, C.c_int, _ip, _dp, _dp, _dp]
            f.restype = C.c_double
        L.ref_torsions.argtypes = [C.c_int, _dp, C.c_int, _ip, _dp, _ip, _dp, _dp]
        L.ref_torsions.restype = C.c_double
        L.ref_exclusions.argtypes = [C.c_int, C.c_int, _ip, C.c_int, _ip, _ip, C.c_long]
        L.ref_exclusions.restype = C.c_long
        L.ref_neighbor_pairs.argtypes = [C.c_int, _dp, _dp, _ip, _ip, C.c_double, _ip, C.c_long]
        L.ref_neighbor_pairs.restype = C.c_long
        L.ref_nonbonded.argtypes = [C.c_int, _dp, _dp, _dp, _dp, _dp, C.c_double, C.c_double,
                                    C.c_int, C.c_double, _ip, _ip, _ip, _dp, _dp]
        L.ref_leapfrog.argtypes = [C.c_int, _dp, _dp, _dp, _dp, C.c_double, _dp]
        L.ref_kinetic.argtypes = [C.c_int, _dp, _dp, _dp, C.c_double]
        L.ref_kinetic.restype = C.c_double
        L.ref_simulate.argtypes = [C.c_char_p] * 4 + [C.c_double, C.c_int, C.c_int, C.c_int]
        L.ref_simulate.restype = C.c_int

    def box(self, pos):
        out = np.zeros(9)
        p = _c(pos, np.float64)
        self.lib.ref_box(len(p), p, out)
        return out

    def bonds(self, pos, idx, prm, box9):
        F = np.zeros((len(pos), 3))
        E = self.lib.ref_bonds(len(pos), _c(pos, np.float64), len(idx), _c(idx, np.int32),
                               _c(prm, np.float64), _c(box9, np.float64), F)
        return E, F

    def angles(self, pos, idx, prm, box9):
        F = np.zeros((len(pos), 3))
        E = self.lib.ref_angles(len(pos), _c(pos, np.float64), len(idx), _c(idx, np.int32),
                                _c(prm, np.float64), _c(box9, np.float64), F)
        return E, F

    def torsions(self, pos, idx, prm, per, box9):
        F = np.zeros((len(pos), 3))
        E = self.lib.ref_torsions(len(pos), _c(pos, np.float64), len(idx), _c(idx, np.int32),
                                  _c(prm, np.float64), _c(per, np.int32), _c(box9, np.float64), F)
        return E, F

    def exclusions(self, n, bonds, depth=3):
        b = _c(bonds, np.int32).reshape(-1)
        off = np.zeros(n + 1, np.int32)
        cap = 8 * n + 16
        while True:
            lst = np.zeros(cap, np.int32)
            ne = self.lib.ref_exclusions(n, len(b) // 2, b, depth, off, lst, cap)
            if ne >= 0:
                return off, lst[:ne].copy()
            cap = -ne

    def neighbor_pairs(self, pos, box9, eoff, elst, cutoff):
        p = _c(pos, np.float64)
        cap = 300 * len(p) + 1024
        while True:
            out = np.zeros(2 * cap, np.int32)
            np_ = self.lib.ref_neighbor_pairs(len(p), p, _c(box9, np.float64), _c(eoff, np.int32),
                                              _c(elst, np.int32), cutoff, out, cap)
            if np_ >= 0:
                return out[:2 * np_].reshape(-1, 2).copy()
            cap = -np_

    def nonbonded(self, s, pos, box9, eoff, elst, grid=None, use_switch=0, switch_dist=0.0):
        F = np.zeros((len(pos), 3))
        E = np.zeros(4)
        g = np.array(grid if grid is not None else (0, 0, 0), np.int32)
        self.lib.ref_nonbonded(len(pos), _c(pos, np.float64), _c(s.charge, np.float64),
                               _c(s.sigma, np.float64), _c(s.epsilon, np.float64),
                               _c(box9, np.float64), s.cutoff, s.ewald_tol, use_switch,
                               switch_dist, g, _c(eoff, np.int32), _c(elst, np.int32), F, E)
        return F, dict(recip=E[0], self=E[1], direct=E[2], exclusion_signed=E[3])

    def leapfrog(self, pos, vel, F, mass, dt, box9):
        p = _c(pos, np.float64).copy()
        v = _c(vel, np.float64).copy()
        self.lib.ref_leapfrog(len(p), p, v, _c(F, np.float64), _c(mass, np.float64), dt,
                              _c(box9, np.float64))
        return p, v

    def kinetic(self, vel, mass, F, dt):
        return self.lib.ref_kinetic(len(vel), _c(vel, np.float64), _c(mass, np.float64),
                                    _c(F, np.float64), dt)

    def simulate(self, system_xml, state_xml, pdb, out, dt, steps, interval, force_mask=15):
        e = lambda s: s.encode()
        return self.lib.ref_simulate(e(system_xml), e(state_xml), e(pdb), e(out), dt, steps,
                                     interval, force_mask)
