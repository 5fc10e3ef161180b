"""Python module with the names of the reference's SWIG module ``NexusMD``.

The reference exposes TaskDispatcher (as a shared_ptr), Coords3D and
SystemXMLParser through SWIG (wrapper/NexusMD.i:1-19).  This module binds the
same names to libnxm_cuda.so's C ABI (include/nxm.h) with ctypes, so a script
written for the reference runs with "GPU" as the processor string:

    import NexusMD
    d = NexusMD.TaskDispatcher.CreateDispatcher("GPU")
    d.EnableHarmonicBondForce(); d.EnableNonbondedForce()
    d.Simulate("system.xml", "state.xml", "in.pdb", "out.pdb", 0.001, 10, 1)

Errors raise RuntimeError (the reference's C++ exceptions surface the same
way through SWIG).  Parsers print the reference's message and return empty
results for an unreadable file.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from .engine import load_library


class _Opts(C.Structure):
    _fields_ = [("precision", C.c_int32), ("skin", C.c_double), ("rebuild_interval", C.c_int32),
                ("device", C.c_int32), ("max_neighbors", C.c_int32), ("exceptions", C.c_int32),
                ("autotune", C.c_int32), ("report_threads", C.c_int32), ("state_velocities", C.c_int32),
                ("fft_path", C.c_int32)]


def _lib():
    L = load_library()
    if not getattr(L, "_nexusmd_bound", False):
        vp = C.c_void_p
        L.nxm_dispatcher_create.argtypes = [C.c_char_p, C.POINTER(vp)]
        L.nxm_dispatcher_destroy.argtypes = [vp]
        L.nxm_dispatcher_destroy.restype = None
        for n in ("harmonic_bond", "harmonic_angle", "periodic_torsion", "nonbonded"):
            getattr(L, "nxm_dispatcher_enable_%s_force" % n).argtypes = [vp]
        L.nxm_dispatcher_set_options.argtypes = [vp, C.POINTER(_Opts)]
        L.nxm_dispatcher_simulate.argtypes = [vp, C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_double,
                                              C.c_int32, C.c_int32]
        L.nxm_parse_files.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(vp)]
        L.nxm_parsed_free.argtypes = [vp]
        L.nxm_parsed_free.restype = None
        L.nxm_parsed_counts.argtypes = [vp, np.ctypeslib.ndpointer(np.int64)]
        L.nxm_parsed_nonbonded.argtypes = [vp, np.ctypeslib.ndpointer(np.float64)]
        L.nxm_parsed_arrays.argtypes = [vp] + [vp] * 12
        L.nxm_parsed_velocities.argtypes = [vp, vp, C.POINTER(C.c_int64)]
        L.nxm_write_state_xml.argtypes = [C.c_char_p, C.c_int32, vp, vp, vp, C.c_int64, C.c_double]
        L._nexusmd_bound = True
    return L


def _err(L, rc, what):
    if rc != 0:
        raise RuntimeError("%s: %s" % (what, L.nxm_last_error().decode(errors="replace")))


# --------------------------------------------------------------- Coords3D

class Coords3D:
    """Three-component vector (core/common/headers/Coords3D.h:15-152)."""

    __slots__ = ("data",)

    def __init__(self, x=0.0, y=0.0, z=0.0):
        self.data = [float(x), float(y), float(z)]

    def __getitem__(self, i):
        return self.data[i]

    def __setitem__(self, i, v):
        self.data[i] = float(v)

    def __eq__(self, o):
        return self.data == list(o.data)

    def __ne__(self, o):
        return not self == o

    def __add__(self, o):
        return Coords3D(*(a + b for a, b in zip(self.data, o.data)))

    def __sub__(self, o):
        return Coords3D(*(a - b for a, b in zip(self.data, o.data)))

    def __neg__(self):
        return Coords3D(*(-a for a in self.data))

    def __mul__(self, s):
        return Coords3D(*(a * s for a in self.data))

    def __truediv__(self, s):
        inv = 1.0 / s
        return Coords3D(*(a * inv for a in self.data))

    def dot(self, o):
        a, b = self.data, o.data
        return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]

    def cross(self, o):
        a, b = self.data, o.data
        return Coords3D(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])

    def length(self):
        return math.sqrt(self.dot(self))

    def normalize(self):
        n = self.length()
        return Coords3D(*(a / n for a in self.data)) if n > 0 else Coords3D()

    def __repr__(self):
        return "Coords3D(%r, %r, %r)" % tuple(self.data)


# ----------------------------------------------------- parameter records

class PTorsionParams:
    def __init__(self, p1=0, p2=0, p3=0, p4=0, k=0.0, phase=0.0, periodicity=0):
        self.p1, self.p2, self.p3, self.p4 = p1, p2, p3, p4
        self.k, self.phase, self.periodicity = k, phase, periodicity


class BondParams:
    def __init__(self, p1=0, p2=0, d=0.0, k=0.0):
        self.p1, self.p2, self.d, self.k = p1, p2, d, k


class AngleParams:
    def __init__(self, p1=0, p2=0, p3=0, a=0.0, k=0.0):
        self.p1, self.p2, self.p3, self.a, self.k = p1, p2, p3, a, k


class NonbondedParticle:
    def __init__(self, q=0.0, sig=0.0, eps=0.0):
        self.q, self.sig, self.eps = q, sig, eps


class NonbondedException:
    def __init__(self, p1=0, p2=0, q=0.0, sig=0.0, eps=0.0):
        self.p1, self.p2, self.q, self.sig, self.eps = p1, p2, q, sig, eps


class NonbondedParams:
    def __init__(self):
        self.alpha = self.cutoff = self.ewaldTolerance = self.rfDielectric = self.switchingDistance = 0.0
        self.dispersionCorrection = self.useSwitchingFunction = self.method = 0
        self.nx = self.ny = self.nz = 0
        self.particles = []
        self.exceptions = []


class _Parsed:
    def __init__(self, system_xml=None, state_xml=None):
        L = _lib()
        h = C.c_void_p()
        L.nxm_parse_files(system_xml.encode() if system_xml else None,
                          state_xml.encode() if state_xml else None, C.byref(h))
        try:
            cnt = np.zeros(7, np.int64)
            L.nxm_parsed_counts(h, cnt)
            nm, npos, nb, na, nt, npart, nex = (int(c) for c in cnt)
            self.masses = np.zeros(nm)
            self.positions = np.zeros((npos, 3))
            self.bond_atoms, self.bond_prm = np.zeros((nb, 2), np.int32), np.zeros((nb, 2))
            self.angle_atoms, self.angle_prm = np.zeros((na, 3), np.int32), np.zeros((na, 2))
            self.tors_atoms, self.tors_prm = np.zeros((nt, 4), np.int32), np.zeros((nt, 2))
            self.tors_per = np.zeros(nt, np.int32)
            self.qse = np.zeros((npart, 3))
            self.ex_atoms, self.ex_prm = np.zeros((nex, 2), np.int32), np.zeros((nex, 3))
            arrs = [self.masses, self.positions, self.bond_atoms, self.bond_prm, self.angle_atoms,
                    self.angle_prm, self.tors_atoms, self.tors_prm, self.tors_per, self.qse,
                    self.ex_atoms, self.ex_prm]
            L.nxm_parsed_arrays(h, *[a.ctypes.data if a.size else None for a in arrs])
            self.nb = np.zeros(11)
            L.nxm_parsed_nonbonded(h, self.nb)
            nv = C.c_int64(0)
            L.nxm_parsed_velocities(h, None, C.byref(nv))
            self.velocities = np.zeros((nv.value, 3))
            if nv.value:
                L.nxm_parsed_velocities(h, self.velocities.ctypes.data, C.byref(nv))
        finally:
            L.nxm_parsed_free(h)


class SystemXMLParser:
    """Static readers of the system XML (core/common/src/SystemXMLParser.cpp:18-196)."""

    @staticmethod
    def MassesParser(filename):
        return [float(m) for m in _Parsed(filename).masses]

    @staticmethod
    def PTorsionParser(filename):
        p = _Parsed(filename)
        return [PTorsionParams(*map(int, a), float(pr[0]), float(pr[1]), int(n))
                for a, pr, n in zip(p.tors_atoms, p.tors_prm, p.tors_per)]

    @staticmethod
    def HBondParser(filename):
        p = _Parsed(filename)
        return [BondParams(int(a[0]), int(a[1]), float(pr[0]), float(pr[1]))
                for a, pr in zip(p.bond_atoms, p.bond_prm)]

    @staticmethod
    def HAngleParser(filename):
        p = _Parsed(filename)
        return [AngleParams(int(a[0]), int(a[1]), int(a[2]), float(pr[0]), float(pr[1]))
                for a, pr in zip(p.angle_atoms, p.angle_prm)]

    @staticmethod
    def NonBondedParser(filename):
        p = _Parsed(filename)
        out = NonbondedParams()
        (out.cutoff, out.ewaldTolerance, out.switchingDistance, usw, out.alpha, out.rfDielectric,
         nx, ny, nz, method, disp) = p.nb.tolist()
        out.useSwitchingFunction, out.nx, out.ny, out.nz = int(usw), int(nx), int(ny), int(nz)
        out.method, out.dispersionCorrection = int(method), int(disp)
        out.particles = [NonbondedParticle(*map(float, r)) for r in p.qse]
        out.exceptions = [NonbondedException(int(a[0]), int(a[1]), *map(float, r))
                          for a, r in zip(p.ex_atoms, p.ex_prm)]
        return out


class StateXMLParser:
    """Reader of the state XML positions (core/common/src/StateXMLParser.cpp:17-37)."""

    @staticmethod
    def parseStateXML(filename):
        return [Coords3D(*r) for r in _Parsed(None, filename).positions]

    @staticmethod
    def parseStateVelocities(filename):
        """The state file's <Velocities> (nm/ps), which the reference does not read;
        empty when the file has none."""
        return [Coords3D(*r) for r in _Parsed(None, filename).velocities]

    @staticmethod
    def writeStateXML(filename, positions, velocities=None, box=(0.0, 0.0, 0.0), step=0, time=0.0):
        """Checkpoint in OpenMM's state format (17 significant digits: reading it back
        gives the same doubles)."""
        L = _lib()
        x = np.ascontiguousarray(np.asarray([tuple(p) for p in positions], np.float64).reshape(-1, 3))
        v = None if velocities is None else np.ascontiguousarray(
            np.asarray([tuple(p) for p in velocities], np.float64).reshape(-1, 3))
        b = np.ascontiguousarray(np.asarray(box, np.float64).reshape(3))
        rc = L.nxm_write_state_xml(str(filename).encode(), len(x), x.ctypes.data,
                                   None if v is None else v.ctypes.data, b.ctypes.data, int(step), float(time))
        _err(L, rc, "writeStateXML")


# ---------------------------------------------------------- dispatcher

PRECISIONS = {"fp64": 0, "double": 0, "mixed": 1}


class TaskDispatcher:
    """CUDA-backed TaskDispatcher (core/dispatcher/headers/TaskDispatcher.h:9-43)."""

    def __init__(self, handle):
        self._h = handle
        self._L = _lib()

    @staticmethod
    def CreateDispatcher(processorChoice):
        L = _lib()
        h = C.c_void_p()
        _err(L, L.nxm_dispatcher_create(str(processorChoice).encode(), C.byref(h)), "CreateDispatcher")
        return TaskDispatcher(h)

    def __del__(self):
        try:
            if self._h:
                self._L.nxm_dispatcher_destroy(self._h)
                self._h = None
        except Exception:
            pass

    def EnableHarmonicBondForce(self):
        self._L.nxm_dispatcher_enable_harmonic_bond_force(self._h)

    def EnableHarmonicAngleForce(self):
        self._L.nxm_dispatcher_enable_harmonic_angle_force(self._h)

    def EnablePeriodicTorsionForce(self):
        self._L.nxm_dispatcher_enable_periodic_torsion_force(self._h)

    def EnableNonbondedForce(self):
        self._L.nxm_dispatcher_enable_nonbonded_force(self._h)

    def SetOptions(self, precision="mixed", skin=0.1, rebuild_interval=10, device=0, max_neighbors=0,
                   exceptions=False, autotune=True, report_threads=4, state_velocities=False):
        """Engine settings the reference hard-codes (precision "mixed" or "fp64").
        exceptions=True applies the system XML's <Exceptions> (scaled 1-4 pairs,
        OpenMM semantics), which the reference parses but ignores; autotune
        times result-neutral launch shapes at set-up and keeps the fastest;
        report_threads > 0 writes the report files on a host thread while the
        GPU steps on (0: before the next step, as the reference; same bytes);
        state_velocities=True starts from the state file's <Velocities>."""
        o = _Opts(PRECISIONS[precision], float(skin), int(rebuild_interval), int(device), int(max_neighbors),
                  1 if exceptions else 0, 1 if autotune else 0, int(report_threads),
                  1 if state_velocities else 0)
        _err(self._L, self._L.nxm_dispatcher_set_options(self._h, C.byref(o)), "SetOptions")

    def Simulate(self, systemFilename, stateFilename, inputFilename, outputFilename, StepSize, TotalSteps,
                 interval):
        rc = self._L.nxm_dispatcher_simulate(self._h, systemFilename.encode(), stateFilename.encode(),
                                             inputFilename.encode(), outputFilename.encode(),
                                             float(StepSize), int(TotalSteps), int(interval))
        _err(self._L, rc, "Simulate")
