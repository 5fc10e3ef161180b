"""ctypes binding of libnxm_cuda.so's engine API (include/nxm.h).

``Engine`` takes one or more :class:`nexusmd_gb300.synthetic.System` (or any
object with the same array attributes), creates a device context and exposes
forces, energies, steps and the neighbour pair set as numpy arrays.  There is
no CPU path: if the CUDA library cannot be loaded or no GPU is present, the
constructor raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnxm_cuda.so")

PRECISION_FP64 = 0
PRECISION_MIXED = 1
FORCE_BOND, FORCE_ANGLE, FORCE_TORSION, FORCE_NONBONDED = 1, 2, 4, 8
FORCE_ALL = 15


class SystemDesc(C.Structure):
    _fields_ = [("n_atoms", C.c_int32), ("masses", C.c_void_p), ("charges", C.c_void_p),
                ("sigmas", C.c_void_p), ("epsilons", C.c_void_p),
                ("n_bonds", C.c_int32), ("bond_atoms", C.c_void_p), ("bond_params", C.c_void_p),
                ("n_angles", C.c_int32), ("angle_atoms", C.c_void_p), ("angle_params", C.c_void_p),
                ("n_torsions", C.c_int32), ("torsion_atoms", C.c_void_p),
                ("torsion_params", C.c_void_p), ("torsion_periodicity", C.c_void_p),
                ("cutoff", C.c_double), ("ewald_tolerance", C.c_double),
                ("use_switching", C.c_int32), ("switching_distance", C.c_double),
                ("grid", C.c_int32 * 3), ("box_from_positions", C.c_int32),
                ("box_lb", C.c_double * 3), ("box_ub", C.c_double * 3),
                ("force_mask", C.c_int32), ("exclusion_depth", C.c_int32),
                ("n_exceptions", C.c_int32), ("exception_atoms", C.c_void_p),
                ("exception_params", C.c_void_p)]


class Options(C.Structure):
    _fields_ = [("precision", C.c_int32), ("skin", C.c_double), ("rebuild_interval", C.c_int32),
                ("device", C.c_int32), ("max_neighbors", C.c_int32), ("exceptions", C.c_int32),
                ("autotune", C.c_int32), ("report_threads", C.c_int32), ("state_velocities", C.c_int32),
                ("fft_path", C.c_int32)]


class Energies(C.Structure):
    _fields_ = [(k, C.c_double) for k in
                ("bond", "angle", "torsion", "recip", "self", "coulomb", "vdw", "exclusion",
                 "kinetic", "potential", "reported_potential", "exception")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Load libnxm_cuda.so (building it first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        from . import build
        build.build()
    L = C.CDLL(path)
    dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
    L.nxm_version.restype = C.c_char_p
    L.nxm_last_error.restype = C.c_char_p
    L.nxm_default_options.argtypes = [C.POINTER(Options)]
    L.nxm_create.argtypes = [C.POINTER(SystemDesc), C.c_int32, C.POINTER(Options), dp,
                             C.POINTER(C.c_void_p)]
    L.nxm_destroy.argtypes = [C.c_void_p]
    L.nxm_destroy.restype = None
    for name in ("nxm_set_positions", "nxm_set_velocities", "nxm_get_positions",
                 "nxm_get_velocities", "nxm_get_forces"):
        getattr(L, name).argtypes = [C.c_void_p, dp]
    L.nxm_get_state.argtypes = [C.c_void_p, dp, dp]
    L.nxm_compute_forces.argtypes = [C.c_void_p]
    L.nxm_step.argtypes = [C.c_void_p, C.c_int32, C.c_double]
    L.nxm_get_energies.argtypes = [C.c_void_p, C.c_int32, C.POINTER(Energies)]
    L.nxm_get_box.argtypes = [C.c_void_p, C.c_int32, dp, dp]
    L.nxm_get_grid.argtypes = [C.c_void_p, C.c_int32, np.ctypeslib.ndpointer(np.int32)]
    L.nxm_get_alpha.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_double)]
    L.nxm_get_pairs.argtypes = [C.c_void_p, C.c_int32, np.ctypeslib.ndpointer(np.int32), C.c_int64]
    L.nxm_get_pairs.restype = C.c_int64
    L.nxm_time_steps.argtypes = [C.c_void_p, C.c_int32, C.c_double, C.POINTER(C.c_double)]
    L.nxm_time_report_steps.argtypes = [C.c_void_p, C.c_int32, C.c_double, C.POINTER(C.c_double)]
    L.nxm_profile_phases.argtypes = [C.c_void_p, C.c_int32, C.c_double, dp, C.c_int32]
    L.nxm_launches_per_step.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    L.nxm_rebuild_count.argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
    L.nxm_get_tuning.argtypes = [C.c_void_p, C.POINTER(C.c_int32)]
    L.nxm_get_fft_plane_threads.argtypes = [C.c_void_p, C.POINTER(C.c_int32)]
    L.nxm_frames_init.argtypes = [C.c_void_p, C.c_int32]
    L.nxm_step_async.argtypes = [C.c_void_p, C.c_int32, C.c_double]
    L.nxm_frame_wait.argtypes = [C.c_void_p, C.POINTER(C.POINTER(C.c_double)), C.POINTER(Energies), C.c_int32]
    L.nxm_get_pme_grids.argtypes = [C.c_void_p, C.c_int32, dp, dp, dp]
    L.nxm_get_create_timing.argtypes = [C.c_void_p, dp, C.POINTER(C.c_int32)]
    L.nxm_get_layout.argtypes = [C.c_void_p, C.c_int32, np.ctypeslib.ndpointer(np.int32)]
    L.nxm_get_fft_radices.argtypes = [C.c_void_p, C.c_int32, C.c_int32, np.ctypeslib.ndpointer(np.int32),
                                      C.c_int32]
    L.nxm_n_atoms.argtypes = [C.c_void_p, C.POINTER(C.c_int32)]
    L.nxm_save_state.argtypes = [C.c_void_p, C.c_int32, C.c_char_p, C.c_int64, C.c_double]
    _lib = L
    return L


class NxmError(RuntimeError):
    pass


def pair_digest(pairs, n_atoms):
    """Order-independent digest of a pair set: (count, sum over pairs of a
    64-bit mix of the key i * n + j, modulo 2^64).  Two sets with equal
    digests are equal except with probability ~2^-64; used where the sets
    (10^8 pairs) are too large to sort and compare in reasonable time."""
    p = np.asarray(pairs).reshape(-1, 2)
    with np.errstate(over="ignore"):
        k = p[:, 0].astype(np.uint64) * np.uint64(n_atoms) + p[:, 1].astype(np.uint64)
        # splitmix64 finaliser
        k = k + np.uint64(0x9E3779B97F4A7C15)
        k = (k ^ (k >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        k = (k ^ (k >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        k = k ^ (k >> np.uint64(31))
        return int(len(p)), int(k.sum(dtype=np.uint64))


def _check(rc, what=""):
    if rc != 0:
        msg = load_library().nxm_last_error().decode(errors="replace")
        raise NxmError("%s failed (%d): %s" % (what, rc, msg))


def _arr(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


class Engine:
    """A device context holding one batch of systems."""

    def __init__(self, systems, precision=PRECISION_MIXED, skin=0.1, rebuild_interval=10,
                 force_mask=FORCE_ALL, box="reference", grid=None, use_switch=0,
                 switch_dist=0.0, exclusion_depth=3, max_neighbors=0, device=0, exceptions=False,
                 fft_path=0, autotune=True):
        """``force_mask``: one mask for every system, or a sequence with one
        per system; ``box``: "reference" (extent + 1%, as the reference) or "explicit"
        (each system's periodic box [0, L)); ``grid``: None = each system's
        ``grid`` attribute, (0,0,0) = the reference's power-of-two rule;
        ``exceptions``: pass each system's ``exc_idx`` / ``exc_prm`` exception
        pairs (OpenMM semantics) when it has them; ``fft_path``: PME FFT
        launch shape, 0 = autotuned, 1 = line path, 2 = plane path where the
        x-planes fit in shared memory; ``autotune``: time the launch shapes
        that change no result at creation and keep the fastest."""
        L = load_library()
        if not isinstance(systems, (list, tuple)):
            systems = [systems]
        self.systems = list(systems)
        self._keep = []
        descs = (SystemDesc * len(systems))()
        pos = []
        masks = list(force_mask) if isinstance(force_mask, (list, tuple)) else [force_mask] * len(systems)
        if len(masks) != len(systems):
            raise ValueError("one force mask per system")
        for d, s, mask in zip(descs, systems, masks):
            k = dict(m=_arr(s.mass, np.float64), q=_arr(s.charge, np.float64),
                     sg=_arr(s.sigma, np.float64), ep=_arr(s.epsilon, np.float64),
                     ba=_arr(s.bonds, np.int32), bp=_arr(s.bond_prm, np.float64),
                     aa=_arr(s.angles, np.int32), ap=_arr(s.angle_prm, np.float64),
                     ta=_arr(s.torsions, np.int32), tp=_arr(s.torsion_prm, np.float64),
                     tn=_arr(s.torsion_n, np.int32))
            self._keep.append(k)
            d.n_atoms = s.n
            d.masses, d.charges = k["m"].ctypes.data, k["q"].ctypes.data
            d.sigmas, d.epsilons = k["sg"].ctypes.data, k["ep"].ctypes.data
            d.n_bonds, d.bond_atoms, d.bond_params = len(k["ba"]), k["ba"].ctypes.data, k["bp"].ctypes.data
            d.n_angles, d.angle_atoms, d.angle_params = len(k["aa"]), k["aa"].ctypes.data, k["ap"].ctypes.data
            d.n_torsions, d.torsion_atoms = len(k["ta"]), k["ta"].ctypes.data
            d.torsion_params, d.torsion_periodicity = k["tp"].ctypes.data, k["tn"].ctypes.data
            d.cutoff, d.ewald_tolerance = float(s.cutoff), float(s.ewald_tol)
            d.use_switching, d.switching_distance = int(use_switch), float(switch_dist)
            g = s.grid if grid is None else grid
            for i in range(3):
                d.grid[i] = int(g[i])
            if box == "reference":
                d.box_from_positions = 1
            else:
                d.box_from_positions = 0
                for i in range(3):
                    d.box_lb[i], d.box_ub[i] = 0.0, float(s.box[i])
            d.force_mask = int(mask)
            d.exclusion_depth = int(exclusion_depth)
            if exceptions and getattr(s, "exc_idx", None) is not None and len(s.exc_idx):
                k["xi"] = _arr(s.exc_idx, np.int32)
                k["xp"] = _arr(s.exc_prm, np.float64)
                d.n_exceptions = len(k["xi"])
                d.exception_atoms, d.exception_params = k["xi"].ctypes.data, k["xp"].ctypes.data
            pos.append(_arr(s.pos, np.float64))
        self.n_atoms = int(sum(s.n for s in systems))
        opt = Options()
        L.nxm_default_options(C.byref(opt))
        opt.precision, opt.skin, opt.rebuild_interval = int(precision), float(skin), int(rebuild_interval)
        opt.device, opt.max_neighbors = int(device), int(max_neighbors)
        opt.fft_path, opt.autotune = int(fft_path), 1 if autotune else 0
        h = C.c_void_p()
        xyz = pos[0] if len(pos) == 1 else np.concatenate(pos)
        _check(L.nxm_create(descs, len(systems), C.byref(opt), xyz, C.byref(h)), "nxm_create")
        self._h = h
        self._L = L
        self.precision = precision

    def close(self):
        if getattr(self, "_h", None):
            self._L.nxm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- state
    def set_positions(self, xyz):
        _check(self._L.nxm_set_positions(self._h, _arr(xyz, np.float64).reshape(-1, 3)), "set_positions")

    def set_velocities(self, xyz):
        _check(self._L.nxm_set_velocities(self._h, _arr(xyz, np.float64).reshape(-1, 3)), "set_velocities")

    def compute_forces(self):
        _check(self._L.nxm_compute_forces(self._h), "compute_forces")
        return self.forces()

    def step(self, nsteps, dt):
        _check(self._L.nxm_step(self._h, int(nsteps), float(dt)), "step")

    def time_steps(self, nsteps, dt):
        ms = C.c_double()
        _check(self._L.nxm_time_steps(self._h, int(nsteps), float(dt), C.byref(ms)), "time_steps")
        return ms.value

    def time_report_steps(self, nsteps, dt):
        """Device milliseconds of nsteps steps that each compute energies and the snapshot."""
        ms = C.c_double()
        _check(self._L.nxm_time_report_steps(self._h, int(nsteps), float(dt), C.byref(ms)), "time_report_steps")
        return ms.value

    def _get(self, fn):
        out = np.zeros((self.n_atoms, 3))
        _check(fn(self._h, out), fn.__name__)
        return out

    def forces(self):
        return self._get(self._L.nxm_get_forces)

    def snapshot_positions(self):
        return self._get(self._L.nxm_get_positions)

    def snapshot_velocities(self):
        return self._get(self._L.nxm_get_velocities)

    def state(self):
        x = np.zeros((self.n_atoms, 3))
        v = np.zeros((self.n_atoms, 3))
        _check(self._L.nxm_get_state(self._h, x, v), "get_state")
        return x, v

    def energies(self, system=0):
        e = Energies()
        _check(self._L.nxm_get_energies(self._h, int(system), C.byref(e)), "get_energies")
        return e.as_dict()

    def box(self, system=0):
        lb, ub = np.zeros(3), np.zeros(3)
        _check(self._L.nxm_get_box(self._h, int(system), lb, ub), "get_box")
        return lb, ub

    def grid(self, system=0):
        g = np.zeros(3, np.int32)
        _check(self._L.nxm_get_grid(self._h, int(system), g), "get_grid")
        return tuple(int(x) for x in g)

    def alpha(self, system=0):
        a = C.c_double()
        _check(self._L.nxm_get_alpha(self._h, int(system), C.byref(a)), "get_alpha")
        return a.value

    def pairs(self, system=0, sort=True):
        """Neighbour pair set within the cutoff, rows (i, j), i > j; sorted
        by (i, j) unless ``sort`` is False."""
        n = self._L.nxm_get_pairs(self._h, int(system), np.zeros(2, np.int32), 0)
        if n < 0:
            _check(int(n), "get_pairs")
        out = np.zeros(2 * max(n, 1), np.int32)
        n2 = self._L.nxm_get_pairs(self._h, int(system), out, n)
        if n2 < 0:
            _check(int(n2), "get_pairs")
        p = out[:2 * n].reshape(-1, 2)
        return p[np.lexsort((p[:, 1], p[:, 0]))] if sort else p

    def step_async(self, nsteps, dt):
        """Enqueue nsteps steps and the copy of the last one's frame into the
        pinned ring; returns without waiting."""
        _check(self._L.nxm_step_async(self._h, int(nsteps), float(dt)), "step_async")

    def frame_wait(self, copy=True):
        """The oldest pending frame: (positions [n][3], energies of system 0).
        With copy=False the positions are a view of the pinned ring slot,
        valid until that slot is filled again."""
        p = C.POINTER(C.c_double)()
        e = Energies()
        _check(self._L.nxm_frame_wait(self._h, C.byref(p), C.byref(e), 1), "frame_wait")
        x = np.ctypeslib.as_array(p, shape=(self.n_atoms, 3))
        return (x.copy() if copy else x), e.as_dict()

    def pme_grids(self, system=0):
        """(charge grid [K0,K1,K2], influence function [K0,K1,K2//2+1], real
        grid after convolution and inverse transform [K0,K1,K2]) of the last
        force evaluation."""
        K = self.grid(system)
        q = np.zeros(K)
        e = np.zeros((K[0], K[1], K[2] // 2 + 1))
        r = np.zeros(K)
        _check(self._L.nxm_get_pme_grids(self._h, int(system), q, e, r), "get_pme_grids")
        return q, e, r

    CREATE_PHASES = ("host_setup", "device_alloc_upload", "pme_tables_fft_plan", "autotune", "graph_builds",
                     "create_total", "of_which_alloc", "of_which_upload", "of_which_exclusions")

    def create_timing(self):
        """Host milliseconds of context creation by phase, and whether the
        autotuned launch shapes came from an earlier context of the same shapes."""
        ms = np.zeros(len(self.CREATE_PHASES))
        cached = C.c_int32()
        _check(self._L.nxm_get_create_timing(self._h, ms, C.byref(cached)), "get_create_timing")
        d = dict(zip(self.CREATE_PHASES, ms.tolist()))
        d["autotune_cached"] = bool(cached.value)
        return d

    LAYOUT = ("cells_per_group", "hood_capacity", "cells_x", "cells_y", "cells_z", "list_stride",
              "fft_path", "fft_plane_chunked", "fft_passes_x", "fft_passes_y", "fft_passes_z")

    def layout(self, system=0):
        """Cell groups, neighbourhood capacity, cells, list stride and FFT
        plan of one system (``fft_path`` 1 = line path, 2 = plane path) plus
        ``fft_radices``: the radix of each FFT pass per axis."""
        out = np.zeros(len(self.LAYOUT), np.int32)
        _check(self._L.nxm_get_layout(self._h, int(system), out), "get_layout")
        d = dict(zip(self.LAYOUT, (int(x) for x in out)))
        r = []
        for ax in range(3):
            buf = np.zeros(16, np.int32)
            k = self._L.nxm_get_fft_radices(self._h, int(system), ax, buf, len(buf))
            if k < 0:
                _check(int(k), "get_fft_radices")
            r.append(tuple(int(x) for x in buf[:k]))
        d["fft_radices"] = tuple(r)
        return d

    PHASES = ("rebuild", "bonded", "pairs", "exclusions", "spread", "fft", "gather", "integrate")

    def profile(self, nsteps, dt):
        """Average device ms per step of each phase (CUDA events on the engine's stream)."""
        ms = np.zeros(len(self.PHASES))
        _check(self._L.nxm_profile_phases(self._h, int(nsteps), float(dt), ms, len(ms)), "profile")
        return dict(zip(self.PHASES, ms.tolist()))

    def launches_per_step(self):
        a, b = C.c_int32(), C.c_int32()
        _check(self._L.nxm_launches_per_step(self._h, C.byref(a), C.byref(b)), "launches")
        return a.value, b.value

    def tuning(self):
        """Launch shapes in use: (FFT lines per z block or 0 on the plane path,
        FFT columns per x block, spread/gather threads)."""
        out = (C.c_int32 * 3)()
        _check(self._L.nxm_get_tuning(self._h, out), "get_tuning")
        return tuple(out)

    def fft_plane_threads(self):
        """Threads per plane-path FFT block, 0 on the line path."""
        t = C.c_int32()
        _check(self._L.nxm_get_fft_plane_threads(self._h, C.byref(t)), "get_fft_plane_threads")
        return t.value

    def rebuilds(self):
        """Neighbour-list rebuilds since the context was created."""
        n = C.c_int64()
        _check(self._L.nxm_rebuild_count(self._h, C.byref(n)), "rebuild_count")
        return n.value

    def save_state(self, path, system=0, step=0, time=0.0):
        """Checkpoint of one system's current positions and velocities in OpenMM's
        state format (17 significant digits: reading it back gives the same doubles)."""
        _check(self._L.nxm_save_state(self._h, int(system), str(path).encode(), int(step), float(time)),
               "save_state")
