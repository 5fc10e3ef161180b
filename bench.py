#!/usr/bin/env python3
"""Throughput of the NexusMD force-and-integrate step on GB300.

Default workload: the ~94,100-atom chain + flexible-water system in a 9.8 nm
periodic box (4 chains x 250 residues + 28,700 waters, seeded synthetic
stand-in), PME grid 100^3, order 5, cutoff 1.0 nm, Ewald tolerance 5e-4,
neighbour list cutoff + 0.1 nm skin rebuilt at most every 10 steps, leapfrog
dt = 0.5 fs, mixed precision (FP32 forces, int64 fixed-point force sums, FP64
positions/velocities/energies).  A "step" is one full force evaluation plus
the integration update.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl native|reference]

Prints one JSON line (rank 0).  value = atom-steps/s over all ranks, timed on
the device with CUDA events on the engine's stream (max over ranks); e2e =
the same metric through the C ABI from the host: context creation from host
arrays plus one nxm_step(1) call per step with the energies and a position
frame copied back each step.  Under torchrun every rank runs an independent
replica on its own GPU (weak scaling; the path has no exchange step).
--impl reference times the CPU oracle (the FP64 restatement of the
reference's algorithm; the reference itself is x86/Windows-built C++ that is
not present on the GPU host) on all host cores as independent processes.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

DT_PS = 0.0005
WORKLOADS = {
    # name: (config number, description); every system carries its 1-4 pairs
    # as exceptions scaled 0.8333 (Coulomb) / 0.5 (LJ), 1-2 and 1-3 excluded
    "c3": (3, "config3: 94,100-atom chain+water, 9.8 nm box, PME 100^3, rc 1.0 nm, skin 0.1 nm / 10 steps, "
              "1-4 scaled 0.8333/0.5"),
    "c2": (2, "config2: 23,800-atom chain+water, 6.2 nm box, PME 64^3, rc 1.0 nm, skin 0.1 nm / 10 steps"),
    "c1": (1, "config1: 2,700-atom chain+water, 3.0 nm box, PME 32^3, rc 1.0 nm, skin 0.1 nm / 10 steps"),
    "c4": (4, "config4: 32 independent lambda-window systems, 2,000-25,000 atoms each (log-uniform), "
              "one context, PME ~0.1 nm grids"),
    "c5": (5, "config5: ~474,000-atom chain+water, 16.8 nm box, PME 180^3, rc 1.2 nm, tol 1e-5"),
}
# algorithmic FP32 flops per in-cutoff pair (FMA = 2): displacement 3,
# minimum image 6, r^2 5, rsqrt 1, r 1, alpha r 1, erfc + exp 16, Coulomb 6,
# LJ 10, force accumulation 9, energy 2
PAIR_FLOPS = 60
# algorithmic bytes per launch of the HBM-bound kernels (N atoms, G = K0 K1 K2
# grid points): spread N*20 (float4 position + charge) + 4G (grid write);
# gather N*20 + 4G (grid read) + N*24 (int64 x 3 force); integrate 152 per
# atom (x, v FP64 read + write, force words read + zeroed, 1/m)
BYTES = {"spread": (20, 4, 0), "gather": (20, 4, 24), "integrate": (152, 0, 0)}


def kernel_bytes(kernel, n_atoms, grid_points):
    a, g, f = BYTES[kernel]
    return a * n_atoms + g * grid_points + f * n_atoms


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init_pg(ws):
    if ws <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo")
    return dist


def replica_throughput(world, atoms, steps, seconds):
    """Whole-job atom-steps/s of `world` independent replicas of `atoms`
    atoms, each running `steps` steps, timed by the slowest rank."""
    return world * atoms * steps / seconds


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allmax(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()

    def summary(self):
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = max(mx, float(r[2]))
                for k, name in enumerate(names):
                    if r[5 + k].strip().lower().startswith("active"):
                        reasons.add(name)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def fp32_peak_tflops(device):
    """FP32 (no TF32) cuBLAS SGEMM throughput, measured here: the FP32-pipe roof."""
    import torch
    torch.backends.cuda.matmul.allow_tf32 = False
    dev = torch.device("cuda", device)
    n = 8192
    a = torch.randn(n, n, device=dev)
    b = torch.randn(n, n, device=dev)
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize(dev)
    best = 0.0
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        torch.matmul(a, b)
        e.record()
        torch.cuda.synchronize(dev)
        best = max(best, 2.0 * n ** 3 / (s.elapsed_time(e) * 1e-3) / 1e12)
    del a, b
    torch.cuda.empty_cache()
    return best


def probe_library():
    """bench_probe.cu's hardware probes (libnxm_probe.so beside this file)."""
    import ctypes as C
    from nexusmd_gb300 import build as B
    if not os.path.exists(B.PROBE_LIB):
        B.build_probe()
    L = C.CDLL(B.PROBE_LIB)
    for f in (L.nxm_probe_fp32_peak, L.nxm_probe_shared_atomics):
        f.argtypes = [C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    return L


def fma_probe_tflops(device):
    """FP32 FMA throughput from the probe kernel: (scalar FFMA, packed FP32x2
    FFMA2) TFLOP/s."""
    import ctypes as C
    a, b = C.c_double(), C.c_double()
    if probe_library().nxm_probe_fp32_peak(int(device), C.byref(a), C.byref(b)) != 0:
        return None, None
    return a.value, b.value


def shared_atomics_probe(device):
    """Shared-memory atomic adds per SM per clock at random addresses: (64-bit, 32-bit)."""
    import ctypes as C
    a, b = C.c_double(), C.c_double()
    if probe_library().nxm_probe_shared_atomics(int(device), C.byref(a), C.byref(b)) != 0:
        return None, None
    return a.value, b.value


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def traffic_from_profiles(kernel, workload):
    """DRAM bytes per launch from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        f = line.split()
        if len(f) >= 3 and f[0] == kernel and f[1] == workload:
            try:
                return float(f[2])
            except ValueError:
                return None
    return None


def make_system(cfg):
    """The named configuration with its 1-4 pairs as scaled exceptions
    (Coulomb 0.8333, LJ 0.5, 1-2/1-3 excluded)."""
    from nexusmd_gb300 import synthetic as sy
    return sy.with_exceptions(sy.config_system(cfg))


def oracle_desc(o, s):
    return o.describe(s, box_mode=1, lb=[0.0, 0.0, 0.0], ub=list(s.box), exceptions=(s.exc_idx, s.exc_prm))


def cpu_baseline(s, steps=2):
    """FP64 oracle (the reference's algorithm restated in C) on one host core."""
    import numpy as np
    from oracle.nxo import Oracle, build
    build(ref=False)
    o = Oracle()
    d = oracle_desc(o, s)
    t0 = time.perf_counter()
    phases = o.run_timed(d, s.pos, np.zeros_like(s.pos), DT_PS, steps)
    dt = time.perf_counter() - t0
    return {"value": s.n * steps / dt, "unit": "atom-steps/s", "cores": 1, "kind": "port",
            "sample": "%d steps of the %d-atom system, FP64 oracle (C restatement), 1 core, %.1f s; "
                      "phase s/step: %s" % (steps, s.n, dt, ", ".join(
                          "%s %.3f" % (k, v / steps) for k, v in phases.items()))}


def sig(x, d=4):
    """x rounded to d significant digits (compact JSON)."""
    if isinstance(x, float) and x != 0.0 and math.isfinite(x):
        return float("%.*g" % (d, x))
    return x


def _oracle():
    from oracle.nxo import Oracle, build
    build(ref=False)
    return Oracle()


def oracle_reference(o, s):
    """FP64 oracle forces, energies and the oracle's neighbour pair set (the
    reference's voxel list) of one physics-mode system at s.pos."""
    box = o.box_explicit([0.0, 0.0, 0.0], list(s.box))
    eoff, el = o.exclusions(s.n, s.bonds)
    eoff, el = o.union_exclusions(eoff, el, s.exc_idx)
    F0, E0 = o.forces(oracle_desc(o, s), s.pos, box, eoff, el)
    pairs = o.neighbor_pairs(s.pos, box, eoff, el, s.cutoff)
    return F0, E0, pairs


def pe_oracle(E0):
    return (E0["bond"] + E0["angle"] + E0["torsion"] + E0["recip"] + E0["self"] + E0["coulomb"] + E0["vdw"]
            - E0["exclusion"] + E0["exception"])


def force_errors(F, F0, E, E0):
    """rel-RMS and max per-atom force error, potential-energy relative error
    (against the sum of the magnitudes of the nonbonded terms)."""
    import numpy as np
    err = float(np.sqrt(((F - F0) ** 2).sum() / (F0 ** 2).sum()))
    dmax = float(np.sqrt(((F - F0) ** 2).sum(1)).max())
    scale = abs(E0["recip"]) + abs(E0["self"]) + abs(E0["coulomb"]) + abs(E0["vdw"])
    return {"force_rel_rms": sig(err), "max_atom_force_err": sig(dmax),
            "pe_rel_err": sig(abs(E["potential"] - pe_oracle(E0)) / scale)}


def pair_set_check(eng, k, s, ref_pairs, exact):
    """The engine's pair set within the cutoff against the oracle's: sorted
    arrays compared element by element (exact), or order-independent 64-bit
    digests where the sets are too large to sort in reasonable time."""
    import numpy as np
    from nexusmd_gb300.engine import pair_digest
    got = eng.pairs(k, sort=False)
    out = {"pairs": int(len(got)), "oracle_pairs": int(len(ref_pairs))}
    if exact:
        kg = np.sort(got[:, 0].astype(np.int64) * s.n + got[:, 1])
        kr = np.sort(ref_pairs[:, 0].astype(np.int64) * s.n + ref_pairs[:, 1])
        out["equal"] = bool(kg.shape == kr.shape and np.array_equal(kg, kr))
        out["compare"] = "sorted arrays"
    else:
        out["equal"] = pair_digest(got, s.n) == pair_digest(ref_pairs, s.n)
        out["compare"] = "count + 64-bit digest"
    return out


def accuracy_check(s, eng_mixed, exact_pairs=True):
    """The mixed engine against the FP64 oracle on identical positions:
    force and energy errors and the neighbour pair set."""
    o = _oracle()
    F0, E0, pairs = oracle_reference(o, s)
    eng_mixed.set_positions(s.pos)
    F = eng_mixed.compute_forces()
    out = force_errors(F, F0, eng_mixed.energies(), E0)
    return out, pair_set_check(eng_mixed, 0, s, pairs, exact_pairs)


def nve_drift_run(eng, s, steps, every):
    """KE + PE sampled every `every` steps; slope in kJ/mol/ns per degree of freedom (3N)."""
    import numpy as np
    t, e = [], []
    for k in range(steps // every):
        eng.step(every, DT_PS)
        E = eng.energies()
        t.append((k + 1) * every * DT_PS)
        e.append(E["kinetic"] + E["potential"])
    t, e = np.array(t), np.array(e)
    slope = float(np.polyfit(t, e, 1)[0])  # kJ/mol/ps
    return {"value": sig(slope * 1000.0 / (3 * s.n)), "e_total_std": sig(float(e.std()))}


def equilibrated_state(s, v0, kw, equil=4000, rescale_every=100):
    """The synthetic structure is not relaxed: `equil` mixed-precision steps
    with the velocities rescaled to 300 K every `rescale_every` steps (on the
    host) come before any drift measurement."""
    import numpy as np
    from nexusmd_gb300.engine import Engine
    eng = Engine(s, precision=1, **kw)
    eng.set_velocities(v0)
    kT = 0.0083144626 * 300.0
    for _ in range(equil // rescale_every):
        eng.step(rescale_every, DT_PS)
        _, v = eng.state()
        ke = 0.5 * float((s.mass[:, None] * v * v).sum())
        eng.set_velocities(v * np.sqrt(1.5 * s.n * kT / ke))
    x, v = eng.state()
    eng.close()
    return x, v


def skin_sweep(s, v0, kw, steps=1000, skins=(0.10, 0.12, 0.15)):
    """Rebuild rate against list length: device ms per step over `steps`
    steps from the same start for several list skins (the named config uses
    0.1 nm, a rebuild at most every 10 steps)."""
    from nexusmd_gb300.engine import Engine
    out = {}
    for skin in skins:
        k = dict(kw, skin=skin)
        eng = Engine(s, precision=1, **k)
        eng.set_velocities(v0)
        rb0 = eng.rebuilds()
        ms = eng.time_steps(steps, DT_PS)
        ph = eng.profile(20, DT_PS)
        out["%.2f" % skin] = {"ms_per_step": sig(ms / steps), "rebuilds_per_1000": sig((eng.rebuilds() - rb0) * 1000 / steps),
                              "list_radius_nm": sig(s.cutoff + skin), "pairs_phase_ms": sig(ph["pairs"], 3)}
        eng.close()
    out["steps"] = steps
    return out


def nve_drift(s, v0, kw, steps=10000, every=20, fp64_steps=0, equil=4000):
    """NVE total-energy drift without a thermostat from an equilibrated
    state: the mixed engine over `steps` steps and, when fp64_steps > 0, the
    FP64 engine from the same state over fp64_steps steps."""
    from nexusmd_gb300.engine import Engine
    x, v = equilibrated_state(s, v0, kw, equil=equil)
    out = {"unit": "kJ/mol/ns/DOF", "equilibration": "%d mixed steps, velocities rescaled to 300 K every 100" % equil,
           "sample_every": every}
    for prec, n, key in ((1, steps, "mixed"), (0, fp64_steps, "fp64")):
        if n <= 0:
            continue
        eng = Engine(s, precision=prec, **kw)
        eng.set_positions(x)
        eng.set_velocities(v)
        r = nve_drift_run(eng, s, n, every)
        r["steps"] = n
        out[key] = r
        eng.close()
    return out


def batch_accuracy(systems, eng, exact_pairs=True):
    """A (batched) engine against the FP64 oracle run per system: force and
    energy errors and each system's pair set."""
    import numpy as np
    o = _oracle()
    F = eng.compute_forces()
    F0, pe_err, sets = [], 0.0, []
    for k, s in enumerate(systems):
        f, E0, pairs = oracle_reference(o, s)
        F0.append(f)
        scale = abs(E0["recip"]) + abs(E0["self"]) + abs(E0["coulomb"]) + abs(E0["vdw"])
        pe_err = max(pe_err, abs(eng.energies(k)["potential"] - pe_oracle(E0)) / scale)
        sets.append(pair_set_check(eng, k, s, pairs, exact_pairs))
        del pairs
    F0 = np.concatenate(F0)
    err = float(np.sqrt(((F - F0) ** 2).sum() / (F0 ** 2).sum()))
    dmax = float(np.sqrt(((F - F0) ** 2).sum(1)).max())
    acc = {"force_rel_rms": sig(err), "max_atom_force_err": sig(dmax), "pe_rel_err_max_over_systems": sig(pe_err)}
    if len(sets) == 1:
        ps = sets[0]
    else:
        ps = {"systems_equal": sum(x["equal"] for x in sets), "systems": len(sets),
              "pairs": sum(x["pairs"] for x in sets), "compare": sets[0]["compare"]}
    return acc, ps


def other_workload(cfg, steps, warmup, device, check=True, fp64_steps=0):
    """Throughput, accuracy and pair set of another named configuration:
    1 = ~2,700 atoms, 2 = ~23,800 atoms, 4 = the 32-system uneven
    lambda-window batch in one context, 5 = ~474k atoms.  fp64_steps > 0
    also times the FP64 form of the engine on the same systems."""
    import numpy as np
    from nexusmd_gb300 import synthetic as sy
    from nexusmd_gb300.engine import Engine
    if cfg == 4:
        systems = [sy.with_exceptions(x) for x in sy.batch_systems()]
    else:
        systems = [make_system(cfg)]
    n = sum(x.n for x in systems)
    v0 = np.concatenate([sy.maxwell_boltzmann(x.mass, 300.0, seed=1000 + cfg + k) for k, x in enumerate(systems)])
    kw = dict(skin=0.1, rebuild_interval=10, box="explicit", device=device, exceptions=True)
    out = {"workload": WORKLOADS["c%d" % cfg][1], "systems": len(systems), "atoms": n}
    pos0 = np.concatenate([x.pos for x in systems])
    for prec, k_steps, key in ((1, steps, "mixed"), (0, fp64_steps, "fp64")):
        if k_steps <= 0:
            continue
        eng = Engine(systems, precision=prec, **kw)
        eng.set_velocities(v0)
        eng.step(warmup if prec else min(warmup, 5), DT_PS)
        rb0 = eng.rebuilds()
        ms = eng.time_steps(k_steps, DT_PS)
        r = {"value": sig(n * k_steps / (ms * 1e-3)), "unit": "atom-steps/s", "ms_per_step": sig(ms / k_steps),
             "ns_per_day": sig((1.0 / (ms / k_steps * 1e-3)) * DT_PS * 1e-3 * 86400.0), "steps": k_steps,
             "list_rebuilds": eng.rebuilds() - rb0}
        if prec == 1:
            r["phase_ms"] = {k: sig(v, 3) for k, v in eng.profile(20, DT_PS).items()}
        if check:
            eng.set_positions(pos0)
            # pair sets of 10^8 pairs (config 5) by digest, the rest sorted
            acc, ps = batch_accuracy(systems, eng, exact_pairs=n < 300000 or cfg == 4)
            r["accuracy_vs_fp64_oracle"] = acc
            r["pair_set"] = ps
        out[key] = r
        eng.close()
    if "fp64" in out:
        out["mixed_over_fp64"] = sig(out["mixed"]["value"] / out["fp64"]["value"])
    return out


def reporting(cfg, steps, interval, device):
    """Simulate through the dispatcher (XML inputs, the three report files):
    wall time with each report written before the next step (report_threads
    = 0, the reference's schedule) and with the asynchronous reporter
    (pinned double-buffered snapshots, files written on host threads)."""
    import shutil
    import tempfile
    import NexusMD
    from nexusmd_gb300 import synthetic as sy
    s = sy.compat_system(sy.config_system(cfg))
    d = tempfile.mkdtemp(prefix="nxm_rep_")
    sp, st, pdb = sy.write_inputs(s, d, "rep")
    out = {"workload": "config%d compat inputs (%d atoms), mixed precision" % (cfg, s.n), "steps": steps,
           "report_interval": interval, "reports": steps // interval + (interval > 1)}
    cwd = os.getcwd()
    saved, null = os.dup(1), os.open(os.devnull, os.O_WRONLY)
    try:
        os.chdir(d)
        # a short untimed run first (one-time costs), then each mode twice, best kept
        for th, key in ((0, None), (0, "sync_s"), (4, "async_s"), (0, "sync_s"), (4, "async_s")):
            disp = NexusMD.TaskDispatcher.CreateDispatcher("GPU")
            disp.EnableHarmonicBondForce()
            disp.EnableHarmonicAngleForce()
            disp.EnablePeriodicTorsionForce()
            disp.EnableNonbondedForce()
            disp.SetOptions(precision="mixed", autotune=False, report_threads=th, device=device)
            sys.stdout.flush()
            os.dup2(null, 1)  # Simulate prints a line per step
            t0 = time.perf_counter()
            try:
                disp.Simulate(sp, st, pdb, "o%d.pdb" % th, DT_PS, steps if key else 2, interval)
            finally:
                os.dup2(saved, 1)
            if key:
                out[key] = min(out.get(key, 1e30), time.perf_counter() - t0)
            del disp
    finally:
        os.chdir(cwd)
        os.close(null)
        os.close(saved)
        shutil.rmtree(d, ignore_errors=True)
    out["async_speedup"] = out["sync_s"] / out["async_s"]
    return out


def e2e_run(s, v0, kw, steps):
    """Wall seconds of: context creation from host arrays, velocities, then
    `steps` steps with every step's energies and position frame read back
    into pinned host memory through the pipelined C ABI calls."""
    from nexusmd_gb300.engine import Engine
    t0 = time.perf_counter()
    eng = Engine(s, precision=1, **kw)
    t1 = time.perf_counter()
    eng.set_velocities(v0)
    t2 = time.perf_counter()
    eng.step_async(1, DT_PS)
    for _ in range(steps - 1):
        eng.step_async(1, DT_PS)
        eng.frame_wait(copy=False)
    eng.frame_wait(copy=False)
    t3 = time.perf_counter()
    dt = t3 - t0
    create = eng.create_timing()
    # wall milliseconds of the parts: the Python constructor (descriptor
    # arrays + nxm_create), the velocities, the steps with their frames
    create["wall_constructor"] = (t1 - t0) * 1e3
    create["wall_velocities"] = (t2 - t1) * 1e3
    create["wall_steps"] = (t3 - t2) * 1e3
    eng.close()
    return dt, create


def fft_paths(cfg, device):
    """Per-step FFT + convolution time (phase profile, CUDA events) of the
    line path and of the plane path on configuration cfg's system."""
    from nexusmd_gb300.engine import Engine
    s = make_system(cfg)
    out = {}
    for path, name in ((1, "lines"), (2, "planes")):
        eng = Engine(s, precision=1, skin=0.1, rebuild_interval=10, box="explicit", device=device,
                     exceptions=True, fft_path=path)
        lay = eng.layout()
        if lay["fft_path"] != path:
            out[name] = None
        else:
            eng.step(3, DT_PS)
            out[name] = {"fft_ms": sig(eng.profile(20, DT_PS)["fft"], 3),
                         "plane_chunked": bool(lay["fft_plane_chunked"]) if path == 2 else None}
        eng.close()
    out["grid"] = list(s.grid)
    out["radices"] = [list(r) for r in lay["fft_radices"]]
    return out


def workload_config(name, s):
    """The workload as both arms name it: a static description of the system
    and the run parameters (no measured values)."""
    cfg, desc = WORKLOADS[name]
    list_mb = s.n * 3 * 512 / 1e6  # three 512-byte list chunks per atom at ~560 entries
    return {"workload": desc, "atoms": s.n, "box_nm": float(s.box[0]), "pme_grid": list(s.grid),
            "cutoff_nm": s.cutoff, "ewald_tolerance": s.ewald_tol, "skin_nm": 0.1, "rebuild_interval": 10,
            "dt_fs": DT_PS * 1000, "v0": "Maxwell-Boltzmann 300 K",
            "exceptions": "1-4 pairs scaled 0.8333 Coulomb / 0.5 LJ, 1-2 and 1-3 excluded",
            "l2": "inputs larger than L2: the neighbour list alone is ~%.0f MB read per step" % list_mb}


def ordered(out, tail):
    """The JSON line with the keys of `tail` last, in that order: the driver
    keeps only the end of the output, so the target comparison (mixed over
    FP64), the errors, the pair-set checks and the phase split go there."""
    head = {k: v for k, v in out.items() if k not in tail}
    head.update((k, out[k]) for k in tail if k in out)
    return head


def native(args):
    import numpy as np
    from nexusmd_gb300.engine import Engine, load_library
    ws, rank, local = dist_env()
    dist = init_pg(ws)
    cfg, desc = WORKLOADS[args.workload]
    s = make_system(cfg)
    load_library()
    from nexusmd_gb300 import synthetic as sy
    v0 = sy.maxwell_boltzmann(s.mass, 300.0, seed=1000 + cfg)
    kw = dict(skin=0.1, rebuild_interval=10, box="explicit", device=local, exceptions=True)
    eng = Engine(s, precision=1, **kw)
    eng.set_velocities(v0)
    eng.step(args.warmup, DT_PS)
    barrier(dist)
    rb0 = eng.rebuilds()
    with Clocks(local) as clk:
        ms = eng.time_steps(args.steps, DT_PS)
    ms = allmax(dist, ms)
    rebuilds = eng.rebuilds() - rb0
    launches, rb_launches = eng.launches_per_step()
    per_step = ms / args.steps
    value = replica_throughput(ws, s.n, args.steps, ms * 1e-3)

    # end to end through the C ABI from host arrays: context creation and
    # upload of the system, then every step's energies and position frame
    # read back into pinned host memory (nxm_step_async + nxm_frame_wait:
    # the copy of frame k overlaps step k+1)
    create_first = eng.create_timing()
    barrier(dist)
    e2e_s, create = e2e_run(s, v0, kw, args.steps)
    e2e_s = allmax(dist, e2e_s)
    h2d = s.n * (3 + 3 + 4) * 8 + (len(s.bonds) * 24 + len(s.angles) * 28 + len(s.torsions) * 36)
    d2h = s.n * 24 + 16 * 8 + 32

    out = {"metric": "atom-steps/s", "value": value, "unit": "atom-steps/s", "n_gpus": ws,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_step,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32 forces / i64 fixed-point sums / f64 x,v,E",
           "data": "synthetic (seeded chain + flexible water, shapes of the named config)",
           "config": workload_config(args.workload, s),
           "precision": "mixed", "replicas": ws, "list_rebuilds_in_timed_steps": rebuilds,
           "autotuned": dict(zip(("fft_lines_per_z_block", "fft_cols_per_yx_block", "pme_threads_per_block"),
                                 eng.tuning()), fft_plane_threads=eng.fft_plane_threads()),
           "e2e": {"value": replica_throughput(ws, s.n, args.steps, e2e_s), "unit": "atom-steps/s",
                   "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h,
                   "calls": "nxm_create + nxm_set_velocities + K x (nxm_step_async(1) + nxm_frame_wait): "
                            "each step's energies and %d-atom position frame into pinned host memory" % s.n,
                   "create_ms": {k: sig(v, 3) for k, v in create.items()},
                   "create_ms_first_context": {k: sig(v, 3) for k, v in create_first.items()}},
           # per step: the step's kernels (one graph launch); per list rebuild: the rebuild kernels
           "gpu_launches": launches * args.steps + rb_launches * rebuilds,
           "clocks": clk.summary()}
    out["ns_per_day"] = sig((1.0 / (per_step * 1e-3)) * DT_PS * 1e-3 * 86400.0)

    if rank == 0 and ws == 1:
        # per-phase device times (CUDA events on the engine's stream)
        ph = eng.profile(max(20, min(200, args.steps)), DT_PS)
        npairs = len(eng.pairs(sort=False))
        peaks, src = measured_peaks()
        sgemm = fp32_peak_tflops(local)
        fma_s, fma_p = fma_probe_tflops(local)
        fp32 = max(sgemm, fma_s or 0.0, fma_p or 0.0)
        top = max(ph, key=ph.get)
        pair_tf = PAIR_FLOPS * npairs / (ph["pairs"] * 1e-3) / 1e12
        gpts = int(np.prod(s.grid))
        hbm = {}
        for k in BYTES:
            if ph.get(k, 0) > 0:
                b = kernel_bytes(k, s.n, gpts)
                gbs = b / (ph[k] * 1e-3) / 1e9
                hbm[k] = {"achieved": sig(gbs), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                          "frac": sig(gbs / peaks["hbm_gbs"]), "bytes_per_launch": b}
        # the spread is bound by L2 atomic throughput, not HBM: 125 int32
        # atomic adds per atom against the probe's rate for the same pattern
        import ctypes as C
        rate = C.c_double()
        if probe_library().nxm_probe_stencil_atomics(local, int(s.grid[0]), C.byref(rate)) == 0 and ph.get("spread"):
            ach = 125.0 * s.n / (ph["spread"] * 1e-3)
            hbm["spread"]["l2_atomics"] = {"achieved": sig(ach), "peak": sig(rate.value), "unit": "atomics/s",
                                           "frac": sig(ach / rate.value),
                                           "peak_source": "int32 atomic adds in 5^3 stencils at random places "
                                                          "of a %d^3 grid (bench_probe.cu), measured here"
                                                          % s.grid[0]}
        u64, u32 = shared_atomics_probe(local)
        out["roofline"] = {"kernel": "k_pairs_mixed (real-space erfc-Coulomb + LJ)", "bound": "fp32",
                           "achieved": sig(pair_tf), "peak": sig(fp32), "unit": "TFLOP/s",
                           "frac": sig(pair_tf / fp32),
                           "peak_source": "best of the FP32 FMA probe (FFMA %.1f, packed FFMA2 %.1f TFLOP/s) and "
                                          "FP32 SGEMM with TF32 off (%.1f), measured in this run"
                                          % (fma_s or 0.0, fma_p or 0.0, sgemm),
                           "algorithmic": "%d flops x %d in-cutoff pairs per launch" % (PAIR_FLOPS, npairs),
                           "traffic": traffic_from_profiles("k_pairs_mixed", args.workload),
                           "top_phase": top,
                           "shared_atomics_per_clk_sm": {"u64": sig(u64 or 0.0), "u32": sig(u32 or 0.0)}}
        out["roofline_hbm"] = dict(hbm, peak_source="MEASURED_PEAKS.json hbm_gbs (%s)" % src)
        out["phase_ms"] = {k: sig(v, 3) for k, v in ph.items()}
        # a step that computes energies and the snapshot (every step of a
        # loop that reports each step, as the end-to-end loop does)
        out["report_step_ms"] = sig(eng.time_report_steps(max(20, min(200, args.steps)), DT_PS) /
                                    max(20, min(200, args.steps)))
        # the same end-to-end measurement over 1,000 steps
        t_long, _ = e2e_run(s, v0, kw, 1000)
        out["e2e"]["value_1000_steps"] = sig(s.n * 1000 / t_long)
        # and the device-timed throughput of the same 1,000 steps from the
        # same start (a fresh context, its first step the forced list build)
        eng_l = Engine(s, precision=1, **kw)
        eng_l.set_velocities(v0)
        ms_l = eng_l.time_steps(1000, DT_PS)
        eng_l.close()
        out["e2e"]["device_value_1000_steps"] = sig(s.n * 1000 / (ms_l * 1e-3))
        # plain FP64 form of the same engine
        eng64 = Engine(s, precision=0, **kw)
        eng64.set_velocities(v0)
        eng64.step(2, DT_PS)
        k64 = 10 if s.n > 50000 else 20
        ms64 = eng64.time_steps(k64, DT_PS)
        v64 = s.n * k64 / (ms64 * 1e-3)
        out["fp64_plain"] = {"value": sig(v64), "ms_per_step": sig(ms64 / k64), "mixed_over_fp64": sig(value / v64)}
        if not args.no_check:
            acc, ps = accuracy_check(s, eng)
            out["accuracy_vs_fp64_oracle"] = acc
            out["pair_set"] = {args.workload: ps}
            # the FP64 form against the oracle on the same positions
            o = _oracle()
            F0, E0, _ = oracle_reference(o, s)
            eng64.set_positions(s.pos)
            out["fp64_plain"]["accuracy_vs_fp64_oracle"] = force_errors(eng64.compute_forces(), F0, eng64.energies(), E0)
        del eng64
        del eng
        if not args.quick:
            out["nve_drift"] = nve_drift(s, v0, kw, fp64_steps=args.drift_fp64_steps)
            out["skin_sweep"] = skin_sweep(s, v0, kw)
            ow = {"c1": other_workload(1, 2000, 50, local, check=not args.no_check),
                  "c2": other_workload(2, 1000, 50, local, check=not args.no_check, fp64_steps=50),
                  "c4": other_workload(4, 200, 10, local, check=not args.no_check),
                  "c5": other_workload(5, 100, 5, local, check=not args.no_check)}
            out["other_workloads"] = ow
            if not args.no_check:
                for k in ("c2", "c4", "c5"):
                    out["pair_set"][k] = ow[k]["mixed"]["pair_set"]
                out["pair_set"]["c2_fp64"] = ow["c2"]["fp64"]["pair_set"]
            out["fft_paths"] = {"c3": fft_paths(3, local), "c5": fft_paths(5, local)}
            out["simulate_reporting"] = [reporting(1, 400, 1, local), reporting(3, 50, 1, local),
                                         reporting(3, 100, 10, local)]
        if not args.no_cpu:
            out["cpu_baseline"] = cpu_baseline(s, steps=args.cpu_steps)
    out = ordered(out, ("roofline_hbm", "roofline", "e2e", "ns_per_day", "phase_ms", "nve_drift",
                        "accuracy_vs_fp64_oracle", "pair_set", "fp64_plain"))
    if rank == 0:
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def _oracle_worker(cfg, steps, warmup, q):
    import numpy as np
    from oracle.nxo import Oracle
    s = make_system(cfg)
    o = Oracle()
    d = oracle_desc(o, s)
    p, v = s.pos.copy(), np.zeros_like(s.pos)
    if warmup:
        o.run_timed(d, p, v, DT_PS, warmup)
    t0 = time.perf_counter()
    o.run_timed(d, s.pos, np.zeros_like(s.pos), DT_PS, steps)
    q.put((s.n, time.perf_counter() - t0))


def reference(args):
    """The reference's algorithm on the host cores: the FP64 C port of the
    reference (its speed within 3% of the reference compiled from its own
    sources on the same system), one independent replica per core."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    import multiprocessing as mp
    from oracle.nxo import build
    build(ref=False)
    cfg, desc = WORKLOADS[args.workload]
    s = make_system(cfg)
    procs = os.cpu_count() or 1
    # bounded sample: K full steps per process when they fit in ~2 minutes
    # at the port's ~2.7 s per step of the 94,100-atom system on one core
    per_step_s = 2.7 * s.n / 94100.0
    steps = max(1, min(args.steps, int(120.0 / per_step_s)))
    warmup = min(args.warmup, max(0, int(30.0 / per_step_s)))
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_oracle_worker, args=(cfg, steps, warmup, q)) for _ in range(procs)]
    t0 = time.perf_counter()
    for p in ps:
        p.start()
    res = [q.get() for _ in ps]
    for p in ps:
        p.join()
    wall = time.perf_counter() - t0
    n = res[0][0]
    slowest = max(r[1] for r in res)
    value = procs * n * steps / slowest
    out = {"impl": "reference", "metric": "atom-steps/s", "value": value, "unit": "atom-steps/s",
           "n_gpus": ws, "steps": steps, "warmup": warmup, "ms_per_step": slowest / steps * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded chain + flexible water, shapes of the named config)",
           "config": workload_config(args.workload, s),
           "precision": "fp64 (the reference's algorithm)", "replicas": procs,
           "cpu_baseline": {"value": value, "unit": "atom-steps/s", "cores": procs, "kind": "port",
                            "sample": "%d independent processes x %d steps (after %d untimed) of the %d-atom "
                                      "system (FP64 C restatement of the reference, single-threaded per "
                                      "process; measured within 3%% of the reference's own compiled code), "
                                      "wall %.1f s" % (procs, steps, warmup, n, wall)},
           "e2e": {"value": value, "unit": "atom-steps/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=50)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    # single-system workloads; the 32-system batch is reported under other_workloads
    ap.add_argument("--workload", default="c3", choices=sorted(k for k in WORKLOADS if k != "c4"))
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--ref-steps", type=int, default=2)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-check", action="store_true")
    ap.add_argument("--quick", action="store_true", help="skip NVE drift and the other workloads")
    ap.add_argument("--drift-fp64-steps", type=int, default=0,
                    help="also run the FP64 engine's NVE drift over this many steps from the same "
                         "equilibrated state as the mixed one")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        reference(args)
    else:
        native(args)


if __name__ == "__main__":
    main()
