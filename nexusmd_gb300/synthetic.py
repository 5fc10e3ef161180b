"""Seeded synthetic chain + flexible-water systems and their OpenMM-style files.

The workloads NexusMD is exercised on are OpenMM-exported systems (a
`<System>` XML with HarmonicBondForce / HarmonicAngleForce /
PeriodicTorsionForce / NonbondedForce blocks, a `<State>` XML with
`<Positions>`, and a PDB whose ATOM records drive the trajectory writer;
see core/common/src/SystemXMLParser.cpp:18-196, StateXMLParser.cpp:17-37 and
core/baseline/src/Reporter.cpp:122-140).  No such input ships with usable
parameters, so this module builds seeded stand-ins with the shapes of the
five benchmark configurations:

* linear chains of 8-particle residues: harmonic bonds (r0 0.10-0.153 nm,
  k 2.5e5-4.6e5 kJ/mol/nm^2), harmonic angles (theta0 104-120 deg,
  k 300-600 kJ/mol/rad^2), periodic torsions (n 1-3, phase 0/180 deg,
  k 0-10 kJ/mol); charges N(0, 0.3 e) neutralised, sigma 0.1-0.35 nm,
  epsilon 0-0.65 kJ/mol;
* flexible 3-site waters (O -0.834 e, H +0.417 e);
* about 100 atoms/nm^3, no non-excluded contact closer than ``min_dist``.

Everything is numpy; the random stream is PCG64 seeded per system.
"""
from __future__ import annotations

import dataclasses
import math
import os
from typing import Optional

import numpy as np

# Flexible 3-site water (TIP3P geometry with harmonic O-H / H-O-H terms).
WATER_ROH = 0.09572
WATER_KOH = 462750.4
WATER_THETA = math.radians(104.52)
WATER_KTHETA = 836.8
WATER_Q_O, WATER_Q_H = -0.834, 0.417
WATER_SIG_O, WATER_EPS_O = 0.315061, 0.636386
# Water H carries a small LJ core so no charged pair is left without repulsion
# (with eps = 0 a water H can fall onto a negatively charged chain bead).
WATER_SIG_H, WATER_EPS_H = 0.1, 0.05
MASS_O, MASS_H = 15.999, 1.008
CHAIN_MASSES = np.array([12.011, 14.007, 15.999, 32.06])
CHAIN_MASS_P = np.array([0.55, 0.2, 0.2, 0.05])
RESIDUE_NAMES = ["ALA", "GLY", "SER", "LEU", "VAL", "THR", "LYS", "GLU"]
CHAIN_ATOM_NAMES = ["N", "CA", "CB", "CG", "CD", "OG", "C", "O"]


@dataclasses.dataclass
class System:
    """One MD system in plain arrays (atom order = file order)."""

    pos: np.ndarray          # (n, 3) float64, nm
    mass: np.ndarray         # (n,)
    charge: np.ndarray       # (n,) e
    sigma: np.ndarray        # (n,) nm
    epsilon: np.ndarray      # (n,) kJ/mol
    bonds: np.ndarray        # (nb, 2) int32
    bond_prm: np.ndarray     # (nb, 2) [d nm, k kJ/mol/nm^2]
    angles: np.ndarray       # (na, 3) int32
    angle_prm: np.ndarray    # (na, 2) [theta0 rad, k]
    torsions: np.ndarray     # (nt, 4) int32
    torsion_prm: np.ndarray  # (nt, 2) [k kJ/mol, phase rad]
    torsion_n: np.ndarray    # (nt,) int32 periodicity
    box: np.ndarray          # (3,) periodic box edge, nm
    cutoff: float = 1.0
    ewald_tol: float = 5e-4
    grid: tuple = (0, 0, 0)  # (0,0,0) = the reference's power-of-two rule
    res_name: Optional[list] = None
    atom_name: Optional[list] = None
    res_seq: Optional[np.ndarray] = None
    # NonbondedForce exceptions (OpenMM semantics): pairs and
    # [chargeProd e^2, sigma nm, epsilon kJ/mol]; None = none
    exc_idx: Optional[np.ndarray] = None
    exc_prm: Optional[np.ndarray] = None

    @property
    def n(self) -> int:
        return int(self.pos.shape[0])


# ---------------------------------------------------------------------------
# geometry helpers

def _place(a, b, c, bond, angle, torsion):
    """Position of d with |cd| = bond, angle(b,c,d) = angle, dihedral(a,b,c,d) = torsion."""
    bc = c - b
    bc /= np.linalg.norm(bc)
    n = np.cross(b - a, bc)
    nn = np.linalg.norm(n)
    if nn < 1e-9:
        n = np.cross(bc, np.array([1.0, 0.0, 0.0]))
        if np.linalg.norm(n) < 1e-6:
            n = np.cross(bc, np.array([0.0, 1.0, 0.0]))
        nn = np.linalg.norm(n)
    n /= nn
    m = np.cross(n, bc)
    d2 = np.array([-bond * math.cos(angle),
                   bond * math.sin(angle) * math.cos(torsion),
                   bond * math.sin(angle) * math.sin(torsion)])
    return c + d2[0] * bc + d2[1] * m + d2[2] * n


class _Grid:
    """Periodic cell hash of growing chain beads (supports removing the newest)."""

    def __init__(self, box, cell, cap):
        self.box = np.asarray(box, float)
        self.nc = np.maximum((self.box / cell).astype(int), 1)
        self.cell = self.box / self.nc
        self.cells: dict = {}
        self.P = np.zeros((cap, 3))
        self.chain = np.zeros(cap, np.int64)
        self.idx = np.zeros(cap, np.int64)
        self.keys: list = []
        self.n = 0

    def _key(self, p):
        return tuple(np.floor(np.mod(p, self.box) / self.cell).astype(int) % self.nc)

    def add(self, p, chain, idx):
        k = self._key(p)
        self.P[self.n], self.chain[self.n], self.idx[self.n] = p, chain, idx
        self.cells.setdefault(k, []).append(self.n)
        self.keys.append(k)
        self.n += 1

    def pop(self):
        self.n -= 1
        self.cells[self.keys.pop()].pop()

    def around(self, p, reach=1):
        c = np.array(self._key(p))
        out = []
        for dx in range(-reach, reach + 1):
            for dy in range(-reach, reach + 1):
                for dz in range(-reach, reach + 1):
                    out.extend(self.cells.get(tuple((c + (dx, dy, dz)) % self.nc), ()))
        return np.asarray(out, np.int64)


def _contacts(p, L, mol, is_h, min_dist, h_min_dist):
    """Intermolecular pairs closer than min_dist (h_min_dist if either atom is a water H)."""
    from scipy.spatial import cKDTree
    tree = cKDTree(p, boxsize=L)
    pr = tree.query_pairs(min_dist, output_type="ndarray")
    if len(pr) == 0:
        return pr
    pr = pr[mol[pr[:, 0]] != mol[pr[:, 1]]]
    d = p[pr[:, 0]] - p[pr[:, 1]]
    d -= L * np.round(d / L)
    r = np.sqrt((d * d).sum(1))
    lim = np.where(is_h[pr[:, 0]] | is_h[pr[:, 1]], h_min_dist, min_dist)
    return pr[r < lim]


# ---------------------------------------------------------------------------
# builders

def _grow_chain(rng, n_beads, center, radius, box, grid, chain_id, min_dist, tries=48):
    """Self-avoiding compact walk confined to a sphere; returns (pos, r0, theta0).

    Each bead is placed at its bond length and bond angle from the previous
    two with a random torsion (away from 0/180 degrees); all ``tries``
    torsions are tested at once against beads of other molecules and beads
    four or more bonds back, and on a dead end the walk backs up."""
    r0 = rng.uniform(0.10, 0.153, size=n_beads - 1)
    th0 = np.radians(rng.uniform(104.0, 120.0, size=n_beads - 2))
    L = np.asarray(box, float)
    pos = np.zeros((n_beads, 3))
    pos[0] = center + rng.normal(0, 0.05, 3)
    v = rng.normal(size=3)
    v /= np.linalg.norm(v)
    pos[1] = pos[0] + r0[0] * v
    w = np.cross(v, rng.normal(size=3))
    w /= np.linalg.norm(w)
    pos[2] = pos[1] + r0[1] * (-math.cos(th0[0]) * v + math.sin(th0[0]) * w)
    for k in range(3):
        grid.add(pos[k], chain_id, k)
    i, iters = 3, 0
    stuck = np.zeros(n_beads, np.int64)
    while i < n_beads:
        iters += 1
        if iters > 200 * n_beads:
            raise RuntimeError("chain growth stuck")
        a, b, c = pos[i - 3], pos[i - 2], pos[i - 1]
        bc = (c - b) / np.linalg.norm(c - b)
        nrm = np.cross(b - a, bc)
        nrm /= np.linalg.norm(nrm)
        m = np.cross(nrm, bc)
        tor = rng.uniform(0.3, math.pi - 0.3, size=tries) * rng.choice([-1.0, 1.0], size=tries)
        bl, an = r0[i - 1], th0[i - 2]
        cand = (c - bl * math.cos(an) * bc
                + (bl * math.sin(an) * np.cos(tor))[:, None] * m
                + (bl * math.sin(an) * np.sin(tor))[:, None] * nrm)
        ok = np.linalg.norm(cand - center, axis=1) <= radius
        ids = grid.around(c)
        if len(ids):
            keep = ~((grid.chain[ids] == chain_id) & (grid.idx[ids] > i - 4))
            ids = ids[keep]
        if len(ids) and ok.any():
            d = cand[:, None, :] - grid.P[ids][None, :, :]
            d -= L * np.round(d / L)
            ok &= ((d * d).sum(-1) >= min_dist * min_dist).all(1)
        hit = np.nonzero(ok)[0]
        if len(hit):
            pos[i] = cand[hit[0]]
            grid.add(pos[i], chain_id, i)
            i += 1
        else:
            # back up further every time the walk dead-ends at this bead
            stuck[i] += 1
            back = int(min(i - 3, stuck[i]))
            if back <= 0:
                raise RuntimeError("chain growth stuck")
            for _ in range(back):
                grid.pop()
            i -= back
    return pos, r0, th0


def make_system(n_chains: int, residues: int, n_waters: int, box: float, seed: int,
                cutoff: float = 1.0, ewald_tol: float = 5e-4, grid=(0, 0, 0),
                beads_per_residue: int = 8, min_dist: float = 0.2, h_min_dist: float = 0.15,
                jitter: float = 0.0015,
                chain_charge_scale: float = 1.0) -> System:
    """Build a periodic chain + water system in a cubic box of edge ``box`` nm."""
    rng = np.random.Generator(np.random.PCG64(seed))
    L = np.array([box, box, box], float)
    n_bead = residues * beads_per_residue
    beads = _Grid(L, 0.4, max(1, n_chains * n_bead))
    # chain globules: about 35 beads/nm^3, centres on a coarse lattice
    radius = (3.0 * n_bead / (4.0 * math.pi * 35.0)) ** (1.0 / 3.0) if n_chains else 0.0
    m = max(1, int(math.ceil(n_chains ** (1.0 / 3.0))))
    centres = []
    for a in range(m):
        for b in range(m):
            for c in range(m):
                centres.append((np.array([a, b, c]) + 0.5) * box / m)
    rng.shuffle(centres)
    chains = []
    for ci in range(n_chains):
        chains.append(_grow_chain(rng, n_bead, centres[ci], radius, L, beads, ci, min_dist + 0.02))
    chain_pos = np.concatenate([c[0] for c in chains]) if chains else np.zeros((0, 3))
    chain_pos = np.mod(chain_pos, L)

    # water oxygen sites: jittered cubic lattice, away from chain beads
    from scipy.spatial import cKDTree
    tree_c = cKDTree(chain_pos, boxsize=L) if len(chain_pos) else None
    frac = 1.0
    for _ in range(40):
        per = int(math.ceil((n_waters * frac) ** (1.0 / 3.0)))
        a = box / per
        g = (np.stack(np.meshgrid(*[np.arange(per)] * 3, indexing="ij"), -1).reshape(-1, 3) + 0.5) * a
        if tree_c is not None:
            d, _ = tree_c.query(g, k=1)
            g = g[d > 0.27]
        if len(g) >= n_waters:
            break
        frac *= 1.06
    else:
        raise RuntimeError("cannot fit waters")
    pick = rng.choice(len(g), size=n_waters, replace=False)
    O = np.mod(g[np.sort(pick)] + rng.uniform(-0.015, 0.015, size=(n_waters, 3)), L)

    def orient(k):
        u = rng.normal(size=(k, 3))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        w = rng.normal(size=(k, 3))
        w -= (w * u).sum(1, keepdims=True) * u
        w /= np.linalg.norm(w, axis=1, keepdims=True)
        h = 0.5 * WATER_THETA
        d1 = math.cos(h) * u + math.sin(h) * w
        d2 = math.cos(h) * u - math.sin(h) * w
        return d1 * WATER_ROH, d2 * WATER_ROH

    H1d, H2d = orient(n_waters)
    nc = len(chain_pos)
    mol = np.concatenate([-1 - np.repeat(np.arange(n_chains), n_bead), np.tile(np.arange(n_waters), 3)])
    is_h = np.concatenate([np.zeros(nc + n_waters, bool), np.ones(2 * n_waters, bool)])
    for _ in range(400):
        H1 = np.mod(O + H1d, L)
        H2 = np.mod(O + H2d, L)
        bad = _contacts(np.concatenate([chain_pos, O, H1, H2]), L, mol, is_h, min_dist, h_min_dist)
        if len(bad) == 0:
            break
        badmol = np.unique(np.concatenate([mol[bad[:, 0]], mol[bad[:, 1]]]))
        badmol = badmol[badmol >= 0]
        if len(badmol) == 0:
            raise RuntimeError("chain-chain contact below min_dist")
        a1, a2 = orient(len(badmol))
        H1d[badmol], H2d[badmol] = a1, a2
        # nudge oxygens a little too so that jammed sites can resolve
        O[badmol] = np.mod(O[badmol] + rng.uniform(-0.01, 0.01, size=(len(badmol), 3)), L)
    else:
        raise RuntimeError("water orientations did not converge (%d contacts)" % len(bad))

    # ---- assemble arrays in file order: chains first, then waters (O, H, H)
    n_total = n_chains * n_bead + 3 * n_waters
    pos = np.zeros((n_total, 3))
    mass = np.zeros(n_total)
    q = np.zeros(n_total)
    sig = np.zeros(n_total)
    eps = np.zeros(n_total)
    bonds, bprm, angles, aprm, tors, tprm, tn = [], [], [], [], [], [], []
    res_name, atom_name, res_seq = [], [], []
    off = 0
    for ci, (cp, r0, th0) in enumerate(chains):
        idx = off + np.arange(n_bead)
        pos[idx] = np.mod(cp, L)
        mass[idx] = rng.choice(CHAIN_MASSES, size=n_bead, p=CHAIN_MASS_P)
        qq = rng.normal(0.0, 0.3, size=n_bead)
        q[idx] = (qq - qq.mean()) * chain_charge_scale
        sig[idx] = rng.uniform(0.1, 0.35, size=n_bead)
        eps[idx] = rng.uniform(0.05, 0.65, size=n_bead)  # within the 0-0.65 range, no bare charges
        for k in range(n_bead - 1):
            bonds.append((idx[k], idx[k + 1]))
            bprm.append((r0[k], rng.uniform(2.5e5, 4.6e5)))
        for k in range(n_bead - 2):
            angles.append((idx[k], idx[k + 1], idx[k + 2]))
            aprm.append((th0[k], rng.uniform(300.0, 600.0)))
        for k in range(n_bead - 3):
            tors.append((idx[k], idx[k + 1], idx[k + 2], idx[k + 3]))
            tprm.append((rng.uniform(0.0, 10.0), math.pi * rng.integers(0, 2)))
            tn.append(int(rng.integers(1, 4)))
        for k in range(n_bead):
            r = k // beads_per_residue
            res_name.append(RESIDUE_NAMES[(r + ci) % len(RESIDUE_NAMES)])
            atom_name.append(CHAIN_ATOM_NAMES[k % beads_per_residue])
            res_seq.append(r + 1)
        off += n_bead
    o = off + 3 * np.arange(n_waters)
    pos[o] = O
    pos[o + 1] = np.mod(O + H1d, L)
    pos[o + 2] = np.mod(O + H2d, L)
    mass[o], mass[o + 1], mass[o + 2] = MASS_O, MASS_H, MASS_H
    q[o], q[o + 1], q[o + 2] = WATER_Q_O, WATER_Q_H, WATER_Q_H
    sig[o], sig[o + 1], sig[o + 2] = WATER_SIG_O, WATER_SIG_H, WATER_SIG_H
    eps[o], eps[o + 1], eps[o + 2] = WATER_EPS_O, WATER_EPS_H, WATER_EPS_H
    if jitter > 0:
        # thermal-scale displacement so that bonds and angles start away from
        # their minima; atoms whose move would create a contact keep their place
        moved = pos + np.clip(rng.normal(0.0, jitter, size=pos.shape), -3 * jitter, 3 * jitter)
        molid = np.concatenate([np.repeat(-1 - np.arange(n_chains), n_bead),
                                off + np.repeat(np.arange(n_waters), 3)])
        isH = np.zeros(n_total, bool)
        isH[o + 1] = True
        isH[o + 2] = True
        bad = _contacts(np.mod(moved, L), L, molid, isH, min_dist, h_min_dist)
        if len(bad):
            back = np.unique(bad.reshape(-1))
            moved[back] = pos[back]
        pos = np.mod(moved, L)
    last_res = (res_seq[-1] if res_seq else 0)
    for w in range(n_waters):
        bonds.append((o[w], o[w] + 1))
        bprm.append((WATER_ROH, WATER_KOH))
        bonds.append((o[w], o[w] + 2))
        bprm.append((WATER_ROH, WATER_KOH))
        angles.append((o[w] + 1, o[w], o[w] + 2))
        aprm.append((WATER_THETA, WATER_KTHETA))
        res_name += ["HOH"] * 3
        atom_name += ["O", "H1", "H2"]
        res_seq += [last_res + 1 + w] * 3

    def arr(x, shape, dt):
        return np.asarray(x, dt).reshape(shape)

    return System(pos=pos, mass=mass, charge=q, sigma=sig, epsilon=eps,
                  bonds=arr(bonds, (-1, 2), np.int32), bond_prm=arr(bprm, (-1, 2), float),
                  angles=arr(angles, (-1, 3), np.int32), angle_prm=arr(aprm, (-1, 2), float),
                  torsions=arr(tors, (-1, 4), np.int32), torsion_prm=arr(tprm, (-1, 2), float),
                  torsion_n=arr(tn, (-1,), np.int32), box=L, cutoff=cutoff,
                  ewald_tol=ewald_tol, grid=tuple(grid), res_name=res_name,
                  atom_name=atom_name, res_seq=np.asarray(res_seq, np.int32))


# ---------------------------------------------------------------------------
# the five benchmark shapes

def config_system(config: int, seed: Optional[int] = None, scale_chain_charge: float = 1.0) -> System:
    """Synthetic stand-in for benchmark configuration ``config`` (1, 2, 3 or 5).

    1: ~2,700 atoms, 3.0 nm box, grid 32^3      2: ~23,800 atoms, 6.2 nm, 64^3
    3: ~94,100 atoms, 9.8 nm, 100^3             5: ~474,000 atoms, 16.8 nm, 180^3,
                                                   cutoff 1.2 nm, Ewald tolerance 1e-5
    Configuration 4 (a batch of uneven systems) is built by ``batch_systems``.
    """
    s = 1000 + config if seed is None else seed
    if config == 1:
        return make_system(1, 60, 740, 3.0, s, grid=(32, 32, 32))
    if config == 2:
        return make_system(1, 200, 7400, 6.2, s, grid=(64, 64, 64))
    if config == 3:
        return make_system(4, 250, 28700, 9.8, s, grid=(100, 100, 100))
    if config == 5:
        return make_system(16, 300, 145000, 16.8, s, cutoff=1.2, ewald_tol=1e-5,
                           grid=(180, 180, 180))
    raise ValueError("config must be 1, 2, 3 or 5 (4 is batch_systems)")


def smooth_grid(n: int) -> int:
    """Smallest 2^a 3^b 5^c >= n."""
    m = n
    while True:
        k = m
        for p in (2, 3, 5):
            while k % p == 0:
                k //= p
        if k == 1:
            return m
        m += 1


def batch_systems(count: int = 32, seed: int = 1004, lo: int = 2000, hi: int = 25000):
    """Uneven lambda-window batch: atom counts log-uniform in [lo, hi], chain charges x lambda."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sizes = np.exp(rng.uniform(math.log(lo), math.log(hi), size=count))
    lams = np.linspace(0.0, 1.0, count)
    out = []
    for k, (n, lam) in enumerate(zip(sizes, lams)):
        L = (n / 100.0) ** (1.0 / 3.0)
        residues = max(2, int(round(0.08 * n / 8)))
        n_w = int(round((n - 8 * residues) / 3))
        K = smooth_grid(int(math.ceil(L / 0.1)))
        out.append(make_system(1, residues, n_w, L, seed * 100 + k, grid=(K, K, K),
                               chain_charge_scale=float(lam)))
    return out


# ---------------------------------------------------------------------------
# the reference's conventions

def reference_box(pos: np.ndarray):
    """Box the reference derives from positions: extent plus 1% on each side.

    core/common/src/PeriodicBoundaryCondition.cpp:20-86 (the water branch, which
    leaves lb/ub at the extent, then applies the 1% margin).
    """
    lb = pos.min(0)
    ub = pos.max(0)
    size = np.abs(ub - lb)
    margin = 0.01 * size
    lb = lb - margin
    ub = ub + margin
    return lb, ub, np.abs(ub - lb)


def compat_system(sys_: System, min_dist: float = 0.2, h_min_dist: float = 0.15,
                  max_iter: int = 50) -> System:
    """Make ``sys_`` well-behaved under the reference's extent-derived box.

    The reference ignores the state file's box and uses the atom extent plus 1%
    per side (PeriodicBoundaryCondition.cpp:20-86).  Molecules are made whole
    (no bond spans the box), then waters that would clash through that box are
    deleted until no intermolecular pair is closer than the contact limits.
    """
    s = dataclasses.replace(sys_)
    pos = s.pos.copy()
    L = s.box
    for b in range(len(s.bonds)):  # bonds are listed along each molecule
        i, j = s.bonds[b]
        d = pos[j] - pos[i]
        pos[j] -= L * np.round(d / L)
    keep = np.ones(s.n, bool)
    mol = _molecule_ids(s.n, s.bonds)
    is_h = np.array([(r == "HOH" and a != "O") for r, a in zip(s.res_name, s.atom_name)])
    is_w = np.array([r == "HOH" for r in s.res_name])
    for _ in range(max_iter):
        idx = np.nonzero(keep)[0]
        lb, ub, size = reference_box(pos[idx])
        p = np.mod(pos[idx] - lb, size)
        pr = _contacts(p, size, mol[idx], is_h[idx], min_dist, h_min_dist)
        if len(pr) == 0:
            break
        bad = set()
        for a, b in pr:
            ia, ib = idx[a], idx[b]
            if is_w[ib]:
                bad.add(mol[ib])
            elif is_w[ia]:
                bad.add(mol[ia])
            else:
                raise RuntimeError("chain atoms clash through the derived box")
        keep &= ~np.isin(mol, list(bad))
    else:
        raise RuntimeError("compat clash removal did not converge")
    return subset(dataclasses.replace(s, pos=pos), np.nonzero(keep)[0])


def _molecule_ids(n, bonds):
    parent = np.arange(n)

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a
    for i, j in bonds:
        ri, rj = find(i), find(j)
        if ri != rj:
            parent[max(ri, rj)] = min(ri, rj)
    return np.array([find(i) for i in range(n)])


def subset(s: System, keep: np.ndarray) -> System:
    """Keep atoms ``keep`` (sorted indices); terms touching dropped atoms go too."""
    remap = -np.ones(s.n, np.int64)
    remap[keep] = np.arange(len(keep))

    def terms(t, *prm):
        ok = np.all(remap[t] >= 0, axis=1) if len(t) else np.zeros(0, bool)
        return (remap[t[ok]].astype(np.int32),) + tuple(p[ok] for p in prm)
    b, bp = terms(s.bonds, s.bond_prm)
    a, ap = terms(s.angles, s.angle_prm)
    t, tp, tn = terms(s.torsions, s.torsion_prm, s.torsion_n)
    pick = lambda lst: [lst[i] for i in keep] if lst is not None else None
    xi = xp = None
    if s.exc_idx is not None:
        xi, xp = terms(np.asarray(s.exc_idx), np.asarray(s.exc_prm))
    return dataclasses.replace(
        s, pos=s.pos[keep].copy(), mass=s.mass[keep].copy(), charge=s.charge[keep].copy(),
        sigma=s.sigma[keep].copy(), epsilon=s.epsilon[keep].copy(), bonds=b, bond_prm=bp,
        angles=a, angle_prm=ap, torsions=t, torsion_prm=tp, torsion_n=tn,
        res_name=pick(s.res_name), atom_name=pick(s.atom_name),
        res_seq=s.res_seq[keep].copy() if s.res_seq is not None else None, exc_idx=xi, exc_prm=xp)


COULOMB14 = 1.0 / 1.2  # 0.8333, the AMBER-style 1-4 Coulomb scale
LJ14 = 0.5


def with_exceptions(s: System, coulomb14: float = COULOMB14, lj14: float = LJ14) -> System:
    """The system with its 1-4 pairs as scaled exceptions, the way OpenMM's
    NonbondedForce.createExceptionsFromBonds makes them: chargeProd =
    coulomb14 q_i q_j, sigma = (sigma_i + sigma_j) / 2, epsilon = lj14
    sqrt(eps_i eps_j).  1-4 pairs are the end atoms of the torsions (the
    chains here have no rings, so no pair is also 1-2 or 1-3)."""
    if len(s.torsions):
        p = np.sort(np.asarray(s.torsions)[:, [0, 3]], axis=1)
        p = np.unique(p, axis=0).astype(np.int32)
    else:
        p = np.zeros((0, 2), np.int32)
    i, j = p[:, 0], p[:, 1]
    prm = np.stack([coulomb14 * s.charge[i] * s.charge[j], 0.5 * (s.sigma[i] + s.sigma[j]),
                    lj14 * np.sqrt(s.epsilon[i] * s.epsilon[j])], axis=1) if len(p) else np.zeros((0, 3))
    return dataclasses.replace(s, exc_idx=p, exc_prm=prm)


# ---------------------------------------------------------------------------
# OpenMM-style files

def write_system_xml(s: System, path: str, use_switch: bool = False, switch_dist: float = 0.0):
    """System XML with the elements/attributes SystemXMLParser.cpp:18-196 reads."""
    out = ['<?xml version="1.0" ?>',
           '<System openmmVersion="8.1.1" type="System" version="1">',
           '\t<PeriodicBoxVectors>',
           '\t\t<A x="%.17g" y="0" z="0"/>' % s.box[0],
           '\t\t<B x="0" y="%.17g" z="0"/>' % s.box[1],
           '\t\t<C x="0" y="0" z="%.17g"/>' % s.box[2],
           '\t</PeriodicBoxVectors>', '\t<Particles>']
    out += ['\t\t<Particle mass="%.17g"/>' % m for m in s.mass]
    out += ['\t</Particles>', '\t<Constraints/>', '\t<Forces>']
    out.append('\t\t<Force forceGroup="0" name="HarmonicBondForce" type="HarmonicBondForce" usesPeriodic="0" version="2">')
    out.append('\t\t\t<Bonds>')
    out += ['\t\t\t\t<Bond d="%.17g" k="%.17g" p1="%d" p2="%d"/>' % (p[0], p[1], b[0], b[1])
            for b, p in zip(s.bonds, s.bond_prm)]
    out += ['\t\t\t</Bonds>', '\t\t</Force>']
    out.append('\t\t<Force forceGroup="0" name="HarmonicAngleForce" type="HarmonicAngleForce" usesPeriodic="0" version="2">')
    out.append('\t\t\t<Angles>')
    out += ['\t\t\t\t<Angle a="%.17g" k="%.17g" p1="%d" p2="%d" p3="%d"/>' % (p[0], p[1], a[0], a[1], a[2])
            for a, p in zip(s.angles, s.angle_prm)]
    out += ['\t\t\t</Angles>', '\t\t</Force>']
    out.append('\t\t<Force forceGroup="0" name="PeriodicTorsionForce" type="PeriodicTorsionForce" usesPeriodic="0" version="2">')
    out.append('\t\t\t<Torsions>')
    out += ['\t\t\t\t<Torsion k="%.17g" p1="%d" p2="%d" p3="%d" p4="%d" periodicity="%d" phase="%.17g"/>'
            % (p[0], t[0], t[1], t[2], t[3], n, p[1])
            for t, p, n in zip(s.torsions, s.torsion_prm, s.torsion_n)]
    out += ['\t\t\t</Torsions>', '\t\t</Force>']
    nx, ny, nz = s.grid
    out.append('\t\t<Force alpha="0" cutoff="%.17g" dispersionCorrection="0" ewaldTolerance="%.17g" '
               'exceptionsUsePeriodic="0" forceGroup="0" includeDirectSpace="1" ljAlpha="0" ljnx="0" '
               'ljny="0" ljnz="0" method="4" name="NonbondedForce" nx="%d" ny="%d" nz="%d" '
               'recipForceGroup="-1" rfDielectric="78.3" switchingDistance="%.17g" type="NonbondedForce" '
               'useSwitchingFunction="%d" version="4">'
               % (s.cutoff, s.ewald_tol, nx, ny, nz, switch_dist, int(use_switch)))
    out.append('\t\t\t<GlobalParameters/>')
    out.append('\t\t\t<ParticleOffsets/>')
    out.append('\t\t\t<ExceptionOffsets/>')
    out.append('\t\t\t<Particles>')
    out += ['\t\t\t\t<Particle eps="%.17g" q="%.17g" sig="%.17g"/>' % (e, c, g)
            for c, g, e in zip(s.charge, s.sigma, s.epsilon)]
    out.append('\t\t\t</Particles>')
    if s.exc_idx is not None and len(s.exc_idx):
        out.append('\t\t\t<Exceptions>')
        out += ['\t\t\t\t<Exception eps="%.17g" p1="%d" p2="%d" q="%.17g" sig="%.17g"/>' % (p[2], e[0], e[1], p[0], p[1])
                for e, p in zip(s.exc_idx, s.exc_prm)]
        out.append('\t\t\t</Exceptions>')
    else:
        out.append('\t\t\t<Exceptions/>')
    out += ['\t\t</Force>', '\t</Forces>', '</System>']
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


def write_state_xml(s: System, path: str):
    """State XML with <PeriodicBoxVectors> and <Positions> (StateXMLParser.cpp:17-37)."""
    out = ['<?xml version="1.0" ?>',
           '<State openmmVersion="8.1.1" stepCount="0" time="0" type="State" version="1">',
           '\t<PeriodicBoxVectors>',
           '\t\t<A x="%.17g" y="0" z="0"/>' % s.box[0],
           '\t\t<B x="0" y="%.17g" z="0"/>' % s.box[1],
           '\t\t<C x="0" y="0" z="%.17g"/>' % s.box[2],
           '\t</PeriodicBoxVectors>', '\t<Positions>']
    out += ['\t\t<Position x="%.17g" y="%.17g" z="%.17g"/>' % tuple(p) for p in s.pos]
    out += ['\t</Positions>', '</State>']
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


def write_pdb(s: System, path: str):
    """PDB whose ATOM records use the whitespace layout Reporter.cpp:109-118 parses."""
    lines = ["REMARK    synthetic chain + water system",
             "CRYST1%9.3f%9.3f%9.3f  90.00  90.00  90.00 P 1           1" % tuple(10.0 * s.box)]
    for i in range(s.n):
        x, y, z = 10.0 * s.pos[i]
        an = s.atom_name[i] if s.atom_name else "C"
        rn = s.res_name[i] if s.res_name else "UNK"
        rs = int(s.res_seq[i]) if s.res_seq is not None else 1
        rs = rs % 10000
        lines.append("ATOM  %5d  %-3s %3s  %4d    %8.3f%8.3f%8.3f  1.00  0.00          %2s"
                     % ((i + 1) % 100000, an, rn, rs, x, y, z, an[0]))
    lines.append("END")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def write_inputs(s: System, directory: str, stem: str, **kw):
    """Write system/state XML and PDB; returns their paths."""
    os.makedirs(directory, exist_ok=True)
    sp = os.path.join(directory, "system_%s.xml" % stem)
    st = os.path.join(directory, "state_%s.xml" % stem)
    pdb = os.path.join(directory, "%s.pdb" % stem)
    write_system_xml(s, sp, **kw)
    write_state_xml(s, st)
    write_pdb(s, pdb)
    return sp, st, pdb


def maxwell_boltzmann(mass: np.ndarray, temperature: float, seed: int) -> np.ndarray:
    """Velocities (nm/ps) drawn at ``temperature`` K with zero net momentum."""
    kB = 0.0083144626  # kJ/mol/K
    rng = np.random.Generator(np.random.PCG64(seed))
    sd = np.sqrt(kB * temperature / mass)[:, None]
    v = rng.normal(size=(len(mass), 3)) * sd
    p = (v * mass[:, None]).sum(0) / mass.sum()
    return v - p
