"""Why the pair kernel walks a full per-atom list rather than a half list of
cluster-pair tiles: interactions evaluated per in-cutoff pair on the
config-2 system (23,800 atoms, rc 1.0 nm, list radius 1.1 nm), CPU only.

* per-atom full list: every atom lists the atoms within the list radius, so
  each pair is evaluated twice: 2 * (pairs within 1.1) / (pairs within 1.0);
* half list of M x M cluster pairs: M consecutive atoms of a z-sorted x-y
  column per cluster, a cluster pair listed once when the bounding boxes
  come within the list radius; M*M interactions per cluster pair, M(M-1)/2
  per cluster with itself (padding lanes counted as evaluated).

The tiles evaluate more than the full list at every cluster size tried, so
halving the list through tiles would not pay even before the cost of
reducing the j-side forces.
"""
import numpy as np
import pytest

scipy_spatial = pytest.importorskip("scipy.spatial")


def _clusters(pos, L, M, col):
    nc = int(L // col)
    cs = L / nc
    cx = np.minimum((pos[:, 0] / cs).astype(int), nc - 1)
    cy = np.minimum((pos[:, 1] / cs).astype(int), nc - 1)
    key = cx * nc + cy
    order = np.lexsort((pos[:, 2], key))
    k = key[order]
    starts = np.searchsorted(k, np.arange(nc * nc))
    ends = np.searchsorted(k, np.arange(nc * nc), side="right")
    return [order[c0:min(c0 + M, b)] for a, b in zip(starts, ends) for c0 in range(a, b, M)]


def _tile_evaluations(pos, L, M, col, rl):
    cl = _clusters(pos, L, M, col)
    lo = np.array([pos[c].min(0) for c in cl])
    hi = np.array([pos[c].max(0) for c in cl])
    cen, half = 0.5 * (lo + hi), 0.5 * (hi - lo)
    rad = np.sqrt((half ** 2).sum(1)).max()
    tree = scipy_spatial.cKDTree(np.mod(cen, L), boxsize=L)
    cand = tree.query_pairs(rl + 2 * rad, output_type="ndarray")
    d = cen[cand[:, 0]] - cen[cand[:, 1]]
    d -= L * np.round(d / L)
    gap = np.maximum(np.abs(d) - half[cand[:, 0]] - half[cand[:, 1]], 0.0)
    n_cp = int(((gap ** 2).sum(1) < rl * rl).sum())
    return n_cp * M * M + len(cl) * M * (M - 1) // 2


def test_full_per_atom_list_evaluates_fewer_than_cluster_tiles():
    from nexusmd_gb300 import synthetic as sy
    s = sy.config_system(2)
    L = float(s.box[0])
    pos = np.mod(s.pos, L)
    tree = scipy_spatial.cKDTree(pos, boxsize=L)
    n = len(pos)
    pairs_rc = (tree.count_neighbors(tree, 1.0) - n) // 2
    pairs_rl = (tree.count_neighbors(tree, 1.1) - n) // 2
    full = 2.0 * pairs_rl / pairs_rc
    tiles = {M: _tile_evaluations(pos, L, M, col, 1.1) / pairs_rc
             for M, col in ((4, 0.35), (8, 0.45), (16, 0.55))}
    print("per in-cutoff pair: full per-atom list %.2f, half list of cluster tiles %s"
          % (full, ", ".join("%dx%d %.2f" % (M, M, v) for M, v in tiles.items())))
    assert 2.5 < full < 2.8
    assert all(v > full for v in tiles.values())
