/*
 * CPU oracle for the NexusMD force-and-integrate path -- TEST INFRASTRUCTURE.
 *
 * FP64 restatement of the reference (paths relative to NexusMD/core/),
 * written operation by operation in the reference's evaluation order so that
 * it agrees with the compiled reference to round-off.  Compile with
 * -ffp-contract=off so that no multiply-add is fused (the reference's x86
 * build never fuses).  Only tests, the smoke check and the CPU-baseline leg
 * of the benchmark use this file.
 */
#define _POSIX_C_SOURCE 199309L
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "nxo_fft.h"

#define PI_ 3.14159265358979323846          /* NonbondedForce.h:12-14 */
#define SQRT_PI_ 1.77245385090551602729     /* NonbondedForce.h:16-18 */
#define TWO_OVER_SQRT_PI_ 1.1283791670955126 /* NonbondedForce.h:20-22 */
#define ONE_4PI_EPS0_ 138.93545764446428693393 /* NonbondedForce.h:25-27 */

/* ---- small vector helpers with Coords3D's arithmetic (Coords3D.h:48-145) */
static inline double dot3(const double *a, const double *b) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
static inline void cross3(const double *a, const double *b, double *c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}
static inline void normalize3(const double *a, double *o) {
    double len = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    o[0] = o[1] = o[2] = 0.0;
    if (len > 0) {
        o[0] = a[0] / len;
        o[1] = a[1] / len;
        o[2] = a[2] / len;
    }
}

/* ------------------------------------------------------------------ box */

/* PeriodicBoundaryCondition.cpp:11-88: lb/ub = extent, then 1% margin each
 * side (the water_availibility branch skips the re-centring code). */
void nxo_box_from_positions(int n, const double *pos, nxo_box *box) {
    for (int d = 0; d < 3; ++d) box->lb[d] = box->ub[d] = pos[d];
    for (int i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) {
            double v = pos[3 * i + d];
            if (v < box->lb[d]) box->lb[d] = v;
            if (v > box->ub[d]) box->ub[d] = v;
        }
    for (int d = 0; d < 3; ++d) box->size[d] = fabs(box->ub[d] - box->lb[d]);
    for (int d = 0; d < 3; ++d) {
        double margin = 0.01 * box->size[d];
        box->lb[d] -= margin;
        box->ub[d] += margin;
    }
    for (int d = 0; d < 3; ++d) box->size[d] = fabs(box->ub[d] - box->lb[d]);
}

void nxo_box_explicit(const double *lb, const double *ub, nxo_box *box) {
    for (int d = 0; d < 3; ++d) {
        box->lb[d] = lb[d];
        box->ub[d] = ub[d];
        box->size[d] = fabs(ub[d] - lb[d]);
    }
}

/* PeriodicBoundaryCondition.cpp:93-104: one +-L shift per component. */
void nxo_min_image(const double *c1, const double *c2, const nxo_box *box, double *d) {
    for (int i = 0; i < 3; ++i) {
        d[i] = c1[i] - c2[i];
        if (d[i] > 0.5 * box->size[i])
            d[i] -= box->size[i];
        else if (d[i] < -0.5 * box->size[i])
            d[i] += box->size[i];
    }
}

/* -------------------------------------------------------------- bonded */

/* Forces.cpp:42-52 + HarmonicBondForce.cpp:20-58 */
double nxo_bonds(const double *pos, int nb, const int *idx, const double *prm, const nxo_box *box,
                 double *F) {
    double E = 0.0;
    for (int b = 0; b < nb; ++b) {
        int p1 = idx[2 * b], p2 = idx[2 * b + 1];
        double d = prm[2 * b], k = prm[2 * b + 1];
        double delta[3];
        nxo_min_image(pos + 3 * p2, pos + 3 * p1, box, delta);
        double r = sqrt(dot3(delta, delta));
        double deltaIdeal = r - d;
        double energy = 0.5 * k * deltaIdeal * deltaIdeal;
        E += energy;
        double dEdR = k * deltaIdeal;
        if (r > 0) {
            double s = dEdR / r;
            delta[0] *= s;
            delta[1] *= s;
            delta[2] *= s;
        } else {
            delta[0] = delta[1] = delta[2] = 0.0;
        }
        for (int c = 0; c < 3; ++c) {
            F[3 * p1 + c] += delta[c];
            F[3 * p2 + c] += -delta[c];
        }
    }
    return E;
}

/* Forces.cpp:54-66 + HarmonicAngleForce.cpp:19-63 */
double nxo_angles(const double *pos, int na, const int *idx, const double *prm,
                  const nxo_box *box, double *F) {
    double E = 0.0;
    for (int a = 0; a < na; ++a) {
        const double *P1 = pos + 3 * idx[3 * a], *P2 = pos + 3 * idx[3 * a + 1],
                     *P3 = pos + 3 * idx[3 * a + 2];
        double theta0 = prm[2 * a], k = prm[2 * a + 1];
        /* calculateAngle (:19-35) */
        double v0[3], v1[3], cp[3];
        nxo_min_image(P2, P1, box, v0);
        nxo_min_image(P2, P3, box, v1);
        cross3(v0, v1, cp);
        double r21 = sqrt(dot3(v0, v0));
        double r23 = sqrt(dot3(v1, v1));
        double dt = dot3(v0, v1);
        double cosine = dt / (r21 * r23);
        if (cosine < -1.0) cosine = -1.0;
        if (cosine > 1.0) cosine = 1.0;
        double theta = acos(cosine);
        /* calculateForces (:37-63) */
        double deltaIdeal = theta - theta0;
        double energy = 0.5 * k * deltaIdeal * deltaIdeal;
        E += energy;
        double dEdAngle = k * deltaIdeal;
        double rp = sqrt(dot3(cp, cp));
        if (rp < 1.0e-06) rp = 1.0e-06;
        double q21 = dot3(v0, v0);
        double q23 = dot3(v1, v1);
        double c1[3], c3[3];
        cross3(v0, cp, c1);
        cross3(cp, v1, c3);
        double s1 = dEdAngle / (q21 * rp);
        double s3 = dEdAngle / (q23 * rp);
        double f1[3], f3[3], f2[3];
        for (int c = 0; c < 3; ++c) {
            f1[c] = c1[c] * s1;
            f3[c] = c3[c] * s3;
            f2[c] = -f1[c] - f3[c];
        }
        for (int c = 0; c < 3; ++c) {
            F[3 * idx[3 * a] + c] += f1[c];
            F[3 * idx[3 * a + 1] + c] += f2[c];
            F[3 * idx[3 * a + 2] + c] += f3[c];
        }
    }
    return E;
}

/* PeriodicTorsionForce.cpp:41-77 (angle) and :81-149 (forces); Forces.cpp:18-39 */
double nxo_torsions(const double *pos, int nt, const int *idx, const double *prm, const int *per,
                    const nxo_box *box, double *F) {
    double E = 0.0;
    for (int t = 0; t < nt; ++t) {
        const double *r1 = pos + 3 * idx[4 * t], *r2 = pos + 3 * idx[4 * t + 1],
                     *r3 = pos + 3 * idx[4 * t + 2], *r4 = pos + 3 * idx[4 * t + 3];
        double k = prm[2 * t], phase = prm[2 * t + 1];
        int periodicity = per[t];
        double v0[3], v1[3], v2[3], cp0[3], cp1[3];
        nxo_min_image(r1, r2, box, v0);
        nxo_min_image(r3, r2, box, v1);
        nxo_min_image(r3, r4, box, v2);
        cross3(v0, v1, cp0);
        cross3(v1, v2, cp1);
        double n0[3], n1[3];
        normalize3(cp0, n0);
        normalize3(cp1, n1);
        double cosangle = dot3(n0, n1);
        double angle;
        if (cosangle > (double)0.99f || cosangle < -(double)0.99f) {
            double cr[3];
            cross3(cp0, cp1, cr);
            double scale = dot3(cp0, cp0) * dot3(cp1, cp1);
            angle = asin(sqrt(dot3(cr, cr) / scale));
            if (cosangle < 0) angle = PI_ - angle;
        } else {
            angle = acos(cosangle);
        }
        angle = (dot3(v0, cp1) >= 0 ? angle : -angle);

        double deltaAngle = periodicity * angle - phase;
        double energy = k * (1.0 + cos(deltaAngle));
        E += energy;
        double dEdPhi = -k * periodicity * sin(deltaAngle);

        double normCross1 = dot3(cp0, cp0);
        double normSqrBC = dot3(v1, v1);
        double normBC = sqrt(normSqrBC);
        double normCross2 = dot3(cp1, cp1);
        double dp = 1.0 / normSqrBC;
        double factor1 = (-dEdPhi * normBC) / normCross1;
        double factor2 = dot3(v0, v1) * dp;
        double factor3 = dot3(v2, v1) * dp;
        double factor4 = (dEdPhi * normBC) / normCross2;
        double f1[3], f4[3], s[3], f2[3], f3[3];
        for (int c = 0; c < 3; ++c) {
            f1[c] = cp0[c] * factor1;
            f4[c] = cp1[c] * factor4;
        }
        for (int c = 0; c < 3; ++c) {
            s[c] = f1[c] * factor2 - f4[c] * factor3;
            f2[c] = s[c] - f1[c];
            f3[c] = -s[c] - f4[c];
        }
        for (int c = 0; c < 3; ++c) {
            F[3 * idx[4 * t] + c] += f1[c];
            F[3 * idx[4 * t + 1] + c] += f2[c];
            F[3 * idx[4 * t + 2] + c] += f3[c];
            F[3 * idx[4 * t + 3] + c] += f4[c];
        }
    }
    return E;
}

/* ---------------------------------------------------------- exclusions */

static int cmp_int(const void *a, const void *b) {
    int x = *(const int *)a, y = *(const int *)b;
    return (x > y) - (x < y);
}

/* Exclusions.cpp:7-44.  With bondCutoff = depth the expansion loop produces
 * every partner reachable by a walk of 1..depth bonds (never the atom
 * itself); that set is built here by breadth-first search per atom. */
long nxo_exclusions(int n, int nb, const int *bonds, int depth, int *off, int *lst, long cap) {
    int *deg = (int *)calloc((size_t)n + 1, sizeof(int));
    for (int b = 0; b < nb; ++b) {
        if (bonds[2 * b] < 0 || bonds[2 * b + 1] < 0 || bonds[2 * b] >= n || bonds[2 * b + 1] >= n) {
            free(deg);
            return -1; /* Exclusions.cpp:12-15 throws here */
        }
        deg[bonds[2 * b]]++;
        deg[bonds[2 * b + 1]]++;
    }
    int *aoff = (int *)malloc(sizeof(int) * ((size_t)n + 1));
    aoff[0] = 0;
    for (int i = 0; i < n; ++i) aoff[i + 1] = aoff[i] + deg[i];
    int *adj = (int *)malloc(sizeof(int) * (size_t)(aoff[n] > 0 ? aoff[n] : 1));
    memset(deg, 0, sizeof(int) * (size_t)n);
    for (int b = 0; b < nb; ++b) {
        int i = bonds[2 * b], j = bonds[2 * b + 1];
        adj[aoff[i] + deg[i]++] = j;
        adj[aoff[j] + deg[j]++] = i;
    }
    int *dist = (int *)malloc(sizeof(int) * (size_t)n);
    int *queue = (int *)malloc(sizeof(int) * (size_t)n);
    for (int i = 0; i < n; ++i) dist[i] = -1;
    long total = 0;
    int overflow = 0;
    for (int i = 0; i < n; ++i) {
        off[i] = (int)(overflow ? 0 : total);
        int qh = 0, qt = 0;
        queue[qt++] = i;
        dist[i] = 0;
        long start = total;
        while (qh < qt) {
            int u = queue[qh++];
            if (dist[u] == depth) continue;
            for (int e = aoff[u]; e < aoff[u + 1]; ++e) {
                int v = adj[e];
                if (dist[v] < 0) {
                    dist[v] = dist[u] + 1;
                    queue[qt++] = v;
                    if (total < cap)
                        lst[total] = v;
                    else
                        overflow = 1;
                    total++;
                }
            }
        }
        if (!overflow) qsort(lst + start, (size_t)(total - start), sizeof(int), cmp_int);
        for (int q = 0; q < qt; ++q) dist[queue[q]] = -1;
    }
    off[n] = (int)(overflow ? 0 : total);
    free(deg);
    free(aoff);
    free(adj);
    free(dist);
    free(queue);
    return overflow ? -total : total;
}

static int is_excluded(const int *eoff, const int *elst, int i, int j) {
    int lo = eoff[i], hi = eoff[i + 1];
    while (lo < hi) {
        int mid = (lo + hi) / 2;
        if (elst[mid] == j) return 1;
        if (elst[mid] < j)
            lo = mid + 1;
        else
            hi = mid;
    }
    return 0;
}

/* ---------------------------------------------------------- neighbours */

/* NeighborList.cpp:129-154 (obtainNeighborList), :12-35 (VoxelHash) and
 * :45-127 (getNeighbors).  std::map<VoxelIndex, Voxel> only matters for
 * which voxels exist; a dense per-voxel list in insertion order visits the
 * same atoms in the same order. */
long nxo_neighbor_pairs(int n, const double *pos, const nxo_box *box, const int *eoff,
                        const int *elst, double cutoff, int *pairs, long cap) {
    double maxDistance = cutoff;
    double edge[3], vs[3];
    int nv[3];
    for (int d = 0; d < 3; ++d) edge[d] = 0.5 * box->size[d] / floor(box->size[d] / maxDistance);
    for (int d = 0; d < 3; ++d) {
        nv[d] = (int)floor(box->size[d] / edge[d] + 0.5);
        vs[d] = box->size[d] / nv[d];
    }
    /* voxel coordinates of every atom (getVoxelIndex, :24-35) */
    int *vc = (int *)malloc(sizeof(int) * 3 * (size_t)n);
    for (int i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) {
            double r = pos[3 * i + d];
            r -= floor(r / box->size[d]) * box->size[d];
            vc[3 * i + d] = (int)floor(r / vs[d]);
        }
    /* a voxel index of nv (r/vs rounding up to the edge) is a real key in the
     * reference's map that the wrapped search never visits */
    long nvox = (long)nv[0] * nv[1] * nv[2];
    int *head = (int *)malloc(sizeof(int) * (size_t)nvox);
    int *tail = (int *)malloc(sizeof(int) * (size_t)nvox);
    int *next = (int *)malloc(sizeof(int) * (size_t)n);
    for (long v = 0; v < nvox; ++v) head[v] = tail[v] = -1;
    double maxD2 = maxDistance * maxDistance;
    double minD2 = 0.0;
    int dI[3];
    for (int d = 0; d < 3; ++d) dI[d] = (int)(maxDistance / vs[d]) + 1;
    long count = 0;
    for (int atomI = 0; atomI < n; ++atomI) {
        const double *locI = pos + 3 * atomI;
        const int *c = vc + 3 * atomI;
        int minz = c[2] - dI[2], maxz = c[2] + dI[2];
        if (maxz > minz + nv[2] - 1) maxz = minz + nv[2] - 1;
        for (int z = minz; z <= maxz; ++z) {
            int miny = c[1] - dI[1], maxy = c[1] + dI[1];
            if (maxy > miny + nv[1] - 1) maxy = miny + nv[1] - 1;
            for (int y = miny; y <= maxy; ++y) {
                int minx = c[0] - dI[0], maxx = c[0] + dI[0];
                if (maxx > minx + nv[0] - 1) maxx = minx + nv[0] - 1;
                for (int x = minx; x <= maxx; ++x) {
                    int X = (x + nv[0]) % nv[0], Y = (y + nv[1]) % nv[1], Z = (z + nv[2]) % nv[2];
                    long key = ((long)X * nv[1] + Y) * nv[2] + Z;
                    for (int atomJ = head[key]; atomJ >= 0; atomJ = next[atomJ]) {
                        if (atomI == atomJ) continue;
                        double dr[3];
                        nxo_min_image(pos + 3 * atomJ, locI, box, dr);
                        double r2 = dot3(dr, dr);
                        if (eoff && is_excluded(eoff, elst, atomI, atomJ)) continue;
                        if (r2 >= minD2 && r2 < maxD2) {
                            if (count < cap) {
                                pairs[2 * count] = atomI;
                                pairs[2 * count + 1] = atomJ;
                            }
                            count++;
                        }
                    }
                }
            }
        }
        /* insert (:37-43); out-of-range voxel indices are never found */
        if (c[0] >= 0 && c[0] < nv[0] && c[1] >= 0 && c[1] < nv[1] && c[2] >= 0 && c[2] < nv[2]) {
            long key = ((long)c[0] * nv[1] + c[1]) * nv[2] + c[2];
            next[atomI] = -1;
            if (tail[key] < 0)
                head[key] = atomI;
            else
                next[tail[key]] = atomI;
            tail[key] = atomI;
        }
    }
    free(vc);
    free(head);
    free(tail);
    free(next);
    return count <= cap ? count : -count;
}

/* ----------------------------------------------------------------- PME */

/* NonbondedForce.cpp:33-48 */
static int fft_dimension(int minimum) {
    minimum = minimum * 10;
    int p = 1;
    while (p < minimum) p *= 2;
    return p;
}
void nxo_pow2_grid(const nxo_box *box, int grid[3]) {
    for (int d = 0; d < 3; ++d) grid[d] = fft_dimension((int)ceil(box->size[d]));
}

/* NonbondedForce.cpp:293-321 ("approximation" branch) */
double nxo_alpha(double cutoff, double tol) { return (1.0 / cutoff) * sqrt(-log(2.0 * tol)); }

#define ORDER 5

/* NonbondedForce.cpp:75-142: spline data and moduli |b(k)|^2 by direct DFT */
void nxo_bspline_moduli(int K, double *mod) {
    double data[ORDER];
    for (int i = 0; i < ORDER; ++i) data[i] = 0.0;
    data[ORDER - 1] = 0.0;
    data[1] = 0.0;
    data[0] = 1.0;
    for (int i = 3; i < ORDER; i++) {
        double div = 1.0 / (i - 1);
        data[i - 1] = 0.0;
        for (int j = 1; j < (i - 1); j++)
            data[i - j - 1] = div * (j * data[i - j - 2] + (i - j) * data[i - j - 1]);
        data[0] = div * data[0];
    }
    double div = 1.0 / (ORDER - 1);
    data[ORDER - 1] = div * data[ORDER - 2];
    for (int i = 1; i < (ORDER - 1); i++)
        data[ORDER - i - 1] = div * (i * data[ORDER - i - 2] + (ORDER - i) * data[ORDER - i - 1]);
    data[0] = div * data[0];
    double *bs = (double *)calloc((size_t)K + ORDER + 1, sizeof(double));
    for (int i = 1; i <= ORDER; i++) bs[i] = data[i - 1];
    for (int i = 0; i < K; i++) {
        double sc = 0.0, ss = 0.0;
        for (int j = 0; j < K; j++) {
            double arg = (2 * PI_ * i * j) / K;
            sc += bs[j] * cos(arg);
            ss += bs[j] * sin(arg);
        }
        mod[i] = sc * sc + ss * ss;
    }
    for (int i = 0; i < K; i++)
        if (mod[i] < 1e-7) mod[i] = (mod[(i - 1 + K) % K] + mod[(i + 1) % K]) / 2.0;
    free(bs);
}

/* NonbondedForce.cpp:51-71 (index, fraction) and :144-182 (theta, dtheta) */
static void spline_atom(const double *x, const double *recip, const int *grid, int *idx,
                        double th[3][ORDER], double dth[3][ORDER]) {
    for (int d = 0; d < 3; d++) {
        double t = x[d] * recip[d];
        t = (t - floor(t)) * grid[d];
        int ti = (int)t;
        double dr = t - ti;
        idx[d] = ti % grid[d];
        double *b = th[d];
        b[ORDER - 1] = 0;
        b[1] = dr;
        b[0] = 1 - dr;
        for (int k = 3; k < ORDER; k++) {
            double div = 1.0 / (k - 1.0);
            b[k - 1] = div * dr * b[k - 2];
            for (int l = 1; l < (k - 1); l++)
                b[k - l - 1] = div * ((dr + l) * b[k - l - 2] + (k - l - dr) * b[k - l - 1]);
            b[0] = div * (1 - dr) * b[0];
        }
        dth[d][0] = -b[0];
        for (int k = 1; k < ORDER; k++) dth[d][k] = b[k - 1] - b[k];
        double div = 1.0 / (ORDER - 1);
        b[ORDER - 1] = div * dr * b[ORDER - 2];
        for (int l = 1; l < (ORDER - 1); l++)
            b[ORDER - l - 1] = div * ((dr + l) * b[ORDER - l - 2] + (ORDER - l - dr) * b[ORDER - l - 1]);
        b[0] = div * (1 - dr) * b[0];
    }
}

/* NonbondedForce.cpp:220-260 */
void nxo_spread(int n, const double *pos, const double *q, const nxo_box *box, const int grid[3],
                double *Q) {
    double recip[3];
    for (int d = 0; d < 3; d++) recip[d] = 1 / box->size[d];
    size_t G = (size_t)grid[0] * grid[1] * grid[2];
    memset(Q, 0, sizeof(double) * 2 * G);
    for (int i = 0; i < n; ++i) {
        int idx[3];
        double th[3][ORDER], dth[3][ORDER];
        spline_atom(pos + 3 * i, recip, grid, idx, th, dth);
        for (int ix = 0; ix < ORDER; ++ix) {
            int xi = (idx[0] + ix) % grid[0];
            for (int iy = 0; iy < ORDER; ++iy) {
                int yi = (idx[1] + iy) % grid[1];
                for (int iz = 0; iz < ORDER; ++iz) {
                    int zi = (idx[2] + iz) % grid[2];
                    size_t index = (size_t)xi * grid[1] * grid[2] + (size_t)yi * grid[2] + zi;
                    Q[2 * index] += q[i] * th[0][ix] * th[1][iy] * th[2][iz];
                }
            }
        }
    }
}

/* NonbondedForce.cpp:467-499 with :323-388 (convolution) and :407-461 (gather) */
double nxo_pme(int n, const double *pos, const double *q, const nxo_box *box, double alpha,
               const int grid[3], double *F) {
    int K0 = grid[0], K1 = grid[1], K2 = grid[2];
    double recip[3];
    for (int d = 0; d < 3; d++) recip[d] = 1 / box->size[d];
    double *mod[3];
    for (int d = 0; d < 3; d++) {
        mod[d] = (double *)malloc(sizeof(double) * (size_t)grid[d]);
        nxo_bspline_moduli(grid[d], mod[d]);
    }
    size_t G = (size_t)K0 * K1 * K2;
    double *Q = (double *)malloc(sizeof(double) * 2 * G);
    nxo_spread(n, pos, q, box, grid, Q);
    nxo_fft3d(Q, K0, K1, K2, -1);

    double one_4pi_eps = ONE_4PI_EPS0_ / 1.0;
    double factor = PI_ * PI_ / (alpha * alpha);
    double boxfactor = PI_ * box->size[0] * box->size[1] * box->size[2];
    double recipE = 0.0;
    int maxkx = (K0 + 1) / 2, maxky = (K1 + 1) / 2, maxkz = (K2 + 1) / 2;
    for (int kx = 0; kx < K0; ++kx) {
        double mx = (kx < maxkx) ? kx : (kx - K0);
        double mhx = mx * recip[0];
        double bx = boxfactor * mod[0][kx];
        for (int ky = 0; ky < K1; ++ky) {
            double my = (ky < maxky) ? ky : (ky - K1);
            double mhy = my * recip[1];
            double by = mod[1][ky];
            for (int kz = 0; kz < K2; ++kz) {
                if (kx == 0 && ky == 0 && kz == 0) continue;
                double mz = (kz < maxkz) ? kz : (kz - K2);
                double mhz = mz * recip[2];
                size_t index = (size_t)kx * K1 * K2 + (size_t)ky * K2 + kz;
                double d1 = Q[2 * index], d2 = Q[2 * index + 1];
                double m2 = mhx * mhx + mhy * mhy + mhz * mhz;
                double bz = mod[2][kz];
                double denom = m2 * bx * by * bz;
                double eterm = one_4pi_eps * exp(-factor * m2) / denom;
                Q[2 * index] = d1 * eterm;
                Q[2 * index + 1] = d2 * eterm;
                double struct2 = d1 * d1 + d2 * d2;
                recipE += eterm * struct2;
            }
        }
    }
    nxo_fft3d(Q, K0, K1, K2, +1);

    for (int i = 0; i < n; ++i) {
        int idx[3];
        double th[3][ORDER], dth[3][ORDER];
        spline_atom(pos + 3 * i, recip, grid, idx, th, dth);
        double fx = 0.0, fy = 0.0, fz = 0.0;
        for (int ix = 0; ix < ORDER; ix++) {
            int xi = (idx[0] + ix) % K0;
            double tx = th[0][ix], dtx = dth[0][ix];
            for (int iy = 0; iy < ORDER; iy++) {
                int yi = (idx[1] + iy) % K1;
                double ty = th[1][iy], dty = dth[1][iy];
                for (int iz = 0; iz < ORDER; iz++) {
                    int zi = (idx[2] + iz) % K2;
                    double tz = th[2][iz], dtz = dth[2][iz];
                    size_t index = (size_t)xi * K1 * K2 + (size_t)yi * K2 + zi;
                    double gv = Q[2 * index];
                    fx += dtx * ty * tz * gv;
                    fy += tx * dty * tz * gv;
                    fz += tx * ty * dtz * gv;
                }
            }
        }
        F[3 * i + 0] -= q[i] * (fx * K0 * recip[0]);
        F[3 * i + 1] -= q[i] * (fy * K1 * recip[1]);
        F[3 * i + 2] -= q[i] * (fz * K2 * recip[2]);
    }
    for (int d = 0; d < 3; d++) free(mod[d]);
    free(Q);
    return 0.5 * recipE;
}

/* ------------------------------------------------------ real space etc */

/* NonbondedForce.cpp:504-513: sigma/2 and 2*sqrt(eps) so that
 * sigma_ij = sg_i + sg_j and 4*sqrt(eps_i eps_j) = ep_i * ep_j */
static void lj_rewrite(int n, const double *sig, const double *eps, double *sg, double *ep) {
    for (int i = 0; i < n; i++) {
        sg[i] = 0.5 * sig[i];
        ep[i] = 2.0 * sqrt(eps[i]);
    }
}

/* NonbondedForce.cpp:515-527 */
static double self_energy(int n, const double *q, double alpha) {
    double selfE = 0.0;
    for (int i = 0; i < n; i++) selfE -= ONE_4PI_EPS0_ * q[i] * q[i] * alpha / SQRT_PI_;
    return selfE;
}

static long pair_list(const nxo_system *s, const double *pos, const nxo_box *box, const int *eoff,
                      const int *elst, int **pairs_out) {
    long cap = (long)s->n * 64 + 1024;
    for (;;) {
        int *pairs = (int *)malloc(sizeof(int) * 2 * (size_t)cap);
        long np = nxo_neighbor_pairs(s->n, pos, box, eoff, elst, s->cutoff, pairs, cap);
        if (np >= 0) {
            *pairs_out = pairs;
            return np;
        }
        free(pairs);
        cap = -np;
    }
}

/* NonbondedForce.cpp:530-585 over a reference-ordered pair list */
static void direct_pairs(const nxo_system *s, const double *pos, const nxo_box *box,
                         const int *pairs, long np, const double *sg, const double *ep,
                         double alpha, double *Fn, double *coulE_out, double *vdwE_out) {
    double vdwE = 0.0, coulE = 0.0;
    double switchValue = 1.0, switchDeriv = 0.0;
    for (long p = 0; p < np; ++p) {
        int ii = pairs[2 * p], jj = pairs[2 * p + 1];
        double d[3];
        nxo_min_image(pos + 3 * ii, pos + 3 * jj, box, d);
        double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        double inverseR = 1.0 / r;
        if (!s->switch_quirk) {
            switchValue = 1.0;
            switchDeriv = 0.0;
        }
        if (s->use_switch && r > s->switch_dist) {
            double t = (r - s->switch_dist) / (s->cutoff - s->switch_dist);
            switchValue = 1 + t * t * t * (-10 + t * (15 - t * 6));
            switchDeriv = t * t * (-30 + t * (60 - t * 30)) / (s->cutoff - s->switch_dist);
        }
        double alphaR = alpha * r;
        double dEdR = ONE_4PI_EPS0_ * s->q[ii] * s->q[jj] * inverseR * inverseR * inverseR;
        dEdR *= (erfc(alphaR) + 2 * alphaR * exp(-alphaR * alphaR) / SQRT_PI_);
        double sig = sg[ii] + sg[jj];
        double sig2 = sig * inverseR;
        sig2 *= sig2;
        double sig6 = sig2 * sig2 * sig2;
        double eps = ep[ii] * ep[jj];
        dEdR += switchValue * eps * (12.0 * sig6 - 6.0) * sig6 * inverseR * inverseR;
        double vdw = eps * (sig6 - 1.0) * sig6;
        if (s->use_switch) {
            dEdR -= vdw * switchDeriv * inverseR;
            vdw *= switchValue;
        }
        for (int c = 0; c < 3; ++c) {
            double f = d[c] * dEdR;
            Fn[3 * ii + c] += f;
            Fn[3 * jj + c] -= f;
        }
        coulE += ONE_4PI_EPS0_ * s->q[ii] * s->q[jj] * inverseR * erfc(alphaR);
        vdwE += vdw;
    }
    *coulE_out = coulE;
    *vdwE_out = vdwE;
}

/* NonbondedForce.cpp:590-630: remove the erf (reciprocal) part of every
 * excluded pair, at any distance; returns the energy to subtract */
static double exclusion_correction(const nxo_system *s, const double *pos, const nxo_box *box,
                                   const int *eoff, const int *elst, double alpha, double *Fn) {
    double exclE = 0.0;
    for (int i = 0; i < s->n; i++) {
        for (int e = eoff[i]; e < eoff[i + 1]; ++e) {
            int jj = elst[e];
            if (jj <= i) continue;
            int ii = i;
            double d[3];
            nxo_min_image(pos + 3 * ii, pos + 3 * jj, box, d);
            double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            double inverseR = 1.0 / r;
            double alphaR = alpha * r;
            double ex;
            if (erf(alphaR) > 1e-6) {
                double dEdR = ONE_4PI_EPS0_ * s->q[ii] * s->q[jj] * inverseR * inverseR * inverseR;
                dEdR = dEdR * (erf(alphaR) - 2 * alphaR * exp(-alphaR * alphaR) / SQRT_PI_);
                for (int c = 0; c < 3; ++c) {
                    double f = d[c] * dEdR;
                    Fn[3 * ii + c] -= f;
                    Fn[3 * jj + c] += f;
                }
                ex = ONE_4PI_EPS0_ * s->q[ii] * s->q[jj] * inverseR * erf(alphaR);
            } else {
                ex = alpha * TWO_OVER_SQRT_PI_ * ONE_4PI_EPS0_ * s->q[ii] * s->q[jj];
            }
            exclE += ex;
        }
    }
    return exclE;
}

static void nb_grid(const nxo_system *s, const nxo_box *box, int grid[3]) {
    grid[0] = s->grid[0];
    grid[1] = s->grid[1];
    grid[2] = s->grid[2];
    if (grid[0] <= 0 || grid[1] <= 0 || grid[2] <= 0) nxo_pow2_grid(box, grid);
}

/* NonbondedForce.cpp:633-647 in its phase order: reciprocal (:467-499),
 * parameter rewrite (:504-513), self (:515-527), direct (:530-585),
 * exclusion correction (:590-630).  The phase forces are summed into a
 * separate vector first and then added to F, as Forces.cpp:69-76 does. */
int nxo_nonbonded(const nxo_system *s, const double *pos, const nxo_box *box, const int *eoff,
                  const int *elst, double *F, nxo_energy *E) {
    int n = s->n;
    double alpha = nxo_alpha(s->cutoff, s->ewald_tol);
    int grid[3];
    nb_grid(s, box, grid);
    double *Fn = (double *)calloc(3 * (size_t)n, sizeof(double));
    E->recip = nxo_pme(n, pos, s->q, box, alpha, grid, Fn);
    double *sg = (double *)malloc(sizeof(double) * (size_t)n);
    double *ep = (double *)malloc(sizeof(double) * (size_t)n);
    lj_rewrite(n, s->sig, s->eps, sg, ep);
    E->self = self_energy(n, s->q, alpha);
    int *pairs;
    long np = pair_list(s, pos, box, eoff, elst, &pairs);
    direct_pairs(s, pos, box, pairs, np, sg, ep, alpha, Fn, &E->coulomb, &E->vdw);
    E->exclusion = exclusion_correction(s, pos, box, eoff, elst, alpha, Fn);
    for (size_t k = 0; k < 3 * (size_t)n; ++k) F[k] += Fn[k];
    free(Fn);
    free(sg);
    free(ep);
    free(pairs);
    return 0;
}

/* Exceptions, OpenMM semantics (the reference has no code for them): one
 * pass over the listed pairs, d = p_i - p_j with the reference's minimum
 * image, dE/dR / r applied as in direct_pairs above. */
double nxo_exceptions(const double *pos, int nexc, const int *idx, const double *prm, const nxo_box *box,
                      double *F) {
    double e = 0.0;
    for (int k = 0; k < nexc; ++k) {
        int ii = idx[2 * k], jj = idx[2 * k + 1];
        double qq = prm[3 * k], sig = prm[3 * k + 1], eps = prm[3 * k + 2];
        double d[3];
        nxo_min_image(pos + 3 * ii, pos + 3 * jj, box, d);
        double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        double inverseR = 1.0 / sqrt(r2);
        double coul = ONE_4PI_EPS0_ * qq * inverseR;
        double s2 = sig * inverseR;
        s2 *= s2;
        double s6 = s2 * s2 * s2;
        double lj = 4.0 * eps * (s6 - 1.0) * s6;
        double dEdR = (coul + 4.0 * eps * (12.0 * s6 - 6.0) * s6) * inverseR * inverseR;
        for (int c = 0; c < 3; ++c) {
            double f = d[c] * dEdR;
            F[3 * ii + c] += f;
            F[3 * jj + c] -= f;
        }
        e += coul + lj;
    }
    return e;
}

/* Engine.cpp:75-95.  reported_pe reproduces the reference's bookkeeping:
 * reciprocalConvolutionAndEnergy *assigns* the reciprocal energy to the
 * running total (NonbondedForce.cpp:387 via :489), which drops the bonded
 * energies accumulated before it. */
int nxo_forces(const nxo_system *s, const double *pos, const nxo_box *box, const int *eoff,
               const int *elst, double *F, nxo_energy *E) {
    memset(E, 0, sizeof(*E));
    memset(F, 0, sizeof(double) * 3 * (size_t)s->n);
    double pe = 0.0;
    if (s->force_mask & 1) {
        E->bond = nxo_bonds(pos, s->nb, s->bonds, s->bond_prm, box, F);
        pe += E->bond;
    }
    if (s->force_mask & 2) {
        E->angle = nxo_angles(pos, s->na, s->angles, s->angle_prm, box, F);
        pe += E->angle;
    }
    if (s->force_mask & 4) {
        E->torsion = nxo_torsions(pos, s->nt, s->torsions, s->torsion_prm, s->torsion_per, box, F);
        pe += E->torsion;
    }
    if (s->force_mask & 8) {
        nxo_nonbonded(s, pos, box, eoff, elst, F, E);
        pe = E->recip;
        pe += E->self;
        pe += E->coulomb + E->vdw;
        pe -= E->exclusion;
        if (s->nexc > 0) {
            E->exception = nxo_exceptions(pos, s->nexc, s->exc_idx, s->exc_prm, box, F);
            pe += E->exception;
        }
    }
    E->reported_pe = pe;
    return 0;
}

/* -------------------------------------------------------- integration */

/* VerletIntegration.cpp:49-89 with dt[0] = dt[1] = dt (Engine.cpp:166) */
void nxo_leapfrog(int n, double *pos, double *vel, const double *F, const double *invm, double dt,
                  const nxo_box *box) {
    double dtPos = dt;
    double dtVel = 0.5 * (dt + dt);
    double scale = dtVel;
    for (int i = 0; i < n; ++i) {
        if (invm[i] == 0.0) continue;
        for (int j = 0; j < 3; ++j) {
            vel[3 * i + j] += invm[i] * F[3 * i + j] * scale;
            double u = pos[3 * i + j] + vel[3 * i + j] * dtPos;
            if (u < box->lb[j])
                u += box->size[j];
            else if (u > box->ub[j])
                u -= box->size[j];
            pos[3 * i + j] = u;
        }
    }
}

/* KineticEnergy.cpp:21-41 */
double nxo_kinetic(int n, const double *vel, const double *mass, const double *F, double dt) {
    double timeShift = 0.5 * dt;
    double total = 0.0;
    for (int i = 0; i < n; ++i) {
        double v[3] = {vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]};
        if (mass[i] > 0) {
            double invMass = 1.0 / mass[i];
            for (int c = 0; c < 3; ++c) v[c] += F[3 * i + c] * invMass * timeShift;
        }
        double ke = 0.5 * mass[i] * dot3(v, v);
        total += ke;
    }
    return total;
}

/* Exclusion CSR united with the exception pairs (both directions), each
 * atom's partners ascending and unique.  Replaces *eoff / *elst. */
static void merge_exceptions(const nxo_system *s, int **eoff, int **elst) {
    int n = s->n;
    int *cnt = (int *)calloc((size_t)n + 1, sizeof(int));
    for (int i = 0; i < n; ++i) cnt[i] = (*eoff)[i + 1] - (*eoff)[i];
    for (int k = 0; k < s->nexc; ++k) {
        cnt[s->exc_idx[2 * k]]++;
        cnt[s->exc_idx[2 * k + 1]]++;
    }
    int *off = (int *)malloc(sizeof(int) * ((size_t)n + 1));
    off[0] = 0;
    for (int i = 0; i < n; ++i) off[i + 1] = off[i] + cnt[i];
    int *lst = (int *)malloc(sizeof(int) * (size_t)(off[n] > 0 ? off[n] : 1));
    for (int i = 0; i < n; ++i) {
        cnt[i] = (*eoff)[i + 1] - (*eoff)[i];
        memcpy(lst + off[i], *elst + (*eoff)[i], sizeof(int) * (size_t)cnt[i]);
    }
    for (int k = 0; k < s->nexc; ++k) {
        int a = s->exc_idx[2 * k], b = s->exc_idx[2 * k + 1];
        lst[off[a] + cnt[a]++] = b;
        lst[off[b] + cnt[b]++] = a;
    }
    /* sort and compact each atom's partners */
    int w = 0;
    int *noff = (int *)malloc(sizeof(int) * ((size_t)n + 1));
    for (int i = 0; i < n; ++i) {
        qsort(lst + off[i], (size_t)cnt[i], sizeof(int), cmp_int);
        noff[i] = w;
        for (int e = 0; e < cnt[i]; ++e) {
            int v = lst[off[i] + e];
            if (e == 0 || v != lst[off[i] + e - 1]) lst[w++] = v;
        }
    }
    noff[n] = w;
    free(*eoff);
    free(*elst);
    free(cnt);
    free(off);
    *eoff = noff;
    *elst = lst;
}

static int setup(const nxo_system *s, const double *pos, nxo_box *box, int **eoff, int **elst,
                 double **invm) {
    if (s->box_mode == 0)
        nxo_box_from_positions(s->n, pos, box);
    else
        nxo_box_explicit(s->lb, s->ub, box);
    *eoff = (int *)malloc(sizeof(int) * ((size_t)s->n + 1));
    long cap = (long)s->n * 8 + 16;
    for (;;) {
        *elst = (int *)malloc(sizeof(int) * (size_t)cap);
        long ne = nxo_exclusions(s->n, s->nb, s->bonds, s->exclusion_depth, *eoff, *elst, cap);
        if (ne == -1 && s->nb > 0) {
            /* bad bond index */
        }
        if (ne >= 0) break;
        free(*elst);
        if (ne == -1) return -1;
        cap = -ne;
    }
    if (s->nexc > 0 && (s->force_mask & 8)) merge_exceptions(s, eoff, elst);
    /* VerletIntegration.cpp:37-45 */
    *invm = (double *)malloc(sizeof(double) * (size_t)s->n);
    for (int i = 0; i < s->n; ++i) (*invm)[i] = (s->mass[i] == 0.0) ? 0.0 : 1.0 / s->mass[i];
    return 0;
}

/* Engine.cpp:162-188 with Report (:117-158) reduced to its energy record. */
int nxo_run(const nxo_system *s, double *pos, double *vel, double *F, double dt, int steps,
            int interval, double *report, nxo_box *box_out) {
    nxo_box box;
    int *eoff, *elst;
    double *invm;
    if (setup(s, pos, &box, &eoff, &elst, &invm)) return -1;
    if (box_out) *box_out = box;
    int nrep = 0;
    nxo_energy E;
    for (int step = 0; step < steps; ++step) {
        nxo_forces(s, pos, &box, eoff, elst, F, &E);
        if (((step + 1) % interval) == 0 || step == 0) {
            double ke = nxo_kinetic(s->n, vel, s->mass, F, dt);
            report[4 * nrep + 0] = step;
            report[4 * nrep + 1] = ke;
            report[4 * nrep + 2] = E.reported_pe;
            report[4 * nrep + 3] = E.reported_pe + ke;
            nrep++;
        }
        nxo_leapfrog(s->n, pos, vel, F, invm, dt, &box);
    }
    free(eoff);
    free(elst);
    free(invm);
    return nrep;
}

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* The same loop with each phase timed separately (no reports). */
int nxo_run_timed(const nxo_system *s, double *pos, double *vel, double dt, int steps,
                  nxo_timing *t) {
    nxo_box box;
    int *eoff, *elst;
    double *invm;
    if (setup(s, pos, &box, &eoff, &elst, &invm)) return -1;
    memset(t, 0, sizeof(*t));
    int n = s->n;
    double *F = (double *)malloc(sizeof(double) * 3 * (size_t)n);
    double *Fn = (double *)malloc(sizeof(double) * 3 * (size_t)n);
    double *sg = (double *)malloc(sizeof(double) * (size_t)n);
    double *ep = (double *)malloc(sizeof(double) * (size_t)n);
    double alpha = nxo_alpha(s->cutoff, s->ewald_tol);
    int grid[3];
    nb_grid(s, &box, grid);
    for (int step = 0; step < steps; ++step) {
        memset(F, 0, sizeof(double) * 3 * (size_t)n);
        double t0 = now_s();
        if (s->force_mask & 1) nxo_bonds(pos, s->nb, s->bonds, s->bond_prm, &box, F);
        if (s->force_mask & 2) nxo_angles(pos, s->na, s->angles, s->angle_prm, &box, F);
        if (s->force_mask & 4)
            nxo_torsions(pos, s->nt, s->torsions, s->torsion_prm, s->torsion_per, &box, F);
        t->bonded += now_s() - t0;
        if (s->force_mask & 8) {
            memset(Fn, 0, sizeof(double) * 3 * (size_t)n);
            double t2 = now_s();
            nxo_pme(n, pos, s->q, &box, alpha, grid, Fn);
            lj_rewrite(n, s->sig, s->eps, sg, ep);
            self_energy(n, s->q, alpha);
            double t3 = now_s();
            int *pairs;
            long np = pair_list(s, pos, &box, eoff, elst, &pairs);
            double t4 = now_s();
            double ce, ve;
            direct_pairs(s, pos, &box, pairs, np, sg, ep, alpha, Fn, &ce, &ve);
            double t5 = now_s();
            exclusion_correction(s, pos, &box, eoff, elst, alpha, Fn);
            for (size_t k = 0; k < 3 * (size_t)n; ++k) F[k] += Fn[k];
            double t6 = now_s();
            free(pairs);
            t->recip += t3 - t2;
            t->nlist += t4 - t3;
            t->direct += t5 - t4;
            t->exclusion += t6 - t5;
        }
        double t7 = now_s();
        nxo_leapfrog(n, pos, vel, F, invm, dt, &box);
        t->integrate += now_s() - t7;
    }
    free(F);
    free(Fn);
    free(sg);
    free(ep);
    free(eoff);
    free(elst);
    free(invm);
    return 0;
}
