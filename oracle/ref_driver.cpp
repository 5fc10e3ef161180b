// Per-phase driver over the reference's own C++ sources -- TEST INFRASTRUCTURE.
//
// Built by oracle/Makefile against the unmodified reference sources into
// oracle/_ref/libnxm_ref.so (never committed, never shipped).  It exposes the
// reference's phase functions through a C ABI so that tests can pin the C
// restatement in oracle.c to the reference itself, and so that golden
// fixtures can be generated from it.  Private members are reached with the
// preprocessor after every standard header is already included.
#include <algorithm>
#include <cassert>
#include <cctype>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "pugixml.hpp"

#define private public
#define protected public
#include "Engine.h"
#include "NonbondedForce.h"
#include "TaskDispatcher.h"
#undef private
#undef protected

using namespace BaseLine;

namespace {

std::vector<Coords3D> to_coords(int n, const double *p) {
    std::vector<Coords3D> v(n);
    for (int i = 0; i < n; ++i) v[i] = Coords3D(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
    return v;
}

void add_coords(const std::vector<Coords3D> &v, double *out) {
    for (size_t i = 0; i < v.size(); ++i)
        for (int c = 0; c < 3; ++c) out[3 * i + c] += v[i][c];
}

PeriodicBoundaryCondition::BoxInfo to_box(const double *b /* lb3 ub3 size3 */) {
    PeriodicBoundaryCondition::BoxInfo box;
    box.lb = Coords3D(b[0], b[1], b[2]);
    box.ub = Coords3D(b[3], b[4], b[5]);
    box.boxSize = Coords3D(b[6], b[7], b[8]);
    return box;
}

std::vector<std::set<int>> to_excl(int n, const int *off, const int *lst) {
    std::vector<std::set<int>> e(n);
    for (int i = 0; i < n; ++i)
        for (int k = off[i]; k < off[i + 1]; ++k) e[i].insert(lst[k]);
    return e;
}

}  // namespace

extern "C" {

void ref_box(int n, const double *pos, double *out9) {
    PeriodicBoundaryCondition::BoxInfo box;
    PeriodicBoundaryCondition::extractBoxBoundaries(to_coords(n, pos), box, "");
    for (int c = 0; c < 3; ++c) {
        out9[c] = box.lb[c];
        out9[3 + c] = box.ub[c];
        out9[6 + c] = box.boxSize[c];
    }
}

double ref_bonds(int n, const double *pos, int nb, const int *idx, const double *prm,
                 const double *box9, double *F) {
    std::vector<BondParams> p(nb);
    for (int b = 0; b < nb; ++b) p[b] = BondParams{idx[2 * b], idx[2 * b + 1], prm[2 * b], prm[2 * b + 1]};
    std::vector<Coords3D> f(n, Coords3D(0, 0, 0));
    double E = 0.0;
    Forces::AddHBond(f, to_coords(n, pos), p, E, to_box(box9));
    add_coords(f, F);
    return E;
}

double ref_angles(int n, const double *pos, int na, const int *idx, const double *prm,
                  const double *box9, double *F) {
    std::vector<AngleParams> p(na);
    for (int a = 0; a < na; ++a)
        p[a] = AngleParams{idx[3 * a], idx[3 * a + 1], idx[3 * a + 2], prm[2 * a], prm[2 * a + 1]};
    std::vector<Coords3D> f(n, Coords3D(0, 0, 0));
    double E = 0.0;
    Forces::AddHAngle(f, to_coords(n, pos), p, E, to_box(box9));
    add_coords(f, F);
    return E;
}

double ref_torsions(int n, const double *pos, int nt, const int *idx, const double *prm,
                    const int *per, const double *box9, double *F) {
    std::vector<PTorsionParams> p(nt);
    for (int t = 0; t < nt; ++t) {
        PTorsionParams tp;
        tp.p1 = idx[4 * t];
        tp.p2 = idx[4 * t + 1];
        tp.p3 = idx[4 * t + 2];
        tp.p4 = idx[4 * t + 3];
        tp.k = prm[2 * t];
        tp.phase = prm[2 * t + 1];
        tp.periodicity = per[t];
        p[t] = tp;
    }
    std::vector<Coords3D> f(n, Coords3D(0, 0, 0));
    double E = 0.0;
    Forces::AddPTorsion(f, to_coords(n, pos), p, E, to_box(box9));
    add_coords(f, F);
    return E;
}

long ref_exclusions(int n, int nb, const int *bonds, int depth, int *off, int *lst, long cap) {
    std::vector<BondParams> p(nb);
    for (int b = 0; b < nb; ++b) p[b] = BondParams{bonds[2 * b], bonds[2 * b + 1], 0.0, 0.0};
    std::vector<std::set<int>> ex(n);
    int nn = n, dd = depth;
    Exclusions::createExclusions(nn, p, ex, dd);
    long total = 0;
    for (int i = 0; i < n; ++i) {
        off[i] = (int)std::min<long>(total, cap);
        for (int j : ex[i]) {
            if (total < cap) lst[total] = j;
            total++;
        }
    }
    off[n] = (int)std::min<long>(total, cap);
    return total <= cap ? total : -total;
}

long ref_neighbor_pairs(int n, const double *pos, const double *box9, const int *eoff,
                        const int *elst, double cutoff, int *pairs, long cap) {
    NeighborList nl;
    obtainNeighborList(nl, to_coords(n, pos), to_box(box9), to_excl(n, eoff, elst), cutoff, 0.0, true);
    long np = (long)nl.pairs.size();
    for (long k = 0; k < np && k < cap; ++k) {
        pairs[2 * k] = nl.pairs[k].first;
        pairs[2 * k + 1] = nl.pairs[k].second;
    }
    return np <= cap ? np : -np;
}

// NonbondedForce::calculateForces (NonbondedForce.cpp:633-647), one phase at
// a time with its own energy accumulator.  grid[0] > 0 overrides gridSize
// after the reference's own initializeGridSize, which is how the benchmark
// grids (64^3, 100^3, 180^3) are reached.  E = {recip, self, direct, -excl}.
void ref_nonbonded(int n, const double *pos, const double *q, const double *sig,
                   const double *eps, const double *box9, double cutoff, double tol,
                   int use_switch, double switch_dist, const int *grid, const int *eoff,
                   const int *elst, double *F, double *E) {
    NonbondedParams params{};
    params.cutoff = cutoff;
    params.ewaldTolerance = tol;
    params.useSwitchingFunction = use_switch;
    params.switchingDistance = switch_dist;
    params.particles.resize(n);
    for (int i = 0; i < n; ++i) params.particles[i] = NonbondedParticle{q[i], sig[i], eps[i]};
    std::vector<Coords3D> atoms = to_coords(n, pos);
    PeriodicBoundaryCondition::BoxInfo box = to_box(box9);
    std::vector<std::set<int>> ex = to_excl(n, eoff, elst);

    NonbondedForce nb;
    std::vector<Coords3D> forces(n, Coords3D(0, 0, 0));
    // ReciprocalPMEcalculateForcesAndEnergy (NonbondedForce.cpp:467-499)
    double e_recip = 0.0;
    nb.initializeReciprocalVectors(box);
    nb.initializeGridSize(box);
    if (grid && grid[0] > 0) nb.gridSize = {grid[0], grid[1], grid[2]};
    const int pmeOrder = 5;
    nb.InitparticleIndexAndFraction(atoms);
    nb.computeBSplineParameters(pmeOrder, atoms);
    ComplexGrid g(nb.gridSize[0] * nb.gridSize[1] * nb.gridSize[2], Complex(0.0, 0.0));
    nb.gridSpreadCharge_Reference(atoms, g, params, box, pmeOrder);
    nb.perform3DFFT(g, true);
    nb.InitializeAlphaEwald(params);
    nb.reciprocalConvolutionAndEnergy(g, params, box, e_recip);
    nb.perform3DFFT(g, false);
    nb.PMEGridForces(forces, atoms, g, params, box, e_recip, pmeOrder);
    // the remaining phases of calculateForces (:638-644)
    nb.NonbondedParamsModifier(atoms, params);
    double e_self = 0.0, e_direct = 0.0, e_excl = 0.0;
    nb.CalculateSelfEnergy(params, e_self);
    nb.DirectForcesAndEnergy(forces, atoms, params, box, ex, e_direct);
    nb.CalculateExclusionEnergyAndForces(forces, atoms, box, ex, e_excl);
    add_coords(forces, F);
    E[0] = e_recip;
    E[1] = e_self;
    E[2] = e_direct;
    E[3] = e_excl;
}

void ref_leapfrog(int n, double *pos, double *vel, const double *F, const double *mass, double dt,
                  const double *box9) {
    std::vector<Coords3D> p = to_coords(n, pos), v = to_coords(n, vel), f = to_coords(n, F);
    std::vector<double> m(mass, mass + n), inv;
    VerletIntegration::InverseMasses(m, inv);
    int step = 0;
    std::vector<double> dts = {dt, dt};
    VerletIntegration::Advance(p, v, f, inv, step, dts, to_box(box9));
    for (int i = 0; i < n; ++i)
        for (int c = 0; c < 3; ++c) {
            pos[3 * i + c] = p[i][c];
            vel[3 * i + c] = v[i][c];
        }
}

double ref_kinetic(int n, const double *vel, const double *mass, const double *F, double dt) {
    std::vector<double> kes(n, 0.0);
    double total = 0.0;
    KineticEnergy::calculateKineticEnergy(to_coords(n, vel), std::vector<double>(mass, mass + n),
                                          to_coords(n, F), dt, n, kes, total);
    return total;
}

// The public entry point: TaskDispatcher::CreateDispatcher("CPU")->Simulate.
int ref_simulate(const char *system_xml, const char *state_xml, const char *input_pdb,
                 const char *output_pdb, double dt, int steps, int interval, int force_mask) {
    try {
        auto d = TaskDispatcher::CreateDispatcher("CPU");
        if (force_mask & 1) d->EnableHarmonicBondForce();
        if (force_mask & 2) d->EnableHarmonicAngleForce();
        if (force_mask & 4) d->EnablePeriodicTorsionForce();
        if (force_mask & 8) d->EnableNonbondedForce();
        d->Simulate(system_xml, state_xml, input_pdb, output_pdb, dt, steps, interval);
    } catch (const std::exception &e) {
        std::cerr << "ref_simulate: " << e.what() << std::endl;
        return -1;
    }
    return 0;
}

}  // extern "C"

extern "C" {
// PME intermediates of the reference: moduli (3 axes concatenated), the
// spread grid and its forward transform (complex interleaved).
void ref_pme_pieces(int n, const double *pos, const double *q, const double *box9,
                    const int *grid, double *moduli, double *spread, double *fwd) {
    NonbondedParams params{};
    params.particles.resize(n);
    for (int i = 0; i < n; ++i) params.particles[i] = NonbondedParticle{q[i], 0.0, 0.0};
    std::vector<Coords3D> atoms = to_coords(n, pos);
    PeriodicBoundaryCondition::BoxInfo box = to_box(box9);
    NonbondedForce nb;
    nb.initializeReciprocalVectors(box);
    nb.initializeGridSize(box);
    if (grid && grid[0] > 0) nb.gridSize = {grid[0], grid[1], grid[2]};
    nb.InitparticleIndexAndFraction(atoms);
    nb.computeBSplineParameters(5, atoms);
    size_t k = 0;
    for (int d = 0; d < 3; ++d)
        for (int i = 0; i < nb.gridSize[d]; ++i) moduli[k++] = nb.bsplines_moduli[d][i];
    ComplexGrid g(nb.gridSize[0] * nb.gridSize[1] * nb.gridSize[2], Complex(0.0, 0.0));
    nb.gridSpreadCharge_Reference(atoms, g, params, box, 5);
    for (size_t i = 0; i < g.size(); ++i) {
        spread[2 * i] = g[i].real();
        spread[2 * i + 1] = g[i].imag();
    }
    nb.perform3DFFT(g, true);
    for (size_t i = 0; i < g.size(); ++i) {
        fwd[2 * i] = g[i].real();
        fwd[2 * i + 1] = g[i].imag();
    }
}
}
