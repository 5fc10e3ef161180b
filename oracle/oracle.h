/*
 * CPU oracle for the NexusMD force-and-integrate path -- TEST INFRASTRUCTURE.
 *
 * A plain-C, FP64 restatement of the reference's algorithm, used only by
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg to check
 * and time the CUDA engine.  The product never calls it.  Every function
 * cites the reference file:line it follows; paths are relative to
 * NexusMD/core/.  Positions, velocities and forces are AoS double[n][3]
 * exactly like the reference's Coords3D vectors.
 */
#ifndef NXO_ORACLE_H
#define NXO_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    double lb[3], ub[3], size[3];
} nxo_box;

typedef struct {
    double bond, angle, torsion;
    double recip, self, coulomb, vdw, exclusion;
    double reported_pe; /* what the reference puts in totalPEnergy */
    double exception;   /* scaled 1-4 (exception) pairs; 0 without exceptions */
} nxo_energy;

typedef struct {
    int n;
    const double *mass, *q, *sig, *eps;
    int nb;
    const int *bonds;        /* nb x 2 */
    const double *bond_prm;  /* nb x 2: d, k */
    int na;
    const int *angles;       /* na x 3 */
    const double *angle_prm; /* na x 2: a, k */
    int nt;
    const int *torsions;       /* nt x 4 */
    const double *torsion_prm; /* nt x 2: k, phase */
    const int *torsion_per;    /* nt */
    double cutoff, ewald_tol;
    int use_switch;
    double switch_dist;
    int switch_quirk; /* 1: keep the reference's un-reset switch state */
    int grid[3];      /* 0,0,0: the reference's power-of-two rule */
    int box_mode;     /* 0: extent + 1% (reference); 1: lb/ub below */
    double lb[3], ub[3];
    int force_mask; /* 1 bond, 2 angle, 4 torsion, 8 nonbonded */
    int exclusion_depth;
    /* NonbondedForce exceptions (OpenMM semantics; the reference parses them,
     * SystemXMLParser.cpp:182-191, but never applies them).  Each pair must
     * also be in the exclusion CSR the caller passes. */
    int nexc;
    const int *exc_idx;    /* nexc x 2 */
    const double *exc_prm; /* nexc x 3: chargeProd (e^2), sigma (nm), epsilon (kJ/mol) */
} nxo_system;

/* PeriodicBoundaryCondition.cpp:11-88 / :93-104 */
void nxo_box_from_positions(int n, const double *pos, nxo_box *box);
void nxo_box_explicit(const double *lb, const double *ub, nxo_box *box);
void nxo_min_image(const double *c1, const double *c2, const nxo_box *box, double *d);

/* Bonded terms: return the energy, add forces into F[n][3]. */
double nxo_bonds(const double *pos, int nb, const int *idx, const double *prm, const nxo_box *box,
                 double *F);
double nxo_angles(const double *pos, int na, const int *idx, const double *prm,
                  const nxo_box *box, double *F);
double nxo_torsions(const double *pos, int nt, const int *idx, const double *prm, const int *per,
                    const nxo_box *box, double *F);

/* Exclusions.cpp:7-44; CSR with ascending partners.  Returns the entry count,
 * or -(needed) when cap is too small. */
long nxo_exclusions(int n, int nb, const int *bonds, int depth, int *off, int *lst, long cap);

/* NonbondedForce.cpp:33-48 and :293-321 */
void nxo_pow2_grid(const nxo_box *box, int grid[3]);
double nxo_alpha(double cutoff, double tol);

/* NeighborList.cpp:12-154.  Pairs (i, j) in the reference's order (i is the
 * atom being inserted, j < i).  Returns the count or -(needed). */
long nxo_neighbor_pairs(int n, const double *pos, const nxo_box *box, const int *eoff,
                        const int *elst, double cutoff, int *pairs, long cap);

/* PME reciprocal space, NonbondedForce.cpp:467-499; returns 0.5*sum eterm|S|^2 */
double nxo_pme(int n, const double *pos, const double *q, const nxo_box *box, double alpha,
               const int grid[3], double *F);
/* the B-spline moduli (NonbondedForce.cpp:75-142), one axis */
void nxo_bspline_moduli(int K, double *mod);
/* the charge grid Q after spreading (NonbondedForce.cpp:220-260), complex interleaved */
void nxo_spread(int n, const double *pos, const double *q, const nxo_box *box, const int grid[3],
                double *grid_out);

/* Exception pairs in OpenMM's NonbondedForce semantics (no counterpart in
 * the reference): E = ke chargeProd / r + 4 eps ((sig/r)^12 - (sig/r)^6),
 * plain Coulomb (the pair is excluded from the Ewald sum and its reciprocal
 * part removed by the exclusion correction), reference minimum image.
 * Returns the energy, adds forces into F[n][3]. */
double nxo_exceptions(const double *pos, int nexc, const int *idx, const double *prm, const nxo_box *box,
                      double *F);

/* Whole NonbondedForce::calculateForces (NonbondedForce.cpp:633-647). */
int nxo_nonbonded(const nxo_system *s, const double *pos, const nxo_box *box, const int *eoff,
                  const int *elst, double *F, nxo_energy *E);

/* Engine::CalculateForces (Engine.cpp:75-95) with per-term energies. */
int nxo_forces(const nxo_system *s, const double *pos, const nxo_box *box, const int *eoff,
               const int *elst, double *F, nxo_energy *E);

/* VerletIntegration.cpp:37-89 and KineticEnergy.cpp:21-41 */
void nxo_leapfrog(int n, double *pos, double *vel, const double *F, const double *invm, double dt,
                  const nxo_box *box);
double nxo_kinetic(int n, const double *vel, const double *mass, const double *F, double dt);

/* Engine::RunSimulation (Engine.cpp:162-188): `steps` steps from pos/vel.
 * report[k] = {step, KE, PE, total} for every report step; returns the count.
 * F receives the forces of the last step; box_out the box used. */
int nxo_run(const nxo_system *s, double *pos, double *vel, double *F, double dt, int steps,
            int interval, double *report, nxo_box *box_out);

/* Seconds of one force evaluation split by phase (for the CPU baseline). */
typedef struct {
    double nlist, direct, recip, bonded, exclusion, integrate;
} nxo_timing;
int nxo_run_timed(const nxo_system *s, double *pos, double *vel, double dt, int steps,
                  nxo_timing *t);

#ifdef __cplusplus
}
#endif
#endif
