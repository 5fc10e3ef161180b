/*
 * nexusmd-gb300: C ABI of the CUDA force-and-integrate engine (libnxm_cuda.so).
 *
 * Plain C types only: pointers, sizes, doubles.  Every function returns
 * NXM_OK (0) or a negative NXM_ERR_* code; the message of the last failure
 * is nxm_last_error() (thread-local).  Positions, velocities and forces are
 * AoS double[n][3] in nm, nm/ps and kJ/mol/nm, the layout of the reference's
 * std::vector<Coords3D> (core/common/headers/Coords3D.h:15-152).  Host
 * buffers are owned by the caller; device memory is owned by the context.
 * One CUDA stream per context; calls are synchronous with respect to the
 * host buffers they take or fill.
 *
 * Reference interfaces each group replaces (paths in the NexusMD project):
 *   nxm_dispatcher_*   TaskDispatcher / BaseLineTaskDispatcher
 *                      (core/dispatcher/headers/TaskDispatcher.h:9-43,
 *                       core/dispatcher/headers/BaseLineTaskDispatcher.h:9-52,
 *                       core/dispatcher/src/TaskDispatcher.cpp:6-23), the
 *                      object the SWIG module exposes (wrapper/NexusMD.i:1-19)
 *   nxm_parse_*        SystemXMLParser / StateXMLParser
 *                      (core/common/headers/SystemXMLParser.h:10-64,
 *                       core/common/headers/StateXMLParser.h:9-18)
 *   nxm_create .. nxm_destroy   BaseLine::Engine and its step loop
 *                      (core/baseline/headers/Engine.h:25-93,
 *                       core/baseline/src/Engine.cpp:75-188)
 */
#ifndef NXM_H
#define NXM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NXM_OK 0
#define NXM_ERR_INVALID -1   /* bad argument or inconsistent system */
#define NXM_ERR_CUDA -2      /* CUDA runtime failure or no device */
#define NXM_ERR_CAPACITY -3  /* neighbour list or exclusion capacity exceeded */
#define NXM_ERR_NUMERIC -4   /* non-finite force */
#define NXM_ERR_IO -5        /* file could not be read or written */

#define NXM_FORCE_BOND 1
#define NXM_FORCE_ANGLE 2
#define NXM_FORCE_TORSION 4
#define NXM_FORCE_NONBONDED 8

#define NXM_PRECISION_FP64 0  /* FP64 everywhere, FP64 atomics */
#define NXM_PRECISION_MIXED 1 /* FP32 forces, int64 fixed-point sums, FP64 x/v/energies */

/* One system.  Index arrays are 0-based atom indices of this system. */
typedef struct {
    int32_t n_atoms;
    const double *masses;   /* [n] */
    const double *charges;  /* [n] e */
    const double *sigmas;   /* [n] nm */
    const double *epsilons; /* [n] kJ/mol */
    int32_t n_bonds;
    const int32_t *bond_atoms;  /* [n_bonds][2] */
    const double *bond_params;  /* [n_bonds][2]: d (nm), k (kJ/mol/nm^2) */
    int32_t n_angles;
    const int32_t *angle_atoms; /* [n_angles][3] */
    const double *angle_params; /* [n_angles][2]: a (rad), k (kJ/mol/rad^2) */
    int32_t n_torsions;
    const int32_t *torsion_atoms;       /* [n_torsions][4] */
    const double *torsion_params;       /* [n_torsions][2]: k (kJ/mol), phase (rad) */
    const int32_t *torsion_periodicity; /* [n_torsions] */
    double cutoff;            /* nm */
    double ewald_tolerance;   /* alpha = sqrt(-ln(2 tol)) / cutoff */
    int32_t use_switching;    /* LJ switching function on/off */
    double switching_distance;
    int32_t grid[3];          /* PME grid; 0,0,0 = the reference's power-of-two rule */
    int32_t box_from_positions; /* 1: atom extent + 1% per side, as the reference */
    double box_lb[3], box_ub[3];  /* used when box_from_positions == 0 */
    int32_t force_mask;       /* NXM_FORCE_* bits */
    int32_t exclusion_depth;  /* bonds within which pairs are excluded; 3 in the reference */
    /* NonbondedForce exceptions in OpenMM's semantics (the reference parses
     * them, SystemXMLParser.cpp:182-191, and ignores them).  Each pair is
     * excluded from the Ewald direct sum and reciprocal-corrected like a
     * bonded exclusion, then interacts by ke*chargeProd/r +
     * 4 eps ((sigma/r)^12 - (sigma/r)^6): scaled 1-4 pairs, or pure
     * exclusions when chargeProd = epsilon = 0.  0 exceptions = the reference. */
    int32_t n_exceptions;
    const int32_t *exception_atoms;  /* [n_exceptions][2] */
    const double *exception_params;  /* [n_exceptions][3]: chargeProd (e^2), sigma (nm), epsilon (kJ/mol) */
} nxm_system_desc;

typedef struct {
    int32_t precision;        /* NXM_PRECISION_* */
    double skin;              /* nm; list radius = cutoff + skin */
    int32_t rebuild_interval; /* max steps between list rebuilds (also rebuilt when an
                                 atom moves more than skin/2); 1 = every step */
    int32_t device;           /* CUDA device ordinal */
    int32_t max_neighbors;    /* list capacity per atom; 0 = from density */
    int32_t exceptions;       /* Simulate only: 1 = apply the system XML's <Exceptions>
                                 (OpenMM semantics); 0 = ignore them, as the reference */
    int32_t autotune;         /* 1 (default): at creation, time candidate launch shapes that
                                 change no result (FFT blocking, spread/gather block size)
                                 and keep the fastest; see nxm_get_tuning */
    int32_t report_threads;   /* Simulate only: 0 = write each report before the next step,
                                 as the reference (Engine.cpp:162-188); N > 0 (default 4) =
                                 copy report snapshots into pinned double buffers and write
                                 the files on a host thread, PVF lines formatted by N threads,
                                 while the GPU steps on.  The files are byte-identical. */
    int32_t state_velocities; /* Simulate only: 1 = start from the state XML's <Velocities>
                                 when it has one per atom; 0 (default) = zero velocities,
                                 as the reference */
    int32_t fft_path;         /* PME FFT launch shape.  0 (default): the line path (5
                                 launches over tiles of lines), or the plane path (one block
                                 per x-plane for the z and y transforms, 3 launches) where
                                 the autotuner finds it faster and every system's K1 is even
                                 -- then both give the same numbers bit for bit; 1 = always
                                 the line path; 2 = the plane path wherever the planes fit
                                 in shared memory (with odd K1 the z transforms pair other
                                 lines than on the line path, which changes the rounding). */
} nxm_options;

/* Energies of one system (kJ/mol) at the last evaluation that computed them. */
typedef struct {
    double bond, angle, torsion;
    double recip, self, coulomb, vdw, exclusion; /* PE(nonbonded) = recip+self+coulomb+vdw-exclusion */
    double kinetic;
    double potential;          /* sum of the enabled terms */
    double reported_potential; /* the reference's TotalEnergy value: reciprocal energy
                                  replaces the bonded sum when nonbonded is on
                                  (NonbondedForce.cpp:387) */
    double exception;          /* exception pairs (0 without exceptions); included in both
                                  potentials above */
} nxm_energies;

typedef struct nxm_ctx nxm_ctx;

const char *nxm_version(void);

const char *nxm_last_error(void);
void nxm_default_options(nxm_options *opt);

/* Create a context for n_systems systems; positions = all systems' atoms
 * concatenated [sum n][3].  Velocities start at zero (Initializer.cpp:18-24).
 * The caller's arrays are read before the call returns.  The call returns
 * with the last set-up kernels and the first neighbour-list build still
 * queued on the context's stream (the autotuner, when it times launch shapes
 * for the first context of its shapes in the process, waits for the set-up
 * before it); a device failure of theirs is reported by the next call that
 * waits for the device.  nxm_set_positions / nxm_set_velocities likewise
 * return once the caller's array is read. */
int nxm_create(const nxm_system_desc *systems, int32_t n_systems, const nxm_options *opt,
               const double *positions, nxm_ctx **out);
void nxm_destroy(nxm_ctx *ctx);

int nxm_n_atoms(const nxm_ctx *ctx, int32_t *n_total);
int nxm_set_positions(nxm_ctx *ctx, const double *xyz);
int nxm_set_velocities(nxm_ctx *ctx, const double *xyz);

/* Forces and energies at the current positions (no integration). */
int nxm_compute_forces(nxm_ctx *ctx);

/* nsteps leapfrog steps of dt ps.  Energies and the x/v/F snapshot are taken
 * on the last step (and the kinetic energy with them). */
int nxm_step(nxm_ctx *ctx, int32_t nsteps, double dt);

/* ---- Pipelined stepping with frames read back into pinned host memory
 * (the reference's Engine::RunSimulation loop with Report, Engine.cpp:162-188,
 * with the report copies overlapped with the next steps).
 * nxm_frames_init: a ring of `depth` frame slots (1..64) in pinned host
 * memory owned by the context; nxm_step_async makes a ring of 2 when none was
 * made.  nxm_step_async: enqueues nsteps steps (the last computes energies and
 * the snapshot) and copies of that step's positions (original atom order,
 * [n][3]), energies and device flags into the next free slot, and returns
 * without waiting; NXM_ERR_INVALID when every slot still holds a frame that
 * nxm_frame_wait has not handed out.  nxm_frame_wait: waits for the oldest
 * pending frame; *xyz (if xyz is not NULL) points at its positions, valid until
 * the slot is filled again `depth` nxm_step_async calls later; energies of
 * the first n_systems systems go to energies[]; device errors of the frame's
 * steps are reported here. */
int nxm_frames_init(nxm_ctx *ctx, int32_t depth);
int nxm_step_async(nxm_ctx *ctx, int32_t nsteps, double dt);
int nxm_frame_wait(nxm_ctx *ctx, const double **xyz, nxm_energies *energies, int32_t n_systems);

/* Snapshot of the last force evaluation: positions and velocities as they
 * were when the forces were computed (before that step's update). */
int nxm_get_positions(nxm_ctx *ctx, double *xyz);
int nxm_get_velocities(nxm_ctx *ctx, double *xyz);
int nxm_get_forces(nxm_ctx *ctx, double *xyz);
/* Positions/velocities now (after the last update). */
int nxm_get_state(nxm_ctx *ctx, double *xyz, double *vel);
int nxm_get_energies(nxm_ctx *ctx, int32_t system, nxm_energies *out);
int nxm_get_box(nxm_ctx *ctx, int32_t system, double lb[3], double ub[3]);
int nxm_get_grid(nxm_ctx *ctx, int32_t system, int32_t grid[3]);
int nxm_get_alpha(nxm_ctx *ctx, int32_t system, double *alpha);

/* Neighbour pair set of one system within the cutoff at the current
 * positions, as the reference's list decides it (NeighborList.cpp:129-154):
 * pairs (i, j), i > j, this system's atom indices, in no particular order.
 * Returns the pair count (>= 0; only min(count, cap) pairs written) or an
 * error code. */
int64_t nxm_get_pairs(nxm_ctx *ctx, int32_t system, int32_t *pairs, int64_t cap);

/* Time one call of nxm_step(nsteps) on the device (CUDA events on the
 * context's stream, after the call's launches); milliseconds. */
int nxm_time_steps(nxm_ctx *ctx, int32_t nsteps, double dt, double *ms);

/* The same for nsteps steps that each compute the energies and the x/v/F
 * snapshot, as the steps of a loop that reports every step do. */
int nxm_time_report_steps(nxm_ctx *ctx, int32_t nsteps, double dt, double *ms);

/* Average device milliseconds per step of each phase over nsteps steps
 * (CUDA events between phases on the context's stream; no energies):
 * [0] list rebuild decision + rebuild, [1] bonded, [2] real-space pairs,
 * [3] exclusion correction, [4] PME spread, [5] FFT + convolution,
 * [6] PME gather, [7] integrate.  cap >= 8. */
int nxm_profile_phases(nxm_ctx *ctx, int32_t nsteps, double dt, double *ms, int32_t cap);

/* Neighbour-list rebuilds since nxm_create (waits for the context's work).
 * The reference rebuilds on every force evaluation (NeighborList.cpp:129-154
 * via NonbondedForce.cpp:474-500); this engine rebuilds when the device
 * decides (list age or displacement beyond half the skin). */
int nxm_rebuild_count(nxm_ctx *ctx, int64_t *count);

/* Launch shapes in use: [0] FFT real lines per z-pass block, or 0 when the
 * FFT runs on the plane path (one block per x-plane for the z and y
 * transforms), [1] FFT columns per x-pass (and y-pass) block, [2] threads per
 * spread/gather block (the autotuner's picks, or the defaults). */
int nxm_get_tuning(nxm_ctx *ctx, int32_t out[3]);

/* Threads per block of the FFT's plane path (the autotuner's pick or the
 * default), or 0 when the FFT runs on the line path. */
int nxm_get_fft_plane_threads(nxm_ctx *ctx, int32_t *threads);

/* One system's PME grids from the last force evaluation, as doubles (any
 * pointer may be NULL): the charge grid the spread summed, [K0][K1][K2]
 * (gridSpreadCharge_Reference, NonbondedForce.cpp:220-260); the influence
 * function on the half spectrum, [K0][K1][K2/2+1] (the eterm of
 * reciprocalConvolutionAndEnergy, :323-388); and the real grid after the
 * forward transform, the convolution and the unnormalised inverse transform,
 * [K0][K1][K2] (what PMEGridForces reads, :407-461).  Waits for the
 * context's work.  For checking the FFT against another implementation. */
int nxm_get_pme_grids(nxm_ctx *ctx, int32_t system, double *charge, double *influence, double *potential);

/* Host wall-clock milliseconds of the context's creation: [0] host set-up
 * (box, per-system constants, exclusions), [1] device allocation and
 * uploads, [2] PME tables (twiddles, B-spline moduli, influence function)
 * and FFT plan, [3] autotuning of launch shapes (about 0 when autotune is
 * off or an earlier context of the same shapes in this process was tuned:
 * *autotune_cached = 1), [4] step-graph builds so far (the first steps
 * build them), [5] the creation total [0] + [1] + [2] + [3]; within [1],
 * [6] device allocation with zeroing and [7] host-to-device copies, and [8]
 * the exclusion sets (built on the device, part of [1]).  The reference
 * builds its Engine per Simulate call (Engine.cpp:19-73). */
int nxm_get_create_timing(nxm_ctx *ctx, double ms[9], int32_t *autotune_cached);

/* Layout of one system of the context: [0] cells per cell group (one block
 * of the list-build and pair kernels per group), [1] atoms a staged
 * neighbourhood can hold, [2..4] neighbour cells per axis, [5] list capacity
 * per atom, [6] PME FFT launch shape in use (1 = line path, 2 = plane path),
 * [7] 1 when the plane path transforms each x-plane in chunks of lines (the
 * plane is larger than its shared-memory scratch), [8..10] FFT passes per
 * axis.  No counterpart in the reference (its list and FFT have no layout). */
int nxm_get_layout(nxm_ctx *ctx, int32_t system, int32_t out[11]);

/* Radices of the FFT passes along one grid axis (0, 1, 2) of one system:
 * returns the number of passes (at most cap radices written) or an error
 * code.  Replaces FFTW's internal plan (NonbondedForce.cpp:264-290). */
int nxm_get_fft_radices(nxm_ctx *ctx, int32_t system, int32_t axis, int32_t *radices, int32_t cap);

/* Kernel launches one step issues (steady state, no list rebuild). */
int nxm_launches_per_step(nxm_ctx *ctx, int32_t *launches, int32_t *rebuild_launches);

/* ---- SystemXMLParser / StateXMLParser (SystemXMLParser.cpp:18-196,
 * StateXMLParser.cpp:17-59).  A parsed system is owned by the library. */
typedef struct nxm_parsed nxm_parsed;
int nxm_parse_files(const char *system_xml, const char *state_xml, nxm_parsed **out);
void nxm_parsed_free(nxm_parsed *p);
/* Counts: atoms (masses), positions, bonds, angles, torsions, nonbonded particles, exceptions. */
int nxm_parsed_counts(const nxm_parsed *p, int64_t counts[7]);
/* Nonbonded scalars: cutoff, ewaldTolerance, switchingDistance, useSwitchingFunction,
 * alpha, rfDielectric, nx, ny, nz, method, dispersionCorrection. */
int nxm_parsed_nonbonded(const nxm_parsed *p, double out[11]);
/* Fill caller arrays (any pointer may be NULL to skip). */
int nxm_parsed_arrays(const nxm_parsed *p, double *masses, double *positions, int32_t *bond_atoms,
                      double *bond_params, int32_t *angle_atoms, double *angle_params,
                      int32_t *torsion_atoms, double *torsion_params, int32_t *torsion_per,
                      double *q_sig_eps, int32_t *exception_atoms, double *exception_params);

/* <Velocities> of the parsed state file (OpenMM writes them beside the
 * positions; the reference's StateXMLParser.cpp:17-37 reads positions only):
 * *n_out = atoms with a velocity (0 when the file has none); vel ([n][3],
 * nm/ps) may be NULL to ask for the count. */
int nxm_parsed_velocities(const nxm_parsed *p, double *vel, int64_t *n_out);

/* ---- State files (checkpoints).  OpenMM's state format: <PeriodicBoxVectors>
 * (orthorhombic edges), <Positions> (nm) and <Velocities> (nm/ps, skipped when
 * vel is NULL), every value with 17 significant digits, so nxm_parse_files /
 * nxm_parsed_velocities read back the same doubles. */
int nxm_write_state_xml(const char *path, int32_t n_atoms, const double *xyz, const double *vel,
                        const double box[3], int64_t step, double time_ps);
/* The current positions and velocities of one system of a context, written
 * as above (box edges = the system's box). */
int nxm_save_state(nxm_ctx *ctx, int32_t system, const char *path, int64_t step, double time_ps);

/* The reporters' number formatter: the text printf("%*.*f", width, prec, x)
 * gives, written to out (cap bytes, NUL-terminated); returns its length or a
 * negative NXM_ERR_* code.  Exact decimal rounding (half to even) in 128-bit
 * integers for finite |x| < 2^40 and prec <= 17, snprintf otherwise. */
int nxm_format_fixed(double x, int32_t prec, int32_t width, char *out, int32_t cap);

/* ---- TaskDispatcher (TaskDispatcher.h:9-43).  "GPU" / "CUDA" select the
 * CUDA engine; any other string prints the reference's complaint and also
 * selects it (this library has no CPU engine). */
typedef struct nxm_dispatcher nxm_dispatcher;
int nxm_dispatcher_create(const char *processor, nxm_dispatcher **out);
void nxm_dispatcher_destroy(nxm_dispatcher *d);
int nxm_dispatcher_enable_harmonic_bond_force(nxm_dispatcher *d);
int nxm_dispatcher_enable_harmonic_angle_force(nxm_dispatcher *d);
int nxm_dispatcher_enable_periodic_torsion_force(nxm_dispatcher *d);
int nxm_dispatcher_enable_nonbonded_force(nxm_dispatcher *d);
/* Engine options the reference hard-codes (precision, list skin, grid). */
int nxm_dispatcher_set_options(nxm_dispatcher *d, const nxm_options *opt);
/* TaskDispatcher::Simulate (BaseLineTaskDispatcher.h:12-40, Engine.cpp:162-188):
 * writes PVFReport<out>, TotalEnergy<out> and <out> in the reference's formats. */
int nxm_dispatcher_simulate(nxm_dispatcher *d, const char *system_xml, const char *state_xml,
                            const char *input_pdb, const char *output_pdb, double step_size,
                            int32_t total_steps, int32_t interval);

/* ---- Reciprocal-space PME that allocates nothing.  No counterpart in the
 * reference (its PME allocates its grids on every evaluation).
 *
 * The engine's mixed-precision PME step (order-5 B-splines, int64
 * fixed-point charge grid, FP32 FFT, influence function and energy) for one
 * system, on caller-owned DEVICE buffers, enqueued on `stream` (a
 * cudaStream_t; NULL = the legacy default stream) and not waited for:
 *   xyz      n_atoms x 3 doubles, nm (read)
 *   charge   n_atoms doubles, e (read)
 *   force    n_atoms x 3 doubles, kJ/mol/nm (overwritten: reciprocal force)
 *   energy   1 double, kJ/mol (overwritten: reciprocal energy)
 * Host arguments: box corners (box edge = |ub - lb|; the grid is anchored at
 * the origin as in the reference), grid sizes, Ewald alpha (1/nm).
 * All intermediates live in one static device array of about 3.7 MB per
 * device, so each grid axis must be 2^a 3^b 5^c with 5 <= K <= 64; a larger
 * grid returns NXM_ERR_CAPACITY.  It calls no cudaMalloc, cudaFree or other
 * allocating routine and copies nothing between host and device.
 * The first call on a device (the current one) looks up the array's address
 * (cudaGetSymbolAddress, which may load the module): make it before any
 * stream capture.  That address is kept for the device's primary context: after
 * cudaDeviceReset, unload and reload the library before calling again.  Every
 * call on a device shares the array and finds the previous call's contents;
 * each call clears what must start at zero, but calls whose work overlaps on
 * the GPU race: serialise them.  A CUDA error already pending on the calling
 * thread is returned as NXM_ERR_CUDA and left pending (not cleared).
 * Results agree with the engine's PME step to force rel-RMS 1e-5 and energy
 * 1e-5 relative, not bit for bit (charge grid rounded to the nearest 2^-32
 * rather than truncated to 2^-31; influence function and moduli formed on
 * the device; force converted from FP32 directly). */
int nxm_pme_reciprocal_noalloc(const double *xyz, const double *charge, int32_t n_atoms,
                               const double box_lb[3], const double box_ub[3], const int32_t grid[3],
                               double alpha, double *force, double *energy, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* NXM_H */
