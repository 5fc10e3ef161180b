// The engine's device state as one POD of device pointers, passed by value
// to every kernel, plus the kernel launchers each .cu file defines.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "nxm_common.cuh"

namespace nxm {

// ints per group of the saved neighbourhood span table (128 spans x 5 ints)
constexpr int kGroupSpanWords = 640;

struct CellGroup {
    int cell;   // first cell (global index)
    int ncell;  // consecutive cells along z in the group
    int sys;
};

struct DevView {
    int N, S;            // atoms (slots) and systems in the batch
    int mixed;           // 1: FP32 force math + int64 fixed point; 0: FP64 throughout
    int force_mask;      // 1 bond, 2 angle, 4 torsion, 8 nonbonded
    int any_switch;      // some system of the batch uses the LJ switching function
    const SysDev *sys;
    int *sys_of;         // slot -> system
    int *orig;           // slot -> original atom index (batch-global)
    int *slot_of;        // original index -> slot
    // state, slot order
    double *x, *y, *z, *vx, *vy, *vz, *mass, *invm;
    double *q;                      // raw per-atom charge
    double *sig, *eps;              // sigma/2 and 2 sqrt(eps), formed once at creation
    // derived per-slot inputs of the pair kernels
    float4 *pf;          // mixed: cell-relative offset (x,y,z), q * sqrt(ke)
    float2 *ljf;         // mixed: sigma/2, 2 sqrt(eps)
    double *qs;          // fp64: q * sqrt(ke)
    double2 *ljd;        // fp64: sigma/2, 2 sqrt(eps)
    int *cell3;          // slot -> packed cell coordinates (x | y<<10 | z<<20)
    // force accumulators (long long in mixed mode, double in fp64 mode)
    void *fx, *fy, *fz;
    // neighbour list
    int total_cells;
    int *cell_key, *cell_count, *cell_start, *cell_fill;
    int *new_orig;
    uint16_t *nl16;      // per-atom list of indices into the cell's staged neighbourhood
    int *ncount;
    int stride;
    struct CellGroup *groups;  // blocks of the tile kernels: runs of cells along z
    int ngroups;
    int hood_cap;        // capacity of a staged neighbourhood (atoms)
    int *gspan;          // [ngroups][kGroupSpanWords]: each group's neighbourhood spans, written by the list build
    int2 *gspan_n;       // [ngroups]: (atoms, spans) of that neighbourhood
    float4 *dtab;        // [S][kDtabStride] cell-image displacement per code
    float2 *cgrid;       // per system and axis, per cell: corner's PME grid coordinate (int part, fraction)
    double *xref;        // [3][N] positions at the last rebuild (mixed: as fix40 integers)
    float4 *oref;        // mixed: cell offsets at the last rebuild, .w = q * sqrt(ke)
    int *excl_off, *excl_lst;  // CSR by original index, partners as original indices
    // scratch used by the permutation
    double *tmp;         // [11][N]
    // bonded terms (original and slot indices)
    int nb, na, nt;
    int2 *bond_orig, *bond_slot;
    double2 *bond_prm;   // d, k
    int4 *angle_orig, *angle_slot;
    double2 *angle_prm;  // a, k
    int4 *tors_orig, *tors_slot;
    double2 *tors_prm;   // k, phase
    int *tors_per;
    float2 *bond_prmf, *angle_prmf, *tors_prmf;  // mixed: the same parameters in FP32
    int nex;
    int2 *ex_orig, *ex_slot;   // excluded pairs (i < j by original index)
    int nxc;                   // exception pairs (OpenMM semantics), also excluded
    int2 *xc_orig, *xc_slot;
    double4 *xc_prm;           // ke * chargeProd, sigma, 4 epsilon, 0
    float4 *xc_prmf;           // mixed: the same in FP32
    int *bond_sys, *angle_sys, *tors_sys, *ex_sys;
    // PME
    long long total_grid, total_cgrid;
    void *grid_acc;      // real grid accumulator: long long (mixed) / double
    void *grid_real;     // real grid after the inverse transform: float / double
    void *grid_cplx;     // half complex grid: float2 / double2
    void *eterm;         // influence function on the half grid: float / double
    void *twiddle;       // float2 / double2 tables, forward sign
    int pme_block;       // threads per block of the spread and gather (tuned at set-up)
    int4 *pme_idx;       // per slot grid base index (x, y, z)
    void *pme_frac;      // per slot fraction: float4 / double4-as-2xdouble2
    // energies, flags, report snapshot (original order, AoS [N][3])
    long long *E;
    Flags *flags;
    double *snap_x, *snap_v, *snap_f;
    double skin_half2;   // (skin/2)^2; 0 disables the displacement check
};

// Context creation: the exclusion sets built on the device
// (k_exclusions_build.cu).  deg, xdeg, afill and xfill are consecutive runs
// of n ints (cleared by one memset).
struct ExclBuild {
    int n, nb, nx;               // atoms, bonds, exception pairs
    const int2 *bonds, *xc;      // batch-global atom indices
    const int *sys_of, *depth, *nb_on;
    int *deg, *xdeg, *afill, *xfill;
    int *aoff, *xoff, *adj, *xadj;
    int *len, *plen, *eoff, *poff;
    int *tile_sum;               // scan scratch: n / 4096 + 1 words
    int *overflow;               // set when a row exceeds the device search's capacity
};
void launch_exclusions_count(const ExclBuild &b, cudaStream_t st);
void launch_exclusions_fill(const ExclBuild &b, int *elst, int2 *pairs, cudaStream_t st);

// kernel launchers (one per .cu file group)
void launch_nlist_rebuild(const DevView &v, cudaStream_t st);
void launch_build(const DevView &v, cudaStream_t st);
void tiles_set_smem(int hood_cap);
void launch_derive_inputs(const DevView &v, cudaStream_t st);
// bonded terms; with pairs != 0 also the exclusion correction and the
// exception pairs, in the same launch.  Returns the number of launches (0, 1).
int launch_bonded(const DevView &v, int energy, cudaStream_t st, int pairs = 0);
void launch_pairs(const DevView &v, int energy, cudaStream_t st);
void launch_exclusions(const DevView &v, int energy, cudaStream_t st);
void launch_exceptions(const DevView &v, int energy, cudaStream_t st);
void launch_pme(const DevView &v, const struct FftPlan &plan, int energy, cudaStream_t st);
void launch_spread(const DevView &v, const struct FftPlan &plan, cudaStream_t st);
void launch_fft_convolve(const DevView &v, const struct FftPlan &plan, int energy, cudaStream_t st);
void launch_gather(const DevView &v, const struct FftPlan &plan, cudaStream_t st);
void launch_integrate(const DevView &v, double dt, int report, cudaStream_t st);
void launch_snapshot_forces(const DevView &v, cudaStream_t st);
void launch_remap_terms(const DevView &v, cudaStream_t st);
long long launch_collect_pairs(const DevView &v, int sys, int *out_pairs, long long cap,
                               cudaStream_t st);

}  // namespace nxm
