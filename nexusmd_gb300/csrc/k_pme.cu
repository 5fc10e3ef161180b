// PME charge spreading and force gathering (B-spline order 5), one thread per
// atom over all systems of the batch.
//
// Grid index and fraction follow InitparticleIndexAndFraction
// (core/baseline/src/Forces/NonbondedForce.cpp:51-71) in FP64: t = x / L,
// t = (t - floor t) K, index = int(t) mod K, fraction = t - int(t) -- the
// grid is anchored at the origin, not at the box's lower bound.  Spline
// weights and derivatives follow computeBSplineParameters (:144-182); the
// spread is :220-260 and the gather :407-461 (its sums regrouped per stencil
// row: the z sums first, then the row's x/y weights).  In mixed mode the
// weights are FP32 and the grid is summed as int32 fixed point in units of
// 2^-24 e (bit-reproducible).
#include <algorithm>

#include "nxm_fft.h"
#include "nxm_view.h"

namespace nxm {

void launch_fft_convolve(const DevView &v, const FftPlan &p, int energy, cudaStream_t st);

template <typename R>
__device__ __forceinline__ void bspline5(R dr, R *th, R *dth) {
    th[4] = 0;
    th[1] = dr;
    th[0] = 1 - dr;
#pragma unroll
    for (int k = 3; k < 5; k++) {
        R div = (R)1 / (R)(k - 1);
        th[k - 1] = div * dr * th[k - 2];
#pragma unroll
        for (int l = 1; l < (k - 1); l++)
            th[k - l - 1] = div * ((dr + l) * th[k - l - 2] + ((R)(k - l) - dr) * th[k - l - 1]);
        th[0] = div * (1 - dr) * th[0];
    }
    dth[0] = -th[0];
#pragma unroll
    for (int k = 1; k < 5; k++) dth[k] = th[k - 1] - th[k];
    R div = (R)0.25;
    th[4] = div * dr * th[3];
#pragma unroll
    for (int l = 1; l < 4; l++) th[4 - l] = div * ((dr + l) * th[3 - l] + ((R)(5 - l) - dr) * th[4 - l]);
    th[0] = div * (1 - dr) * th[0];
}

// Mixed-mode grid word: int32 fixed point in units of 2^-24 e, for |Q| <
// 128 e per point.  A point holds q wx wy wz summed over the atoms whose
// 5-point stencils cover it, each weight at most 115/192 per axis (< 0.22 per
// atom), so physical charge densities stay two orders of magnitude inside the
// range.  Half the bytes of an int64 word per atomic: the spread's L2 atomic
// traffic is its bound (38 -> 33 us at 94,100 atoms on a 100^3 grid).
__device__ __forceinline__ int to_grid_fixed(float v) { return __float2int_rn(v * 16777216.0f); }
__device__ __forceinline__ void grid_add(int *g, float v) { atomicAdd(g, to_grid_fixed(v)); }
__device__ __forceinline__ void grid_add(double *g, double v) { atomicAdd(g, v); }

template <typename R, typename Acc>
__global__ void __launch_bounds__(256) k_spread(DevView v, const FftSysDev *fs) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= v.N) return;
    int sys = v.sys_of[s];
    const SysDev &S = v.sys[sys];
    if (!S.nb_on) return;
    const FftSysDev &F = fs[sys];
    double p[3] = {v.x[s], v.y[s], v.z[s]};
    int idx[3];
    R fr[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        double t = p[d] * S.invL[d];
        t = (t - floor(t)) * F.K[d];
        int ti = (int)t;
        fr[d] = (R)(t - ti);
        idx[d] = ti % F.K[d];
    }
    v.pme_idx[s] = make_int4(idx[0], idx[1], idx[2], 0);
    if (sizeof(R) == 4) {
        static_cast<float4 *>(v.pme_frac)[s] = make_float4((float)fr[0], (float)fr[1], (float)fr[2], 0.f);
    } else {
        double2 *f = static_cast<double2 *>(v.pme_frac);
        f[2 * s] = make_double2((double)fr[0], (double)fr[1]);
        f[2 * s + 1] = make_double2((double)fr[2], 0.0);
    }
    R th[3][5], dth[3][5];
#pragma unroll
    for (int d = 0; d < 3; ++d) bspline5<R>(fr[d], th[d], dth[d]);
    R q = (R)v.q[s];
    Acc *g = static_cast<Acc *>(v.grid_acc) + F.roff;
    int K1 = F.K[1], K2 = F.K[2];
#pragma unroll
    for (int ix = 0; ix < 5; ++ix) {
        int xi = idx[0] + ix;
        xi -= xi >= F.K[0] ? F.K[0] : 0;
        R qx = q * th[0][ix];
#pragma unroll
        for (int iy = 0; iy < 5; ++iy) {
            int yi = idx[1] + iy;
            yi -= yi >= K1 ? K1 : 0;
            R qxy = qx * th[1][iy];
            long long row = ((long long)xi * K1 + yi) * K2;
#pragma unroll
            for (int iz = 0; iz < 5; ++iz) {
                int zi = idx[2] + iz;
                zi -= zi >= K2 ? K2 : 0;
                grid_add(g + row + zi, qxy * th[2][iz]);
            }
        }
    }
}

// Mixed-precision spread with the warp's lanes on one atom's points: each
// of the first kSpreadAtoms lanes prepares one atom of the warp (grid index,
// fraction, weights), then the warp walks those atoms and spreads each
// atom's 125 points with 32 consecutive points per instruction.
// Consecutive points share grid rows (5 contiguous words per row), so one
// atomic instruction touches ~13 memory sectors instead of the 32 of
// one-atom-per-lane; 16 atoms per warp keep twice as many warps in flight as
// 32 would.  The values are the per-atom kernel's ((q wx) wy) wz, so the
// grid is identical.
constexpr int kSpreadWarps = 8, kSpreadAtoms = 16;  // atoms per warp

__global__ void __launch_bounds__(kSpreadWarps * 32) k_spread_warp(DevView v, const FftSysDev *fs) {
    __shared__ float s_w[kSpreadWarps][kSpreadAtoms][16];  // wx[5] wy[5] wz[5] q
    __shared__ int s_i[kSpreadWarps][kSpreadAtoms][4];     // grid index x y z, system (-1: none)
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int s = (blockIdx.x * kSpreadWarps + warp) * kSpreadAtoms + lane;
    if (lane < kSpreadAtoms) {
        int sys = -1;
        if (s < v.N) {
            sys = v.sys_of[s];
            const SysDev &S = v.sys[sys];
            if (S.nb_on) {
                const FftSysDev &F = fs[sys];
                int idx[3];
                float fr[3];
                // grid coordinate = the atom's cell corner's (a table built in
                // FP64 on the host) + the FP32 offset in the cell times K / L:
                // no FP64 arithmetic, which is narrow on this GPU
                const float4 pq = v.pf[s];
                const float po[3] = {pq.x, pq.y, pq.z};
                const int c3 = v.cell3[s];
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    const float2 cg = v.cgrid[S.cg_off[d] + ((c3 >> (10 * d)) & 1023)];
                    const float u = fmaf(po[d], S.kl[d], cg.y);
                    const float fl = floorf(u);
                    int ti = ((int)cg.x + (int)fl) % F.K[d];  // a cell spans several grid points
                    ti += ti < 0 ? F.K[d] : 0;
                    fr[d] = u - fl;
                    idx[d] = ti;
                    s_i[warp][lane][d] = idx[d];
                }
                v.pme_idx[s] = make_int4(idx[0], idx[1], idx[2], 0);
                static_cast<float4 *>(v.pme_frac)[s] = make_float4(fr[0], fr[1], fr[2], 0.f);
                float th[5], dth[5];
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    bspline5<float>(fr[d], th, dth);
#pragma unroll
                    for (int k = 0; k < 5; ++k) s_w[warp][lane][5 * d + k] = th[k];
                }
                s_w[warp][lane][15] = (float)v.q[s];
            } else {
                sys = -1;
            }
        }
        s_i[warp][lane][3] = sys;
    }
    __syncwarp();
    const unsigned full = 0xffffffffu;
    for (int a = 0; a < kSpreadAtoms; ++a) {
        const int sys = s_i[warp][a][3];
        if (sys < 0) continue;
        const FftSysDev &F = fs[sys];
        const int K0 = F.K[0], K1 = F.K[1], K2 = F.K[2];
        int *g = static_cast<int *>(v.grid_acc) + F.roff;
        const float *w = s_w[warp][a];
        // lane r < 25: grid row (ix, iy) = (r / 5, r % 5) of the atom, its
        // offset and its weight (q wx) wy
        long long row_off = 0;
        float row_w = 0.f;
        if (lane < 25) {
            const int ix = lane / 5, iy = lane - 5 * ix;
            int xi = s_i[warp][a][0] + ix, yi = s_i[warp][a][1] + iy;
            xi -= xi >= K0 ? K0 : 0;
            yi -= yi >= K1 ? K1 : 0;
            row_off = ((long long)xi * K1 + yi) * K2;
            row_w = w[15] * w[ix] * w[5 + iy];
        }
        const int z0 = s_i[warp][a][2];
        // point p = 5 row + iz: 32 consecutive points per instruction
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int p = lane + 32 * k;
            const int row = min(p / 5, 24), iz = min(p - 5 * row, 4);  // (clamped past point 124)
            const long long off = __shfl_sync(full, row_off, row);
            const float rw = __shfl_sync(full, row_w, row);
            int zi = z0 + iz;
            zi -= zi >= K2 ? K2 : 0;
            if (p < 125) atomicAdd(g + off + zi, to_grid_fixed(rw * w[10 + iz]));
        }
    }
}

template <typename R, typename Acc>
__global__ void __launch_bounds__(256) k_gather(DevView v, const FftSysDev *fs) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= v.N) return;
    int sys = v.sys_of[s];
    const SysDev &S = v.sys[sys];
    if (!S.nb_on) return;
    const FftSysDev &F = fs[sys];
    int4 id = v.pme_idx[s];
    R fr[3];
    if (sizeof(R) == 4) {
        float4 f = static_cast<const float4 *>(v.pme_frac)[s];
        fr[0] = (R)f.x;
        fr[1] = (R)f.y;
        fr[2] = (R)f.z;
    } else {
        const double2 *f = static_cast<const double2 *>(v.pme_frac);
        double2 a = f[2 * s], b = f[2 * s + 1];
        fr[0] = (R)a.x;
        fr[1] = (R)a.y;
        fr[2] = (R)b.x;
    }
    R th[3][5], dth[3][5];
#pragma unroll
    for (int d = 0; d < 3; ++d) bspline5<R>(fr[d], th[d], dth[d]);
    const R *g = static_cast<const R *>(v.grid_real) + F.roff;
    int K1 = F.K[1], K2 = F.K[2];
    // the five z indices of the stencil, wrapped once
    int zo[5];
#pragma unroll
    for (int iz = 0; iz < 5; ++iz) {
        const int zi = id.z + iz;
        zo[iz] = zi >= K2 ? zi - K2 : zi;
    }
    R fx = 0, fy = 0, fz = 0;
#pragma unroll
    for (int ix = 0; ix < 5; ++ix) {
        int xi = id.x + ix;
        xi -= xi >= F.K[0] ? F.K[0] : 0;
#pragma unroll
        for (int iy = 0; iy < 5; ++iy) {
            int yi = id.y + iy;
            yi -= yi >= K1 ? K1 : 0;
            const R *row = g + ((long long)xi * K1 + yi) * K2;
            // the row's two z sums, sum_z theta_z g and sum_z dtheta_z g, then
            // the row's x/y weights once: (dx ty, tx dy, tx ty) applied to them
            R sz = 0, sdz = 0;
#pragma unroll
            for (int iz = 0; iz < 5; ++iz) {
                const R gv = row[zo[iz]];
                sz += th[2][iz] * gv;
                sdz += dth[2][iz] * gv;
            }
            const R ty = th[1][iy], dy = dth[1][iy];
            fx += (dth[0][ix] * ty) * sz;
            fy += (th[0][ix] * dy) * sz;
            fz += (th[0][ix] * ty) * sdz;
        }
    }
    R q = (R)v.q[s];
    // K / L per axis: precomputed in FP32 for the mixed engine (the same
    // rounding of the same FP64 product), in FP64 otherwise
    R kl[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) kl[d] = sizeof(R) == 4 ? (R)S.kl[d] : (R)(F.K[d] * S.invL[d]);
    using Acc_ = Acc;
    acc_add(static_cast<Acc_ *>(v.fx) + s, -(q * (fx * kl[0])));
    acc_add(static_cast<Acc_ *>(v.fy) + s, -(q * (fy * kl[1])));
    acc_add(static_cast<Acc_ *>(v.fz) + s, -(q * (fz * kl[2])));
}

// Spread: bound by the L2 atomics (125 int32 per atom), and by how many
// memory sectors each atomic instruction touches -- hence the warp-per-atom
// layout in mixed mode (the FP64 engine keeps one atom per thread).
// Alternatives measured slower at 94,100 atoms and dropped: one block per
// 8x8x8 grid tile summing its points in shared memory with no global
// atomics (the search for the atoms that reach a tile costs ~155
// instructions per contribution), a shared-memory sub-grid per box of cells
// or per 32-slot clump flushed by one atomic per point (fewer global
// atomics, no faster; with the int32 grid and native 32-bit shared atomics,
// one block per run of cells of a column with its box in shared memory and
// one thread per atom: 32.8 vs 32.9 us at 94,100 atoms, 112 vs 97 us at
// 473,400), and five threads per atom (one x-plane each).
void launch_spread(const DevView &v, const FftPlan &plan, cudaStream_t st) {
    // the accumulator (int64 fixed point or double, 8 bytes per point) starts at zero
    cudaMemsetAsync(v.grid_acc, 0, (v.mixed ? sizeof(int) : sizeof(double)) * (size_t)v.total_grid, st);
    int t = v.pme_block, nb = (v.N + t - 1) / t;
    if (v.mixed)
        k_spread_warp<<<(v.N + kSpreadWarps * kSpreadAtoms - 1) / (kSpreadWarps * kSpreadAtoms), kSpreadWarps * 32, 0,
                        st>>>(v, plan.dsys);
    else
        k_spread<double, double><<<nb, t, 0, st>>>(v, plan.dsys);
}

void launch_gather(const DevView &v, const FftPlan &plan, cudaStream_t st) {
    int t = v.pme_block, nb = (v.N + t - 1) / t;
    if (v.mixed)
        k_gather<float, long long><<<nb, t, 0, st>>>(v, plan.dsys);
    else
        k_gather<double, double><<<nb, t, 0, st>>>(v, plan.dsys);
}

void launch_pme(const DevView &v, const FftPlan &plan, int energy, cudaStream_t st) {
    if (v.N == 0 || plan.nz == 0) return;
    launch_spread(v, plan, st);
    launch_fft_convolve(v, plan, energy, st);
    launch_gather(v, plan, st);
}

}  // namespace nxm
