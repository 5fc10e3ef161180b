// Neighbour-list rebuild: cell binning, a deterministic spatial sort of the
// slots, permutation of the per-atom state, and a full (both directions)
// per-atom Verlet list built one warp per atom with ballot compaction.
//
// Replaces the reference's per-step std::map voxel hash
// (core/baseline/src/Forces/NeighborList.cpp:12-154).  The set of pairs that
// reach the force kernels is the reference's: every non-excluded pair whose
// single-shift minimum-image r^2 (FP64, PeriodicBoundaryCondition.cpp:93-104)
// is below cutoff^2; the list holds a superset (cutoff + skin, with an FP32
// safety margin) and the exact test is made per step in the pair kernels.
#include "nxm_view.h"

namespace nxm {

__device__ __forceinline__ int wrapi(int a, int n) {
    a %= n;
    return a < 0 ? a + n : a;
}

__device__ __forceinline__ void cell_of(const SysDev &S, double x, double y, double z, int c[3]) {
    double p[3] = {x, y, z};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        double u = (p[d] - S.lb[d]) * S.invL[d];
        u -= floor(u);
        int k = (int)(u * S.nc[d]);
        c[d] = k < 0 ? 0 : (k >= S.nc[d] ? S.nc[d] - 1 : k);
    }
}

__global__ void k_assign(DevView v) {
    if (!v.flags->rebuild) return;
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= v.N) return;
    const SysDev &S = v.sys[v.sys_of[s]];
    int c[3];
    cell_of(S, v.x[s], v.y[s], v.z[s], c);
    int key = S.cell_off + (c[0] * S.nc[1] + c[1]) * S.nc[2] + c[2];
    v.cell_key[s] = key;
    atomicAdd(&v.cell_count[key], 1);
}

// Exclusive scan of n ints by one block, four consecutive values per
// thread per round; out[n] = total.
__global__ void __launch_bounds__(1024) k_scan(const Flags *flags, const int *in, int *out, int n) {
    if (!flags->rebuild) return;
    __shared__ int wsum[32];
    __shared__ int carry;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < n; base += 4 * blockDim.x) {
        const int i0 = base + 4 * threadIdx.x;
        int a[4], val = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            a[k] = i0 + k < n ? in[i0 + k] : 0;
            val += a[k];
        }
        int xs = val;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(full, xs, o);
            if (lane >= o) xs += y;
        }
        if (lane == 31) wsum[w] = xs;
        __syncthreads();
        if (w == 0) {
            int ws = lane < nw ? wsum[lane] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(full, ws, o);
                if (lane >= o) ws += y;
            }
            wsum[lane] = ws;
        }
        __syncthreads();
        int prefix = carry + (w > 0 ? wsum[w - 1] : 0) + xs - val;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (i0 + k < n) out[i0 + k] = prefix;
            prefix += a[k];
        }
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = prefix;
        __syncthreads();
    }
    if (threadIdx.x == 0) out[n] = carry;
}

__global__ void k_scatter(DevView v) {
    if (!v.flags->rebuild) return;
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= v.N) return;
    int key = v.cell_key[s];
    int pos = atomicAdd(&v.cell_fill[key], 1);
    v.new_orig[v.cell_start[key] + pos] = v.orig[s];
}

// Order inside a cell by z (the fractional box coordinate the cell binning
// uses), ties by original index: the layout (and every sum that follows it)
// does not depend on atomic arrival order, and each z-row of cells in a
// staged neighbourhood is sorted by z, which lets the list build bound its
// scan to the atom's z window.  One warp per cell: each lane ranks its
// elements against all of the cell's (shared memory); cells of more than
// kSortMax atoms fall back to an insertion sort by one lane.  The key, a
// fraction in [0, 1), is compared as the integer of its bits (the same
// order for non-negative doubles), which keeps the n^2 comparisons off the
// narrow FP64 pipe.
constexpr int kSortWarps = 4, kSortMax = 64;

__global__ void __launch_bounds__(kSortWarps * 32) k_cellsort(DevView v) {
    if (!v.flags->rebuild) return;
    __shared__ long long s_key[kSortWarps][kSortMax];
    __shared__ int s_org[kSortWarps][kSortMax];
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int c = blockIdx.x * kSortWarps + warp;
    if (c >= v.total_cells) return;
    int a = v.cell_start[c], n = v.cell_start[c + 1] - a;
    // the cell's count and fill words, done with, start the next rebuild at zero
    if (lane == 0) {
        v.cell_count[c] = 0;
        v.cell_fill[c] = 0;
    }
    if (n <= 1) return;
    auto key_of = [&](int o) {
        int s = v.slot_of[o];
        const SysDev &S = v.sys[v.sys_of[s]];
        double u = (v.z[s] - S.lb[2]) * S.invL[2];
        return __double_as_longlong(u - floor(u));
    };
    if (n > kSortMax) {
        if (lane == 0)
            for (int i = a + 1; i < a + n; ++i) {
                int o = v.new_orig[i];
                const long long k = key_of(o);
                int j = i - 1;
                while (j >= a) {
                    int oj = v.new_orig[j];
                    const long long kj = key_of(oj);
                    if (kj < k || (kj == k && oj < o)) break;
                    v.new_orig[j + 1] = oj;
                    --j;
                }
                v.new_orig[j + 1] = o;
            }
        return;
    }
    for (int e = lane; e < n; e += 32) {
        int o = v.new_orig[a + e];
        s_org[warp][e] = o;
        s_key[warp][e] = key_of(o);
    }
    __syncwarp();
    int dst[2], val[2], m = 0;
    for (int e = lane; e < n; e += 32) {
        const long long k = s_key[warp][e];
        int o = s_org[warp][e], r = 0;
        for (int f = 0; f < n; ++f) {
            const long long kf = s_key[warp][f];
            r += kf < k || (kf == k && s_org[warp][f] < o);
        }
        dst[m] = r;
        val[m] = o;
        ++m;
    }
    for (int t = 0; t < m; ++t) v.new_orig[a + dst[t]] = val[t];
}

constexpr int kPermArrays = 11;

__global__ void k_permute_gather(DevView v) {
    if (!v.flags->rebuild) return;
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= v.N) return;
    int so = v.slot_of[v.new_orig[s]];
    const double *src[kPermArrays] = {v.x, v.y, v.z, v.vx, v.vy, v.vz, v.mass, v.invm, v.q, v.sig, v.eps};
#pragma unroll
    for (int k = 0; k < kPermArrays; ++k) v.tmp[(size_t)k * v.N + s] = src[k][so];
}

// Per-slot derived inputs: cell coordinates, cell-relative FP32 offsets,
// scaled charges and combined LJ parameters (NonbondedForce.cpp:504-513:
// sigma/2 and 2 sqrt(eps), kept in sig / eps since creation), and the
// rebuild-time reference positions.
__device__ __forceinline__ void derive_slot(const DevView &v, int s, double x, double y, double z, double q,
                                            double sg, double ep) {
    const SysDev &S = v.sys[v.sys_of[s]];
    int c[3];
    cell_of(S, x, y, z, c);
    v.cell3[s] = c[0] | (c[1] << 10) | (c[2] << 20);
    double qs = q * sqrt(kOne4PiEps0);
    if (v.mixed) {
        double p[3] = {x, y, z};
        float o[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            double org = S.lb[d] + c[d] * S.cs[d];
            o[d] = (float)min_image(p[d] - org, S.L[d], S.halfL[d]);
        }
        v.pf[s] = make_float4(o[0], o[1], o[2], (float)qs);
        v.oref[s] = make_float4(o[0], o[1], o[2], (float)qs);
        v.ljf[s] = make_float2((float)sg, (float)ep);
        // the mixed integrator's skin test and cell offsets take
        // displacements from these in fixed point (fix40)
        long long *x40 = reinterpret_cast<long long *>(v.xref);
        x40[s] = fix40(x);
        x40[v.N + s] = fix40(y);
        x40[2 * v.N + s] = fix40(z);
    } else {
        v.qs[s] = qs;
        v.ljd[s] = make_double2(sg, ep);
        v.xref[s] = x;
        v.xref[v.N + s] = y;
        v.xref[2 * v.N + s] = z;
    }
}

// The permuted arrays into place, the slot maps, and the slot's derived
// inputs from the same values.
__global__ void k_permute_scatter(DevView v) {
    if (!v.flags->rebuild) return;
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= v.N) return;
    double *dst[kPermArrays] = {v.x, v.y, v.z, v.vx, v.vy, v.vz, v.mass, v.invm, v.q, v.sig, v.eps};
    double val[kPermArrays];
#pragma unroll
    for (int k = 0; k < kPermArrays; ++k) {
        val[k] = v.tmp[(size_t)k * v.N + s];
        dst[k][s] = val[k];
    }
    int o = v.new_orig[s];
    v.orig[s] = o;
    v.slot_of[o] = s;
    derive_slot(v, s, val[0], val[1], val[2], val[8], val[9], val[10]);
}

// The derived inputs alone (context creation, new positions).
__global__ void k_derive(DevView v) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= v.N) return;
    derive_slot(v, s, v.x[s], v.y[s], v.z[s], v.q[s], v.sig[s], v.eps[s]);
}

__global__ void k_remap(DevView v) {
    if (!v.flags->rebuild) return;
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < v.nb) {
        int2 b = v.bond_orig[t];
        v.bond_slot[t] = make_int2(v.slot_of[b.x], v.slot_of[b.y]);
        return;
    }
    t -= v.nb;
    if (t < v.na) {
        int4 a = v.angle_orig[t];
        v.angle_slot[t] = make_int4(v.slot_of[a.x], v.slot_of[a.y], v.slot_of[a.z], 0);
        return;
    }
    t -= v.na;
    if (t < v.nt) {
        int4 a = v.tors_orig[t];
        v.tors_slot[t] = make_int4(v.slot_of[a.x], v.slot_of[a.y], v.slot_of[a.z], v.slot_of[a.w]);
        return;
    }
    t -= v.nt;
    if (t < v.nex) {
        int2 e = v.ex_orig[t];
        v.ex_slot[t] = make_int2(v.slot_of[e.x], v.slot_of[e.y]);
        return;
    }
    t -= v.nex;
    if (t < v.nxc) {
        int2 e = v.xc_orig[t];
        v.xc_slot[t] = make_int2(v.slot_of[e.x], v.slot_of[e.y]);
    }
}

static inline int blocks(long long n, int t) { return (int)((n + t - 1) / t); }

void launch_derive_inputs(const DevView &v, cudaStream_t st) {
    k_derive<<<blocks(v.N, 256), 256, 0, st>>>(v);
}

void launch_remap_terms(const DevView &v, cudaStream_t st) {
    long long n = (long long)v.nb + v.na + v.nt + v.nex + v.nxc;
    if (n > 0) k_remap<<<blocks(n, 256), 256, 0, st>>>(v);
}

void launch_nlist_rebuild(const DevView &v, cudaStream_t st) {
    k_assign<<<blocks(v.N, 256), 256, 0, st>>>(v);
    k_scan<<<1, 1024, 0, st>>>(v.flags, v.cell_count, v.cell_start, v.total_cells);
    k_scatter<<<blocks(v.N, 256), 256, 0, st>>>(v);
    k_cellsort<<<blocks(v.total_cells, kSortWarps), kSortWarps * 32, 0, st>>>(v);
    k_permute_gather<<<blocks(v.N, 256), 256, 0, st>>>(v);
    k_permute_scatter<<<blocks(v.N, 256), 256, 0, st>>>(v);
    long long nt = (long long)v.nb + v.na + v.nt + v.nex + v.nxc;
    if (nt > 0) k_remap<<<blocks(nt, 256), 256, 0, st>>>(v);
    launch_build(v, st);
}

}  // namespace nxm
