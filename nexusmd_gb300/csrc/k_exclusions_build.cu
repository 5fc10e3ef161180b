// Exclusion sets on the device at context creation.
//
// createExclusions (core/baseline/src/Exclusions.cpp) excludes, for every
// atom, the atoms within `depth` bonds of it (a breadth-first search over the
// bond graph); the engine unites each set with the atom's exception partners
// (OpenMM semantics: exceptions leave the Ewald direct sum too).  Here one
// thread per atom runs that search over a CSR adjacency built with atomics,
// sorts its row and writes it at its offset from an exclusive scan of the
// row lengths: the same CSR (excl_off / excl_lst, rows ascending) and the same
// list of excluded pairs j > i (ordered by i, then j; systems with the
// nonbonded force only) as a serial pass over the atoms.  A row longer than
// kExclRowMax sets an overflow word and the host builds the sets itself.
#include "nxm_view.h"

namespace nxm {

constexpr int kExclRowMax = 96;

// degree counts: items [0, nb) are bonds, [nb, nb + nx) exception pairs
__global__ void k_ex_degree(const int2 *bonds, int nb, const int2 *xc, int nx, int *deg, int *xdeg) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nb) {
        const int2 b = bonds[t];
        atomicAdd(deg + b.x, 1);
        atomicAdd(deg + b.y, 1);
    } else if (t < nb + nx) {
        const int2 p = xc[t - nb];
        atomicAdd(xdeg + p.x, 1);
        atomicAdd(xdeg + p.y, 1);
    }
}

// adjacency rows in arrival order (each row is a set; the search sorts)
__global__ void k_ex_adjacency(const int2 *bonds, int nb, const int2 *xc, int nx, const int *aoff, const int *xoff,
                               int *afill, int *xfill, int *adj, int *xadj) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nb) {
        const int2 b = bonds[t];
        adj[aoff[b.x] + atomicAdd(afill + b.x, 1)] = b.y;
        adj[aoff[b.y] + atomicAdd(afill + b.y, 1)] = b.x;
    } else if (t < nb + nx) {
        const int2 p = xc[t - nb];
        xadj[xoff[p.x] + atomicAdd(xfill + p.x, 1)] = p.y;
        xadj[xoff[p.y] + atomicAdd(xfill + p.y, 1)] = p.x;
    }
}

struct ExclInput {
    const int *sys_of, *depth, *nb_on;  // per atom: system; per system: search depth, nonbonded force on
    const int *aoff, *adj, *xoff, *xadj;
    int n;
    int *overflow;
};

// Atom i's row, ascending, into row[]; returns its length (-1: longer than
// kExclRowMax).  Levels of the search are consecutive runs of row[].
__device__ int ex_row(const ExclInput &in, int i, int *row) {
    int n = 0;
    auto add = [&](int w) {
        if (w == i) return true;
        for (int k = 0; k < n; ++k)
            if (row[k] == w) return true;
        if (n == kExclRowMax) return false;
        row[n++] = w;
        return true;
    };
    const int depth = in.depth[in.sys_of[i]];
    if (depth >= 1) {
        for (int k = in.aoff[i]; k < in.aoff[i + 1]; ++k)
            if (!add(in.adj[k])) return -1;
        int lo = 0;
        for (int d = 2; d <= depth; ++d) {
            const int hi = n;
            for (int u = lo; u < hi; ++u) {
                const int a = row[u];
                for (int k = in.aoff[a]; k < in.aoff[a + 1]; ++k)
                    if (!add(in.adj[k])) return -1;
            }
            lo = hi;
        }
    }
    for (int k = in.xoff[i]; k < in.xoff[i + 1]; ++k)
        if (!add(in.xadj[k])) return -1;
    for (int a = 1; a < n; ++a) {  // insertion sort (a few dozen entries)
        const int w = row[a];
        int b = a - 1;
        while (b >= 0 && row[b] > w) {
            row[b + 1] = row[b];
            --b;
        }
        row[b + 1] = w;
    }
    return n;
}

__device__ __forceinline__ int ex_upper(const ExclInput &in, int i, const int *row, int n) {
    if (!in.nb_on[in.sys_of[i]]) return 0;
    int u = 0;
    for (int k = 0; k < n; ++k) u += row[k] > i;
    return u;
}

__global__ void k_ex_count(ExclInput in, int *len, int *plen) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= in.n) return;
    int row[kExclRowMax];
    const int n = ex_row(in, i, row);
    if (n < 0) {
        atomicOr(in.overflow, 1);
        len[i] = plen[i] = 0;
        return;
    }
    len[i] = n;
    plen[i] = ex_upper(in, i, row, n);
}

__global__ void k_ex_fill(ExclInput in, const int *eoff, const int *poff, int *elst, int2 *pairs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= in.n) return;
    int row[kExclRowMax];
    const int n = ex_row(in, i, row);
    if (n < 0) return;
    int *dst = elst + eoff[i];
    for (int k = 0; k < n; ++k) dst[k] = row[k];
    if (!in.nb_on[in.sys_of[i]]) return;
    int2 *pd = pairs + poff[i];
    for (int k = 0; k < n; ++k)
        if (row[k] > i) *pd++ = make_int2(i, row[k]);
}

// Exclusive scan of n ints by one block; out[n] = total.
__global__ void k_ex_scan(const int *in, int *out, int n) {
    __shared__ int wsum[32];
    __shared__ int carry;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < n; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const int val = i < n ? in[i] : 0;
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
        const int prefix = carry + (w > 0 ? wsum[w - 1] : 0) + xs - val;
        if (i < n) out[i] = prefix;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = prefix + val;
        __syncthreads();
    }
    if (threadIdx.x == 0) out[n] = carry;
}

static int nblocks(long long n, int t) { return (int)((n + t - 1) / t); }

void launch_exclusions_count(const ExclBuild &b, cudaStream_t st) {
    const long long items = (long long)b.nb + b.nx;
    cudaMemsetAsync(b.deg, 0, sizeof(int) * 4 * (size_t)b.n, st);  // deg, xdeg, afill, xfill
    if (items > 0) k_ex_degree<<<nblocks(items, 256), 256, 0, st>>>(b.bonds, b.nb, b.xc, b.nx, b.deg, b.xdeg);
    k_ex_scan<<<1, 1024, 0, st>>>(b.deg, b.aoff, b.n);
    k_ex_scan<<<1, 1024, 0, st>>>(b.xdeg, b.xoff, b.n);
    if (items > 0)
        k_ex_adjacency<<<nblocks(items, 256), 256, 0, st>>>(b.bonds, b.nb, b.xc, b.nx, b.aoff, b.xoff, b.afill,
                                                             b.xfill, b.adj, b.xadj);
    const ExclInput in{b.sys_of, b.depth, b.nb_on, b.aoff, b.adj, b.xoff, b.xadj, b.n, b.overflow};
    if (b.n > 0) k_ex_count<<<nblocks(b.n, 128), 128, 0, st>>>(in, b.len, b.plen);
    k_ex_scan<<<1, 1024, 0, st>>>(b.len, b.eoff, b.n);
    k_ex_scan<<<1, 1024, 0, st>>>(b.plen, b.poff, b.n);
}

void launch_exclusions_fill(const ExclBuild &b, int *elst, int2 *pairs, cudaStream_t st) {
    const ExclInput in{b.sys_of, b.depth, b.nb_on, b.aoff, b.adj, b.xoff, b.xadj, b.n, b.overflow};
    if (b.n > 0) k_ex_fill<<<nblocks(b.n, 128), 128, 0, st>>>(in, b.eoff, b.poff, elst, pairs);
}

}  // namespace nxm
