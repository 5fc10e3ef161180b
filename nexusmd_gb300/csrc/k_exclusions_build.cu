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

// Exclusive scan of n ints, out[n] = total: each block scans kScanTile
// consecutive values (four per thread) and records its total, one block
// scans the totals, and every block adds its offset.
constexpr int kScanThreads = 1024, kScanTile = 4 * kScanThreads;

// Exclusive scan of the block's values in place (v: this thread's value);
// returns the block total to every thread.
__device__ __forceinline__ int block_scan(int &v) {
    __shared__ int wsum[32];
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int xs = v;
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
    const int total = wsum[nw - 1];
    v = (w > 0 ? wsum[w - 1] : 0) + xs - v;
    __syncthreads();  // wsum is reused by the next call
    return total;
}

__global__ void __launch_bounds__(kScanThreads) k_ex_scan_tiles(const int *in, int *out, int *tile_sum, int n) {
    const int base = blockIdx.x * kScanTile + 4 * threadIdx.x;
    int a[4], s = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        a[k] = base + k < n ? in[base + k] : 0;
        s += a[k];
    }
    int pre = s;
    const int total = block_scan(pre);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (base + k < n) out[base + k] = pre;
        pre += a[k];
    }
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
}

// the tile totals (at most kScanTile of them, so one tile) and out[n]
__global__ void __launch_bounds__(kScanThreads) k_ex_scan_sums(int *tile_sum, int ntiles, int *out, int n) {
    const int base = 4 * threadIdx.x;
    int a[4], s = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        a[k] = base + k < ntiles ? tile_sum[base + k] : 0;
        s += a[k];
    }
    int pre = s;
    const int total = block_scan(pre);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (base + k < ntiles) tile_sum[base + k] = pre;
        pre += a[k];
    }
    if (threadIdx.x == 0) out[n] = total;
}

__global__ void k_ex_scan_add(int *out, const int *tile_sum, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += tile_sum[i / kScanTile];
}

// Scan of n <= kScanTile^2 values (tile_sum holds n / kScanTile + 1 words).
static void ex_scan(const int *in, int *out, int *tile_sum, int n, cudaStream_t st) {
    const int ntiles = (n + kScanTile - 1) / kScanTile;
    if (ntiles > 0) k_ex_scan_tiles<<<ntiles, kScanThreads, 0, st>>>(in, out, tile_sum, n);
    k_ex_scan_sums<<<1, kScanThreads, 0, st>>>(tile_sum, ntiles, out, n);
    if (ntiles > 1) k_ex_scan_add<<<(n + 255) / 256, 256, 0, st>>>(out, tile_sum, n);
}

static int nblocks(long long n, int t) { return (int)((n + t - 1) / t); }

// A batch beyond the scans' reach (over 16.7 M atoms) reports overflow: the
// host builds its sets.
__global__ void k_ex_too_large(int *overflow) { *overflow = 1; }

void launch_exclusions_count(const ExclBuild &b, cudaStream_t st) {
    if ((long long)b.n > (long long)kScanTile * kScanTile) {
        k_ex_too_large<<<1, 1, 0, st>>>(b.overflow);
        return;
    }
    const long long items = (long long)b.nb + b.nx;
    cudaMemsetAsync(b.deg, 0, sizeof(int) * 4 * (size_t)b.n, st);  // deg, xdeg, afill, xfill
    if (items > 0) k_ex_degree<<<nblocks(items, 256), 256, 0, st>>>(b.bonds, b.nb, b.xc, b.nx, b.deg, b.xdeg);
    ex_scan(b.deg, b.aoff, b.tile_sum, b.n, st);
    ex_scan(b.xdeg, b.xoff, b.tile_sum, b.n, st);
    if (items > 0)
        k_ex_adjacency<<<nblocks(items, 256), 256, 0, st>>>(b.bonds, b.nb, b.xc, b.nx, b.aoff, b.xoff, b.afill,
                                                             b.xfill, b.adj, b.xadj);
    const ExclInput in{b.sys_of, b.depth, b.nb_on, b.aoff, b.adj, b.xoff, b.xadj, b.n, b.overflow};
    if (b.n > 0) k_ex_count<<<nblocks(b.n, 128), 128, 0, st>>>(in, b.len, b.plen);
    ex_scan(b.len, b.eoff, b.tile_sum, b.n, st);
    ex_scan(b.plen, b.poff, b.tile_sum, b.n, st);
}

void launch_exclusions_fill(const ExclBuild &b, int *elst, int2 *pairs, cudaStream_t st) {
    const ExclInput in{b.sys_of, b.depth, b.nb_on, b.aoff, b.adj, b.xoff, b.xadj, b.n, b.overflow};
    if (b.n > 0) k_ex_fill<<<nblocks(b.n, 128), 128, 0, st>>>(in, b.eoff, b.poff, elst, pairs);
}

}  // namespace nxm
