// The neighbourhood of a group of cells staged in shared memory.
//
// A group is G consecutive cells of one z-row of one system's cell grid.
// Its neighbourhood is the block of cells x-2..x+2, y-2..y+2,
// z0-2..z0+G+1 (cells are >= (cutoff + skin)/2 wide, so it holds every
// atom within the list radius of any atom of the group).  In slot order the
// cells of one (ox, oy) row are adjacent, so the neighbourhood is a few
// contiguous slot spans per row, enumerated in a fixed order: rows
// ox = -2..2, oy = -2..2, then z.  Entry k of the staged tile is the k-th
// atom of that enumeration and neighbour lists store k (16 bits), so the
// pair kernel reads j from shared memory rather than by scattered global
// loads.  Positions are staged shifted into the frame of the group's first
// cell, so a pair displacement is one subtraction.
#pragma once

#include "nxm_view.h"

namespace nxm {

constexpr int kHoodWarps = 16;   // warps per group block
constexpr int kMaxSpans = 128;
constexpr int kMaxGroup = kMaxGroupCells;
constexpr int kRowCells = kMaxGroup + 4;  // cells of one neighbourhood row, at most

struct HoodSpan {
    int start;   // first slot
    int count;   // atoms
    int offset;  // first tile index
    int code0;   // cell-image code of the span's first cell (row * kRowCells + oz + 2)
    int cz0;     // z index of that cell
};
constexpr int kSpanWords = sizeof(HoodSpan) / sizeof(int);
static_assert(kMaxSpans * kSpanWords == kGroupSpanWords, "per-group span record size");

__device__ __forceinline__ int hood_wrap(int a, int n) {
    a %= n;
    return a < 0 ? a + n : a;
}

// a in (-n, 2n): one periodic shift
__device__ __forceinline__ int wrap_once(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

// Warp 0 enumerates the neighbourhood of the group whose first cell has
// packed coordinates c3 and which holds g cells.  Lane r < 25 takes row r
// (ox = r / 5 - 2, oy = r % 5 - 2) and reads the slot range of each of its
// g + 4 cells at once; runs of cells adjacent in slot order become spans.
// With bnd, it also records the tile index of the first atom of every cell
// of every row, bnd[r * (kRowCells + 1) + oz + 2] (oz = -2 .. g + 1), and
// of the row's end (index g + 4).  Every thread gets the tile size after
// the barrier; s_n[1] holds the span count (above kMaxSpans: overflow).
__device__ __forceinline__ int hood_setup(const DevView &v, const SysDev &S, int c3, int g, HoodSpan *spans,
                                          int *s_n, int *bnd) {
    if (threadIdx.x < 32) {
        const unsigned full = 0xffffffffu;
        int lane = threadIdx.x;
        int ncz = S.nc[2], cz0 = (c3 >> 20) & 1023;
        int rowkey = 0;
        if (lane < 25) {
            int nx = hood_wrap((c3 & 1023) + lane / 5 - 2, S.nc[0]);
            int ny = hood_wrap(((c3 >> 10) & 1023) + lane % 5 - 2, S.nc[1]);
            rowkey = S.cell_off + (nx * S.nc[1] + ny) * ncz;
        }
        int a[kRowCells], b[kRowCells];
#pragma unroll
        for (int q = 0; q < kRowCells; ++q) {
            a[q] = 0;
            b[q] = 0;
            if (lane < 25 && q < g + 4) {
                int cz = wrap_once(cz0 + q - 2, ncz);
                a[q] = v.cell_start[rowkey + cz];
                b[q] = v.cell_start[rowkey + cz + 1];
            }
        }
        // spans: maximal runs of non-empty cells that continue one another in slot order
        int tot = 0, nm = 0, end = -1;
#pragma unroll
        for (int q = 0; q < kRowCells; ++q) {
            if (b[q] > a[q]) {
                nm += (a[q] != end);
                end = b[q];
            }
            tot += b[q] - a[q];
        }
        int nsp = nm, ntot = tot;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int x = __shfl_up_sync(full, nsp, o), y = __shfl_up_sync(full, ntot, o);
            if (lane >= o) {
                nsp += x;
                ntot += y;
            }
        }
        int sp = nsp - nm, off = ntot - tot;
        if (lane < 25) {
            end = -1;
            int cur = -1;
            int *bd = bnd ? bnd + lane * (kRowCells + 1) : nullptr;
#pragma unroll
            for (int q = 0; q < kRowCells; ++q) {
                if (q < g + 4) {
                    if (bd) bd[q] = off;
                    int c = b[q] - a[q];
                    if (c > 0) {
                        if (a[q] != end) {
                            cur = sp++;
                            if (cur < kMaxSpans)
                                spans[cur] = HoodSpan{a[q], c, off, lane * kRowCells + q, wrap_once(cz0 + q - 2, ncz)};
                        } else if (cur < kMaxSpans) {
                            spans[cur].count += c;
                        }
                        end = b[q];
                    }
                    off += c;
                }
            }
            if (bd) bd[g + 4] = off;
        }
        if (lane == 31) {
            s_n[0] = ntot;
            s_n[1] = nsp;
        }
    }
    __syncthreads();
    return s_n[0];
}

// Slot of tile entry k (binary search over the spans; for rare paths).
__device__ __forceinline__ int hood_slot(const HoodSpan *spans, int nsp, int k) {
    int lo = 0, hi = nsp - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (spans[mid].offset <= k)
            lo = mid;
        else
            hi = mid - 1;
    }
    return spans[lo].start + (k - spans[lo].offset);
}

}  // namespace nxm
