// The neighbourhood of a group of cells staged in shared memory.
//
// A group is G consecutive cells of one z-row of one system's cell grid.
// Its neighbourhood is the block of cells x-2..x+2, y-2..y+2,
// z0-2..z0+G+1 (cells are >= (cutoff + skin)/2 wide, so it holds every
// atom within the list radius of any atom of the group).  In slot order the
// cells of one (ox, oy) row are adjacent, so the neighbourhood is a few
// contiguous slot spans per row, enumerated in a fixed order: rows
// ox = -2..2, oy = -2..2, then z merged into spans.  Entry k of the staged
// tile is the k-th atom of that enumeration and neighbour lists store k
// (16 bits), so the pair kernel reads j from shared memory rather than by
// scattered global loads.  Positions are staged already shifted into the
// frame of the group's first cell (the cell-image displacement is applied
// while loading), so a pair displacement is one subtraction.
#pragma once

#include "nxm_view.h"

namespace nxm {

constexpr int kHoodWarps = 16;   // warps per group block
constexpr int kMaxSpans = 128;
constexpr int kMaxGroup = kMaxGroupCells;

struct HoodSpan {
    int start;   // first slot
    int count;   // atoms
    int offset;  // first tile index
    int code0;   // cell-image code of the span's first cell (relative to the group's first cell)
    int cz0;     // z index of that cell
};

__device__ __forceinline__ int hood_wrap(int a, int n) {
    a %= n;
    return a < 0 ? a + n : a;
}

// Warp 0 lists the spans of the neighbourhood of the group whose first cell
// has packed coordinates c3 and which holds g cells; every thread gets the
// tile size after the barrier.  Cell-image codes stay in [-2, 2]^3 relative
// to the group's first cell except along z, where they run to g + 1; the
// displacement table is indexed by (ox+2)*25 + (oy+2)*5 + (oz+2) with oz up
// to kMaxGroup + 1, hence its 5 x 5 x (kMaxGroup + 4) layout.
__device__ __forceinline__ int hood_spans(const DevView &v, const SysDev &S, int c3, int g, HoodSpan *spans,
                                          int *s_n) {
    int ci[3] = {c3 & 1023, (c3 >> 10) & 1023, (c3 >> 20) & 1023};
    if (threadIdx.x < 32) {
        int lane = threadIdx.x;
        HoodSpan mine[4];
        int nm = 0, tot = 0;
        if (lane < 25) {
            int ox = lane / 5 - 2, oy = lane % 5 - 2;
            int nx = hood_wrap(ci[0] + ox, S.nc[0]), ny = hood_wrap(ci[1] + oy, S.nc[1]);
            int ncz = S.nc[2];
            int rowkey = S.cell_off + (nx * S.nc[1] + ny) * ncz;
            int codexy = ((ox + 2) * 5 + (oy + 2)) * (kMaxGroup + 4);
            int ozmax = g + 1;
            int oz = -2;
            while (oz <= ozmax && nm < 4) {
                int cz0 = hood_wrap(ci[2] + oz, ncz), oz0 = oz, cz = cz0;
                while (oz < ozmax && cz + 1 < ncz && hood_wrap(ci[2] + oz + 1, ncz) == cz + 1) {
                    ++oz;
                    ++cz;
                }
                ++oz;
                int a = v.cell_start[rowkey + cz0], b = v.cell_start[rowkey + cz + 1];
                mine[nm].start = a;
                mine[nm].count = b - a;
                mine[nm].code0 = codexy + oz0 + 2;
                mine[nm].cz0 = cz0;
                tot += b - a;
                ++nm;
            }
            if (oz <= ozmax) tot = 1 << 24;  // more spans than the enumeration holds: reported as overflow
        }
        int nsp = nm, ntot = tot;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int a = __shfl_up_sync(0xffffffffu, nsp, o), b = __shfl_up_sync(0xffffffffu, ntot, o);
            if (lane >= o) {
                nsp += a;
                ntot += b;
            }
        }
        int sp0 = nsp - nm, at0 = ntot - tot;
        for (int k = 0; k < nm; ++k) {
            HoodSpan h = mine[k];
            h.offset = at0;
            at0 += h.count;
            if (sp0 + k < kMaxSpans) spans[sp0 + k] = h;
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
