// Neighbour-list build and real-space pair forces on shared-memory tiles.
//
// One block per group of consecutive cells (nxm_hood.cuh): the block stages
// the group's neighbourhood once, then each warp takes atoms of the group.
//
// Physics follows NonbondedForce::DirectForcesAndEnergy
// (core/baseline/src/Forces/NonbondedForce.cpp:530-585): sigma_ij =
// sigma_i/2 + sigma_j/2, eps_ij = (2 sqrt eps_i)(2 sqrt eps_j), no LJ shift,
// no dispersion correction.  The optional switching function is applied per
// pair (the reference never resets its switch state between pairs, :541;
// that order-dependent carry-over is not reproduced).  Pair membership is
// decided exactly as the reference's list does (NeighborList.cpp:106-116):
// FP64 single-shift minimum image (PeriodicBoundaryCondition.cpp:93-104),
// r^2 < cutoff^2.  The list holds a superset (cutoff + skin, FP32 test with
// a safety margin); in mixed mode the FP32 r^2 settles every pair except
// those within 1e-5 relative of the cutoff, which are re-tested in FP64.
#include <mutex>
#include <type_traits>

#include "nxm_hood.cuh"
#include "nxm_view.h"

namespace nxm {

// r^2 of the pair exactly as the reference forms it: d = p_j - p_i with one
// shift per component, then (dx*dx + dy*dy) + dz*dz with no fused multiply-add.
__device__ __forceinline__ double exact_r2(const DevView &v, const SysDev &S, int i, int j) {
    double dx = min_image(__dsub_rn(v.x[j], v.x[i]), S.L[0], S.halfL[0]);
    double dy = min_image(__dsub_rn(v.y[j], v.y[i]), S.L[1], S.halfL[1]);
    double dz = min_image(__dsub_rn(v.z[j], v.z[i]), S.L[2], S.halfL[2]);
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

__device__ __forceinline__ void offset_in_cell(const DevView &v, const SysDev &S, int s, int c3, float o[3]) {
    int c[3] = {c3 & 1023, (c3 >> 10) & 1023, (c3 >> 20) & 1023};
    double p[3] = {v.x[s], v.y[s], v.z[s]};
#pragma unroll
    for (int d = 0; d < 3; ++d) o[d] = (float)min_image(p[d] - (S.lb[d] + c[d] * S.cs[d]), S.L[d], S.halfL[d]);
}

// Atom i's position in the frame of the group's first cell.
__device__ __forceinline__ void i_in_group_frame(const DevView &v, const SysDev &S, int i, int cz_first, float p[3]) {
    int c3 = v.cell3[i];
    float gz = (float)wrap_once(((c3 >> 20) & 1023) - cz_first, S.nc[2]) * S.csf[2];
    if (v.mixed) {
        float4 q = v.pf[i];
        p[0] = q.x;
        p[1] = q.y;
        p[2] = q.z + gz;
    } else {
        offset_in_cell(v, S, i, c3, p);
        p[2] += gz;
    }
}

// This system's cell-image displacements (v.dtab: code r * kRowCells +
// oz + 2 -> -(ox, oy, oz) * cell edge) copied into shared memory by the
// threads outside warp 0 while warp 0 enumerates the neighbourhood; read
// after the barrier that follows.
__device__ __forceinline__ void load_dtab(const DevView &v, int sys, float4 *s_dt) {
    const float4 *dt = v.dtab + sys * kDtabStride;
    for (int e = (int)threadIdx.x - 32; e < 25 * kRowCells; e += blockDim.x - 32)
        if (e >= 0) s_dt[e] = __ldg(dt + e);
}

// Stage the group's neighbourhood (spans already in shared memory):
// positions shifted into the group frame, .w = the scaled charge (pair
// kernel, mixed mode) or the original index's bits (build), and the LJ
// parameters (pair kernel).  Each atom's
// own-cell offset is shifted by its cell's displacement from the group's
// first cell (a span's cells are consecutive in z, so the code is the
// span's first code plus the z step).  In mixed mode each lane loads four
// atoms of its span before it stores any, so the loads of a span are in
// flight together.
template <bool BUILD, bool MIXED>
__device__ void stage(const DevView &v, const SysDev &S, float4 *s_q, float2 *s_lj, const HoodSpan *spans, int nsp,
                      const float4 *s_dt) {
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int sp = warp; sp < nsp; sp += nw) {
        HoodSpan h = spans[sp];
        if (MIXED) {
            constexpr int U = 4;
            for (int t0 = 0; t0 < h.count; t0 += 32 * U) {
                int cj[U], oj[U];
                float4 p[U];
                float2 l[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    int t = t0 + lane + 32 * u;
                    if (t < h.count) {
                        int j = h.start + t;
                        cj[u] = v.cell3[j];
                        p[u] = v.pf[j];
                        if (BUILD)
                            oj[u] = v.orig[j];
                        else
                            l[u] = v.ljf[j];
                    }
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    int t = t0 + lane + 32 * u;
                    if (t < h.count) {
                        int k = h.offset + t;
                        float4 D = s_dt[h.code0 + (((cj[u] >> 20) & 1023) - h.cz0)];
                        s_q[k] = make_float4(p[u].x - D.x, p[u].y - D.y, p[u].z - D.z,
                                             BUILD ? __int_as_float(oj[u]) : p[u].w);
                        if (!BUILD) s_lj[k] = l[u];
                    }
                }
            }
        } else {
            for (int t = lane; t < h.count; t += 32) {
                int j = h.start + t, k = h.offset + t;
                int cj = v.cell3[j];
                float4 D = s_dt[h.code0 + (((cj >> 20) & 1023) - h.cz0)];
                float o[3];
                offset_in_cell(v, S, j, cj, o);
                s_q[k] = make_float4(o[0] - D.x, o[1] - D.y, o[2] - D.z, BUILD ? __int_as_float(v.orig[j]) : 0.f);
            }
        }
    }
    __syncthreads();
}

// List layout: each 256-entry chunk of an atom's list is stored transposed,
// entry p of the chunk at position 8 * (p mod 32) + p / 32, so that lane L
// of a warp fetches entries L, L+32, ..., L+224 with one 16-byte load.
// An entry holds 8 times the tile index (the byte offset of the atom's LJ
// pair in the pair kernel's staged tile; tile indices stay below 8,192).
__device__ __forceinline__ int list_pos(int p) { return (p & ~255) | ((p & 31) << 3) | ((p >> 5) & 7); }
constexpr int kEntryShift = 3;

// ------------------------------------------------------------------ build

// Each warp takes atoms of the group; every staged atom within the list
// radius that is not i itself and not excluded is appended to i's list as
// its 16-bit tile index (ballot compaction: deterministic order).  An atom
// scans only the rows of the neighbourhood its list sphere reaches, and in
// each row (z-sorted: k_cellsort orders every cell by z) only the atoms
// within the z extent the sphere has over that row, found by binary search
// (0.01 nm margin), in tile order: the list is the one a scan of the whole
// tile gives.
// Stores one 256-entry list chunk held in order in shared memory as the list
// layout wants it: lane l writes 16 bytes, entries l + 32 q for q = 0..7.
__device__ __forceinline__ void store_chunk(uint16_t *dst, const uint16_t *src, int lane) {
    uint32_t w[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) w[q] = (uint32_t)src[lane + 64 * q] | ((uint32_t)src[lane + 64 * q + 32] << 16);
    reinterpret_cast<uint4 *>(dst)[lane] = make_uint4(w[0], w[1], w[2], w[3]);
}

// W warps per block: 16 (two blocks per SM) or, when two blocks' shared
// memory does not fit on an SM, 32 (one block per SM, the same 32 warps).
template <int W>
__global__ void __launch_bounds__(W * 32, W == kHoodWarps ? 2 : 1) k_build(DevView v) {
    extern __shared__ __align__(16) unsigned char smem[];
    if (!v.flags->rebuild) return;
    const unsigned full = 0xffffffffu;
    CellGroup G = v.groups[blockIdx.x];
    int a0 = v.cell_start[G.cell], a1 = v.cell_start[G.cell + G.ncell];
    if (a0 == a1) return;
    const SysDev &S = v.sys[G.sys];
    if (!S.nb_on) {
        for (int i = a0 + threadIdx.x; i < a1; i += blockDim.x) v.ncount[i] = 0;
        return;
    }
    int cap = v.hood_cap;
    float4 *s_q = reinterpret_cast<float4 *>(smem);  // .w: the original index's bits
    uint16_t *s_buf = reinterpret_cast<uint16_t *>(s_q + cap);  // [W][2][256], 16-byte aligned
    int *s_bnd = reinterpret_cast<int *>(s_buf + W * 512);
    HoodSpan *spans = reinterpret_cast<HoodSpan *>(s_bnd + 25 * (kRowCells + 1));
    int *s_n = reinterpret_cast<int *>(spans + kMaxSpans);
    __shared__ float4 s_dt[25 * kRowCells];
    int c3f = v.cell3[a0];
    load_dtab(v, G.sys, s_dt);
    int n = hood_setup(v, S, c3f, G.ncell, spans, s_n, s_bnd);
    int nsp = s_n[1];
    // the spans, for the pair kernel's steps until the next rebuild
    {
        const int *src = reinterpret_cast<const int *>(spans);
        int *dst = v.gspan + (size_t)blockIdx.x * kGroupSpanWords;
        for (int e = threadIdx.x; e < min(nsp, kMaxSpans) * kSpanWords; e += blockDim.x) dst[e] = src[e];
        if (threadIdx.x == 0) v.gspan_n[blockIdx.x] = make_int2(n, nsp);
    }
    if (n > v.hood_cap || nsp > kMaxSpans) {
        if (threadIdx.x == 0) atomicOr(&v.flags->error, ERR_NLIST_OVERFLOW);
        return;
    }
    if (v.mixed)
        stage<true, true>(v, S, s_q, nullptr, spans, nsp, s_dt);
    else
        stage<true, false>(v, S, s_q, nullptr, spans, nsp, s_dt);
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    float rl2 = S.rlist2f * 1.0001f + 1e-6f;
    const float margin = 0.01f;
    const float rlm = sqrtf(rl2) + margin;
    const float csx = (float)S.cs[0], csy = (float)S.cs[1], csz = (float)S.cs[2], icsz = 1.0f / csz;
    int czf = (c3f >> 20) & 1023;
    int g = G.ncell;
    for (int i = a0 + warp; i < a1; i += nw) {
        float pi3[3];
        i_in_group_frame(v, S, i, czf, pi3);
        int oi = v.orig[i];
        int e0 = v.excl_off[oi];
        int ne = v.excl_off[oi + 1] - e0;
        int my_ex = lane < ne ? v.excl_lst[e0 + lane] : -1;
        int nfast = ne < 32 ? ne : 32;
        // Index window [ex_lo, ex_lo + ex_win] of i itself and its exclusion
        // partners (rows ascending): a candidate outside it needs no
        // membership test.  i is left out by its index too, so every image
        // of i is (the far one lies beyond the list radius anyway).
        const int ex_lo = ne ? min(v.excl_lst[e0], oi) : oi;
        const unsigned ex_win = (unsigned)((ne ? max(v.excl_lst[e0 + ne - 1], oi) : oi) - ex_lo);
        int count = 0;
        uint16_t *out = v.nl16 + (size_t)i * v.stride;
        // lane r < 25: the tile range [kb, ke) of row r that i's sphere reaches
        int kb = 0, ke = 0;
        if (lane < 25) {
            // distance from i to the row's cell column in x and y
            float ox = (float)(lane / 5 - 2), oy = (float)(lane % 5 - 2);
            float ddx = fmaxf(fmaxf(ox * csx - pi3[0], pi3[0] - (ox + 1.0f) * csx), 0.0f);
            float ddy = fmaxf(fmaxf(oy * csy - pi3[1], pi3[1] - (oy + 1.0f) * csy), 0.0f);
            float rem = rlm * rlm - (ddx * ddx + ddy * ddy);
            if (rem >= 0.0f) {
                float h = sqrtf(rem) + margin;
                int zlo = max((int)floorf((pi3[2] - h) * icsz), -2);
                int zhi = min((int)floorf((pi3[2] + h) * icsz), g + 1);
                if (zlo <= zhi) {
                    const int *b = s_bnd + lane * (kRowCells + 1);
                    // the row is sorted by z (cells in z order, atoms in a
                    // cell by z): narrow to the atoms with z in pz +- h.  The
                    // first such atom lies in cell zlo and the last in cell
                    // zhi, so each search covers one cell.
                    const float zl = pi3[2] - h, zh = pi3[2] + h;
                    int l = b[zlo + 2], r = b[zlo + 3];
                    while (l < r) {
                        int mid = (l + r) >> 1;
                        if (s_q[mid].z < zl)
                            l = mid + 1;
                        else
                            r = mid;
                    }
                    kb = l;
                    l = max(b[zhi + 2], kb);
                    r = b[zhi + 3];
                    while (l < r) {
                        int mid = (l + r) >> 1;
                        if (s_q[mid].z <= zh)
                            l = mid + 1;
                        else
                            r = mid;
                    }
                    ke = l;
                }
            }
        }
        // i's list is assembled per 256-entry chunk in two halves per warp
        // (entry p at p & 511), so an iteration that completes a chunk writes
        // on into the other half; a completed chunk is stored transposed as
        // in memory (lane l's 16 bytes hold entries l + 32 q, q = 0..7)
        uint16_t *buf = s_buf + warp * 512;
        const unsigned lt = (1u << lane) - 1u;
        unsigned rows = __ballot_sync(full, ke > kb);
        while (rows) {
            int r = __ffs(rows) - 1;
            rows &= rows - 1;
            const int rb = __shfl_sync(full, kb, r), re = __shfl_sync(full, ke, r);
            for (int k0 = rb; k0 < re; k0 += 32) {
                // k past the row's end reads a later row or the chunk
                // buffers behind the tile, inside the block's shared
                // memory; such a lane is no candidate
                const int k = k0 + lane;
                const float4 q = s_q[k];
                const float dx = pi3[0] - q.x, dy = pi3[1] - q.y, dz = pi3[2] - q.z;
                bool cand = (k < re) & (fmaf(dz, dz, fmaf(dy, dy, dx * dx)) < rl2);
                const int oj = __float_as_int(q.w);
                if (__any_sync(full, cand && (unsigned)(oj - ex_lo) <= ex_win)) {
                    bool ex = oj == oi;
                    for (int e = 0; e < nfast; ++e) ex |= (__shfl_sync(full, my_ex, e) == oj);
                    if (ne > 32 && cand)
                        for (int e = 32; e < ne; ++e) ex |= (v.excl_lst[e0 + e] == oj);
                    cand = cand && !ex;
                }
                const unsigned m = __ballot_sync(full, cand);
                const int newc = count + __popc(m);
                // every lane stores: a rejected candidate goes to count + 32 +
                // lane, past the entries of this iteration -- a slot that a
                // later entry overwrites or that lies beyond the list's count
                // (never in the half being stored: at most 32 entries come
                // per iteration)
                buf[(cand ? count + __popc(m & lt) : count + 32 + lane) & 511] = (uint16_t)(k << kEntryShift);
                if ((newc ^ count) >> 8) {
                    // chunk count >> 8 complete: one 16-byte store per lane
                    __syncwarp();
                    const int c = count >> 8;
                    if ((c + 1) * 256 <= v.stride) store_chunk(out + c * 256, buf + (c & 1) * 256, lane);
                    __syncwarp();
                }
                count = newc;
            }
        }
        __syncwarp();
        {
            const int c = count >> 8;
            if ((count & 255) && c * 256 < v.stride) store_chunk(out + c * 256, buf + (c & 1) * 256, lane);
        }
        __syncwarp();
        if (lane == 0) {
            v.ncount[i] = count < v.stride ? count : v.stride;
            if (count > v.stride) atomicOr(&v.flags->error, ERR_NLIST_OVERFLOW);
        }
    }
}

// ------------------------------------------------------------------ pairs

struct PairPrm {
    float ex2c, a04, k2a, sw, cut;  // SysDev::ex2c, a04, k2a
    int use_sw;
};

__device__ __forceinline__ float fast_ex2(float x) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// FP32 force (and energy) of one list entry, accumulated into the lane's
// partial sums when `in` (inside the cutoff), NonbondedForce.cpp:559-581 in
// single precision.  Evaluated without branches: an entry outside the cutoff
// (r^2 up to 1e30 for padding) gives finite values that the select drops, so
// two entries per lane run as independent instruction streams.
template <bool ENERGY, bool SW>
__device__ __forceinline__ void pair_mixed(bool in, float dx, float dy, float dz, float r2, float qq, float sg,
                                           float eps, const PairPrm &P, float &fx, float &fy, float &fz,
                                           float &ec, float &ev) {
    float rinv = fast_rsqrt(r2);
    float rinv2 = rinv * rinv;
    float r = r2 * rinv;
    // exp(-(alpha r)^2) straight from r^2; erfc(alpha r) = exp(-(alpha r)^2) g(t),
    // t = 1 / (1 + 0.4 alpha r); 2 alpha r / sqrt(pi) as k2a * r
    float ex = fast_ex2(r2 * P.ex2c);
    float erfcv = ex * erfcx_fit(fast_rcp(fmaf(P.a04, r, 1.0f)));
    float qr = qq * rinv;
    float dEdR = qr * rinv2 * fmaf(P.k2a * r, ex, erfcv);
    float s2 = sg * sg * rinv2;
    float s6 = s2 * s2 * s2;
    float evdw = eps * (s6 - 1.0f) * s6;
    float sw = 1.0f;
    if (SW && P.use_sw && r > P.sw) {
        float w = P.cut - P.sw;
        float t = (r - P.sw) / w;
        sw = 1.0f + t * t * t * (-10.0f + t * (15.0f - t * 6.0f));
        float dsw = t * t * (-30.0f + t * (60.0f - t * 30.0f)) / w;
        dEdR -= evdw * dsw * rinv;
    }
    float lj = eps * (12.0f * s6 - 6.0f) * s6;
    if (SW) lj *= sw;
    dEdR = fmaf(lj, rinv2, dEdR);
    dEdR = in ? dEdR : 0.0f;
    fx = fmaf(dx, dEdR, fx);
    fy = fmaf(dy, dEdR, fy);
    fz = fmaf(dz, dEdR, fz);
    if (ENERGY) {
        ec += in ? qr * erfcv : 0.0f;
        ev += in ? (SW ? sw * evdw : evdw) : 0.0f;
    }
}

// Per-system constants of pair_mixed2, each in both halves of a float2.
struct PairPrm2 {
    float2 ex2c, a04, k2a, one, twelve, msix, mone;
};

__device__ __forceinline__ float2 dup2(float a) { return make_float2(a, a); }

__device__ __forceinline__ float2 erfcx_fit2(float2 t) {
    float2 g = dup2(-2.164941738e-01f);
    g = __ffma2_rn(g, t, dup2(7.803782561e-01f));
    g = __ffma2_rn(g, t, dup2(-4.985805536e-01f));
    g = __ffma2_rn(g, t, dup2(5.875147125e-01f));
    g = __ffma2_rn(g, t, dup2(1.009222009e-01f));
    g = __ffma2_rn(g, t, dup2(2.479314205e-01f));
    g = __ffma2_rn(g, t, dup2(-1.671998421e-03f));
    return g;
}

// pair_mixed for a lane's two entries at once (no switching function): the
// same chain of operations per entry in the two halves of packed FP32x2
// arithmetic, one instruction for both entries (the reciprocal square root,
// exponential and reciprocal stay scalar); about a sixth fewer instructions
// per entry.  The displacements come as j - i, so the force sums (fxy = x,
// y; fz) are negated sums; the caller flips their sign.
template <bool ENERGY>
__device__ __forceinline__ void pair_mixed2(bool in0, bool in1, float2 dxy0, float dz0, float2 dxy1, float dz1,
                                            float2 r2, float2 qq, float2 sg, float2 eps, const PairPrm2 &P,
                                            float2 &fxy, float &fz, float2 &ecv) {
    float2 rinv = make_float2(fast_rsqrt(r2.x), fast_rsqrt(r2.y));
    float2 rinv2 = __fmul2_rn(rinv, rinv);
    float2 r = __fmul2_rn(r2, rinv);
    float2 ea = __fmul2_rn(r2, P.ex2c);
    float2 ex = make_float2(fast_ex2(ea.x), fast_ex2(ea.y));
    float2 tt = __ffma2_rn(P.a04, r, P.one);
    float2 erfcv = __fmul2_rn(ex, erfcx_fit2(make_float2(fast_rcp(tt.x), fast_rcp(tt.y))));
    float2 qr = __fmul2_rn(qq, rinv);
    float2 dEdR = __fmul2_rn(__fmul2_rn(qr, rinv2), __ffma2_rn(__fmul2_rn(P.k2a, r), ex, erfcv));
    float2 s2 = __fmul2_rn(__fmul2_rn(sg, sg), rinv2);
    float2 s6 = __fmul2_rn(__fmul2_rn(s2, s2), s2);

    float2 lj = __fmul2_rn(__fmul2_rn(eps, __ffma2_rn(P.twelve, s6, P.msix)), s6);
    dEdR = __ffma2_rn(lj, rinv2, dEdR);
    const float d0 = in0 ? dEdR.x : 0.0f, d1 = in1 ? dEdR.y : 0.0f;
    fxy = __ffma2_rn(dxy0, dup2(d0), fxy);
    fz = fmaf(dz0, d0, fz);
    fxy = __ffma2_rn(dxy1, dup2(d1), fxy);
    fz = fmaf(dz1, d1, fz);
    if (ENERGY) {
        // (Coulomb, LJ) as one packed sum, entry 0 then entry 1 (entries
        // outside the cutoff add zero)
        const float2 e = __fmul2_rn(qr, erfcv);
        const float2 l = __fmul2_rn(__fmul2_rn(eps, __fadd2_rn(s6, P.mone)), s6);
        ecv = __fadd2_rn(ecv, make_float2(in0 ? e.x : 0.0f, in0 ? l.x : 0.0f));
        ecv = __fadd2_rn(ecv, make_float2(in1 ? e.y : 0.0f, in1 ? l.y : 0.0f));
    }
}

// Mixed precision: each lane keeps two list entries in flight; j comes from
// the staged tile.  SW: some system of the batch uses the switching function.
template <bool ENERGY, bool SW, int W>
__global__ void __launch_bounds__(W * 32, W == kHoodWarps ? 2 : 1) k_pairs_mixed(DevView v) {
    extern __shared__ __align__(16) unsigned char smem[];
    const unsigned full = 0xffffffffu;
    CellGroup G = v.groups[blockIdx.x];
    int a0 = v.cell_start[G.cell], a1 = v.cell_start[G.cell + G.ncell];
    if (a0 == a1) return;
    const SysDev &S = v.sys[G.sys];
    if (!S.nb_on) return;
    int cap = v.hood_cap;
    // tile: LJ pairs first (a list entry is the byte offset of its atom's
    // pair), then positions at twice that offset past them (cap is a
    // multiple of 32, so the positions stay 16-byte aligned)
    float2 *s_lj = reinterpret_cast<float2 *>(smem);
    float4 *s_q = reinterpret_cast<float4 *>(s_lj + cap);
    HoodSpan *spans = reinterpret_cast<HoodSpan *>(s_q + cap);
    const unsigned char *q_base = reinterpret_cast<const unsigned char *>(s_q);
    __shared__ float4 s_dt[25 * kRowCells];
    __shared__ int2 s_nn;
    int c3f = v.cell3[a0];
    // the neighbourhood's spans as the list build enumerated them (the
    // cells have not changed since), and the displacement table
    {
        const int *src = v.gspan + (size_t)blockIdx.x * kGroupSpanWords;
        int *dst = reinterpret_cast<int *>(spans);
        for (int e = threadIdx.x; e < kGroupSpanWords; e += blockDim.x) dst[e] = src[e];
        if (threadIdx.x == 0) s_nn = v.gspan_n[blockIdx.x];
        const float4 *dt = v.dtab + G.sys * kDtabStride;
        for (int e = threadIdx.x; e < 25 * kRowCells; e += blockDim.x) s_dt[e] = __ldg(dt + e);
    }
    __syncthreads();
    const int n = s_nn.x, nsp = s_nn.y;
    if (n > v.hood_cap || nsp > kMaxSpans) {
        if (threadIdx.x == 0) atomicOr(&v.flags->error, ERR_NLIST_OVERFLOW);
        return;
    }
    stage<false, true>(v, S, s_q, s_lj, spans, nsp, s_dt);
    int czf = (c3f >> 20) & 1023;
    const float lo = S.cut2f_lo, hi = S.cut2f_hi;
    const PairPrm P{S.ex2c, S.a04, S.k2a, S.sw_distf, S.cutofff, S.use_switch};
    const PairPrm2 P2{dup2(S.ex2c), dup2(S.a04), dup2(S.k2a), dup2(1.0f), dup2(12.0f), dup2(-6.0f), dup2(-1.0f)};
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    float ec = 0.f, ev = 0.f;
    float2 ecv = make_float2(0.f, 0.f);  // pair_mixed2's (Coulomb, LJ) sums
    for (int i = a0 + warp; i < a1; i += nw) {
        float pi3[3];
        i_in_group_frame(v, S, i, czf, pi3);
        const float qi = v.pf[i].w;
        const float2 li = v.ljf[i];
        const int cnt = v.ncount[i];
        const uint4 *lst4 = reinterpret_cast<const uint4 *>(v.nl16 + (size_t)i * v.stride) + lane;
        float fx = 0.f, fy = 0.f, fz = 0.f;
        // without the switching function: negated x, y sums as a pair (pair_mixed2)
        float2 fxy = make_float2(0.f, 0.f);
        const float2 nxy = make_float2(-pi3[0], -pi3[1]);
        const float nz = -pi3[2];
        // the first chunk's slot always exists: its load need not wait for the count
        uint4 cur = __ldg(lst4);
        for (int c0 = 0; c0 < cnt; c0 += 256) {
            // this lane's entries c0 + lane + 32u, u = 0..7, and the next chunk in flight
            uint4 nxt = c0 + 256 < cnt ? __ldg(lst4 + (c0 + 256) / 8) : make_uint4(0, 0, 0, 0);
            uint32_t wds[4] = {cur.x, cur.y, cur.z, cur.w};
            // bit u: entry u's FP32 r^2 lies within 1e-5 of the cutoff, so
            // the FP32 test (which left it out) is re-done in FP64 below
            unsigned amb = 0;
            // FULL: all 256 entries of the chunk are valid (every chunk but
            // the last), so the per-entry range checks compile away
            auto walk = [&](auto full_chunk) {
                constexpr bool FULL = decltype(full_chunk)::value;
#pragma unroll
                for (int u = 0; u < 8; u += 2) {
                    if (!FULL && c0 + 32 * u >= cnt) break;  // rest of the last chunk is empty (warp-uniform)
                    int k0 = c0 + lane + 32 * u;
                    bool v0 = FULL || k0 < cnt, v1 = FULL || k0 + 32 < cnt;
                    const unsigned e0 = v0 ? (wds[u >> 1] & 0xffffu) : 0u;
                    const unsigned e1 = v1 ? (wds[u >> 1] >> 16) : 0u;
                    const float4 p0 = *reinterpret_cast<const float4 *>(q_base + 2 * e0);
                    const float4 p1 = *reinterpret_cast<const float4 *>(q_base + 2 * e1);
                    const float2 l0 = *reinterpret_cast<const float2 *>(smem + e0);
                    const float2 l1 = *reinterpret_cast<const float2 *>(smem + e1);
                    // j - i: x and y as one pair per entry
                    const float2 dxy0 = __fadd2_rn(make_float2(p0.x, p0.y), nxy);
                    const float2 dxy1 = __fadd2_rn(make_float2(p1.x, p1.y), nxy);
                    const float dz0 = p0.z + nz, dz1 = p1.z + nz;
                    float r20 = v0 ? fmaf(dz0, dz0, fmaf(dxy0.y, dxy0.y, dxy0.x * dxy0.x)) : 1e30f;
                    float r21 = v1 ? fmaf(dz1, dz1, fmaf(dxy1.y, dxy1.y, dxy1.x * dxy1.x)) : 1e30f;
                    const bool in0 = r20 < lo, in1 = r21 < lo;
                    amb |= ((!in0 && r20 < hi) ? 1u : 0u) << u;
                    amb |= ((!in1 && r21 < hi) ? 1u : 0u) << (u + 1);
                    if (SW) {
                        pair_mixed<ENERGY, SW>(in0, -dxy0.x, -dxy0.y, -dz0, r20, qi * p0.w, li.x + l0.x,
                                               li.y * l0.y, P, fx, fy, fz, ec, ev);
                        pair_mixed<ENERGY, SW>(in1, -dxy1.x, -dxy1.y, -dz1, r21, qi * p1.w, li.x + l1.x,
                                               li.y * l1.y, P, fx, fy, fz, ec, ev);
                    } else {
                        pair_mixed2<ENERGY>(in0, in1, dxy0, dz0, dxy1, dz1, make_float2(r20, r21),
                                            make_float2(qi * p0.w, qi * p1.w), make_float2(li.x + l0.x, li.x + l1.x),
                                            make_float2(li.y * l0.y, li.y * l1.y), P2, fxy, fz, ecv);
                    }
                }
            };
            if (c0 + 256 <= cnt)
                walk(std::true_type{});
            else
                walk(std::false_type{});
            if (__any_sync(full, amb != 0)) {
                // near the cutoff: decide in FP64 exactly as the reference;
                // an entry within the cutoff is evaluated here (the walk
                // dropped it)
                for (int u = 0; u < 8; ++u) {
                    if (!((amb >> u) & 1u)) continue;
                    const unsigned e = (wds[u >> 1] >> (16 * (u & 1))) & 0xffffu;
                    if (!(exact_r2(v, S, i, hood_slot(spans, nsp, (int)(e >> kEntryShift))) < S.cut2)) continue;
                    const float4 pj = *reinterpret_cast<const float4 *>(q_base + 2 * e);
                    const float2 lj = *reinterpret_cast<const float2 *>(smem + e);
                    // j - i, the walk's convention (the sums are negated at the end)
                    const float dx = pj.x - pi3[0], dy = pj.y - pi3[1], dz = pj.z - pi3[2];
                    const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                    if (SW)
                        pair_mixed<ENERGY, SW>(true, -dx, -dy, -dz, r2, qi * pj.w, li.x + lj.x, li.y * lj.y, P, fx,
                                               fy, fz, ec, ev);
                    else
                        pair_mixed<ENERGY, SW>(true, dx, dy, dz, r2, qi * pj.w, li.x + lj.x, li.y * lj.y, P, fxy.x,
                                               fxy.y, fz, ec, ev);
                }
            }
            cur = nxt;
        }
        if (!SW) {
            fx = -fxy.x;
            fy = -fxy.y;
            fz = -fz;
        }
        fx = warp_sum(fx);
        fy = warp_sum(fy);
        fz = warp_sum(fz);
        if (lane == 0) {
            acc_add(static_cast<long long *>(v.fx) + i, fx);
            acc_add(static_cast<long long *>(v.fy) + i, fy);
            acc_add(static_cast<long long *>(v.fz) + i, fz);
        }
    }
    if (ENERGY) {
        // the packed sums, and the near-cutoff corrections (scalar)
        ec += ecv.x;
        ev += ecv.y;
        // each pair sits in both partners' lists
        energy_add_f(v.E, G.sys, E_COUL, 0.5f * ec);
        energy_add_f(v.E, G.sys, E_VDW, 0.5f * ev);
    }
}

// FP64 form: the same list; every pair in double precision from the FP64
// positions with the reference's minimum image (NonbondedForce.cpp:548-581).
template <bool ENERGY>
__global__ void __launch_bounds__(kHoodWarps * 32) k_pairs_fp64(DevView v) {
    extern __shared__ __align__(16) unsigned char smem[];
    CellGroup G = v.groups[blockIdx.x];
    int a0 = v.cell_start[G.cell], a1 = v.cell_start[G.cell + G.ncell];
    if (a0 == a1) return;
    const SysDev &S = v.sys[G.sys];
    if (!S.nb_on) return;
    HoodSpan *spans = reinterpret_cast<HoodSpan *>(smem);
    int *s_n = reinterpret_cast<int *>(spans + kMaxSpans);
    int n = hood_setup(v, S, v.cell3[a0], G.ncell, spans, s_n, nullptr);
    if (n > v.hood_cap || s_n[1] > kMaxSpans) {
        if (threadIdx.x == 0) atomicOr(&v.flags->error, ERR_NLIST_OVERFLOW);
        return;
    }
    int nsp = s_n[1];
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    double ec = 0, ev = 0;
    for (int i = a0 + warp; i < a1; i += nw) {
        double xi = v.x[i], yi = v.y[i], zi = v.z[i];
        double qi = v.qs[i];
        double2 li = v.ljd[i];
        int cnt = v.ncount[i];
        const uint16_t *lst = v.nl16 + (size_t)i * v.stride;
        double fx = 0, fy = 0, fz = 0;
        for (int k = lane; k < cnt; k += 32) {
            int j = hood_slot(spans, nsp, lst[list_pos(k)] >> kEntryShift);
            if (!(exact_r2(v, S, i, j) < S.cut2)) continue;
            // deltaR = minimumImageVector(p_i, p_j) (NonbondedForce.cpp:548)
            double dx = min_image(xi - v.x[j], S.L[0], S.halfL[0]);
            double dy = min_image(yi - v.y[j], S.L[1], S.halfL[1]);
            double dz = min_image(zi - v.z[j], S.L[2], S.halfL[2]);
            double r = sqrt(dx * dx + dy * dy + dz * dz);
            double rinv = 1.0 / r;
            double sw = 1.0, dsw = 0.0;
            if (S.use_switch && r > S.sw_dist) {
                double t = (r - S.sw_dist) / (S.cutoff - S.sw_dist);
                sw = 1 + t * t * t * (-10 + t * (15 - t * 6));
                dsw = t * t * (-30 + t * (60 - t * 30)) / (S.cutoff - S.sw_dist);
            }
            double xa = S.alpha * r;
            double qq = qi * v.qs[j];
            double erfcv = erfc(xa);
            double dEdR = qq * rinv * rinv * rinv * (erfcv + 2 * xa * exp(-xa * xa) / kSqrtPi);
            double2 lj = v.ljd[j];
            double sg = li.x + lj.x;
            double s2 = sg * rinv;
            s2 *= s2;
            double s6 = s2 * s2 * s2;
            double eps = li.y * lj.y;
            dEdR += sw * eps * (12.0 * s6 - 6.0) * s6 * rinv * rinv;
            double evdw = eps * (s6 - 1.0) * s6;
            if (S.use_switch) {
                dEdR -= evdw * dsw * rinv;
                evdw *= sw;
            }
            fx += dx * dEdR;
            fy += dy * dEdR;
            fz += dz * dEdR;
            if (ENERGY) {
                ec += qq * rinv * erfcv;
                ev += evdw;
            }
        }
        fx = warp_sum(fx);
        fy = warp_sum(fy);
        fz = warp_sum(fz);
        if (lane == 0) {
            atomicAdd(static_cast<double *>(v.fx) + i, fx);
            atomicAdd(static_cast<double *>(v.fy) + i, fy);
            atomicAdd(static_cast<double *>(v.fz) + i, fz);
        }
    }
    if (ENERGY) {
        energy_add(v.E, G.sys, E_COUL, 0.5 * ec);
        energy_add(v.E, G.sys, E_VDW, 0.5 * ev);
    }
}

// ---- test support: the neighbour pair set within the cutoff, exactly as
// the reference decides it, as (larger, smaller) original indices.
__global__ void k_collect(DevView v, int sys_sel, int *out, long long cap, unsigned long long *n_out) {
    extern __shared__ __align__(16) unsigned char smem[];
    CellGroup G = v.groups[blockIdx.x];
    if (G.sys != sys_sel) return;
    int a0 = v.cell_start[G.cell], a1 = v.cell_start[G.cell + G.ncell];
    if (a0 == a1) return;
    const SysDev &S = v.sys[G.sys];
    if (!S.nb_on) return;
    HoodSpan *spans = reinterpret_cast<HoodSpan *>(smem);
    int *s_n = reinterpret_cast<int *>(spans + kMaxSpans);
    hood_setup(v, S, v.cell3[a0], G.ncell, spans, s_n, nullptr);
    if (s_n[1] > kMaxSpans) return;
    int nsp = s_n[1];
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int i = a0 + warp; i < a1; i += nw) {
        int oi = v.orig[i];
        int cnt = v.ncount[i];
        for (int k = lane; k < cnt; k += 32) {
            int j = hood_slot(spans, nsp, v.nl16[(size_t)i * v.stride + list_pos(k)] >> kEntryShift);
            int oj = v.orig[j];
            if (oi <= oj) continue;
            if (!(exact_r2(v, S, i, j) < S.cut2)) continue;
            unsigned long long p = atomicAdd(n_out, 1ull);
            if ((long long)p < cap) {
                out[2 * p] = oi - S.atom_off;
                out[2 * p + 1] = oj - S.atom_off;
            }
        }
    }
}

// ------------------------------------------------------------------ launch

static size_t tail_bytes() { return kMaxSpans * sizeof(HoodSpan) + 4 * sizeof(int); }
static size_t smem_build(int cap, int warps) {
    return (size_t)cap * sizeof(float4) + (size_t)warps * 512 * sizeof(uint16_t) +
           25 * (kRowCells + 1) * sizeof(int) + tail_bytes();
}
static size_t smem_pairs(int cap, int mixed) {
    return mixed ? (size_t)cap * (sizeof(float4) + sizeof(float2)) + tail_bytes() : tail_bytes();
}
// static shared memory of the tile kernels (displacement table and counts)
constexpr size_t kTileStatic = 25 * kRowCells * sizeof(float4) + 16;

// Two blocks of 16 warps per SM when both blocks' shared memory fits (228 KB
// per SM, 1 KB reserved per block); otherwise one block of 32 warps, which
// keeps 32 warps on the SM at the same 64 registers per thread.  (Dense
// neighbourhoods -- one-cell groups of large cells -- need the latter.)
static bool wide(size_t dynamic_smem) { return 2 * (dynamic_smem + kTileStatic + 1024) > 228 * 1024; }
static int build_warps(int cap) { return wide(smem_build(cap, kHoodWarps)) ? 2 * kHoodWarps : kHoodWarps; }
static int pair_warps(int cap) { return wide(smem_pairs(cap, 1)) ? 2 * kHoodWarps : kHoodWarps; }

template <int W>
static void set_pairs_smem(int m) {
    cudaFuncSetAttribute(k_pairs_mixed<true, false, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_pairs_mixed<false, false, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_pairs_mixed<true, true, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_pairs_mixed<false, true, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
}

// The dynamic shared-memory limit is a per-kernel attribute shared by every
// context of the process on a device: it is only ever raised, so a context
// with a smaller neighbourhood cannot lower it under another one.
void tiles_set_smem(int cap) {
    static std::mutex mu;
    static int seen_build[2][kMaxSmemDevices] = {}, seen_pairs[2][kMaxSmemDevices] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= kMaxSmemDevices) dev = 0;
    const int bw = build_warps(cap), pw = pair_warps(cap);
    const int b = (int)smem_build(cap, bw), m = (int)smem_pairs(cap, 1);
    const int bi = bw == kHoodWarps ? 0 : 1, pi = pw == kHoodWarps ? 0 : 1;
    std::lock_guard<std::mutex> lock(mu);
    // launches up to 48 KB need no attribute
    if (b > 48 * 1024 && b > seen_build[bi][dev]) {
        if (bi)
            cudaFuncSetAttribute(k_build<2 * kHoodWarps>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
        else
            cudaFuncSetAttribute(k_build<kHoodWarps>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
        seen_build[bi][dev] = b;
    }
    if (m > 48 * 1024 && m > seen_pairs[pi][dev]) {
        if (pi)
            set_pairs_smem<2 * kHoodWarps>(m);
        else
            set_pairs_smem<kHoodWarps>(m);
        seen_pairs[pi][dev] = m;
    }
}

void launch_build(const DevView &v, cudaStream_t st) {
    if (!v.ngroups) return;
    if (build_warps(v.hood_cap) == kHoodWarps)
        k_build<kHoodWarps><<<v.ngroups, kHoodWarps * 32, smem_build(v.hood_cap, kHoodWarps), st>>>(v);
    else
        k_build<2 * kHoodWarps>
            <<<v.ngroups, 2 * kHoodWarps * 32, smem_build(v.hood_cap, 2 * kHoodWarps), st>>>(v);
}

template <int W>
static void launch_pairs_mixed(const DevView &v, int energy, cudaStream_t st) {
    const int g = v.ngroups, t = W * 32;
    const size_t sm = smem_pairs(v.hood_cap, 1);
    if (v.any_switch) {
        if (energy)
            k_pairs_mixed<true, true, W><<<g, t, sm, st>>>(v);
        else
            k_pairs_mixed<false, true, W><<<g, t, sm, st>>>(v);
    } else {
        if (energy)
            k_pairs_mixed<true, false, W><<<g, t, sm, st>>>(v);
        else
            k_pairs_mixed<false, false, W><<<g, t, sm, st>>>(v);
    }
}

void launch_pairs(const DevView &v, int energy, cudaStream_t st) {
    if (v.N == 0 || v.ngroups == 0) return;
    if (v.mixed) {
        if (pair_warps(v.hood_cap) == kHoodWarps)
            launch_pairs_mixed<kHoodWarps>(v, energy, st);
        else
            launch_pairs_mixed<2 * kHoodWarps>(v, energy, st);
        return;
    }
    int g = v.ngroups, t = kHoodWarps * 32;
    size_t sm = smem_pairs(v.hood_cap, 0);
    if (energy)
        k_pairs_fp64<true><<<g, t, sm, st>>>(v);
    else
        k_pairs_fp64<false><<<g, t, sm, st>>>(v);
}

long long launch_collect_pairs(const DevView &v, int sys, int *out_pairs, long long cap, cudaStream_t st) {
    unsigned long long *dn;
    cudaMallocAsync(&dn, sizeof(unsigned long long), st);
    cudaMemsetAsync(dn, 0, sizeof(unsigned long long), st);
    k_collect<<<v.ngroups, kHoodWarps * 32, tail_bytes(), st>>>(v, sys, out_pairs, cap, dn);
    unsigned long long n = 0;
    cudaMemcpyAsync(&n, dn, sizeof(n), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    cudaFreeAsync(dn, st);
    return (long long)n;
}

}  // namespace nxm
