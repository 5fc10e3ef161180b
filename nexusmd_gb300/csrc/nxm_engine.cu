// Host orchestration of the CUDA engine.
//
// Set-up reproduces the reference's per-run constants once (box from the
// atom extent, PME grid rule, Ewald alpha, exclusion sets, B-spline moduli,
// self energy), where the reference recomputes several of them every step
// (core/baseline/src/Forces/NonbondedForce.cpp:19-183, :293-321, :515-527).
// The step is the reference's CalculateForces -> Report -> Integrate
// (core/baseline/src/Engine.cpp:162-188) as a fixed sequence of kernel
// launches on one stream, everything resident on the device.
#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <queue>
#include <string>

#include <thread>
#include <tuple>

#include "nxm_engine.h"

namespace nxm {

// ------------------------------------------------------------ rebuild gate

// force 1: a rebuild in this step; 2: the context's first list, built
// before any step (the interval then counts from the first step).
__global__ void k_decide(DevView v, int force) {
    Flags *f = v.flags;
    int rb = force || f->since >= f->interval || f->skin_hit;
    f->rebuild = rb;
    f->skin_hit = 0;
    f->since = rb ? (force == 2 ? 0 : 1) : f->since + 1;
    if (rb) f->nrebuild += 1;
}

void launch_decide_rebuild(const DevView &v, int force, cudaStream_t st) { k_decide<<<1, 1, 0, st>>>(v, force); }

// The same decision inside a step graph: it also opens or closes the
// graph's conditional rebuild node.
__global__ void k_decide_graph(DevView v, cudaGraphConditionalHandle h) {
    Flags *f = v.flags;
    int rb = f->since >= f->interval || f->skin_hit;
    f->rebuild = rb;
    f->skin_hit = 0;
    f->since = rb ? 1 : f->since + 1;
    if (rb) f->nrebuild += 1;
    cudaGraphSetConditional(h, rb ? 1u : 0u);
}

// Context creation: positions given per atom as (x, y, z) into x, y, z;
// 1/m (0 for a massless particle, VerletIntegration.cpp:37-45; the division
// rounds as the host's); the LJ parameters as the combination rule uses
// them, sigma/2 and 2 sqrt(eps) (NonbondedForce.cpp:504-513), once here
// instead of at every list rebuild; slot = original index until the first
// sort.
__global__ void k_init_atoms(DevView v, const double *xyz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.N) return;
    v.x[i] = xyz[3 * (size_t)i];
    v.y[i] = xyz[3 * (size_t)i + 1];
    v.z[i] = xyz[3 * (size_t)i + 2];
    const double m = v.mass[i];
    v.invm[i] = m == 0.0 ? 0.0 : 1.0 / m;
    v.sig[i] = 0.5 * v.sig[i];
    v.eps[i] = 2.0 * sqrt(v.eps[i]);
    v.orig[i] = i;
    v.slot_of[i] = i;
}

static void launch_init_atoms(const DevView &v, const double *xyz, cudaStream_t st) {
    if (v.N > 0) k_init_atoms<<<(v.N + 255) / 256, 256, 0, st>>>(v, xyz);
}

// A state vector given per original atom as (x, y, z) into slot order.
__global__ void k_state_to_slots(DevView v, const double *xyz, double *dx, double *dy, double *dz) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= v.N) return;
    const size_t o = 3 * (size_t)v.orig[s];
    dx[s] = xyz[o];
    dy[s] = xyz[o + 1];
    dz[s] = xyz[o + 2];
}

// Term ingest at context creation: term t of one kind (per = 2, 3 or 4
// atoms; its system s found in the kind's per-system term offsets toff) has
// its atom indices checked against the system's atom count and shifted by the
// system's first atom, into int2 (per 2) or int4 (per 3, 4; unused word 0)
// words.  An invalid term sets `errbit` in *err and takes the system's first
// atom for every index, so later set-up kernels stay in range.  in and out may
// be the same array when per is 2 or 4.
__global__ void k_terms_ingest(const int *in, int per, int *out, int n, const int *toff, const int *first,
                               const int *count, int S, int errbit, int *err) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int lo = 0, hi = S - 1;  // the last system whose terms start at or before t
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (toff[mid] <= t)
            lo = mid;
        else
            hi = mid - 1;
    }
    int a[4] = {0, 0, 0, 0};
    bool bad = false;
    for (int k = 0; k < per; ++k) {
        a[k] = in[(size_t)t * per + k];
        bad |= a[k] < 0 || a[k] >= count[lo];
    }
    if (bad) atomicOr(err, errbit);
    const int ow = per == 2 ? 2 : 4;
    for (int k = 0; k < ow; ++k) out[(size_t)t * ow + k] = k < per ? first[lo] + (bad ? 0 : a[k]) : 0;
}

// FP32 copies of the bonded parameters (each double rounded once, as the
// FP64 terms' values).
__global__ void k_params_f32(const double2 *a, float2 *b, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) b[k] = make_float2((float)a[k].x, (float)a[k].y);
}

// The exceptions' (q_i q_j / 4 pi eps0, sigma, 4 eps) in FP32.
__global__ void k_xc_params_f32(const double4 *a, float4 *b, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) b[k] = make_float4((float)a[k].x, (float)a[k].y, (float)a[k].z, 0.f);
}

// ------------------------------------------------------------ host maths

static bool smooth235(int n) {
    if (n < 1) return false;
    for (int p : {2, 3, 5})
        while (n % p == 0) n /= p;
    return n == 1;
}

// PeriodicBoundaryCondition.cpp:11-88 (water branch: extent, then 1% margin)
static void box_from_positions(int n, const double *pos, double lb[3], double ub[3], double L[3]) {
    for (int d = 0; d < 3; ++d) lb[d] = ub[d] = pos[d];
    for (int i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) {
            lb[d] = std::min(lb[d], pos[3 * i + d]);
            ub[d] = std::max(ub[d], pos[3 * i + d]);
        }
    double size[3];
    for (int d = 0; d < 3; ++d) size[d] = std::fabs(ub[d] - lb[d]);
    for (int d = 0; d < 3; ++d) {
        double m = 0.01 * size[d];
        lb[d] -= m;
        ub[d] += m;
        L[d] = std::fabs(ub[d] - lb[d]);
    }
}

// NonbondedForce.cpp:33-48
static int pow2_dimension(double box) {
    int minimum = (int)std::ceil(box) * 10;
    int p = 1;
    while (p < minimum) p *= 2;
    return p;
}

// NonbondedForce.cpp:75-142: |b(k)|^2 by the direct DFT, with the
// neighbour average for values below 1e-7.
static void bspline_moduli(int K, std::vector<double> &mod) {
    const int ORDER = kOrder;
    double data[ORDER] = {0, 0, 0, 0, 0};
    data[ORDER - 1] = 0.0;
    data[1] = 0.0;
    data[0] = 1.0;
    for (int i = 3; i < ORDER; i++) {
        double div = 1.0 / (i - 1);
        data[i - 1] = 0.0;
        for (int j = 1; j < (i - 1); j++) data[i - j - 1] = div * (j * data[i - j - 2] + (i - j) * data[i - j - 1]);
        data[0] = div * data[0];
    }
    double div = 1.0 / (ORDER - 1);
    data[ORDER - 1] = div * data[ORDER - 2];
    for (int i = 1; i < (ORDER - 1); i++)
        data[ORDER - i - 1] = div * (i * data[ORDER - i - 2] + (ORDER - i) * data[ORDER - i - 1]);
    data[0] = div * data[0];
    std::vector<double> bs(K + ORDER + 1, 0.0);
    for (int i = 1; i <= ORDER; i++) bs[i] = data[i - 1];
    mod.assign(K, 0.0);
    // bs[j] is zero outside 1..ORDER, and the terms j < K it would add there
    // are zeros that leave the sums' bits unchanged: the sums run over the
    // non-zero terms only, in the same order
    const int jmax = std::min(ORDER, K - 1);
    for (int i = 0; i < K; i++) {
        double sc = 0.0, ss = 0.0;
        for (int j = 1; j <= jmax; j++) {
            double arg = (2 * kPi * i * j) / K;
            sc += bs[j] * std::cos(arg);
            ss += bs[j] * std::sin(arg);
        }
        mod[i] = sc * sc + ss * ss;
    }
    for (int i = 0; i < K; i++)
        if (mod[i] < 1e-7) mod[i] = (mod[(i - 1 + K) % K] + mod[(i + 1) % K]) / 2.0;
}

// Exclusions.cpp:7-44 with bondCutoff = depth: every atom reachable through
// 1..depth bonds, united with the exception partners (pairs `exc`, which are
// excluded from the Ewald direct sum too).  Appends one sorted row per atom
// of the system to the batch CSR (eoff, elst), indices shifted by `off`, and
// the pairs with j > i to ex_pairs.  Flat arrays only: the bonds' adjacency
// by a counting sort, one breadth-first search per atom into a shared
// buffer, then a merge with the atom's sorted exception partners.  The
// creation builds the same sets on the device (k_exclusions_build.cu); this
// host form serves a batch with a row longer than the device search holds.
static std::string exclusion_rows(const HostSystem &s, int off, std::vector<int> &eoff, std::vector<int> &elst,
                                  std::vector<int2> &ex_pairs) {
    const int n = s.n;
    const size_t nbond = s.bonds.size() / 2;
    std::vector<int> aoff(n + 1, 0), adj(2 * nbond);
    for (size_t b = 0; b < nbond; ++b) {
        int i = s.bonds[2 * b], j = s.bonds[2 * b + 1];
        if (i < 0 || j < 0 || i >= n || j >= n) return "createExclusions: Illegal particle index in list of bonds";
        ++aoff[i + 1];
        ++aoff[j + 1];
    }
    for (int i = 0; i < n; ++i) aoff[i + 1] += aoff[i];
    {
        std::vector<int> fill(aoff.begin(), aoff.end() - 1);
        for (size_t b = 0; b < nbond; ++b) {
            int i = s.bonds[2 * b], j = s.bonds[2 * b + 1];
            adj[fill[i]++] = j;
            adj[fill[j]++] = i;
        }
    }
    // exception partners, sorted per atom
    const size_t nexc = s.exc.size() / 2;
    std::vector<int> xoff(n + 1, 0), xadj(2 * nexc);
    for (size_t k = 0; k < nexc; ++k) {
        ++xoff[s.exc[2 * k] + 1];
        ++xoff[s.exc[2 * k + 1] + 1];
    }
    for (int i = 0; i < n; ++i) xoff[i + 1] += xoff[i];
    {
        std::vector<int> fill(xoff.begin(), xoff.end() - 1);
        for (size_t k = 0; k < nexc; ++k) {
            int a = s.exc[2 * k], b = s.exc[2 * k + 1];
            xadj[fill[a]++] = b;
            xadj[fill[b]++] = a;
        }
        for (int i = 0; i < n; ++i) std::sort(xadj.begin() + xoff[i], xadj.begin() + xoff[i + 1]);
    }
    // one breadth-first search per atom; atoms split into contiguous ranges
    // over the host's threads, each range's rows and pairs appended in
    // order afterwards (the same CSR as one pass)
    struct Part {
        std::vector<int> len, lst;
        std::vector<int2> pairs;
    };
    const int nth = n < 16384 ? 1 : std::max(1, std::min(15, (int)std::thread::hardware_concurrency() - 1));
    std::vector<Part> parts(nth);
    auto run = [&](int t) {
        const int i0 = (int)((long long)n * t / nth), i1 = (int)((long long)n * (t + 1) / nth);
        Part &P = parts[t];
        P.len.reserve(i1 - i0);
        P.lst.reserve((size_t)(i1 - i0) * 4);
        // the search's queue with each atom's depth; a depth-limited search
        // visits a few dozen atoms at most, so "visited" is a scan of it
        std::vector<int> queue, depth, row;
        queue.reserve(64);
        depth.reserve(64);
        row.reserve(64);
        for (int i = i0; i < i1; ++i) {
            row.clear();
            if (s.excl_depth >= 1) {
                queue.clear();
                depth.clear();
                queue.push_back(i);
                depth.push_back(0);
                for (size_t h = 0; h < queue.size(); ++h) {
                    const int u = queue[h], du = depth[h];
                    if (du == s.excl_depth) continue;
                    for (int k = aoff[u]; k < aoff[u + 1]; ++k) {
                        const int w = adj[k];
                        if (std::find(queue.begin(), queue.end(), w) != queue.end()) continue;
                        queue.push_back(w);
                        depth.push_back(du + 1);
                        row.push_back(w);
                    }
                }
                std::sort(row.begin(), row.end());
            }
            // sorted union with the exception partners
            const size_t base = P.lst.size();
            size_t p = 0;
            int q = xoff[i];
            while (p < row.size() || q < xoff[i + 1]) {
                int v;
                if (q >= xoff[i + 1] || (p < row.size() && row[p] < xadj[q]))
                    v = row[p++];
                else if (p >= row.size() || xadj[q] < row[p])
                    v = xadj[q++];
                else {
                    v = row[p++];
                    ++q;
                }
                if (P.lst.size() > base && P.lst.back() == off + v) continue;  // repeated exception pair
                P.lst.push_back(off + v);
                if (v > i) P.pairs.push_back(make_int2(off + i, off + v));
            }
            P.len.push_back((int)(P.lst.size() - base));
        }
    };
    if (nth == 1) {
        run(0);
    } else {
        std::vector<std::thread> pool;
        for (int t = 1; t < nth; ++t) pool.emplace_back(run, t);
        run(0);
        for (auto &th : pool) th.join();
    }
    size_t nl = 0, np = 0;
    for (const Part &P : parts) {
        nl += P.lst.size();
        np += P.pairs.size();
    }
    eoff.reserve(eoff.size() + n);
    elst.reserve(elst.size() + nl);
    ex_pairs.reserve(ex_pairs.size() + np);
    for (const Part &P : parts) {
        int e = eoff.back();
        for (int l : P.len) eoff.push_back(e += l);
        elst.insert(elst.end(), P.lst.begin(), P.lst.end());
        ex_pairs.insert(ex_pairs.end(), P.pairs.begin(), P.pairs.end());
    }
    return "";
}

// reciprocalConvolutionAndEnergy's eterm (NonbondedForce.cpp:323-388) on one
// system's half spectrum, one thread per element, in FP64 with the host's
// order of operations written out (round-to-nearest multiplies and adds, no
// fused multiply-adds); the element (0, 0, 0) is zero.  mod: the three axes'
// B-spline moduli, concatenated.
template <typename T>
__global__ void k_influence(T *eterm, const double *mod, int K0, int K1, int K2, double r0, double r1, double r2,
                            double factor, double boxfactor) {
    const int Kh = K2 / 2 + 1;
    const long long n = (long long)K0 * K1 * Kh;
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= n) return;
    const int kz = (int)(idx % Kh);
    const long long t = idx / Kh;
    const int ky = (int)(t % K1), kx = (int)(t / K1);
    if (idx == 0) {
        eterm[0] = (T)0;
        return;
    }
    const double mx = kx < (K0 + 1) / 2 ? kx : kx - K0;
    const double my = ky < (K1 + 1) / 2 ? ky : ky - K1;
    const double mz = kz < (K2 + 1) / 2 ? kz : kz - K2;
    const double mhx = __dmul_rn(mx, r0), mhy = __dmul_rn(my, r1), mhz = __dmul_rn(mz, r2);
    const double m2 = __dadd_rn(__dadd_rn(__dmul_rn(mhx, mhx), __dmul_rn(mhy, mhy)), __dmul_rn(mhz, mhz));
    const double bx = __dmul_rn(boxfactor, mod[kx]), by = mod[K0 + ky], bz = mod[K0 + K1 + kz];
    const double denom = __dmul_rn(__dmul_rn(__dmul_rn(m2, bx), by), bz);
    eterm[idx] = (T)__ddiv_rn(__dmul_rn(kOne4PiEps0, exp(__dmul_rn(-factor, m2))), denom);
}

static void launch_influence(void *eterm, int mixed, long long coff, const double *mod, const int K[3],
                             const double L[3], double alpha, cudaStream_t st) {
    const long long n = (long long)K[0] * K[1] * (K[2] / 2 + 1);
    const int nb = (int)((n + 255) / 256);
    const double r0 = 1 / L[0], r1 = 1 / L[1], r2 = 1 / L[2];
    const double factor = kPi * kPi / (alpha * alpha);
    const double boxfactor = kPi * L[0] * L[1] * L[2];
    if (mixed)
        k_influence<float><<<nb, 256, 0, st>>>(static_cast<float *>(eterm) + coff, mod, K[0], K[1], K[2], r0, r1, r2,
                                               factor, boxfactor);
    else
        k_influence<double><<<nb, 256, 0, st>>>(static_cast<double *>(eterm) + coff, mod, K[0], K[1], K[2], r0, r1,
                                                r2, factor, boxfactor);
}

// ------------------------------------------------------------ engine

static size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

// Page-locked host memory: a page-aligned allocation registered with the
// driver (for a few MB about ten times cheaper than cudaMallocHost here).
static void *pinned_alloc(size_t b) {
    b = (b + 65535) & ~(size_t)65535;
    void *p = std::aligned_alloc(65536, b);
    if (!p) return nullptr;
    if (cudaHostRegister(p, b, cudaHostRegisterDefault) != cudaSuccess) {
        cudaGetLastError();
        std::free(p);
        return nullptr;
    }
    return p;
}

static void pinned_free(void *p) {
    if (!p) return;
    cudaHostUnregister(p);
    std::free(p);
}

static double now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Zeroed device arrays, 256-byte aligned, carved out of chunks: one
// cudaMalloc (~30 us whatever its size) and one memset per chunk, not per
// array.  The set-up first reserves one chunk sized for all of the context's
// arrays; what does not fit comes out of further 32 MB chunks, or gets a
// chunk of its own above 8 MB.  Freed with the engine.
constexpr size_t kArenaChunk = 32u << 20;

// The compute stream, after the set-up's uploads and zeroing queued so far
// on the copy stream.  The set-up uploads on the copy stream because an
// upload from pageable memory returns only once every earlier operation of
// its stream has run: on the compute stream each would wait for the
// set-up's kernels.
cudaStream_t Engine::kst() {
    if (uploads_pending_) {
        cudaEventRecord(ev_uploaded_, st_copy_);
        cudaStreamWaitEvent(st_, ev_uploaded_, 0);
        uploads_pending_ = false;
    }
    return st_;
}

char *Engine::chunk(size_t b) {
    const double t0 = now_ms();
    void *p = nullptr;
    if (cudaMalloc(&p, b) != cudaSuccess) {
        alloc_failed_ = true;
        return nullptr;
    }
    // zeroed in the order of the set-up's uploads (copy stream), which the
    // compute stream joins before its first kernel on them (kst)
    cudaMemsetAsync(p, 0, b, st_copy_);
    uploads_pending_ = true;
    allocs_.push_back(p);
    create_ms_[6] += now_ms() - t0;
    return static_cast<char *>(p);
}

void Engine::arena_reserve(size_t b) {
    b = (b + 255) & ~(size_t)255;
    if (b <= arena_left_) return;
    arena_ptr_ = chunk(b);
    arena_left_ = arena_ptr_ ? b : 0;
}

template <typename T>
T *Engine::dalloc(size_t n) {
    if (n == 0) n = 1;
    const size_t bytes = (n * sizeof(T) + 255) & ~(size_t)255;
    if (arena_left_ < bytes) {
        if (bytes > kArenaChunk / 4) return reinterpret_cast<T *>(chunk(bytes));
        arena_ptr_ = chunk(kArenaChunk);
        arena_left_ = arena_ptr_ ? kArenaChunk : 0;
        if (!arena_ptr_) return nullptr;
    }
    T *r = reinterpret_cast<T *>(arena_ptr_);
    arena_ptr_ += bytes;
    arena_left_ -= bytes;
    return r;
}

Engine::~Engine() {
    if (st_) cudaStreamSynchronize(st_);
    free_frames();
    for (int b = 0; b < 2; ++b)
        if (buf_free_[b]) cudaEventDestroy(buf_free_[b]);
    if (step_done_) cudaEventDestroy(step_done_);
    for (cudaEvent_t ev : {ev_setup_, ev_staged_, ev_stage_free_, ev_uploaded_})
        if (ev) cudaEventDestroy(ev);
    if (st_copy_) cudaStreamDestroy(st_copy_);
    free_graphs();
    for (void *p : allocs_) cudaFree(p);
    fft_plan_free(plan_);
    pinned_free(h_E_);  // h_flags_ and h_tail_ lie in the same block
    if (ev_fork_) cudaEventDestroy(ev_fork_);
    if (ev_join_) cudaEventDestroy(ev_join_);
    if (st_pme_) cudaStreamDestroy(st_pme_);
    if (st_) cudaStreamDestroy(st_);
}

std::string Engine::check(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return std::string(what) + ": " + cudaGetErrorString(e);
    return "";
}

std::string Engine::init(const std::vector<HostSystem> &systems, const nxm_options &opt,
                         const double *positions) {
    const double t_start = now_ms();
    if (systems.empty()) return "no systems";
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return "no CUDA device";
    if (opt.device < 0 || opt.device >= ndev) return "bad device ordinal";
    if (opt.fft_path < 0 || opt.fft_path > 2) return "bad fft_path";
    fft_path_ = opt.fft_path;
    cudaSetDevice(opt.device);
    device_ = opt.device;
    mixed_ = opt.precision == NXM_PRECISION_MIXED ? 1 : 0;
    interval_ = opt.rebuild_interval > 0 ? opt.rebuild_interval : 1;
    int S = (int)systems.size();
    N_ = 0;
    for (auto &s : systems) {
        if (s.n <= 0) return "a system has no atoms";
        N_ += s.n;
    }
    if (N_ > (int)kSlotMask) return "too many atoms for the list entry format";

    // ---- per-system constants
    sysd_.assign(S, SysDev{});
    sysh_.assign(S, SysHost{});
    plan_.S = S;
    plan_.hsys.assign(S, FftSysDev{});
    // exclusion sets as batch CSR (original indices), filled per system
    std::vector<int> eoff(1, 0), elst;
    std::vector<int2> ex_pairs;
    std::vector<int2> xc_pairs;      // exception pairs, batch-global original indices
    std::vector<double4> xc_prm;
    // Self energies (NonbondedForce.cpp:515-527), in the reference's serial
    // order, on a helper thread while this one sets up the device (a chain
    // of ~N dependent adds and N divisions); joined before init returns.
    std::vector<double> self_e(S, 0.0);
    struct Joiner {
        std::thread t;
        ~Joiner() {
            if (t.joinable()) t.join();
        }
    } self_th;
    {
        bool big = false;
        for (const HostSystem &h : systems) big |= h.n > 4096;
        auto sum_self = [&systems, &self_e, S] {
            for (int s = 0; s < S; ++s) {
                const HostSystem &h = systems[s];
                const double alpha = (1.0 / h.cutoff) * std::sqrt(-std::log(2.0 * h.tol));
                double self = 0.0;
                for (int i = 0; i < h.n; ++i) self -= kOne4PiEps0 * h.q[i] * h.q[i] * alpha / kSqrtPi;
                self_e[s] = self;
            }
        };
        if (big)
            self_th.t = std::thread(sum_self);
        else
            sum_self();
    }
    int off = 0, cell_off = 0, cg_total = 0;
    long long roff = 0, coff = 0;
    int tw_total = 0;
    double skin = opt.skin > 0 ? opt.skin : 0.0;
    int stride = 0, hood_cap = 0;
    std::vector<int> group_g(S, 1);
    std::vector<double> cell_atoms_s(S, 0.0);  // mean atoms per cell
    for (int s = 0; s < S; ++s) {
        const HostSystem &h = systems[s];
        SysDev &D = sysd_[s];
        SysHost &H = sysh_[s];
        const double *p = positions + 3 * (size_t)off;
        if (h.box_from_positions) {
            box_from_positions(h.n, p, H.lb, H.ub, H.L);
        } else {
            for (int d = 0; d < 3; ++d) {
                H.lb[d] = h.lb[d];
                H.ub[d] = h.ub[d];
                H.L[d] = std::fabs(h.ub[d] - h.lb[d]);
            }
        }
        if (!(h.cutoff > 0)) return "cutoff must be positive";
        for (int d = 0; d < 3; ++d)
            if (!(H.L[d] >= 2 * h.cutoff)) return "box edge shorter than twice the cutoff";
        if (!(h.tol > 0 && h.tol < 0.5)) return "ewald tolerance must be in (0, 0.5)";
        for (int d = 0; d < 3; ++d) {
            H.K[d] = h.grid[0] > 0 ? h.grid[d] : pow2_dimension(H.L[d]);
            if (!smooth235(H.K[d]) || H.K[d] < 5) return "PME grid sizes must be 2^a 3^b 5^c and >= 5";
            if (H.K[d] > 1024) return "PME grid size above 1024";
        }
        H.alpha = (1.0 / h.cutoff) * std::sqrt(-std::log(2.0 * h.tol));
        double sk = skin;
        for (int d = 0; d < 3; ++d) sk = std::min(sk, 0.5 * H.L[d] - h.cutoff);
        H.rlist = h.cutoff + std::max(sk, 0.0);
        H.atom_off = off;
        H.natoms = h.n;
        H.force_mask = h.force_mask;
        H.self_energy = 0.0;  // summed by the helper thread below

        for (int d = 0; d < 3; ++d) {
            D.lb[d] = H.lb[d];
            D.ub[d] = H.ub[d];
            D.L[d] = H.L[d];
            D.invL[d] = 1 / H.L[d];
            D.halfL[d] = 0.5 * H.L[d];
            D.Lf[d] = (float)H.L[d];
            D.halfLf[d] = (float)(0.5 * H.L[d]);
            D.K[d] = H.K[d];
            int nc = (int)std::floor(H.L[d] / (0.5 * H.rlist));
            nc = std::max(1, std::min(nc, 1023));
            D.nc[d] = nc;
            D.cs[d] = H.L[d] / nc;
        }
        D.cutoff = h.cutoff;
        D.cut2 = h.cutoff * h.cutoff;
        D.alpha = H.alpha;
        D.rlist2 = H.rlist * H.rlist;
        D.sw_dist = h.sw_dist;
        D.use_switch = h.use_switch;
        D.nb_on = (h.force_mask & NXM_FORCE_NONBONDED) ? 1 : 0;
        D.cut2f = (float)D.cut2;
        D.cut2f_lo = (float)(D.cut2 * (1.0 - 1e-5));
        D.cut2f_hi = (float)(D.cut2 * (1.0 + 1e-5));
        D.alphaf = (float)H.alpha;
        D.ex2c = (float)(-H.alpha * H.alpha * 1.4426950408889634);  // log2(e)
        D.a04 = (float)(0.4 * H.alpha);
        D.k2a = (float)(2.0 * H.alpha / kSqrtPi);
        for (int d = 0; d < 3; ++d) D.csf[d] = (float)D.cs[d];
        for (int d = 0; d < 3; ++d) {
            D.L40[d] = fix40(H.L[d]);
            D.halfL40[d] = fix40(0.5 * H.L[d]);
            D.lbkey[d] = dkey(H.lb[d]);
            D.ubkey[d] = dkey(H.ub[d]);
        }
        D.rlist2f = (float)D.rlist2;
        D.sw_distf = (float)h.sw_dist;
        D.cutofff = (float)h.cutoff;
        D.atom_off = off;
        D.natoms = h.n;
        D.Kh = H.K[2] / 2 + 1;
        D.grid_off = roff;
        D.cgrid_off = coff;
        D.cell_off = cell_off;
        cell_off += D.nc[0] * D.nc[1] * D.nc[2];
        for (int d = 0; d < 3; ++d) {
            D.cg_off[d] = cg_total;
            cg_total += D.nc[d];
            D.kl[d] = (float)((double)H.K[d] * D.invL[d]);
        }

        FftSysDev &F = plan_.hsys[s];
        for (int d = 0; d < 3; ++d) F.K[d] = H.K[d];
        F.Kh = D.Kh;
        F.roff = roff;
        F.coff = coff;
        for (int d = 0; d < 3; ++d) {
            F.tw[d] = tw_total;
            D.tw_off[d] = tw_total;
            tw_total += H.K[d];
        }
        roff += (long long)H.K[0] * H.K[1] * H.K[2];
        coff += (long long)H.K[0] * H.K[1] * D.Kh;

        // exclusions (batch-global original indices), united with the
        // exception pairs, which are excluded from the Ewald direct sum too
        if (h.exc.size() != 2 * (h.exc_prm.size() / 3)) return "exception arrays disagree in length";
        for (size_t k = 0; k < h.exc.size() / 2; ++k) {
            int a = h.exc[2 * k], b = h.exc[2 * k + 1];
            if (a < 0 || b < 0 || a >= h.n || b >= h.n || a == b) return "exception: illegal particle index";
            if (h.force_mask & NXM_FORCE_NONBONDED) {
                xc_pairs.push_back(make_int2(off + a, off + b));
                const double *p = &h.exc_prm[3 * k];
                xc_prm.push_back(make_double4(kOne4PiEps0 * p[0], p[1], 4.0 * p[2], 0.0));
            }
        }
        // list capacity from the density
        double vol = H.L[0] * H.L[1] * H.L[2];
        double expect = 4.0 / 3.0 * kPi * H.rlist * H.rlist * H.rlist * h.n / vol;
        int cap = (int)(1.6 * expect + 64);
        stride = std::max(stride, cap);
        // tile kernels: groups of G cells along z; the staged neighbourhood
        // holds 5 x 5 x (G + 4) cells.  The largest G whose neighbourhood
        // (with 25% headroom over the mean density) holds at most 4,400
        // atoms -- ~109 KB of shared memory per block, so two blocks of the
        // pair kernel and of the list build share an SM -- and at most
        // nz - 4, so no cell appears twice.  (Larger groups stage fewer
        // atoms per atom of the group: at 94k atoms G = 3 runs the pair
        // kernel 7% faster than G = 2.)
        double cell_atoms = sysd_[s].cs[0] * sysd_[s].cs[1] * sysd_[s].cs[2] * h.n / vol;
        int gmax = std::max(1, std::min(kMaxGroupCells, sysd_[s].nc[2] - 4));
        int G = 1;
        for (int g = gmax; g >= 1; --g)
            if (25.0 * (g + 4) * cell_atoms * 1.25 + 128 <= 4400.0) {
                G = g;
                break;
            }
        group_g[s] = G;
        int hood = (int)(25.0 * (G + 4) * cell_atoms * 1.25 + 128);
        hood_cap = std::max(hood_cap, hood);
        cell_atoms_s[s] = cell_atoms;
        off += h.n;
    }
    if (hood_cap > 4400) {
        // Some system's one-cell neighbourhood exceeds what two blocks per
        // SM can stage, so the tile kernels run one block of 32 warps per SM
        // (k_pairs.cu): then every system takes the longest groups, up to
        // kMaxGroupCellsWide cells, whose neighbourhood stays within ~8,000
        // atoms (one block's shared memory; 16-bit list entries address
        // 8,191), split evenly along the column, up to the whole column --
        // beyond nz - 4 a cell enters the neighbourhood twice, as two
        // periodic images at least a box edge (> twice the list radius)
        // apart, so at most one image of an atom is within the list radius,
        // as in boxes of four cells.  A block's 32 warps then have 40-130
        // atoms to take instead of 17-58, and each atom stages about half
        // as many neighbours.  The cap keeps the tile's FP32 coordinates
        // (relative to the group's first cell) within about six cells: at
        // config 4 (32 systems) groups of up to 4 cells took the step 1.04
        // -> 0.93 ms with the largest per-atom force error 0.077 kJ/mol/nm
        // against the FP64 oracle; up to 5 or 8 cells, 0.89 / 0.86 ms but
        // 0.35 kJ/mol/nm.
        hood_cap = 0;
        for (int s = 0; s < S; ++s) {
            const int nz = sysd_[s].nc[2];
            int G = 1;
            for (int g = std::min(kMaxGroupCellsWide, nz); g >= 1; --g)
                if (25.0 * (g + 4) * cell_atoms_s[s] * 1.25 + 128 <= 8000.0) {
                    G = g;
                    break;
                }
            const int ng = (nz + G - 1) / G;  // groups per column, of near-equal length
            G = (nz + ng - 1) / ng;
            group_g[s] = G;
            hood_cap = std::max(hood_cap, (int)(25.0 * (G + 4) * cell_atoms_s[s] * 1.25 + 128));
        }
    }
    group_g_ = group_g;
    if (opt.max_neighbors > 0) stride = opt.max_neighbors;
    stride = (stride + 255) / 256 * 256;  // whole 256-entry chunks (transposed list layout)

    // ---- device memory
    const double t_host = now_ms();
    create_ms_[0] = t_host - t_start;
    cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking);
    // second stream and fork/join events: the PME branch of the step graph
    cudaStreamCreateWithFlags(&st_pme_, cudaStreamNonBlocking);
    cudaEventCreateWithFlags(&ev_fork_, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&ev_join_, cudaEventDisableTiming);
    energies_.assign((size_t)S * E_SLOTS, 0.0);
    {
        // page-locked host memory in one block: the energy words, the
        // flags and the exclusion build's totals (the frame ring of
        // nxm_step_async comes with the first frame step, while the device
        // builds the first list)
        const size_t be = al256(sizeof(long long) * energies_.size()), bf = al256(sizeof(Flags)), bt = 256;
        void *hp = pinned_alloc(be + bf + bt);
        if (!hp) return "device: pinned host allocation failed";
        h_E_ = static_cast<long long *>(hp);
        h_flags_ = reinterpret_cast<int *>(static_cast<char *>(hp) + be);
        h_tail_ = reinterpret_cast<int *>(static_cast<char *>(hp) + be + bf);
    }
    // the frame copies' stream and events
    for (int b = 0; b < 2; ++b) cudaEventCreateWithFlags(&buf_free_[b], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&step_done_, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&ev_setup_, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&ev_staged_, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&ev_uploaded_, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&ev_stage_free_, cudaEventDisableTiming);
    cudaStreamCreateWithFlags(&st_copy_, cudaStreamNonBlocking);
    v_ = DevView{};
    v_.N = N_;
    v_.S = S;
    v_.mixed = mixed_;
    v_.stride = stride;
    {
        // one reservation for the context's device arrays (an upper
        // estimate; a shortfall comes out of further chunks): per atom the
        // state, derived inputs, cell keys, exclusion build, PME stencils,
        // snapshots and frames (~600 B) and the list; per cell, group, term,
        // exception and grid point their tables
        size_t nb = 0, na = 0, nt = 0, nx = 0, ngr = 0;
        for (int s = 0; s < S; ++s) {
            const HostSystem &h = systems[s];
            nb += h.bonds.size() / 2;
            na += h.angles.size() / 3;
            nt += h.torsions.size() / 4;
            nx += h.exc.size() / 2;
            const SysDev &D = sysd_[s];
            ngr += (size_t)D.nc[0] * D.nc[1] * ((D.nc[2] + group_g[s] - 1) / group_g[s]);
        }
        const size_t est = (size_t)N_ * (600 + 2 * (size_t)stride) + 12 * ((size_t)cell_off + 1) +
                           ngr * (sizeof(CellGroup) + 4 * (size_t)kGroupSpanWords + 8) +
                           (size_t)S * (kDtabStride * sizeof(float4) + 24 * E_SLOTS + sizeof(SysDev)) +
                           8 * (size_t)cg_total + 56 * nb + 56 * na + 60 * nt + 88 * nx + 16 * (size_t)roff +
                           24 * (size_t)coff + 24 * (size_t)tw_total + (256u << 10);
        arena_reserve(est);
    }
    SysDev *dsys = dalloc<SysDev>(S);
    cudaMemcpyAsync(dsys, sysd_.data(), sizeof(SysDev) * S, cudaMemcpyHostToDevice, st_copy_);
    v_.sys = dsys;
    v_.sys_of = dalloc<int>(N_);
    v_.orig = dalloc<int>(N_);
    v_.slot_of = dalloc<int>(N_);
    double **dbl[] = {&v_.x, &v_.y, &v_.z, &v_.vx, &v_.vy, &v_.vz, &v_.mass, &v_.invm, &v_.q, &v_.sig, &v_.eps};
    for (double **d : dbl) *d = dalloc<double>(N_);
    if (mixed_) {
        v_.pf = dalloc<float4>(N_);
        v_.ljf = dalloc<float2>(N_);
        v_.fx = dalloc<long long>(N_);
        v_.fy = dalloc<long long>(N_);
        v_.fz = dalloc<long long>(N_);
    } else {
        v_.qs = dalloc<double>(N_);
        v_.ljd = dalloc<double2>(N_);
        v_.fx = dalloc<double>(N_);
        v_.fy = dalloc<double>(N_);
        v_.fz = dalloc<double>(N_);
    }
    v_.cell3 = dalloc<int>(N_);
    v_.total_cells = cell_off;
    v_.cell_key = dalloc<int>(N_);
    v_.cell_count = dalloc<int>(cell_off + 1);
    v_.cell_start = dalloc<int>(cell_off + 1);
    v_.cell_fill = dalloc<int>(cell_off + 1);
    v_.new_orig = dalloc<int>(N_);
    hood_cap = (hood_cap + 31) / 32 * 32;
    if (hood_cap > 8191) return "neighbourhood too dense for 16-bit list entries";
    v_.hood_cap = hood_cap;
    v_.nl16 = dalloc<uint16_t>((size_t)N_ * stride);
    {
        // groups of G consecutive cells along each z-row of every system
        std::vector<CellGroup> gr;
        for (int s = 0; s < S; ++s) {
            const SysDev &D = sysd_[s];
            int G = group_g[s];
            for (int cx = 0; cx < D.nc[0]; ++cx)
                for (int cy = 0; cy < D.nc[1]; ++cy)
                    for (int cz = 0; cz < D.nc[2]; cz += G) {
                        CellGroup g;
                        g.cell = D.cell_off + (cx * D.nc[1] + cy) * D.nc[2] + cz;
                        g.ncell = std::min(G, D.nc[2] - cz);
                        g.sys = s;
                        gr.push_back(g);
                    }
        }
        v_.ngroups = (int)gr.size();
        v_.groups = dalloc<CellGroup>(gr.size());
        v_.gspan = dalloc<int>(gr.size() * (size_t)kGroupSpanWords);
        v_.gspan_n = dalloc<int2>(gr.size());
        cudaMemcpyAsync(v_.groups, gr.data(), sizeof(CellGroup) * gr.size(), cudaMemcpyHostToDevice, st_copy_);
    }
    tiles_set_smem(hood_cap);
    v_.ncount = dalloc<int>(N_);
    v_.dtab = dalloc<float4>((size_t)S * kDtabStride);
    v_.xref = dalloc<double>(3 * (size_t)N_);
    v_.oref = dalloc<float4>(N_);
    v_.tmp = dalloc<double>(11 * (size_t)N_);
    if (!v_.nl16 || !v_.tmp) return "device allocation failed (neighbour list)";

    // per-atom inputs in original order (slot = original index until the
    // first sort): each array from the caller's in one copy (a batch's
    // systems concatenated), the positions as given (x, y, z per atom) into
    // scratch, split and 1/m formed on the device (k_init_atoms)
    // uploads in the stream's order (the kernels of the set-up follow them
    // there); from pageable memory the call returns once the source is
    // consumed
    auto up = [&](void *dst, const void *src, size_t bytes) {
        const double t0 = now_ms();
        cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st_copy_);
        uploads_pending_ = true;
        create_ms_[7] += now_ms() - t0;
    };
    // each atom's system (one system: the zeroed array as it is)
    std::vector<int> sys_of;
    if (S > 1) {
        sys_of.resize(N_);
        int o = 0;
        for (int s = 0; s < S; ++s) {
            std::fill(sys_of.begin() + o, sys_of.begin() + o + systems[s].n, s);
            o += systems[s].n;
        }
        up(v_.sys_of, sys_of.data(), sizeof(int) * N_);
    }
    {
        std::vector<double> cat;
        auto atoms = [&](double *dst, const Span<double> HostSystem::*field) {
            const double *src = (systems[0].*field).data();
            if (S > 1) {
                cat.clear();
                cat.reserve(N_);
                for (const HostSystem &h : systems) cat.insert(cat.end(), (h.*field).begin(), (h.*field).end());
                src = cat.data();
            }
            up(dst, src, sizeof(double) * N_);
        };
        atoms(v_.mass, &HostSystem::mass);
        atoms(v_.q, &HostSystem::q);
        atoms(v_.sig, &HostSystem::sig);
        atoms(v_.eps, &HostSystem::eps);
    }
    up(v_.tmp, positions, sizeof(double) * 3 * (size_t)N_);
    launch_init_atoms(v_, v_.tmp, kst());

    // cell-image displacement table: code ((ox+2)*5 + (oy+2))*12 + (oz+2) -> -(o . cs),
    // o relative to the first cell of a group (oz from -2 to kMaxGroupCells + 1)
    std::vector<float4> dt((size_t)S * kDtabStride, make_float4(0, 0, 0, 0));
    for (int s = 0; s < S; ++s)
        for (int ox = -2; ox <= 2; ++ox)
            for (int oy = -2; oy <= 2; ++oy)
                for (int oz = -2; oz <= kMaxGroupCells + 1; ++oz) {
                    int code = ((ox + 2) * 5 + (oy + 2)) * (kMaxGroupCells + 4) + (oz + 2);
                    dt[(size_t)s * kDtabStride + code] =
                        make_float4((float)(-ox * sysd_[s].cs[0]), (float)(-oy * sysd_[s].cs[1]),
                                    (float)(-oz * sysd_[s].cs[2]), 0.f);
                }
    up(v_.dtab, dt.data(), sizeof(float4) * dt.size());

    // PME grid coordinate of every cell's lower corner, per axis, as the
    // reference forms a particle's (t = frac(x / L) K, NonbondedForce.cpp:51-71)
    {
        std::vector<float2> cg(std::max(cg_total, 1), make_float2(0.f, 0.f));
        for (int s = 0; s < S; ++s) {
            const SysDev &D = sysd_[s];
            for (int d = 0; d < 3; ++d)
                for (int c = 0; c < D.nc[d]; ++c) {
                    double t = (D.lb[d] + c * D.cs[d]) * D.invL[d];
                    t = (t - std::floor(t)) * D.K[d];
                    int ti = std::min((int)t, D.K[d] - 1);
                    cg[(size_t)D.cg_off[d] + c] = make_float2((float)ti, (float)(t - ti));
                }
        }
        v_.cgrid = dalloc<float2>(cg.size());
        up(v_.cgrid, cg.data(), sizeof(float2) * cg.size());
    }

    // ---- bonds and terms (batch-global original indices).  Each kind's
    // arrays go up as given -- one system's straight from the caller's
    // array, several systems' concatenated with one host copy each -- and
    // k_terms_ingest checks every atom index against its system's atom count
    // and adds the system's first atom.  An invalid index is reported with
    // the exclusion totals below.  Every bond feeds the exclusion sets; the
    // bond, angle and torsion terms of a system come only with its force
    // mask's bit.
    int *ingest_err = dalloc<int>(1);
    int2 *bonds_all = nullptr;
    int nb_all = 0;
    int *dtab = nullptr;  // [depth S][nonbonded on S][first atom S][atoms S][term offsets 4 x (S + 1)]
    {
        std::vector<int> tab(8 * (size_t)S + 4, 0);
        int *depth = tab.data(), *nb_on = depth + S, *first = nb_on + S, *count = first + S;
        int *o_all = count + S, *o_b = o_all + S + 1, *o_a = o_b + S + 1, *o_t = o_a + S + 1;
        const unsigned bits[3] = {NXM_FORCE_BOND, NXM_FORCE_ANGLE, NXM_FORCE_TORSION};
        int o = 0;
        for (int s = 0; s < S; ++s) {
            const HostSystem &h = systems[s];
            depth[s] = h.excl_depth;
            nb_on[s] = (h.force_mask & NXM_FORCE_NONBONDED) ? 1 : 0;
            first[s] = o;
            count[s] = h.n;
            o += h.n;
            const int m[3] = {(int)(h.bonds.size() / 2), (int)(h.angles.size() / 3), (int)(h.torsions.size() / 4)};
            o_all[s + 1] = o_all[s] + m[0];
            int *ok[3] = {o_b, o_a, o_t};
            for (int k = 0; k < 3; ++k) ok[k][s + 1] = ok[k][s] + ((h.force_mask & bits[k]) ? m[k] : 0);
        }
        nb_all = o_all[S];
        v_.nb = o_b[S];
        v_.na = o_a[S];
        v_.nt = o_t[S];
        dtab = dalloc<int>(tab.size());
        up(dtab, tab.data(), sizeof(int) * tab.size());
        const int *d_first = dtab + 2 * S, *d_count = dtab + 3 * S, *d_oall = dtab + 4 * S,
                  *d_ob = d_oall + S + 1, *d_oa = d_ob + S + 1, *d_ot = d_oa + S + 1;

        // one field of the systems selected by `on`, concatenated in system order
        std::vector<char> cat;
        auto put = [&](void *dst, auto field, auto on) {
            size_t bytes = 0;
            int ns = 0, one = 0;
            for (int s = 0; s < S; ++s) {
                const auto &f = systems[s].*field;
                if (on(s) && f.size()) {
                    bytes += f.size() * sizeof(*f.data());
                    ++ns;
                    one = s;
                }
            }
            if (!bytes) return;
            if (ns == 1) {
                up(dst, (systems[one].*field).data(), bytes);
                return;
            }
            cat.resize(bytes);
            size_t k = 0;
            for (int s = 0; s < S; ++s) {
                const auto &f = systems[s].*field;
                if (on(s) && f.size()) {
                    std::memcpy(cat.data() + k, f.data(), f.size() * sizeof(*f.data()));
                    k += f.size() * sizeof(*f.data());
                }
            }
            up(dst, cat.data(), bytes);
        };
        auto every = [](int) { return true; };
        auto has = [&](unsigned bit) { return [&systems, bit](int s) { return (systems[s].force_mask & bit) != 0; }; };
        auto ingest = [&](const void *in, int per, void *out, int n, const int *toff, int errbit) {
            if (n > 0)
                k_terms_ingest<<<(n + 255) / 256, 256, 0, kst()>>>(static_cast<const int *>(in), per,
                                                                 static_cast<int *>(out), n, toff, d_first, d_count,
                                                                 S, errbit, ingest_err);
        };
        bonds_all = dalloc<int2>(nb_all);
        put(bonds_all, &HostSystem::bonds, every);
        ingest(bonds_all, 2, bonds_all, nb_all, d_oall, 1);
        if (v_.nb == nb_all) {
            v_.bond_orig = bonds_all;  // every system's bonds are terms too
        } else {
            v_.bond_orig = dalloc<int2>(v_.nb);
            put(v_.bond_orig, &HostSystem::bonds, has(NXM_FORCE_BOND));
            ingest(v_.bond_orig, 2, v_.bond_orig, v_.nb, d_ob, 1);
        }
        v_.bond_prm = dalloc<double2>(v_.nb);
        put(v_.bond_prm, &HostSystem::bprm, has(NXM_FORCE_BOND));
        int *araw = dalloc<int>(3 * (size_t)v_.na);
        put(araw, &HostSystem::angles, has(NXM_FORCE_ANGLE));
        v_.angle_orig = dalloc<int4>(v_.na);
        ingest(araw, 3, v_.angle_orig, v_.na, d_oa, 2);
        v_.angle_prm = dalloc<double2>(v_.na);
        put(v_.angle_prm, &HostSystem::aprm, has(NXM_FORCE_ANGLE));
        v_.tors_orig = dalloc<int4>(v_.nt);
        put(v_.tors_orig, &HostSystem::torsions, has(NXM_FORCE_TORSION));
        ingest(v_.tors_orig, 4, v_.tors_orig, v_.nt, d_ot, 4);
        v_.tors_prm = dalloc<double2>(v_.nt);
        put(v_.tors_prm, &HostSystem::tprm, has(NXM_FORCE_TORSION));
        v_.tors_per = dalloc<int>(v_.nt);
        put(v_.tors_per, &HostSystem::tper, has(NXM_FORCE_TORSION));
        v_.bond_slot = dalloc<int2>(v_.nb);
        v_.angle_slot = dalloc<int4>(v_.na);
        v_.tors_slot = dalloc<int4>(v_.nt);
    }

    // exclusion CSR (batch-global original indices) and the excluded pairs
    // j > i of the systems with the nonbonded force, built on the device
    // (k_exclusions_build.cu); a row too long for it: built on the host
    bool ex_on_host = false;
    ExclBuild B{};
    {
        const double t0 = now_ms();
        v_.nxc = (int)xc_pairs.size();
        v_.xc_orig = dalloc<int2>(v_.nxc);
        if (v_.nxc) up(v_.xc_orig, xc_pairs.data(), sizeof(int2) * v_.nxc);
        B.n = N_;
        B.nb = nb_all;
        B.nx = v_.nxc;
        B.bonds = bonds_all;
        B.xc = v_.xc_orig;
        B.sys_of = v_.sys_of;
        B.depth = dtab;
        B.nb_on = dtab + S;
        int *w4 = dalloc<int>(4 * (size_t)N_);
        B.deg = w4;
        B.xdeg = w4 + N_;
        B.afill = w4 + 2 * (size_t)N_;
        B.xfill = w4 + 3 * (size_t)N_;
        B.aoff = dalloc<int>(N_ + 1);
        B.xoff = dalloc<int>(N_ + 1);
        B.adj = dalloc<int>(std::max<size_t>(2 * (size_t)nb_all, 1));
        B.xadj = dalloc<int>(std::max<size_t>(2 * xc_pairs.size(), 1));
        B.len = dalloc<int>(N_);
        B.plen = dalloc<int>(N_);
        B.eoff = dalloc<int>(N_ + 1);
        B.poff = dalloc<int>(N_ + 1);
        B.tile_sum = dalloc<int>(N_ / 4096 + 2);
        B.overflow = dalloc<int>(1);
        if (alloc_failed_) return "device allocation failed (exclusions)";
        launch_exclusions_count(B, kst());
        // the totals (list length, pair count, overflow) and the terms'
        // index check are read once the host has prepared the PME tables
        cudaMemcpyAsync(h_tail_, B.eoff + N_, sizeof(int), cudaMemcpyDeviceToHost, st_);
        cudaMemcpyAsync(h_tail_ + 1, B.poff + N_, sizeof(int), cudaMemcpyDeviceToHost, st_);
        cudaMemcpyAsync(h_tail_ + 2, B.overflow, sizeof(int), cudaMemcpyDeviceToHost, st_);
        cudaMemcpyAsync(h_tail_ + 3, ingest_err, sizeof(int), cudaMemcpyDeviceToHost, st_);
        cudaEventRecord(ev_setup_, st_);
        std::string e = check("exclusions");
        if (!e.empty()) return e;
        create_ms_[8] = now_ms() - t0;
    }

    if (mixed_) {
        // the FP32 engine's parameters rounded once here rather than in
        // every evaluation (the same values: the kernels round the same doubles)
        v_.bond_prmf = dalloc<float2>(v_.nb);
        v_.angle_prmf = dalloc<float2>(v_.na);
        v_.tors_prmf = dalloc<float2>(v_.nt);
        if (alloc_failed_) return "device allocation failed (terms)";
        const std::pair<const double2 *, float2 *> pr[3] = {
            {v_.bond_prm, v_.bond_prmf}, {v_.angle_prm, v_.angle_prmf}, {v_.tors_prm, v_.tors_prmf}};
        const int cnt[3] = {v_.nb, v_.na, v_.nt};
        for (int k = 0; k < 3; ++k)
            if (cnt[k]) k_params_f32<<<(cnt[k] + 255) / 256, 256, 0, kst()>>>(pr[k].first, pr[k].second, cnt[k]);
    }
    v_.xc_slot = dalloc<int2>(v_.nxc);
    v_.xc_prm = dalloc<double4>(v_.nxc);
    if (v_.nxc) up(v_.xc_prm, xc_prm.data(), sizeof(double4) * v_.nxc);
    if (mixed_) {
        v_.xc_prmf = dalloc<float4>(v_.nxc);
        if (v_.nxc) k_xc_params_f32<<<(v_.nxc + 255) / 256, 256, 0, kst()>>>(v_.xc_prm, v_.xc_prmf, v_.nxc);
    }

    // ---- PME
    const double t_dev = now_ms();
    create_ms_[1] = t_dev - t_host;
    bool any_nb = false;
    for (auto &h : sysh_) any_nb |= (h.force_mask & NXM_FORCE_NONBONDED) != 0;
    v_.total_grid = roff;
    v_.total_cgrid = coff;
    bool tuned = false;
    int tv[5] = {0, 0, 0, 0, 0};
    if (any_nb) {
        v_.grid_acc = mixed_ ? (void *)dalloc<int>(roff) : (void *)dalloc<double>(roff);
        v_.grid_real = mixed_ ? (void *)dalloc<float>(roff) : (void *)dalloc<double>(roff);
        v_.grid_cplx = mixed_ ? (void *)dalloc<float2>(coff) : (void *)dalloc<double2>(coff);
        v_.eterm = mixed_ ? (void *)dalloc<float>(coff) : (void *)dalloc<double>(coff);
        v_.twiddle = mixed_ ? (void *)dalloc<float2>(tw_total) : (void *)dalloc<double2>(tw_total);
        if (!v_.grid_acc || !v_.grid_cplx) return "device allocation failed (PME grids)";
        // twiddles exp(-2 pi i t / K)
        std::vector<double> tw(2 * (size_t)tw_total);
        for (int s = 0; s < S; ++s)
            for (int d = 0; d < 3; ++d) {
                int K = sysh_[s].K[d];
                for (int t = 0; t < K; ++t) {
                    double a = -2.0 * kPi * (double)t / (double)K;
                    tw[2 * ((size_t)plan_.hsys[s].tw[d] + t)] = std::cos(a);
                    tw[2 * ((size_t)plan_.hsys[s].tw[d] + t) + 1] = std::sin(a);
                }
            }
        if (mixed_) {
            std::vector<float> twf(tw.begin(), tw.end());
            up(v_.twiddle, twf.data(), sizeof(float) * twf.size());
        } else {
            up(v_.twiddle, tw.data(), sizeof(double) * tw.size());
        }
        // influence function on the half spectrum, NonbondedForce.cpp:323-388:
        // B-spline moduli on the host (once per distinct grid length), the
        // elements on the device (k_influence)
        std::vector<double> mods;
        std::vector<size_t> mod_off(S);
        {
            std::map<int, std::vector<double>> by_len;
            for (int s = 0; s < S; ++s) {
                mod_off[s] = mods.size();
                for (int d = 0; d < 3; ++d) {
                    const int K = sysh_[s].K[d];
                    auto it = by_len.find(K);
                    if (it == by_len.end()) {
                        std::vector<double> m;
                        bspline_moduli(K, m);
                        it = by_len.emplace(K, std::move(m)).first;
                    }
                    mods.insert(mods.end(), it->second.begin(), it->second.end());
                }
            }
        }
        double *dmod = dalloc<double>(mods.size());
        up(dmod, mods.data(), sizeof(double) * mods.size());
        for (int s = 0; s < S; ++s) {
            const SysHost &H = sysh_[s];
            if (!(H.force_mask & NXM_FORCE_NONBONDED)) continue;
            launch_influence(v_.eterm, mixed_, plan_.hsys[s].coff, dmod + mod_off[s], H.K, H.L, H.alpha, kst());
        }
        v_.pme_idx = dalloc<int4>(N_);
        v_.pme_frac = mixed_ ? (void *)dalloc<float4>(N_) : (void *)dalloc<double2>(2 * (size_t)N_);
        // FFT work lists only for systems with nonbonded forces: systems
        // without them keep an empty grid that no block touches
        // launch shapes an earlier context of the same shapes tuned, else
        // the defaults until the autotuner has timed the candidates
        plan_.ext_cap = fft_plan_bytes_max(plan_);
        plan_.ext = dalloc<char>(plan_.ext_cap);
        tuned = opt.autotune && tune_lookup(tv);
        if (tuned) {
            plan_.zlines = tv[0];
            plan_.cols = tv[1];
        }
        fft_plan_build(plan_, mixed_, st_copy_);
        uploads_pending_ = true;
        plan_.plane = tuned ? (tv[2] && plan_.plane_ok) : (plan_.plane_ok && fft_path_ == 2);
        if (tuned) plan_.plane_threads = tv[3];
        tune_[0] = plan_.plane ? 0 : plan_.zlines;
        tune_[1] = plan_.cols;
        if (tuned) tune_[2] = tv[4];
    }
    v_.pme_block = tuned ? tv[4] : 128;
    const double t_pme = now_ms();
    create_ms_[2] = t_pme - t_dev;
    {
        // the exclusion sets: their build on the device ran while the host
        // prepared the terms and the PME tables; a row too long for it, or a
        // batch beyond its scans' reach, is built on the host instead
        const double t0 = now_ms();
        cudaEventSynchronize(ev_setup_);
        std::string e = check("exclusions");
        if (!e.empty()) return e;
        if (h_tail_[3] & 1) return "createExclusions: Illegal particle index in list of bonds";
        if (h_tail_[3] & 2) return "angle atom index out of range";
        if (h_tail_[3] & 4) return "torsion atom index out of range";
        if (h_tail_[2]) {
            ex_on_host = true;
            int o = 0;
            for (const HostSystem &h : systems) {
                e = exclusion_rows(h, o, eoff, elst, ex_pairs);
                if (!e.empty()) return e;
                o += h.n;
            }
            v_.excl_off = dalloc<int>(N_ + 1);
            v_.excl_lst = dalloc<int>(std::max<size_t>(elst.size(), 1));
            up(v_.excl_off, eoff.data(), sizeof(int) * (N_ + 1));
            if (!elst.empty()) up(v_.excl_lst, elst.data(), sizeof(int) * elst.size());
            // exclusion correction pairs: only for systems with nonbonded enabled
            std::vector<int2> keep;
            for (auto &x : ex_pairs)
                if (sysh_[S > 1 ? sys_of[x.x] : 0].force_mask & NXM_FORCE_NONBONDED) keep.push_back(x);
            ex_pairs.swap(keep);
            v_.nex = (int)ex_pairs.size();
            v_.ex_orig = dalloc<int2>(v_.nex);
            if (v_.nex) up(v_.ex_orig, ex_pairs.data(), sizeof(int2) * v_.nex);
        } else {
            v_.excl_off = B.eoff;
            v_.excl_lst = dalloc<int>(std::max(h_tail_[0], 1));
            v_.nex = h_tail_[1];
            v_.ex_orig = dalloc<int2>(std::max(v_.nex, 1));
            if (alloc_failed_) return "device allocation failed (exclusions)";
            launch_exclusions_fill(B, v_.excl_lst, v_.ex_orig, kst());
        }
        v_.ex_slot = dalloc<int2>(v_.nex);
        create_ms_[8] += now_ms() - t0;
    }
    // systems without nonbonded forces: zero their charges in the PME and
    // pair paths by skipping them entirely (no list, no grid)
    v_.E = dalloc<long long>((size_t)S * E_SLOTS);
    v_.flags = dalloc<Flags>(1);
    {
        Flags f{};
        f.interval = interval_;
        up(v_.flags, &f, sizeof(f));
    }
    v_.snap_x = dalloc<double>(3 * (size_t)N_);
    v_.snap_v = dalloc<double>(3 * (size_t)N_);
    v_.snap_f = dalloc<double>(3 * (size_t)N_);
    stage3_ = dalloc<double>(3 * (size_t)N_);  // state uploads (set_positions, set_velocities)
    // frame steps' device buffers A and B (nxm_step_async)
    for (int b = 0; b < 2; ++b) {
        frame_x_[b] = dalloc<double>(3 * (size_t)N_);
        frame_E_[b] = dalloc<long long>(energies_.size());
    }
    v_.skin_half2 = skin > 0 ? 0.25 * skin * skin : 0.0;
    v_.force_mask = 0;
    for (auto &h : sysh_) v_.force_mask |= h.force_mask;
    v_.any_switch = 0;
    for (auto &d : sysd_) v_.any_switch |= d.use_switch ? 1 : 0;
    if (alloc_failed_) return "device allocation failed";
    launch_derive_inputs(v_, kst());
    force_rebuild_ = true;
    std::string e = check("set-up");
    if (!e.empty()) return e;
    // the allocations and uploads after the PME tables count with [1]
    const double t_rest = now_ms();
    create_ms_[1] += t_rest - t_pme;
    // Without candidates to time, creation returns with its last kernels
    // still queued: the next call that waits for the device reports a
    // failure of theirs.
    autotune_cached_ = tuned ? 1 : 0;
    if (opt.autotune && !tuned && (v_.force_mask & NXM_FORCE_NONBONDED) && plan_.nz) {
        cudaStreamSynchronize(st_);
        e = check("set-up");
        if (!e.empty()) return e;
        e = autotune();
    }
    if (!e.empty()) return e;
    if (self_th.t.joinable()) self_th.t.join();
    for (int s = 0; s < S; ++s) sysh_[s].self_energy = self_e[s];
    // the first neighbour list, built on the device while the caller goes on
    launch_decide_rebuild(v_, 2, kst());
    launch_nlist_rebuild(v_, st_);
    force_rebuild_ = false;
    e = check("first neighbour list");
    create_ms_[3] = now_ms() - t_rest;
    create_ms_[5] = create_ms_[0] + create_ms_[1] + create_ms_[2] + create_ms_[3];
    return e;
}

namespace {
// Autotuned launch shapes per shape of batch within the process: the picks
// change no result (see Engine::autotune), so a context with the same
// device, precision, FFT path option, atom count and grids takes them
// without timing the candidates again.
struct TuneKey {
    int device, mixed, fft_path, n;
    std::vector<int> grids;
    bool operator<(const TuneKey &o) const {
        return std::tie(device, mixed, fft_path, n, grids) < std::tie(o.device, o.mixed, o.fft_path, o.n, o.grids);
    }
};
struct TuneVal {
    int zlines, cols, plane, plane_threads, pme_block;
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneVal> g_tune_cache;
}  // namespace

// Launch shapes that change no result, chosen by timing each candidate on
// this context's own buffers (grid contents do not matter for the timing;
// what the timed kernels accumulate is cleared afterwards):
//  * FFT: threads per plane block (plane path) or real lines per z-pass
//    block (line path), x columns per x-pass (and y-pass) block -- every line
//    is transformed by the same arithmetic whatever the blocking;
//  * spread / gather: threads per block -- the sums are integer atomics.
// The neighbour-list cell groups are not tuned: their size changes the
// summation order of the pair forces, and a choice that followed timing
// noise would break run-to-run bit reproducibility.
bool Engine::tune_lookup(int out[5]) {
    TuneKey key{device_, mixed_, fft_path_, N_, {}};
    for (auto &h : sysh_)
        for (int d = 0; d < 3; ++d) key.grids.push_back(h.K[d]);
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it == g_tune_cache.end()) return false;
    const TuneVal &t = it->second;
    const int v[5] = {t.zlines, t.cols, t.plane, t.plane_threads, t.pme_block};
    std::copy(v, v + 5, out);
    return true;
}

std::string Engine::autotune() {
    TuneKey key{device_, mixed_, fft_path_, N_, {}};
    for (auto &h : sysh_)
        for (int d = 0; d < 3; ++d) key.grids.push_back(h.K[d]);
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    auto time3 = [&](auto &&launch) {
        launch();  // warm-up
        cudaEventRecord(a, st_);
        for (int r = 0; r < 3; ++r) launch();
        cudaEventRecord(b, st_);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        return ms;
    };
    // The plane path joins the line path as a candidate only where the two
    // give the same numbers bit for bit (every system's K1 even: the z
    // transforms pair the same real lines), so that a pick that follows
    // timing noise cannot change results; fft_path 1 / 2 fix the path.
    bool even_k1 = true;
    for (int s = 0; s < plan_.S; ++s) even_k1 = even_k1 && plan_.hsys[s].K[1] % 2 == 0;
    const bool try_line = fft_path_ != 2 || !plan_.plane_ok;
    const bool try_plane = plan_.plane_ok && (fft_path_ == 2 || (fft_path_ == 0 && even_k1));
    float best = 1e30f;
    int bz = plan_.zlines, bc = plan_.cols, bp = plan_.plane, bpt = plan_.plane_threads;
    for (int cols : {4, 8, 16}) {
        for (int zl : {8, 16, 32}) {
            if (!try_line && zl != 16) continue;  // the z blocking is unused on the plane path
            plan_.zlines = zl;
            plan_.cols = cols;
            fft_plan_build(plan_, mixed_, st_);
            for (int plane = 0; plane < 2; ++plane) {
                if (plane ? !(try_plane && zl == 16) : !try_line) continue;
                plan_.plane = plane;
                for (int th : {256, 512, 1024}) {
                    if (!plane && th != 256) continue;
                    plan_.plane_threads = th;
                    float t = time3([&] { launch_fft_convolve(v_, plan_, 0, st_); });
                    if (t < best) {
                        best = t;
                        bz = zl;
                        bc = cols;
                        bp = plane;
                        bpt = th;
                    }
                }
            }
        }
    }
    plan_.zlines = bz;
    plan_.cols = bc;
    fft_plan_build(plan_, mixed_, st_);
    plan_.plane = bp;
    plan_.plane_threads = bpt;
    best = 1e30f;
    int bt = v_.pme_block;
    for (int t : {64, 128, 256}) {
        v_.pme_block = t;
        float ms = time3([&] {
            launch_spread(v_, plan_, st_);
            launch_gather(v_, plan_, st_);
        });
        if (ms < best) {
            best = ms;
            bt = t;
        }
    }
    v_.pme_block = bt;
    // the gather added into the force words
    size_t fb = sizeof(long long) * (size_t)N_;
    cudaMemsetAsync(v_.fx, 0, fb, st_);
    cudaMemsetAsync(v_.fy, 0, fb, st_);
    cudaMemsetAsync(v_.fz, 0, fb, st_);
    cudaStreamSynchronize(st_);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    tune_[0] = plan_.plane ? 0 : bz;
    tune_[1] = bc;
    tune_[2] = bt;
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tune_cache[key] = TuneVal{bz, bc, bp, bpt, bt};
    }
    return check("autotune");
}

// A state array from the caller (original order, x y z per atom) into
// slot order.  It goes up on the copy stream into a staging buffer -- an
// upload from pageable memory returns once its source is consumed, and on
// that stream it waits for no work queued on the compute stream -- and the
// gather runs on the compute stream after it.  The staging buffer is written
// again only after the last gather from it.
std::string Engine::stage_state(const double *xyz, double *dx, double *dy, double *dz) {
    if (stage_used_) cudaStreamWaitEvent(st_copy_, ev_stage_free_, 0);
    cudaMemcpyAsync(stage3_, xyz, sizeof(double) * 3 * (size_t)N_, cudaMemcpyHostToDevice, st_copy_);
    cudaEventRecord(ev_staged_, st_copy_);
    cudaStreamWaitEvent(st_, ev_staged_, 0);
    if (N_ > 0) k_state_to_slots<<<(N_ + 255) / 256, 256, 0, st_>>>(v_, stage3_, dx, dy, dz);
    cudaEventRecord(ev_stage_free_, st_);
    stage_used_ = true;
    return check("state upload");
}

std::string Engine::set_positions(const double *xyz) {
    // the slot order is re-derived from the new positions by the forced
    // rebuild of the next evaluation
    std::string e = stage_state(xyz, v_.x, v_.y, v_.z);
    if (!e.empty()) return e;
    launch_derive_inputs(v_, st_);
    force_rebuild_ = true;
    return check("set_positions");
}

std::string Engine::set_velocities(const double *xyz) { return stage_state(xyz, v_.vx, v_.vy, v_.vz); }

// Force kernels of one evaluation (everything but the integrator).
// Kernel launches of force_launches below, without launching.
static int pme_launch_count(const DevView &v, const FftPlan &plan) {
    return (v.N == 0 || plan.nz == 0) ? 0 : 2 + fft_launch_count(plan);
}
static int force_launch_count(const DevView &v, const FftPlan &plan) {
    bool nb = (v.force_mask & NXM_FORCE_NONBONDED) != 0;
    int n = (v.nb + v.na + v.nt + (nb ? v.nex + v.nxc : 0)) ? 1 : 0;
    if (nb) n += 1 + pme_launch_count(v, plan);
    return n;
}

// All force kernels.  With a second stream `pme_st`, the PME chain (spread,
// FFT, gather) runs there as an independent branch: it shares nothing with
// the bonded / pair / exclusion kernels but the force words, which both add
// to with integer atomics (order-free); the caller joins the streams before
// the update.
static int force_launches(const DevView &v, const FftPlan &plan, int energy, cudaStream_t st,
                          cudaStream_t pme_st = nullptr) {
    int n = 0;
    bool nb = (v.force_mask & NXM_FORCE_NONBONDED) != 0;
    if (nb && pme_st) {
        launch_pme(v, plan, energy, pme_st);
        n += pme_launch_count(v, plan);
    }
    // bonded terms, exclusion correction and exceptions: one launch
    n += launch_bonded(v, energy, st, nb ? 1 : 0);
    if (nb) {
        launch_pairs(v, energy, st);
        ++n;
        if (!pme_st) {
            launch_pme(v, plan, energy, st);
            n += pme_launch_count(v, plan);
        }
    }
    return n;
}

void Engine::free_graphs() {
    for (auto &G : graph_) {
        if (G.exec) cudaGraphExecDestroy(G.exec);
        if (G.graph) cudaGraphDestroy(G.graph);
        G = StepGraph{};
    }
}

std::string Engine::build_graph(double dt, int report) {
    const double t0 = now_ms();
    std::string r = build_graph_timed(dt, report);
    create_ms_[4] += now_ms() - t0;
    return r;
}

std::string Engine::build_graph_timed(double dt, int report) {
    StepGraph &G = graph_[report];
    const DevView vv = view_for(report);
    if (G.exec) cudaGraphExecDestroy(G.exec);
    if (G.graph) cudaGraphDestroy(G.graph);
    G = StepGraph{};
    const cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
    cudaGraph_t g = nullptr, captured = nullptr;
    auto fail_capture = [&](const char *what, cudaError_t e) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st_, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone)
            cudaStreamEndCapture(st_, &captured);
        cudaGetLastError();
        return std::string("step graph: ") + what + ": " + cudaGetErrorString(e);
    };
    cudaError_t e = cudaGraphCreate(&g, 0);
    if (e != cudaSuccess) return fail_capture("create", e);
    G.graph = g;
    cudaGraphConditionalHandle h;
    e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) return fail_capture("conditional handle", e);
    // head: energy reset and the decision
    e = cudaStreamBeginCaptureToGraph(st_, g, nullptr, nullptr, 0, mode);
    if (e != cudaSuccess) return fail_capture("capture head", e);
    if (report) cudaMemsetAsync(vv.E, 0, sizeof(long long) * v_.S * E_SLOTS, st_);
    k_decide_graph<<<1, 1, 0, st_>>>(vv, h);
    cudaStreamCaptureStatus cs;
    const cudaGraphNode_t *deps = nullptr;
    size_t nd = 0;
    e = cudaStreamGetCaptureInfo(st_, &cs, nullptr, nullptr, &deps, nullptr, &nd);
    if (e != cudaSuccess) return fail_capture("capture info", e);
    std::vector<cudaGraphNode_t> head(deps, deps + nd);
    e = cudaStreamEndCapture(st_, &captured);
    if (e != cudaSuccess) return fail_capture("end head", e);
    // the conditional rebuild node and its body
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeIf;
    cp.conditional.size = 1;
    cudaGraphNode_t cnode;
    e = cudaGraphAddNode(&cnode, g, head.data(), nullptr, head.size(), &cp);
    if (e != cudaSuccess) return fail_capture("conditional node", e);
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    e = cudaStreamBeginCaptureToGraph(st_, body, nullptr, nullptr, 0, mode);
    if (e != cudaSuccess) return fail_capture("capture rebuild", e);
    launch_nlist_rebuild(vv, st_);
    e = cudaStreamEndCapture(st_, &captured);
    if (e != cudaSuccess) return fail_capture("end rebuild", e);
    // tail: forces and update, after the conditional node
    e = cudaStreamBeginCaptureToGraph(st_, g, &cnode, nullptr, 1, mode);
    if (e != cudaSuccess) return fail_capture("capture tail", e);
    // PME as a parallel branch on the second stream, joined before the update
    cudaEventRecord(ev_fork_, st_);
    cudaStreamWaitEvent(st_pme_, ev_fork_, 0);
    force_launches(vv, plan_, report ? 1 : 0, st_, st_pme_);
    cudaEventRecord(ev_join_, st_pme_);
    cudaStreamWaitEvent(st_, ev_join_, 0);
    launch_integrate(vv, dt, report >= 2 ? 2 : report, st_);
    e = cudaStreamEndCapture(st_, &captured);
    if (e != cudaSuccess) return fail_capture("end tail", e);
    e = cudaGraphInstantiate(&G.exec, g, 0);
    if (e != cudaSuccess) return fail_capture("instantiate", e);
    G.dt = dt;
    G.ok = true;
    return "";
}

// One step of report kind `report` (0 none, 1 energies and the x/v/F
// snapshot, 2 / 3 a frame into frame buffer A / B).
std::string Engine::one_step(double dt, int report) {
    launches_per_rebuild_ = 8;  // kernels of one list rebuild
    if (!force_rebuild_) {
        StepGraph &G = graph_[report];
        if (!G.ok || G.dt != dt) {
            std::string e = build_graph(dt, report);
            if (!e.empty()) return e;
        }
        cudaError_t e = cudaGraphLaunch(G.exec, st_);
        if (e != cudaSuccess) return std::string("step graph launch: ") + cudaGetErrorString(e);
        // decide + forces + integrate; the rebuild kernels run on rebuild steps only
        launches_per_step_ = force_launch_count(v_, plan_) + 2;
        return check("step");
    }
    const DevView vv = view_for(report);
    if (report) cudaMemsetAsync(vv.E, 0, sizeof(long long) * v_.S * E_SLOTS, st_);
    launch_decide_rebuild(vv, 1, st_);
    force_rebuild_ = false;
    launch_nlist_rebuild(vv, st_);
    int n = force_launches(vv, plan_, report ? 1 : 0, st_);
    launch_integrate(vv, dt, report >= 2 ? 2 : report, st_);
    launches_per_step_ = n + 2 + launches_per_rebuild_;
    return check("step");
}

void Engine::fetch_energies() {
    cudaMemcpyAsync(h_E_, v_.E, sizeof(long long) * v_.S * E_SLOTS, cudaMemcpyDeviceToHost, st_);
}

std::string Engine::finish_call() {
    fetch_energies();
    cudaMemcpyAsync(h_flags_, v_.flags, sizeof(Flags), cudaMemcpyDeviceToHost, st_);
    cudaError_t e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return std::string("device: ") + cudaGetErrorString(e);
    for (size_t k = 0; k < energies_.size(); ++k) energies_[k] = (double)h_E_[k] * kEnergyUnscale;
    return flag_error(h_flags_[0]);
}

std::string Engine::flag_error(int err) {
    if (err & ERR_NLIST_OVERFLOW) return "neighbour list capacity exceeded (raise max_neighbors)";
    if (err & ERR_NONFINITE) return "non-finite force";
    return "";
}

std::string Engine::enqueue_report(double *x, double *v, double *f, long long *E, int *flags, cudaEvent_t done) {
    size_t b = sizeof(double) * 3 * (size_t)N_;
    cudaMemcpyAsync(x, v_.snap_x, b, cudaMemcpyDeviceToHost, st_);
    cudaMemcpyAsync(v, v_.snap_v, b, cudaMemcpyDeviceToHost, st_);
    cudaMemcpyAsync(f, v_.snap_f, b, cudaMemcpyDeviceToHost, st_);
    cudaMemcpyAsync(E, v_.E, sizeof(long long) * energies_.size(), cudaMemcpyDeviceToHost, st_);
    cudaMemcpyAsync(flags, v_.flags, sizeof(Flags), cudaMemcpyDeviceToHost, st_);
    cudaEventRecord(done, st_);
    return check("report copies");
}

void Engine::free_frames() {
    if (st_copy_) cudaStreamSynchronize(st_copy_);
    for (Frame &f : ring_) {
        if (f.done) cudaEventSynchronize(f.done);
        if (f.done) cudaEventDestroy(f.done);
    }
    pinned_free(ring_mem_);
    ring_mem_ = nullptr;
    ring_.clear();
    ring_next_ = ring_pending_ = 0;
}

DevView Engine::view_for(int kind) const {
    DevView v = v_;
    if (kind >= 2) {
        v.E = frame_E_[kind - 2];
        v.snap_x = frame_x_[kind - 2];
    }
    return v;
}

size_t Engine::frame_slot_bytes() const {
    return al256(sizeof(double) * 3 * (size_t)N_) + al256(sizeof(long long) * energies_.size()) + al256(sizeof(Flags));
}

std::string Engine::frames_init(int depth) {
    if (depth < 1 || depth > 64) return "frame ring depth must be 1..64";
    if (ring_pending_) return "frames still pending: wait for them first";
    free_frames();
    // one page-locked block; per slot the positions, the energy words and
    // the flags, 256-byte aligned
    const size_t bx = al256(sizeof(double) * 3 * (size_t)N_), be = al256(sizeof(long long) * energies_.size()),
                 slot = frame_slot_bytes();
    ring_mem_ = pinned_alloc(slot * depth);
    if (!ring_mem_) return "device: pinned frame buffers could not be allocated";
    char *mem = static_cast<char *>(ring_mem_);
    for (int b = 0; b < 2; ++b) buf_used_[b] = false;
    ring_.resize(depth);
    for (int k = 0; k < depth; ++k) {
        char *base = mem + slot * k;
        Frame &f = ring_[k];
        f.x = reinterpret_cast<double *>(base);
        f.E = reinterpret_cast<long long *>(base + bx);
        f.flags = reinterpret_cast<int *>(base + bx + be);
        if (cudaEventCreateWithFlags(&f.done, cudaEventDisableTiming) != cudaSuccess) {
            free_frames();
            return "device: frame events could not be created";
        }
    }
    return check("frames");
}

std::string Engine::step_async(int nsteps, double dt) {
    if (ring_.empty()) {
        std::string e = frames_init(2);
        if (!e.empty()) return e;
    }
    Frame &f = ring_[ring_next_];
    if (f.pending) return "frame ring full: wait for a frame before the next nxm_step_async";
    const int b = frame_buf_;
    for (int k = 0; k < nsteps; ++k) {
        const bool last = k == nsteps - 1;
        // frame buffer b is written again only after its last copy finished
        if (last && buf_used_[b]) cudaStreamWaitEvent(st_, buf_free_[b], 0);
        std::string e = one_step(dt, last ? 2 + b : 0);
        if (!e.empty()) return e;
    }
    // the flags after the step, in stream order; then the positions and
    // energies on the copy stream while the next step runs
    cudaMemcpyAsync(f.flags, v_.flags, sizeof(Flags), cudaMemcpyDeviceToHost, st_);
    cudaEventRecord(step_done_, st_);
    cudaStreamWaitEvent(st_copy_, step_done_, 0);
    cudaMemcpyAsync(f.x, frame_x_[b], sizeof(double) * 3 * (size_t)N_, cudaMemcpyDeviceToHost, st_copy_);
    cudaMemcpyAsync(f.E, frame_E_[b], sizeof(long long) * energies_.size(), cudaMemcpyDeviceToHost, st_copy_);
    cudaEventRecord(buf_free_[b], st_copy_);
    cudaEventRecord(f.done, st_copy_);
    buf_used_[b] = true;
    frame_buf_ ^= 1;
    f.pending = true;
    ring_next_ = (ring_next_ + 1) % (int)ring_.size();
    ++ring_pending_;
    return check("step_async");
}

std::string Engine::frame_wait(const double **xyz, nxm_energies *out, int n_out) {
    if (!ring_pending_) return "no frame pending";
    const int depth = (int)ring_.size();
    Frame &f = ring_[(ring_next_ - ring_pending_ + depth) % depth];
    cudaError_t ce = cudaEventSynchronize(f.done);
    f.pending = false;
    --ring_pending_;
    if (ce != cudaSuccess) return std::string("device: ") + cudaGetErrorString(ce);
    std::memcpy(h_flags_, f.flags, sizeof(Flags));
    std::string e = flag_error(f.flags[0]);
    if (!e.empty()) return e;
    for (size_t k = 0; k < energies_.size(); ++k) energies_[k] = (double)f.E[k] * kEnergyUnscale;
    for (int s = 0; s < n_out && s < (int)sysh_.size(); ++s) energies(s, &out[s]);
    if (xyz) *xyz = f.x;
    return "";
}

std::string Engine::step(int nsteps, double dt) {
    for (int k = 0; k < nsteps; ++k) {
        std::string e = one_step(dt, k == nsteps - 1);
        if (!e.empty()) return e;
    }
    return finish_call();
}

std::string Engine::compute_forces() {
    cudaMemsetAsync(v_.E, 0, sizeof(long long) * v_.S * E_SLOTS, st_);
    launch_decide_rebuild(v_, 1, st_);
    force_rebuild_ = false;
    launch_nlist_rebuild(v_, st_);
    force_launches(v_, plan_, 1, st_);
    launch_export(v_, 1, st_);
    std::string e = check("compute_forces");
    if (!e.empty()) return e;
    return finish_call();
}

std::string Engine::time_steps(int nsteps, double dt, double *ms, int report) {
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, st_);
    for (int k = 0; k < nsteps; ++k) {
        std::string e = one_step(dt, report);
        if (!e.empty()) return e;
    }
    cudaEventRecord(b, st_);
    std::string e = finish_call();
    float t = 0;
    cudaEventElapsedTime(&t, a, b);
    *ms = t;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return e;
}

// Average device time per step of each phase over nsteps steps, from CUDA
// events recorded on the engine's stream between the phases:
// 0 list decision + rebuild, 1 bonded, 2 pairs, 3 exclusions, 4 spread,
// 5 FFT + convolution, 6 gather, 7 integrate.
std::string Engine::profile(int nsteps, double dt, double *ms) {
    const int P = kProfilePhases;
    cudaEvent_t ev[P + 1];
    for (auto &e : ev) cudaEventCreate(&e);
    double acc[P] = {0};
    for (int k = 0; k < nsteps; ++k) {
        cudaEventRecord(ev[0], st_);
        launch_decide_rebuild(v_, force_rebuild_ ? 1 : 0, st_);
        force_rebuild_ = false;
        launch_nlist_rebuild(v_, st_);
        cudaEventRecord(ev[1], st_);
        if (v_.nb + v_.na + v_.nt) launch_bonded(v_, 0, st_);
        cudaEventRecord(ev[2], st_);
        bool nb = (v_.force_mask & NXM_FORCE_NONBONDED) != 0;
        if (nb) launch_pairs(v_, 0, st_);
        cudaEventRecord(ev[3], st_);
        if (nb && v_.nex) launch_exclusions(v_, 0, st_);
        if (nb && v_.nxc) launch_exceptions(v_, 0, st_);
        cudaEventRecord(ev[4], st_);
        if (nb && plan_.nz) launch_spread(v_, plan_, st_);
        cudaEventRecord(ev[5], st_);
        if (nb && plan_.nz) launch_fft_convolve(v_, plan_, 0, st_);
        cudaEventRecord(ev[6], st_);
        if (nb && plan_.nz) launch_gather(v_, plan_, st_);
        cudaEventRecord(ev[7], st_);
        launch_integrate(v_, dt, 0, st_);
        cudaEventRecord(ev[8], st_);
        cudaError_t e = cudaEventSynchronize(ev[8]);
        if (e != cudaSuccess) return std::string("profile: ") + cudaGetErrorString(e);
        for (int p = 0; p < P; ++p) {
            float t = 0;
            cudaEventElapsedTime(&t, ev[p], ev[p + 1]);
            acc[p] += t;
        }
    }
    for (auto &e : ev) cudaEventDestroy(e);
    for (int p = 0; p < P; ++p) ms[p] = acc[p] / nsteps;
    return finish_call();
}

std::string Engine::get_snapshot(double *x, double *v, double *f) {
    cudaStreamSynchronize(st_);
    size_t b = sizeof(double) * 3 * (size_t)N_;
    if (x) cudaMemcpy(x, v_.snap_x, b, cudaMemcpyDeviceToHost);
    if (v) cudaMemcpy(v, v_.snap_v, b, cudaMemcpyDeviceToHost);
    if (f) cudaMemcpy(f, v_.snap_f, b, cudaMemcpyDeviceToHost);
    return check("snapshot");
}

std::string Engine::get_state(double *x, double *v) {
    // export current x and v (not forces) into the snapshot buffers' copies
    std::vector<int> orig(N_);
    cudaStreamSynchronize(st_);
    cudaMemcpy(orig.data(), v_.orig, sizeof(int) * N_, cudaMemcpyDeviceToHost);
    std::vector<double> a(N_), b(N_), c(N_);
    double *src[2][3] = {{v_.x, v_.y, v_.z}, {v_.vx, v_.vy, v_.vz}};
    double *dst[2] = {x, v};
    for (int k = 0; k < 2; ++k) {
        if (!dst[k]) continue;
        cudaMemcpy(a.data(), src[k][0], sizeof(double) * N_, cudaMemcpyDeviceToHost);
        cudaMemcpy(b.data(), src[k][1], sizeof(double) * N_, cudaMemcpyDeviceToHost);
        cudaMemcpy(c.data(), src[k][2], sizeof(double) * N_, cudaMemcpyDeviceToHost);
        for (int s = 0; s < N_; ++s) {
            int o = orig[s];
            dst[k][3 * (size_t)o] = a[s];
            dst[k][3 * (size_t)o + 1] = b[s];
            dst[k][3 * (size_t)o + 2] = c[s];
        }
    }
    return check("state");
}

void Engine::energies_from(const long long *raw, int s, nxm_energies *out) const {
    double e[E_SLOTS];
    for (int k = 0; k < E_SLOTS; ++k) e[k] = (double)raw[(size_t)s * E_SLOTS + k] * kEnergyUnscale;
    decode_energies(e, sysh_[s], out);
}

void Engine::energies(int s, nxm_energies *out) const { decode_energies(energies_.data() + (size_t)s * E_SLOTS, sysh_[s], out); }

void Engine::decode_energies(const double *e, const SysHost &H, nxm_energies *out) {
    std::memset(out, 0, sizeof(*out));
    out->bond = e[E_BOND];
    out->angle = e[E_ANGLE];
    out->torsion = e[E_TORSION];
    out->kinetic = e[E_KIN];
    double pe = 0.0;
    if (H.force_mask & NXM_FORCE_BOND) pe += out->bond;
    if (H.force_mask & NXM_FORCE_ANGLE) pe += out->angle;
    if (H.force_mask & NXM_FORCE_TORSION) pe += out->torsion;
    double reported = pe;
    if (H.force_mask & NXM_FORCE_NONBONDED) {
        out->recip = e[E_RECIP];
        out->self = H.self_energy;
        out->coulomb = e[E_COUL];
        out->vdw = e[E_VDW];
        out->exclusion = e[E_EXCL];
        out->exception = e[E_EXCEPT];
        double nb = out->recip + out->self + out->coulomb + out->vdw - out->exclusion + out->exception;
        pe += nb;
        // NonbondedForce.cpp:387 assigns the reciprocal energy to the running
        // total, then self, direct and exclusion terms are added to it
        // (exceptions, which the reference never applies, come last)
        reported = out->recip;
        reported += out->self;
        reported += out->coulomb + out->vdw;
        reported -= out->exclusion;
        reported += out->exception;
    }
    out->potential = pe;
    out->reported_potential = reported;
}

std::string Engine::pme_grids(int s, double *charge, double *influence, double *potential) {
    if (!v_.grid_acc || !(sysh_[s].force_mask & NXM_FORCE_NONBONDED)) return "no PME grids (nonbonded force off)";
    cudaError_t ce = cudaStreamSynchronize(st_);
    if (ce != cudaSuccess) return std::string("device: ") + cudaGetErrorString(ce);
    const FftSysDev &F = plan_.hsys[s];
    const size_t nr = (size_t)F.K[0] * F.K[1] * F.K[2], nc = (size_t)F.K[0] * F.K[1] * F.Kh;
    auto fetch = [&](const void *base, size_t off, size_t n, size_t esz, std::vector<unsigned char> &h) {
        h.resize(n * esz);
        return cudaMemcpy(h.data(), static_cast<const unsigned char *>(base) + off * esz, n * esz,
                          cudaMemcpyDeviceToHost);
    };
    std::vector<unsigned char> h;
    if (charge) {
        if (fetch(v_.grid_acc, F.roff, nr, mixed_ ? 4 : 8, h) != cudaSuccess) return check("pme_grids");
        for (size_t k = 0; k < nr; ++k) {
            if (mixed_) {
                int w;
                std::memcpy(&w, &h[4 * k], 4);
                charge[k] = (double)w * kGridUnscale;
            } else {
                std::memcpy(&charge[k], &h[8 * k], 8);
            }
        }
    }
    const size_t fsz = mixed_ ? 4 : 8;
    auto to_double = [&](double *out, size_t n) {
        for (size_t k = 0; k < n; ++k) {
            if (mixed_) {
                float f;
                std::memcpy(&f, &h[4 * k], 4);
                out[k] = f;
            } else {
                std::memcpy(&out[k], &h[8 * k], 8);
            }
        }
    };
    if (influence) {
        if (fetch(v_.eterm, F.coff, nc, fsz, h) != cudaSuccess) return check("pme_grids");
        to_double(influence, nc);
    }
    if (potential) {
        if (fetch(v_.grid_real, F.roff, nr, fsz, h) != cudaSuccess) return check("pme_grids");
        to_double(potential, nr);
    }
    return check("pme_grids");
}

void Engine::layout(int s, int out[kLayoutWords]) const {
    const SysDev &D = sysd_[s];
    out[0] = group_g_[s];
    out[1] = v_.hood_cap;
    for (int d = 0; d < 3; ++d) out[2 + d] = D.nc[d];
    out[5] = v_.stride;
    out[6] = plan_.plane ? 2 : 1;
    out[7] = plan_.plane_chunked;
    for (int d = 0; d < 3; ++d) out[8 + d] = plan_.hsys[s].ax[d].np;
}

int Engine::fft_radices(int s, int d, int *out, int cap) const {
    const FftPasses &P = plan_.hsys[s].ax[d];
    for (int p = 0; p < P.np && p < cap; ++p) out[p] = P.R[p];
    return P.np;
}

std::string Engine::pairs(int s, std::vector<int> &out) {
    cudaStreamSynchronize(st_);
    long long cap = 400LL * sysh_[s].natoms + 1024;
    int *d = nullptr;
    if (cudaMalloc(&d, sizeof(int) * 2 * cap) != cudaSuccess) return "allocation failed";
    long long n = launch_collect_pairs(v_, s, d, cap, st_);
    if (n > cap) {
        cudaFree(d);
        cap = n;
        if (cudaMalloc(&d, sizeof(int) * 2 * cap) != cudaSuccess) return "allocation failed";
        n = launch_collect_pairs(v_, s, d, cap, st_);
    }
    out.resize(2 * (size_t)n);
    if (n) cudaMemcpy(out.data(), d, sizeof(int) * 2 * n, cudaMemcpyDeviceToHost);
    cudaFree(d);
    return check("pairs");
}

}  // namespace nxm
