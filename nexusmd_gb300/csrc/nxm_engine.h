// Host side of the CUDA engine: set-up of a batch of systems, device memory,
// and the per-step launch sequence.
#pragma once

#include <string>
#include <vector>

#include "../../include/nxm.h"
#include "nxm_fft.h"
#include "nxm_view.h"

namespace nxm {

constexpr int kProfilePhases = 8;
constexpr int kLayoutWords = 11;
constexpr int kCreatePhases = 9;

// A read-only view of a caller's array (valid for the duration of the call
// that receives it): context creation reads the inputs in place.
template <class T>
struct Span {
    const T *p = nullptr;
    size_t n = 0;
    Span() = default;
    Span(const T *ptr, size_t count) : p(ptr), n(count) {}
    Span(const std::vector<T> &v) : p(v.data()), n(v.size()) {}  // NOLINT: views a vector the caller keeps
    const T *data() const { return p; }
    size_t size() const { return n; }
    bool empty() const { return n == 0; }
    const T &operator[](size_t i) const { return p[i]; }
    const T *begin() const { return p; }
    const T *end() const { return p + n; }
};

// One system's inputs to Engine::init, viewed in the caller's arrays.
struct HostSystem {
    int n = 0;
    Span<double> mass, q, sig, eps;
    Span<int> bonds, angles, torsions, tper;  // flattened atom indices
    Span<double> bprm, aprm, tprm;
    double cutoff = 1.0, tol = 5e-4;
    int use_switch = 0;
    double sw_dist = 0.0;
    int grid[3] = {0, 0, 0};
    int box_from_positions = 1;
    double lb[3] = {0, 0, 0}, ub[3] = {0, 0, 0};
    int force_mask = 15;
    int excl_depth = 3;
    // exception pairs (OpenMM semantics): atoms, and chargeProd / sigma / epsilon
    Span<int> exc;
    Span<double> exc_prm;
};

struct SysHost {
    double lb[3], ub[3], L[3];
    double alpha, rlist;
    int K[3];
    double self_energy;
    int atom_off, natoms;
    int force_mask;
};

class Engine {
public:
    Engine() = default;
    ~Engine();
    // Returns an empty string on success, else the error.
    std::string init(const std::vector<HostSystem> &systems, const nxm_options &opt,
                     const double *positions);
    std::string set_positions(const double *xyz);
    std::string set_velocities(const double *xyz);
    std::string compute_forces();
    std::string step(int nsteps, double dt);
    // Steps with a snapshot on the schedule of the reference's Report
    // (step 0 and every `interval`-th); `on_report(step)` runs after each.
    template <typename F>
    std::string run_reporting(int nsteps, double dt, int interval, F on_report);
    // One step; with report != 0 the energies and the x/v/F snapshot of the
    // step are taken and the call waits for them.
    std::string advance(double dt, int report) {
        std::string e = one_step(dt, report);
        if (!e.empty()) return e;
        return report ? finish_call() : std::string();
    }
    std::string sync() { return finish_call(); }
    // One step enqueued on the engine stream, not waited for; report != 0
    // computes the step's energies and x/v/F snapshot.
    std::string launch_step(double dt, int report) { return one_step(dt, report); }
    // Enqueues, behind the work already on the engine stream, copies of the
    // last report step's snapshot (x, v, F in original atom order, 3N
    // doubles each), the raw energy accumulators (energy_words() fixed-point
    // words) and the device flags (8 ints) into caller-owned pinned host
    // buffers, then records `done`.  Nothing waits.
    std::string enqueue_report(double *x, double *v, double *f, long long *E, int *flags, cudaEvent_t done);
    // Pipelined stepping: a ring of pinned host slots owned by the engine,
    // each holding one report step's positions (original order, 3N
    // doubles), energy words and flags, filled by copies on the engine
    // stream.  step_async enqueues nsteps steps (the last a report step) and
    // the copies into the next free slot and returns; frame_wait waits for
    // the oldest filled slot and hands out its positions (valid until that
    // slot is filled again) and the energies of the first n_out systems.
    std::string frames_init(int depth);
    std::string step_async(int nsteps, double dt);
    std::string frame_wait(const double **xyz, nxm_energies *out, int n_out);
    int energy_words() const { return (int)energies_.size(); }
    // Energies of system s from accumulators copied by enqueue_report.
    void energies_from(const long long *raw, int s, nxm_energies *out) const;
    // The error a device flags word reports ("" for none).
    static std::string flag_error(int err);
    int device() const { return device_; }
    std::string get_snapshot(double *x, double *v, double *f);
    std::string get_state(double *x, double *v);
    void energies(int sys, nxm_energies *out) const;
    std::string pairs(int sys, std::vector<int> &out);
    // System s's PME grids of the last evaluation, as doubles: the charge
    // grid the spread summed (K0 K1 K2), the influence function on the half
    // spectrum (K0 K1 (K2/2+1)) and the real grid after the convolution and
    // inverse transform (K0 K1 K2); any pointer may be null.
    std::string pme_grids(int s, double *charge, double *influence, double *potential);
    // Device milliseconds of nsteps steps (report != 0: every step computes
    // energies and the snapshot, as a reporting loop's steps do).
    std::string time_steps(int nsteps, double dt, double *ms, int report = 0);
    std::string profile(int nsteps, double dt, double *ms);
    int n_total() const { return N_; }
    int n_systems() const { return (int)sysh_.size(); }
    const SysHost &sys(int s) const { return sysh_[s]; }
    int launches_per_step() const { return launches_per_step_; }
    int launches_per_rebuild() const { return launches_per_rebuild_; }
    const int *tuning() const { return tune_; }
    // threads per plane-path FFT block, 0 on the line path
    int fft_plane_threads() const { return plan_.plane ? plan_.plane_threads : 0; }
    // System s's layout: [0] cells per group, [1] neighbourhood capacity
    // (atoms), [2..4] cells per axis, [5] list stride, [6] FFT path in use
    // (1 lines, 2 planes), [7] 1 when the plane path works through a plane in
    // chunks of lines, [8..10] FFT passes per axis.
    void layout(int s, int out[kLayoutWords]) const;
    // Radices of system s's FFT passes along axis d (count returned, at most
    // cap written).
    int fft_radices(int s, int d, int *out, int cap) const;
    // Host wall milliseconds of context creation: [0] host set-up (box,
    // constants, exclusions), [1] device allocation and uploads, [2] PME
    // tables and FFT plan, [3] autotuning (0 when skipped or cached),
    // [4] step-graph builds so far, [5] creation total ([0]..[3]); of [1]:
    // [6] cudaMalloc and zeroing, [7] host-to-device copies; [8] the
    // exclusion sets, built on a host thread alongside [1].
    const double *create_ms() const { return create_ms_; }
    // 1 when the launch shapes came from an earlier context of the same shapes
    int autotune_cached() const { return autotune_cached_; }
    // neighbour-list rebuilds since creation, as of the last finished call
    long long rebuild_count() const { return h_flags_ ? reinterpret_cast<const Flags *>(h_flags_)->nrebuild : 0; }

private:
    // One step as a CUDA graph: energy reset (report steps), the list
    // decision, a conditional node whose body is the rebuild sequence (run
    // only when the decision kernel sets it), the force kernels and the
    // update.  One graph per report flag, rebuilt when dt changes.
    struct StepGraph {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        double dt = 0.0;
        bool ok = false;
    };
    // report kinds: 0 none, 1 energies and the x/v/F snapshot, 2 / 3 a
    // frame (energies and positions) into frame buffer A / B
    StepGraph graph_[4];
    // Launch shapes tuned at set-up: FFT real lines per z-pass block (0 on
    // the plane path), FFT columns per y/x-pass block, threads per
    // spread/gather block.
    int tune_[3] = {0, 8, 128};
    std::string autotune();
    // launch shapes tuned by an earlier context of the same shapes in this
    // process: FFT z lines, columns, plane path, plane threads, PME threads
    bool tune_lookup(int out[5]);
    std::string build_graph(double dt, int report);
    std::string build_graph_timed(double dt, int report);
    void free_graphs();
    std::string one_step(double dt, int report);
    std::string check(const char *what);
    std::string finish_call();
    static void decode_energies(const double *e, const SysHost &H, nxm_energies *out);
    void fetch_energies();

    DevView v_{};
    FftPlan plan_;
    std::vector<SysDev> sysd_;
    std::vector<SysHost> sysh_;
    cudaStream_t st_ = nullptr;
    cudaStream_t st_pme_ = nullptr;  // PME branch of the step graph (captured only)
    cudaEvent_t ev_fork_ = nullptr, ev_join_ = nullptr;
    int N_ = 0;
    int device_ = 0;
    int mixed_ = 1;
    int interval_ = 1;
    int fft_path_ = 0;  // nxm_options::fft_path
    std::vector<int> group_g_;  // cells per group, per system
    double create_ms_[kCreatePhases] = {};
    struct Frame {
        double *x = nullptr;      // pinned, 3N
        long long *E = nullptr;   // pinned, energy words
        int *flags = nullptr;     // pinned, Flags
        cudaEvent_t done = nullptr;
        bool pending = false;
    };
    std::vector<Frame> ring_;
    void *ring_mem_ = nullptr;  // one page-locked block holding every slot
    size_t frame_slot_bytes() const;
    int ring_next_ = 0, ring_pending_ = 0;
    // Frame steps write their energies and positions into one of two device
    // buffers (A, B: report kinds 2, 3), alternately, so the copy of frame k
    // on st_copy_ overlaps step k+1; a buffer is written again only after
    // its copy has finished (buf_free_).
    double *frame_x_[2] = {nullptr, nullptr};
    long long *frame_E_[2] = {nullptr, nullptr};
    cudaEvent_t buf_free_[2] = {nullptr, nullptr}, step_done_ = nullptr;
    bool buf_used_[2] = {false, false};
    int frame_buf_ = 0;
    cudaStream_t st_copy_ = nullptr;
    void free_frames();
    // the device view a step of report kind `kind` runs with
    DevView view_for(int kind) const;
    int autotune_cached_ = 0;
    bool force_rebuild_ = true;
    int since_rebuild_ = 0;
    std::vector<void *> allocs_;
    // bump allocation of the engine's many small device arrays out of a few
    // zeroed chunks (one cudaMalloc and one memset per chunk, not per array)
    char *arena_ptr_ = nullptr;
    size_t arena_left_ = 0;
    bool alloc_failed_ = false;
    std::vector<double> energies_;  // [S][E_SLOTS] decoded
    long long *h_E_ = nullptr;       // pinned
    int *h_flags_ = nullptr;         // pinned
    int *h_tail_ = nullptr;          // pinned: the exclusion build's totals
    cudaEvent_t ev_setup_ = nullptr; // the set-up's point where those totals are in host memory
    // state uploads: staging buffer (3N doubles) and its events
    double *stage3_ = nullptr;
    cudaEvent_t ev_staged_ = nullptr, ev_stage_free_ = nullptr;
    bool stage_used_ = false;
    std::string stage_state(const double *xyz, double *dx, double *dy, double *dz);
    int launches_per_step_ = 0, launches_per_rebuild_ = 0;
    template <typename T>
    T *dalloc(size_t n);
    char *chunk(size_t bytes);
    cudaStream_t kst();
    bool uploads_pending_ = false;   // set-up uploads on the copy stream the compute stream has not joined
    cudaEvent_t ev_uploaded_ = nullptr;
    void arena_reserve(size_t bytes);
};

void launch_export(const DevView &v, int with_forces, cudaStream_t st);
void launch_decide_rebuild(const DevView &v, int force, cudaStream_t st);

template <typename F>
std::string Engine::run_reporting(int nsteps, double dt, int interval, F on_report) {
    for (int step = 0; step < nsteps; ++step) {
        int report = (((step + 1) % interval) == 0) || step == 0;
        std::string e = one_step(dt, report);
        if (!e.empty()) return e;
        if (report) {
            e = finish_call();
            if (!e.empty()) return e;
            if (!on_report(step)) return "report callback failed";
        }
    }
    return finish_call();
}

}  // namespace nxm
