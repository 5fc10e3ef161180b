// Asynchronous reporter: pinned double-buffered snapshot copies, files
// formatted and written on a host thread.
#include "nxm_report.h"

#include <algorithm>

namespace nxm {

AsyncReporter::AsyncReporter(Engine &eng, ReportWriter &rep, int n_atoms, int format_threads)
    : eng_(eng), rep_(rep), n_(n_atoms), threads_(std::max(1, format_threads)) {}

std::string AsyncReporter::init() {
    size_t b = sizeof(double) * 3 * (size_t)n_;
    for (Slot &s : slot_) {
        if (cudaMallocHost(&s.x, b) != cudaSuccess || cudaMallocHost(&s.v, b) != cudaSuccess ||
            cudaMallocHost(&s.f, b) != cudaSuccess ||
            cudaMallocHost(&s.E, sizeof(long long) * std::max(1, eng_.energy_words())) != cudaSuccess ||
            cudaMallocHost(&s.flags, 8 * sizeof(int)) != cudaSuccess)
            return "pinned host allocation failed (reporter)";
        if (cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming) != cudaSuccess)
            return "event creation failed (reporter)";
    }
    th_ = std::thread(&AsyncReporter::run, this);
    return "";
}

AsyncReporter::~AsyncReporter() {
    {
        std::lock_guard<std::mutex> lk(mu_);
        stop_ = true;
    }
    cv_.notify_all();
    if (th_.joinable()) th_.join();
    for (Slot &s : slot_) {
        if (s.x) cudaFreeHost(s.x);
        if (s.v) cudaFreeHost(s.v);
        if (s.f) cudaFreeHost(s.f);
        if (s.E) cudaFreeHost(s.E);
        if (s.flags) cudaFreeHost(s.flags);
        if (s.done) cudaEventDestroy(s.done);
    }
}

std::string AsyncReporter::submit(int step, int model) {
    std::unique_lock<std::mutex> lk(mu_);
    Slot &s = slot_[next_];
    cv_.wait(lk, [&] { return !s.busy || !err_.empty(); });
    if (!err_.empty()) return err_;
    s.busy = true;
    s.step = step;
    s.model = model;
    lk.unlock();
    std::string e = eng_.enqueue_report(s.x, s.v, s.f, s.E, s.flags, s.done);
    lk.lock();
    if (!e.empty()) {
        s.busy = false;
        return e;
    }
    queue_.push_back(next_);
    next_ = (next_ + 1) % kSlots;
    cv_.notify_all();
    return "";
}

std::string AsyncReporter::drain() {
    std::unique_lock<std::mutex> lk(mu_);
    cv_.wait(lk, [&] {
        if (!queue_.empty()) return false;
        for (const Slot &s : slot_)
            if (s.busy) return false;
        return true;
    });
    return err_;
}

void AsyncReporter::run() {
    cudaSetDevice(eng_.device());
    for (;;) {
        int k;
        {
            std::unique_lock<std::mutex> lk(mu_);
            cv_.wait(lk, [&] { return stop_ || !queue_.empty(); });
            if (queue_.empty()) return;
            k = queue_.front();
            queue_.pop_front();
        }
        Slot &s = slot_[k];
        std::string e;
        cudaError_t ce = cudaEventSynchronize(s.done);
        if (ce != cudaSuccess)
            e = std::string("device: ") + cudaGetErrorString(ce);
        else
            e = Engine::flag_error(s.flags[0]);
        if (e.empty()) {
            // Engine::Report (Engine.cpp:117-160) order: PDB, TotalEnergy, PVF
            nxm_energies E;
            eng_.energies_from(s.E, 0, &E);
            double pe = E.reported_potential, ke = E.kinetic;
            if (s.step == 0) rep_.pdb_part1();
            rep_.pdb_part2(s.x, s.model, false);
            rep_.total_energy(ke, pe, pe + ke, s.step);
            rep_.pvf(s.x, s.v, s.f, n_, s.step, threads_);
        }
        {
            std::lock_guard<std::mutex> lk(mu_);
            if (!e.empty() && err_.empty()) err_ = e;
            s.busy = false;
        }
        cv_.notify_all();
    }
}

}  // namespace nxm
