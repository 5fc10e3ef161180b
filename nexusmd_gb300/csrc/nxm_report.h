// Report files written behind the step loop (Reporter.cpp:26-229 formats,
// Engine::Report schedule, Engine.cpp:117-160).
//
// At a report step the step's snapshot (x, v, F), its raw energy
// accumulators and the device flags are copied on the engine stream into one
// of two pinned host buffer sets, after the step's kernels and before the
// next step's.  A writer thread waits for that copy's event, formats the
// three files (the PVF lines over several threads) and hands the set back.
// The step loop waits only when both sets are still being written, so the
// GPU keeps stepping while the host formats.  The files are byte-identical
// to those of the synchronous loop.
#pragma once

#include <cuda_runtime.h>

#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>

#include "nxm_engine.h"
#include "nxm_io.h"

namespace nxm {

class AsyncReporter {
public:
    AsyncReporter(Engine &eng, ReportWriter &rep, int n_atoms, int format_threads);
    ~AsyncReporter();
    // Pinned buffers, events and the writer thread; "" on success.
    std::string init();
    // After eng.launch_step(dt, 1) of `step`: queue its report (`model` is
    // the PDB model number).  Returns the first error met so far.
    std::string submit(int step, int model);
    // Waits until every queued report is written; the first error, if any.
    std::string drain();

private:
    struct Slot {
        double *x = nullptr, *v = nullptr, *f = nullptr;
        long long *E = nullptr;
        int *flags = nullptr;
        cudaEvent_t done = nullptr;
        int step = 0, model = 0;
        bool busy = false;
    };
    static constexpr int kSlots = 2;
    void run();

    Engine &eng_;
    ReportWriter &rep_;
    int n_, threads_;
    Slot slot_[kSlots];
    int next_ = 0;
    std::deque<int> queue_;
    std::mutex mu_;
    std::condition_variable cv_;
    std::string err_;
    bool stop_ = false;
    std::thread th_;
};

}  // namespace nxm
