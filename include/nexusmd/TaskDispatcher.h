// C++ interface of the NexusMD dispatcher, backed by the CUDA engine.
//
// Same shape as the reference's class (core/dispatcher/headers/
// TaskDispatcher.h:9-43): a factory, four Enable*Force switches and Simulate,
// which reads the OpenMM-style system/state XML and writes PVFReport<out>,
// TotalEnergy<out> and the <out> PDB trajectory.  CreateDispatcher("GPU") or
// ("CUDA") returns the CUDA dispatcher; any other string prints the
// reference's complaint and returns it too (there is no CPU engine here).
// Errors throw std::runtime_error, as the reference's do.
#pragma once

#include <memory>
#include <string>

#include "../nxm.h"

class TaskDispatcher {
public:
    virtual void Simulate(const std::string &systemFilename, const std::string &stateFilename,
                          const std::string &inputFilename, const std::string &outputFilename, double StepSize,
                          int TotalSteps, int interval) = 0;
    virtual ~TaskDispatcher() = default;

    static std::shared_ptr<TaskDispatcher> CreateDispatcher(const std::string &processorChoice);

    void EnableHarmonicBondForce() { harmonicBondForceEnabled = true; }
    void EnableHarmonicAngleForce() { harmonicAngleForceEnabled = true; }
    void EnablePeriodicTorsionForce() { periodicTorsionForceEnabled = true; }
    void EnableNonbondedForce() { nonbondedForceEnabled = true; }

    // Engine settings the reference hard-codes: precision, list skin and
    // rebuild interval, device (defaults: mixed precision, 0.1 nm, 10, 0).
    void SetOptions(const nxm_options &opt) {
        options = opt;
        have_options = true;
    }

protected:
    bool harmonicBondForceEnabled = false;
    bool harmonicAngleForceEnabled = false;
    bool periodicTorsionForceEnabled = false;
    bool nonbondedForceEnabled = false;
    nxm_options options{};
    bool have_options = false;
};
