// TaskDispatcher on the CUDA engine, and the C ABI of the dispatcher and of
// the XML readers.
//
// Simulate follows BaseLineTaskDispatcher::Simulate
// (core/dispatcher/headers/BaseLineTaskDispatcher.h:12-40) and
// Engine::RunSimulation / Engine::Report (core/baseline/src/Engine.cpp:117-188):
// parse the inputs, box from the atom extent, velocities zero, exclusions
// from the bonds (three bonds deep), then per step CalculateForces -> Report
// on step 0 and every `interval`-th step -> Integrate.  With report_threads
// > 0 the report files are written by a host thread from pinned copies of
// the report step's snapshot while the GPU steps on (nxm_report.h); the
// bytes are those of the synchronous loop.  state_velocities = 1 starts from
// the state file's <Velocities> instead of zero.
#include <cstring>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/nexusmd/TaskDispatcher.h"
#include "nxm_engine.h"
#include "nxm_io.h"
#include "nxm_report.h"

namespace nxm {
extern thread_local std::string g_last_error;
int fail(int code, const std::string &msg);
}  // namespace nxm

namespace {

class CudaTaskDispatcher : public TaskDispatcher {
public:
    void Simulate(const std::string &systemFilename, const std::string &stateFilename,
                  const std::string &inputFilename, const std::string &outputFilename, double StepSize,
                  int TotalSteps, int interval) override {
        if (harmonicBondForceEnabled) std::cout << "Harmonic Bond Force is enabled" << std::endl;
        if (harmonicAngleForceEnabled) std::cout << "Harmonic Angle Force is enabled" << std::endl;
        if (periodicTorsionForceEnabled) std::cout << "Periodic Torsion Force is enabled" << std::endl;
        if (nonbondedForceEnabled) std::cout << "Nonbonded Force is enabled" << std::endl;
        if (interval <= 0) throw std::runtime_error("Simulate: interval must be positive");
        nxm::ParsedSystem ps = nxm::parse_all(systemFilename, stateFilename);
        if (ps.positions.empty()) throw std::runtime_error("No atom positions available to extract boundaries.");
        int n = (int)(ps.positions.size() / 3);
        nxm::HostSystem h;
        h.n = n;
        // the arrays the engine reads during its creation
        std::vector<double> mass = ps.masses, q(n, 0.0), sig(n, 0.0), eps(n, 0.0), bprm, aprm, tprm, exc_prm;
        std::vector<int> bonds, angles, torsions, tper, exc;
        mass.resize(n, 0.0);
        if (nonbondedForceEnabled) {
            if ((int)ps.nb.particles.size() < n)
                throw std::runtime_error("NonbondedForce has fewer particles than the state has positions");
            for (int i = 0; i < n; ++i) {
                q[i] = ps.nb.particles[i].q;
                sig[i] = ps.nb.particles[i].sig;
                eps[i] = ps.nb.particles[i].eps;
            }
            h.cutoff = ps.nb.cutoff;
            h.tol = ps.nb.ewaldTolerance;
            h.use_switch = ps.nb.useSwitchingFunction;
            h.sw_dist = ps.nb.switchingDistance;
        }
        for (auto &b : ps.bonds) {
            bonds.push_back(b.p1);
            bonds.push_back(b.p2);
            bprm.push_back(b.d);
            bprm.push_back(b.k);
        }
        for (auto &a : ps.angles) {
            angles.insert(angles.end(), {a.p1, a.p2, a.p3});
            aprm.push_back(a.a);
            aprm.push_back(a.k);
        }
        for (auto &t : ps.torsions) {
            torsions.insert(torsions.end(), {t.p1, t.p2, t.p3, t.p4});
            tprm.push_back(t.k);
            tprm.push_back(t.phase);
            tper.push_back(t.periodicity);
        }
        h.force_mask = (harmonicBondForceEnabled ? NXM_FORCE_BOND : 0) | (harmonicAngleForceEnabled ? NXM_FORCE_ANGLE : 0) |
                       (periodicTorsionForceEnabled ? NXM_FORCE_TORSION : 0) |
                       (nonbondedForceEnabled ? NXM_FORCE_NONBONDED : 0);
        h.box_from_positions = 1;
        h.excl_depth = 3;  // Engine.h:58
        nxm_options opt;
        nxm_default_options(&opt);
        if (have_options) opt = options;
        if (opt.exceptions && nonbondedForceEnabled) {
            // <Exceptions> of the system XML in OpenMM semantics (the reference ignores them)
            for (auto &x : ps.nb.exceptions) {
                exc.push_back(x.p1);
                exc.push_back(x.p2);
                exc_prm.insert(exc_prm.end(), {x.q, x.sig, x.eps});
            }
        }
        h.mass = mass;
        h.q = q;
        h.sig = sig;
        h.eps = eps;
        h.bonds = bonds;
        h.bprm = bprm;
        h.angles = angles;
        h.aprm = aprm;
        h.torsions = torsions;
        h.tprm = tprm;
        h.tper = tper;
        h.exc = exc;
        h.exc_prm = exc_prm;
        auto eng = std::make_unique<nxm::Engine>();
        std::string err = eng->init({h}, opt, ps.positions.data());
        if (!err.empty()) throw std::runtime_error(err);
        if (opt.state_velocities && ps.velocities.size() == ps.positions.size()) {
            err = eng->set_velocities(ps.velocities.data());
            if (!err.empty()) throw std::runtime_error(err);
        }

        nxm::ReportWriter rep(inputFilename, outputFilename);
        if (opt.report_threads > 0) {
            // reports written by a host thread while the GPU steps on
            nxm::AsyncReporter ar(*eng, rep, n, opt.report_threads);
            err = ar.init();
            if (!err.empty()) throw std::runtime_error(err);
            for (int step = 0; step < TotalSteps; ++step) {
                int report = (((step + 1) % interval) == 0) || step == 0;
                err = eng->launch_step(StepSize, report);
                if (!err.empty()) throw std::runtime_error(err);
                if (report) {
                    int model = (step + 1) / interval;
                    std::cout << model << "   ";
                    err = ar.submit(step, model);
                    if (!err.empty()) throw std::runtime_error(err);
                }
                std::cout << "Simulation Step #" << step + 1 << " is completed" << std::endl;
            }
            err = ar.drain();
            if (!err.empty()) throw std::runtime_error(err);
            err = eng->sync();
            if (!err.empty()) throw std::runtime_error(err);
            return;
        }
        std::vector<double> x(3 * (size_t)n), v(3 * (size_t)n), f(3 * (size_t)n);
        for (int step = 0; step < TotalSteps; ++step) {
            int report = (((step + 1) % interval) == 0) || step == 0;
            err = eng->advance(StepSize, report);
            if (!err.empty()) throw std::runtime_error(err);
            if (report) {
                err = eng->get_snapshot(x.data(), v.data(), f.data());
                if (!err.empty()) throw std::runtime_error(err);
                nxm_energies E;
                eng->energies(0, &E);
                double pe = E.reported_potential, ke = E.kinetic;
                int model = (step + 1) / interval;
                if (step == 0) rep.pdb_part1();
                rep.pdb_part2(x.data(), model);
                rep.total_energy(ke, pe, pe + ke, step);
                rep.pvf(x.data(), v.data(), f.data(), n, step);
            }
            std::cout << "Simulation Step #" << step + 1 << " is completed" << std::endl;
        }
        err = eng->sync();
        if (!err.empty()) throw std::runtime_error(err);
    }
};

}  // namespace

std::shared_ptr<TaskDispatcher> TaskDispatcher::CreateDispatcher(const std::string &processorChoice) {
    if (processorChoice != "GPU" && processorChoice != "CUDA")
        std::cerr << "Invalid processor type. Defaulting to GPU." << std::endl;
    return std::make_shared<CudaTaskDispatcher>();
}

// ------------------------------------------------------------------ C ABI

struct nxm_dispatcher {
    std::shared_ptr<TaskDispatcher> d;
};

struct nxm_parsed {
    nxm::ParsedSystem ps;
};

using nxm::fail;

extern "C" {

int nxm_dispatcher_create(const char *processor, nxm_dispatcher **out) {
    if (!out) return fail(NXM_ERR_INVALID, "null argument");
    *out = new nxm_dispatcher{TaskDispatcher::CreateDispatcher(processor ? processor : "")};
    return NXM_OK;
}

void nxm_dispatcher_destroy(nxm_dispatcher *d) { delete d; }

int nxm_dispatcher_enable_harmonic_bond_force(nxm_dispatcher *d) {
    if (!d) return fail(NXM_ERR_INVALID, "null dispatcher");
    d->d->EnableHarmonicBondForce();
    return NXM_OK;
}
int nxm_dispatcher_enable_harmonic_angle_force(nxm_dispatcher *d) {
    if (!d) return fail(NXM_ERR_INVALID, "null dispatcher");
    d->d->EnableHarmonicAngleForce();
    return NXM_OK;
}
int nxm_dispatcher_enable_periodic_torsion_force(nxm_dispatcher *d) {
    if (!d) return fail(NXM_ERR_INVALID, "null dispatcher");
    d->d->EnablePeriodicTorsionForce();
    return NXM_OK;
}
int nxm_dispatcher_enable_nonbonded_force(nxm_dispatcher *d) {
    if (!d) return fail(NXM_ERR_INVALID, "null dispatcher");
    d->d->EnableNonbondedForce();
    return NXM_OK;
}
int nxm_dispatcher_set_options(nxm_dispatcher *d, const nxm_options *opt) {
    if (!d || !opt) return fail(NXM_ERR_INVALID, "null argument");
    d->d->SetOptions(*opt);
    return NXM_OK;
}

int nxm_dispatcher_simulate(nxm_dispatcher *d, const char *system_xml, const char *state_xml, const char *input_pdb,
                            const char *output_pdb, double step_size, int32_t total_steps, int32_t interval) {
    if (!d || !system_xml || !state_xml || !input_pdb || !output_pdb) return fail(NXM_ERR_INVALID, "null argument");
    try {
        d->d->Simulate(system_xml, state_xml, input_pdb, output_pdb, step_size, total_steps, interval);
    } catch (const std::exception &e) {
        std::string m = e.what();
        int code = m.find("CUDA") != std::string::npos || m.find("device") != std::string::npos ? NXM_ERR_CUDA
                                                                                                   : NXM_ERR_INVALID;
        return fail(code, m);
    }
    return NXM_OK;
}

int nxm_parse_files(const char *system_xml, const char *state_xml, nxm_parsed **out) {
    if (!out) return fail(NXM_ERR_INVALID, "null argument");
    auto *p = new nxm_parsed;
    std::string sx = system_xml ? system_xml : "", st = state_xml ? state_xml : "";
    p->ps = nxm::parse_all(sx, st);
    *out = p;
    bool bad = (!sx.empty() && !nxm::xml_ok(sx)) || (!st.empty() && !nxm::xml_ok(st));
    return bad ? fail(NXM_ERR_IO, "input file did not parse") : NXM_OK;
}

void nxm_parsed_free(nxm_parsed *p) { delete p; }

int nxm_parsed_counts(const nxm_parsed *p, int64_t counts[7]) {
    if (!p || !counts) return fail(NXM_ERR_INVALID, "null argument");
    counts[0] = (int64_t)p->ps.masses.size();
    counts[1] = (int64_t)p->ps.positions.size() / 3;
    counts[2] = (int64_t)p->ps.bonds.size();
    counts[3] = (int64_t)p->ps.angles.size();
    counts[4] = (int64_t)p->ps.torsions.size();
    counts[5] = (int64_t)p->ps.nb.particles.size();
    counts[6] = (int64_t)p->ps.nb.exceptions.size();
    return NXM_OK;
}

int nxm_parsed_velocities(const nxm_parsed *p, double *vel, int64_t *n_out) {
    if (!p || !n_out) return fail(NXM_ERR_INVALID, "null argument");
    *n_out = (int64_t)p->ps.velocities.size() / 3;
    if (vel && !p->ps.velocities.empty())
        std::memcpy(vel, p->ps.velocities.data(), sizeof(double) * p->ps.velocities.size());
    return NXM_OK;
}

int nxm_write_state_xml(const char *path, int32_t n_atoms, const double *xyz, const double *vel, const double box[3],
                        int64_t step, double time_ps) {
    if (!path || !xyz || !box || n_atoms < 0) return fail(NXM_ERR_INVALID, "bad argument");
    if (!nxm::write_state_xml(path, n_atoms, xyz, vel, box, (long long)step, time_ps))
        return fail(NXM_ERR_IO, std::string("cannot write ") + path);
    return NXM_OK;
}

int nxm_format_fixed(double x, int32_t prec, int32_t width, char *out, int32_t cap) {
    if (!out || prec < 0 || width < 0 || width > 64) return fail(NXM_ERR_INVALID, "bad argument");
    char buf[nxm::kFixedCharsMax];
    int n = nxm::fixed_chars(x, prec, width, buf);
    if (n + 1 > cap) return fail(NXM_ERR_CAPACITY, "output buffer too small");
    std::memcpy(out, buf, (size_t)n + 1);
    return n;
}

int nxm_parsed_nonbonded(const nxm_parsed *p, double out[11]) {
    if (!p || !out) return fail(NXM_ERR_INVALID, "null argument");
    const nxm::NbParams &n = p->ps.nb;
    double v[11] = {n.cutoff, n.ewaldTolerance, n.switchingDistance, (double)n.useSwitchingFunction, n.alpha,
                    n.rfDielectric, (double)n.nx, (double)n.ny, (double)n.nz, (double)n.method,
                    (double)n.dispersionCorrection};
    std::memcpy(out, v, sizeof v);
    return NXM_OK;
}

int nxm_parsed_arrays(const nxm_parsed *p, double *masses, double *positions, int32_t *bond_atoms,
                      double *bond_params, int32_t *angle_atoms, double *angle_params, int32_t *torsion_atoms,
                      double *torsion_params, int32_t *torsion_per, double *q_sig_eps, int32_t *exception_atoms,
                      double *exception_params) {
    if (!p) return fail(NXM_ERR_INVALID, "null argument");
    const nxm::ParsedSystem &s = p->ps;
    if (masses) std::memcpy(masses, s.masses.data(), sizeof(double) * s.masses.size());
    if (positions) std::memcpy(positions, s.positions.data(), sizeof(double) * s.positions.size());
    for (size_t k = 0; k < s.bonds.size(); ++k) {
        if (bond_atoms) {
            bond_atoms[2 * k] = s.bonds[k].p1;
            bond_atoms[2 * k + 1] = s.bonds[k].p2;
        }
        if (bond_params) {
            bond_params[2 * k] = s.bonds[k].d;
            bond_params[2 * k + 1] = s.bonds[k].k;
        }
    }
    for (size_t k = 0; k < s.angles.size(); ++k) {
        if (angle_atoms) {
            angle_atoms[3 * k] = s.angles[k].p1;
            angle_atoms[3 * k + 1] = s.angles[k].p2;
            angle_atoms[3 * k + 2] = s.angles[k].p3;
        }
        if (angle_params) {
            angle_params[2 * k] = s.angles[k].a;
            angle_params[2 * k + 1] = s.angles[k].k;
        }
    }
    for (size_t k = 0; k < s.torsions.size(); ++k) {
        const nxm::TorsionP &t = s.torsions[k];
        if (torsion_atoms) {
            torsion_atoms[4 * k] = t.p1;
            torsion_atoms[4 * k + 1] = t.p2;
            torsion_atoms[4 * k + 2] = t.p3;
            torsion_atoms[4 * k + 3] = t.p4;
        }
        if (torsion_params) {
            torsion_params[2 * k] = t.k;
            torsion_params[2 * k + 1] = t.phase;
        }
        if (torsion_per) torsion_per[k] = t.periodicity;
    }
    for (size_t k = 0; k < s.nb.particles.size(); ++k)
        if (q_sig_eps) {
            q_sig_eps[3 * k] = s.nb.particles[k].q;
            q_sig_eps[3 * k + 1] = s.nb.particles[k].sig;
            q_sig_eps[3 * k + 2] = s.nb.particles[k].eps;
        }
    for (size_t k = 0; k < s.nb.exceptions.size(); ++k) {
        const nxm::NbException &e = s.nb.exceptions[k];
        if (exception_atoms) {
            exception_atoms[2 * k] = e.p1;
            exception_atoms[2 * k + 1] = e.p2;
        }
        if (exception_params) {
            exception_params[3 * k] = e.q;
            exception_params[3 * k + 1] = e.sig;
            exception_params[3 * k + 2] = e.eps;
        }
    }
    return NXM_OK;
}

}  // extern "C"
