// extern "C" entry points of libnxm_cuda.so for the engine (include/nxm.h).
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/nxm.h"
#include "nxm_engine.h"
#include "nxm_io.h"

struct nxm_ctx {
    nxm::Engine eng;
};

namespace nxm {
thread_local std::string g_last_error;
int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}
}  // namespace nxm

using nxm::fail;

extern "C" {

const char *nxm_version(void) { return "nexusmd-gb300 0.1 (sm_103a)"; }

const char *nxm_last_error(void) { return nxm::g_last_error.c_str(); }

void nxm_default_options(nxm_options *opt) {
    if (!opt) return;
    std::memset(opt, 0, sizeof(*opt));
    opt->precision = NXM_PRECISION_MIXED;
    opt->skin = 0.1;
    opt->rebuild_interval = 10;
    opt->device = 0;
    opt->max_neighbors = 0;
    opt->exceptions = 0;
    opt->autotune = 1;
    opt->report_threads = 4;
    opt->state_velocities = 0;
    opt->fft_path = 0;
}

static int code_for(const std::string &e) {
    if (e.find("capacity") != std::string::npos) return NXM_ERR_CAPACITY;
    if (e.find("non-finite") != std::string::npos) return NXM_ERR_NUMERIC;
    if (e.find("device") != std::string::npos || e.find("CUDA") != std::string::npos) return NXM_ERR_CUDA;
    return NXM_ERR_INVALID;
}

int nxm_create(const nxm_system_desc *systems, int32_t n_systems, const nxm_options *opt,
               const double *positions, nxm_ctx **out) {
    if (!systems || n_systems <= 0 || !positions || !out) return fail(NXM_ERR_INVALID, "nxm_create: null argument");
    *out = nullptr;
    nxm_options o;
    nxm_default_options(&o);
    if (opt) o = *opt;
    std::vector<nxm::HostSystem> hs(n_systems);
    for (int s = 0; s < n_systems; ++s) {
        const nxm_system_desc &d = systems[s];
        nxm::HostSystem &h = hs[s];
        if (d.n_atoms <= 0 || !d.masses || !d.charges || !d.sigmas || !d.epsilons)
            return fail(NXM_ERR_INVALID, "nxm_create: system needs atoms, masses and nonbonded parameters");
        if ((d.n_bonds > 0 && (!d.bond_atoms || !d.bond_params)) ||
            (d.n_angles > 0 && (!d.angle_atoms || !d.angle_params)) ||
            (d.n_torsions > 0 && (!d.torsion_atoms || !d.torsion_params || !d.torsion_periodicity)))
            return fail(NXM_ERR_INVALID, "nxm_create: term count without arrays");
        int n = d.n_atoms;
        h.n = n;
        // the caller's arrays, read in place during the creation
        h.mass = {d.masses, (size_t)n};
        h.q = {d.charges, (size_t)n};
        h.sig = {d.sigmas, (size_t)n};
        h.eps = {d.epsilons, (size_t)n};
        if (d.n_bonds > 0) {
            h.bonds = {d.bond_atoms, 2 * (size_t)d.n_bonds};
            h.bprm = {d.bond_params, 2 * (size_t)d.n_bonds};
        }
        if (d.n_angles > 0) {
            h.angles = {d.angle_atoms, 3 * (size_t)d.n_angles};
            h.aprm = {d.angle_params, 2 * (size_t)d.n_angles};
        }
        if (d.n_torsions > 0) {
            h.torsions = {d.torsion_atoms, 4 * (size_t)d.n_torsions};
            h.tprm = {d.torsion_params, 2 * (size_t)d.n_torsions};
            h.tper = {d.torsion_periodicity, (size_t)d.n_torsions};
        }
        h.cutoff = d.cutoff;
        h.tol = d.ewald_tolerance;
        h.use_switch = d.use_switching;
        h.sw_dist = d.switching_distance;
        for (int k = 0; k < 3; ++k) {
            h.grid[k] = d.grid[k];
            h.lb[k] = d.box_lb[k];
            h.ub[k] = d.box_ub[k];
        }
        h.box_from_positions = d.box_from_positions;
        h.force_mask = d.force_mask;
        h.excl_depth = d.exclusion_depth;
        if (d.n_exceptions < 0 || (d.n_exceptions > 0 && (!d.exception_atoms || !d.exception_params)))
            return fail(NXM_ERR_INVALID, "nxm_create: exception count without arrays");
        if (d.n_exceptions > 0) {
            h.exc = {d.exception_atoms, 2 * (size_t)d.n_exceptions};
            h.exc_prm = {d.exception_params, 3 * (size_t)d.n_exceptions};
        }
    }
    nxm_ctx *c = new (std::nothrow) nxm_ctx;
    if (!c) return fail(NXM_ERR_INVALID, "out of host memory");
    std::string e = c->eng.init(hs, o, positions);
    if (!e.empty()) {
        delete c;
        return fail(code_for(e), "nxm_create: " + e);
    }
    *out = c;
    return NXM_OK;
}

void nxm_destroy(nxm_ctx *ctx) { delete ctx; }

int nxm_n_atoms(const nxm_ctx *ctx, int32_t *n) {
    if (!ctx || !n) return fail(NXM_ERR_INVALID, "null argument");
    *n = ctx->eng.n_total();
    return NXM_OK;
}

#define NXM_CALL(expr)                                          \
    do {                                                        \
        std::string e_ = (expr);                                \
        if (!e_.empty()) return fail(code_for(e_), e_);         \
        return NXM_OK;                                          \
    } while (0)

int nxm_set_positions(nxm_ctx *ctx, const double *xyz) {
    if (!ctx || !xyz) return fail(NXM_ERR_INVALID, "null argument");
    NXM_CALL(ctx->eng.set_positions(xyz));
}

int nxm_set_velocities(nxm_ctx *ctx, const double *xyz) {
    if (!ctx || !xyz) return fail(NXM_ERR_INVALID, "null argument");
    NXM_CALL(ctx->eng.set_velocities(xyz));
}

int nxm_compute_forces(nxm_ctx *ctx) {
    if (!ctx) return fail(NXM_ERR_INVALID, "null argument");
    NXM_CALL(ctx->eng.compute_forces());
}

int nxm_step(nxm_ctx *ctx, int32_t nsteps, double dt) {
    if (!ctx || nsteps < 0) return fail(NXM_ERR_INVALID, "bad argument");
    if (nsteps == 0) return NXM_OK;
    NXM_CALL(ctx->eng.step(nsteps, dt));
}

int nxm_get_positions(nxm_ctx *ctx, double *xyz) {
    if (!ctx || !xyz) return fail(NXM_ERR_INVALID, "null argument");
    NXM_CALL(ctx->eng.get_snapshot(xyz, nullptr, nullptr));
}

int nxm_get_velocities(nxm_ctx *ctx, double *xyz) {
    if (!ctx || !xyz) return fail(NXM_ERR_INVALID, "null argument");
    NXM_CALL(ctx->eng.get_snapshot(nullptr, xyz, nullptr));
}

int nxm_get_forces(nxm_ctx *ctx, double *xyz) {
    if (!ctx || !xyz) return fail(NXM_ERR_INVALID, "null argument");
    NXM_CALL(ctx->eng.get_snapshot(nullptr, nullptr, xyz));
}

int nxm_get_state(nxm_ctx *ctx, double *xyz, double *vel) {
    if (!ctx) return fail(NXM_ERR_INVALID, "null argument");
    NXM_CALL(ctx->eng.get_state(xyz, vel));
}

int nxm_save_state(nxm_ctx *ctx, int32_t system, const char *path, int64_t step, double time_ps) {
    if (!ctx || !path || system < 0 || system >= ctx->eng.n_systems()) return fail(NXM_ERR_INVALID, "bad argument");
    int n = ctx->eng.n_total();
    std::vector<double> x(3 * (size_t)n), v(3 * (size_t)n);
    std::string e = ctx->eng.get_state(x.data(), v.data());
    if (!e.empty()) return fail(code_for(e), e);
    const nxm::SysHost &h = ctx->eng.sys(system);
    double box[3] = {h.L[0], h.L[1], h.L[2]};
    size_t o = 3 * (size_t)h.atom_off;
    if (!nxm::write_state_xml(path, h.natoms, x.data() + o, v.data() + o, box, (long long)step, time_ps))
        return fail(NXM_ERR_IO, std::string("cannot write ") + path);
    return NXM_OK;
}

int nxm_get_energies(nxm_ctx *ctx, int32_t system, nxm_energies *out) {
    if (!ctx || !out || system < 0 || system >= ctx->eng.n_systems()) return fail(NXM_ERR_INVALID, "bad argument");
    ctx->eng.energies(system, out);
    return NXM_OK;
}

int nxm_get_box(nxm_ctx *ctx, int32_t system, double lb[3], double ub[3]) {
    if (!ctx || system < 0 || system >= ctx->eng.n_systems()) return fail(NXM_ERR_INVALID, "bad argument");
    const nxm::SysHost &h = ctx->eng.sys(system);
    for (int d = 0; d < 3; ++d) {
        if (lb) lb[d] = h.lb[d];
        if (ub) ub[d] = h.ub[d];
    }
    return NXM_OK;
}

int nxm_get_grid(nxm_ctx *ctx, int32_t system, int32_t grid[3]) {
    if (!ctx || !grid || system < 0 || system >= ctx->eng.n_systems()) return fail(NXM_ERR_INVALID, "bad argument");
    for (int d = 0; d < 3; ++d) grid[d] = ctx->eng.sys(system).K[d];
    return NXM_OK;
}

int nxm_get_alpha(nxm_ctx *ctx, int32_t system, double *alpha) {
    if (!ctx || !alpha || system < 0 || system >= ctx->eng.n_systems()) return fail(NXM_ERR_INVALID, "bad argument");
    *alpha = ctx->eng.sys(system).alpha;
    return NXM_OK;
}

int64_t nxm_get_pairs(nxm_ctx *ctx, int32_t system, int32_t *pairs, int64_t cap) {
    if (!ctx || system < 0 || system >= ctx->eng.n_systems() || cap < 0 || (cap > 0 && !pairs))
        return fail(NXM_ERR_INVALID, "bad argument");
    std::vector<int> p;
    std::string e = ctx->eng.pairs(system, p);
    if (!e.empty()) return fail(code_for(e), e);
    int64_t n = (int64_t)p.size() / 2;
    int64_t w = n < cap ? n : cap;
    if (w > 0) std::memcpy(pairs, p.data(), sizeof(int32_t) * 2 * (size_t)w);
    return n;
}

int nxm_time_steps(nxm_ctx *ctx, int32_t nsteps, double dt, double *ms) {
    if (!ctx || !ms || nsteps <= 0) return fail(NXM_ERR_INVALID, "bad argument");
    NXM_CALL(ctx->eng.time_steps(nsteps, dt, ms));
}

int nxm_time_report_steps(nxm_ctx *ctx, int32_t nsteps, double dt, double *ms) {
    if (!ctx || !ms || nsteps <= 0) return fail(NXM_ERR_INVALID, "bad argument");
    NXM_CALL(ctx->eng.time_steps(nsteps, dt, ms, 1));
}

int nxm_profile_phases(nxm_ctx *ctx, int32_t nsteps, double dt, double *ms, int32_t cap) {
    if (!ctx || !ms || nsteps <= 0 || cap < nxm::kProfilePhases) return fail(NXM_ERR_INVALID, "bad argument");
    NXM_CALL(ctx->eng.profile(nsteps, dt, ms));
}

int nxm_get_tuning(nxm_ctx *ctx, int32_t out[3]) {
    if (!ctx || !out) return fail(NXM_ERR_INVALID, "null argument");
    const int *t = ctx->eng.tuning();
    for (int k = 0; k < 3; ++k) out[k] = t[k];
    return NXM_OK;
}

int nxm_get_fft_plane_threads(nxm_ctx *ctx, int32_t *threads) {
    if (!ctx || !threads) return fail(NXM_ERR_INVALID, "null argument");
    *threads = ctx->eng.fft_plane_threads();
    return NXM_OK;
}

int nxm_frames_init(nxm_ctx *ctx, int32_t depth) {
    if (!ctx) return fail(NXM_ERR_INVALID, "null argument");
    NXM_CALL(ctx->eng.frames_init(depth));
}

int nxm_step_async(nxm_ctx *ctx, int32_t nsteps, double dt) {
    if (!ctx || nsteps <= 0) return fail(NXM_ERR_INVALID, "bad argument");
    NXM_CALL(ctx->eng.step_async(nsteps, dt));
}

int nxm_frame_wait(nxm_ctx *ctx, const double **xyz, nxm_energies *energies, int32_t n_systems) {
    if (!ctx || n_systems < 0 || (n_systems > 0 && !energies)) return fail(NXM_ERR_INVALID, "bad argument");
    NXM_CALL(ctx->eng.frame_wait(xyz, energies, n_systems));
}

int nxm_get_create_timing(nxm_ctx *ctx, double ms[9], int32_t *autotune_cached) {
    if (!ctx || !ms) return fail(NXM_ERR_INVALID, "null argument");
    const double *c = ctx->eng.create_ms();
    for (int k = 0; k < nxm::kCreatePhases; ++k) ms[k] = c[k];
    if (autotune_cached) *autotune_cached = ctx->eng.autotune_cached();
    return NXM_OK;
}

int nxm_get_pme_grids(nxm_ctx *ctx, int32_t system, double *charge, double *influence, double *potential) {
    if (!ctx || system < 0 || system >= ctx->eng.n_systems()) return fail(NXM_ERR_INVALID, "bad argument");
    NXM_CALL(ctx->eng.pme_grids(system, charge, influence, potential));
}

int nxm_get_layout(nxm_ctx *ctx, int32_t system, int32_t out[11]) {
    if (!ctx || !out || system < 0 || system >= ctx->eng.n_systems()) return fail(NXM_ERR_INVALID, "bad argument");
    int w[nxm::kLayoutWords];
    ctx->eng.layout(system, w);
    for (int k = 0; k < nxm::kLayoutWords; ++k) out[k] = w[k];
    return NXM_OK;
}

int nxm_get_fft_radices(nxm_ctx *ctx, int32_t system, int32_t axis, int32_t *radices, int32_t cap) {
    if (!ctx || system < 0 || system >= ctx->eng.n_systems() || axis < 0 || axis > 2 || cap < 0 ||
        (cap > 0 && !radices))
        return fail(NXM_ERR_INVALID, "bad argument");
    int r[nxm::kMaxPasses];
    int np = ctx->eng.fft_radices(system, axis, r, nxm::kMaxPasses);
    for (int p = 0; p < np && p < cap; ++p) radices[p] = r[p];
    return np;
}

int nxm_rebuild_count(nxm_ctx *ctx, int64_t *count) {
    if (!ctx || !count) return fail(NXM_ERR_INVALID, "null argument");
    std::string e = ctx->eng.sync();
    if (!e.empty()) return fail(code_for(e), e);
    *count = ctx->eng.rebuild_count();
    return NXM_OK;
}

int nxm_launches_per_step(nxm_ctx *ctx, int32_t *launches, int32_t *rebuild_launches) {
    if (!ctx) return fail(NXM_ERR_INVALID, "null argument");
    if (launches) *launches = ctx->eng.launches_per_step();
    if (rebuild_launches) *rebuild_launches = ctx->eng.launches_per_rebuild();
    return NXM_OK;
}

}  // extern "C"
