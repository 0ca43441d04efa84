/*
 * gbfwi_reference_shim.h — the in-process binding of libgbfwi.so into the
 * reference's own program (libccy/inv.cu).
 *
 * The reference chooses its solver and filter by integer id (lib/index.h:32-64)
 * and drives them through the virtual members of class Solver
 * (solver/solver.h:7-268) and class Filter (filter/filter.h:3-15). GbSolver and
 * GbFilter implement those members by forwarding to the C ABI (gbfwi.h), so
 * the reference's Misfit (misfit/misfit.h:15-151) and Optimizer
 * (optimizer/optimizer.h) run unchanged on the GB300 kernels: the shim
 * publishes the library's device buffers (traces, adjoint sources, model,
 * kernels) in the reference's public pointers, in the reference's layout.
 *
 * Include it after the reference's own headers (lib/index.h up to
 * filter/gaussian.h), then register the classes in lib/index.h:
 *     module::solver: case 1: return new GbSolver();
 *     module::filter: case 1: return new GbFilter();
 * and link with -lgbfwi. A status other than GB_OK from the library is
 * printed with gb_last_error() (the reference's members return void).
 */
#pragma once

#include <cstdio>
#include <string>
#include <vector>

#include "gbfwi.h"

namespace gbfwi_shim {
inline void report(const char *what, int rc) {
    if (rc != GB_OK) std::fprintf(stderr, "gbfwi: %s failed: %s\n", what, gb_last_error());
}
}  // namespace gbfwi_shim

class GbSolver : public Solver {
    gb_config *gcfg = nullptr;
    gb_solver *gs = nullptr;

    // the library's buffers become the reference's public device pointers
    void publish() {
        out_x = gb_solver_ptr(gs, GB_OUT_X);
        out_y = gb_solver_ptr(gs, GB_OUT_Y);
        out_z = gb_solver_ptr(gs, GB_OUT_Z);
        adstf_x = gb_solver_ptr(gs, GB_ADSTF_X);
        adstf_y = gb_solver_ptr(gs, GB_ADSTF_Y);
        adstf_z = gb_solver_ptr(gs, GB_ADSTF_Z);
        lambda = gb_solver_ptr(gs, GB_LAMBDA);
        mu = gb_solver_ptr(gs, GB_MU);
        rho = gb_solver_ptr(gs, GB_RHO);
        k_lambda = gb_solver_ptr(gs, GB_K_LAMBDA);
        k_mu = gb_solver_ptr(gs, GB_K_MU);
        k_rho = gb_solver_ptr(gs, GB_K_RHO);
    }

public:
    // Solver::init + FdmSolver::init (solver/solver.h:158-224, solver/fdm.h:350-462)
    void init(Config *config) override {
        Solver::init(config);  // the public scalars: nt, dt, nsrc, nrec, sh, psv, adj, inv_*, ...
        // every parsed key, at float precision, wins over config.ini as in the reference
        std::vector<std::string> kv;
        char buf[64];
        for (auto &p : config->f) {
            std::snprintf(buf, sizeof buf, "%.9g", (double)p.second);
            kv.push_back(p.first + "=" + buf);
        }
        std::vector<const char *> ov;
        for (auto &s : kv) ov.push_back(s.c_str());
        gcfg = gb_config_load(config->path.c_str(), (int)ov.size(), ov.data());
        if (!gcfg) {
            gbfwi_shim::report("gb_config_load", GB_ERR_IO);
            return;
        }
        gs = gb_solver_create(gcfg);
        if (!gs) {
            gbfwi_shim::report("gb_solver_create", GB_ERR_ARG);
            return;
        }
        int nx = 0, nz = 0;
        gb_solver_dims(gs, &nx, &nz, nullptr, nullptr, nullptr);
        dim.init(nx, nz);
        gb_solver_steps(gs, &dx, &dz, nullptr);
        publish();
    }
    // Solver::importModel + FdmSolver::importModel (solver/solver.h:225-252, solver/fdm.h:463-476)
    void importModel(bool model) override { gbfwi_shim::report("gb_import_model", gb_import_model(gs, model)); }
    // FdmSolver::runForward / runAdjoint (solver/fdm.h:515-612)
    void runForward(int isrc, bool trace = false, bool snapshot = false) override {
        gbfwi_shim::report("gb_run_forward", gb_run_forward(gs, isrc, trace, snapshot));
    }
    void runAdjoint(int isrc, bool snapshot = false) override {
        gbfwi_shim::report("gb_run_adjoint", gb_run_adjoint(gs, isrc, snapshot));
    }
    // FdmSolver::initKernels / exportAxis, Solver::exportKernel / exportModel
    void initKernels() override { gbfwi_shim::report("gb_init_kernels", gb_init_kernels(gs)); }
    void exportAxis() override { gbfwi_shim::report("gb_export_axis", gb_export_axis(gs)); }
    void exportKernel(size_t n = 0) override { gbfwi_shim::report("gb_export_kernel", gb_export_kernel(gs, (int)n)); }
    void exportModel(size_t n = 0) override { gbfwi_shim::report("gb_export_model", gb_export_model(gs, (int)n)); }
    ~GbSolver() override {
        gb_solver_destroy(gs);
        gb_config_free(gcfg);
    }
};

// GaussianFilter (filter/gaussian.h:37-61): the same one-sided smoothing
class GbFilter : public Filter {
    gb_filter *gf = nullptr;

public:
    void init(size_t nx, size_t nz, size_t sigma) override {
        Filter::init(nx, nz, sigma);
        gf = gb_filter_create((int)nx, (int)nz, (int)sigma);
        if (!gf) gbfwi_shim::report("gb_filter_create", GB_ERR_ARG);
    }
    void apply(float *data) override { gbfwi_shim::report("gb_filter_apply", gb_filter_apply(gf, data)); }
    ~GbFilter() override { gb_filter_destroy(gf); }
};
