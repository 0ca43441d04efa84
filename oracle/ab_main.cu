// A/B driver of the in-process binding: TEST INFRASTRUCTURE ONLY.
//
// Built from the reference's own headers (lib/index.h and everything it
// includes) plus include/gbfwi_reference_shim.h, and linked with libgbfwi.so,
// by oracle/Makefile (target `ab`, only where the reference sources are
// present). It runs the reference's main for mode 2 (inv.cu:57-67): its own
// Config, Misfit::init and Misfit::run(kernel = true), with the solver and
// the filter chosen by id as lib/index.h does, where id 1 is the GB300 shim
// (GbSolver, GbFilter) and id 0 the reference's FdmSolver / GaussianFilter.
// It prints the misfit and writes the kernels with Solver::exportKernel, so
// two runs (solver=0 filter=0 against solver=1 filter=1) compare the
// reference's whole gradient with the same reference code driving the GB300
// kernels.
//     ab_harness <dir> -solver=<0|1> -filter=<0|1> [-key=value ...]
#include "lib/index.h"

#include "gbfwi_reference_shim.h"

int main(int argc, const char *argv[]) {
    std::map<std::string, std::string> cfg;
    for (int i = 1; i < argc; i++) {
        std::string arg = argv[i];
        const size_t pos = arg.find("=");
        if (arg[0] == '-') {
            if (pos != std::string::npos) cfg[arg.substr(1, pos - 1)] = arg.substr(pos + 1);
        } else {
            cfg["config"] = arg;
        }
    }
    if (!cfg["config"].size()) {
        std::fprintf(stderr, "usage: ab_harness <dir> -solver=<0|1> -filter=<0|1> [-key=value ...]\n");
        return 2;
    }
    cublasCreate(&device::cublas_handle);
    Config *config = new Config(cfg);
    const int sid = config->i["solver"], fid = config->i["filter"];
    Solver *solver = sid == 1 ? new GbSolver() : module::solver(sid);
    Filter *filter = fid == 1 ? new GbFilter() : module::filter(fid);
    Misfit *misfit = module::misfit(config->i["misfit"]);
    if (!solver || !filter || !misfit) {
        std::fprintf(stderr, "ab_harness: unknown solver, filter or misfit id\n");
        return 2;
    }
    misfit->init(config, solver, filter);
    const float value = misfit->run(true, false);
    std::printf("misfit %.9g\n", (double)value);
    solver->exportKernel();
    cudaError_t e = cudaDeviceSynchronize();
    cublasDestroy(device::cublas_handle);
    return e == cudaSuccess ? 0 : 1;
}
