// gbinv: command-line drop-in for inv.cu's main (inv.cu:6-92).
//
//   gbinv [dir] [-key=value ...]
//
// Same arguments, config files, output files and stdout lines; modes:
//   0 inversion, 1 forward with snapshots (all sources at once),
//   2 adjoint kernels, 3 traces per shot, 4 device query, 5 model export.
#include <cuda_runtime.h>

#include <cstdio>
#include <iostream>
#include <string>
#include <vector>

#include "gbfwi.h"

static int fail(const char *what) {
    std::cerr << "gbinv: " << what << ": " << gb_last_error() << std::endl;
    return 1;
}

static void memory_report(size_t before) {
    size_t freeb = 0, total = 0;
    if (cudaMemGetInfo(&freeb, &total) != cudaSuccess) return;
    const double mb = 1024.0 * 1024.0;
    std::printf("Memory usage: %.1fMB / %.1fMB\n", (before - (double)freeb) / mb, before / mb);
}

static void device_query() {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) {
        std::cout << "Failed to get device info: " << cudaGetErrorString(e) << std::endl;
        return;
    }
    for (int d = 0; d < n; d++) {
        cudaDeviceProp p;
        cudaGetDeviceProperties(&p, d);
        std::cout << "Device " << d << ": " << p.name << "\n  compute capability " << p.major << "." << p.minor
                  << "\n  multiprocessors " << p.multiProcessorCount << "\n  global memory "
                  << p.totalGlobalMem / (1024 * 1024) << " MB\n  shared memory per block " << p.sharedMemPerBlock
                  << " B\n  L2 cache " << p.l2CacheSize / 1024 << " KB" << std::endl;
    }
}

int main(int argc, const char *argv[]) {
    size_t free0 = 0, total0 = 0;
    cudaMemGetInfo(&free0, &total0);
    std::string dir;
    std::vector<std::string> over;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        if (!a.empty() && a[0] == '-') {
            if (a.find('=') != std::string::npos) over.push_back(a);
        } else {
            dir = a;
        }
    }
    if (dir.empty()) {
        std::cout << "Using default directory example/checker" << std::endl;
        dir = "example/checker";
    }
    std::vector<const char *> ov;
    for (auto &s : over) ov.push_back(s.c_str());
    gb_config *cfg = gb_config_load(dir.c_str(), (int)ov.size(), ov.data());
    if (!cfg) return fail("config");
    const int mode = gb_config_i(cfg, "mode");
    int rc = 0;
    switch (mode) {
        case 0: {
            gb_solver *s = gb_solver_create(cfg);
            if (!s) return fail("solver");
            gb_misfit *m = gb_misfit_create(cfg, s, nullptr);
            if (!m) return fail("misfit");
            gb_optimizer *o = gb_optimizer_create(cfg, s, m);
            if (!o) return fail("optimizer");
            if (gb_optimizer_run(o)) return fail("optimizer run");
            memory_report(free0);
            gb_optimizer_destroy(o);
            gb_misfit_destroy(m);
            gb_solver_destroy(s);
            break;
        }
        case 1: {
            gb_solver *s = gb_solver_create(cfg);
            if (!s) return fail("solver");
            if (gb_import_model(s, 1) || gb_export_axis(s) || gb_run_forward(s, -1, 1, 1)) return fail("forward");
            memory_report(free0);
            gb_solver_destroy(s);
            break;
        }
        case 2: {
            gb_solver *s = gb_solver_create(cfg);
            if (!s) return fail("solver");
            gb_misfit *m = gb_misfit_create(cfg, s, nullptr);
            if (!m) return fail("misfit");
            double v = 0;
            if (gb_misfit_run(m, 1, 1, &v) || gb_export_axis(s) || gb_export_kernel(s, 0)) return fail("adjoint");
            memory_report(free0);
            gb_misfit_destroy(m);
            gb_solver_destroy(s);
            break;
        }
        case 3: {
            gb_solver *s = gb_solver_create(cfg);
            if (!s) return fail("solver");
            if (gb_import_model(s, 1)) return fail("model");
            int nsrc = 0;
            gb_solver_dims(s, nullptr, nullptr, nullptr, &nsrc, nullptr);
            for (int is = 0; is < nsrc; is++)
                if (gb_run_forward(s, is, 1, 0)) return fail("forward");
            gb_solver_destroy(s);
            break;
        }
        case 4:
            device_query();
            break;
        case 5: {
            gb_solver *s = gb_solver_create(cfg);
            if (!s) return fail("solver");
            if (gb_import_model(s, 1) || gb_export_axis(s) || gb_export_model(s, 0)) return fail("export");
            gb_solver_destroy(s);
            break;
        }
        default:
            break;
    }
    gb_config_free(cfg);
    return rc;
}
