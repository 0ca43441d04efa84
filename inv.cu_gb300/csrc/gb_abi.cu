// C ABI of the solver (include/gbfwi.h): thin wrappers over gb::Solver that
// keep the reference's calling conventions (solver/solver.h, solver/fdm.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "gb_solver.h"

using namespace gb;

namespace {

// Grid inference of FdmSolver::init (solver/fdm.h:354-391): xmax/zmax are
// the largest x/z values of model_true (floor 0), nx solves
// a*y^2 + (a+1)*y + 1 - npt = 0 for y = nx-1 with a = zmax/xmax, and
// nz = npt / nx in integer division.
int infer_grid(const std::string &dir, int *nx, int *nz, float *xmax, float *zmax, int *npt) {
    std::vector<float> x, z;
    int rc = read_bin(dir + "/model_true/proc000000_x.bin", x);
    if (rc) return rc;
    rc = read_bin(dir + "/model_true/proc000000_z.bin", z);
    if (rc) return rc;
    if (x.size() != z.size() || x.empty()) {
        set_error("error: invalid model (x and z point counts differ or are empty)");
        return GB_ERR_MODEL;
    }
    float xm = 0, zm = 0;
    for (float v : x)
        if (v > xm) xm = v;
    for (float v : z)
        if (v > zm) zm = v;
    const size_t n = x.size();
    if (!(xm > 0) || !(zm > 0)) {
        set_error("error: invalid model (xmax and zmax must be positive)");
        return GB_ERR_MODEL;
    }
    const float a = zm / xm;
    const float b = a + 1;
    const float c = 1 - (int)n;
    const size_t gx = (size_t)std::round((-b + std::sqrt(b * b - 4 * a * c)) / (2 * a)) + 1;
    const size_t gz = (size_t)std::round((float)(n / gx));
    *nx = (int)gx;
    *nz = (int)gz;
    *xmax = xm;
    *zmax = zm;
    *npt = (int)n;
    return GB_OK;
}

gb_solver *make_solver(const gb_config *cfg, int nx, int nz, float xmax, float zmax, int npt) {
    gb_solver *s = new gb_solver();
    int rc = s->s.init(*reinterpret_cast<const Config *>(cfg), nx, nz, xmax, zmax);
    if (rc) {
        s->s.release();
        delete s;
        return nullptr;
    }
    s->s.model_npt = npt;
    return s;
}

}  // namespace

extern "C" {

int gb_infer_grid(const char *dir, int *nx, int *nz, float *xmax, float *zmax, int *npt) {
    if (!dir || !nx || !nz || !xmax || !zmax || !npt) {
        set_error("gb_infer_grid: null argument");
        return GB_ERR_ARG;
    }
    return infer_grid(dir, nx, nz, xmax, zmax, npt);
}

gb_solver *gb_solver_create(const gb_config *cfg) {
    if (!cfg) {
        set_error("gb_solver_create: null config");
        return nullptr;
    }
    int nx, nz, npt;
    float xmax, zmax;
    if (infer_grid(reinterpret_cast<const Config *>(cfg)->path, &nx, &nz, &xmax, &zmax, &npt)) return nullptr;
    return make_solver(cfg, nx, nz, xmax, zmax, npt);
}

gb_solver *gb_solver_create_grid(const gb_config *cfg, int nx, int nz, float xmax, float zmax) {
    if (!cfg || nx < 2 || nz < 2 || !(xmax > 0) || !(zmax > 0)) {
        gb::set_error("gb_solver_create_grid: need nx, nz >= 2 and positive extents");
        return nullptr;
    }
    return make_solver(cfg, nx, nz, xmax, zmax, 0);
}

void gb_solver_destroy(gb_solver *s) {
    if (!s) return;
    s->s.release();
    delete s;
}

int gb_import_model(gb_solver *s, int model_true) {
    if (!s) return GB_ERR_ARG;
    return s->s.import_model(model_true != 0);
}

int gb_set_model_points(gb_solver *s, int npt, const float *x, const float *z, const float *a, const float *b,
                        const float *rho) {
    if (!s) return GB_ERR_ARG;
    return s->s.set_model_points(npt, x, z, a, b, rho);
}

int gb_set_model_grid(gb_solver *s, const float *lambda, const float *mu, const float *rho) {
    if (!s || !lambda || !mu || !rho) return GB_ERR_ARG;
    Solver &v = s->s;
    const size_t n = v.ncell() * 4;
    GB_CUDA_TRY(cudaMemcpyAsync(v.lambda, lambda, n, cudaMemcpyHostToDevice, v.st));
    GB_CUDA_TRY(cudaMemcpyAsync(v.mu, mu, n, cudaMemcpyHostToDevice, v.st));
    GB_CUDA_TRY(cudaMemcpyAsync(v.rho, rho, n, cudaMemcpyHostToDevice, v.st));
    GB_CUDA_TRY(cudaStreamSynchronize(v.st));
    return GB_OK;
}

int gb_run_forward(gb_solver *s, int isrc, int trace, int snapshot) {
    if (!s) return GB_ERR_ARG;
    Solver &v = s->s;
    int rc = v.forward(&isrc, 1, true, v.adj || v.trace_type == 1, snapshot != 0);
    if (rc) return rc;
    if (trace) return gb_export_traces(s, std::max(isrc, 0));
    return GB_OK;
}

int gb_run_adjoint(gb_solver *s, int isrc, int snapshot) {
    if (!s) return GB_ERR_ARG;
    return s->s.adjoint(&isrc, 1, snapshot != 0, isrc);
}

int gb_run_forward_batch(gb_solver *s, const int *isrc, int n) {
    if (!s || !isrc || n < 0) return GB_ERR_ARG;
    Solver &v = s->s;
    return v.forward(isrc, n, true, v.adj || v.trace_type == 1, false);
}

int gb_run_adjoint_batch(gb_solver *s, const int *isrc, int n) {
    if (!s || !isrc || n < 0) return GB_ERR_ARG;
    return s->s.adjoint(isrc, n, false, -1);
}

int gb_init_kernels(gb_solver *s) {
    if (!s) return GB_ERR_ARG;
    return s->s.init_kernels();
}

int gb_export_axis(gb_solver *s) {
    if (!s) return GB_ERR_ARG;
    Solver &v = s->s;
    std::vector<float> x(v.ncell()), z(v.ncell());
    for (int i = 0; i < v.nx; i++)
        for (int j = 0; j < v.nz; j++) {
            const size_t k = (size_t)i * v.nz + j;
            x[k] = i * v.dx;
            z[k] = j * v.dz;
        }
    int rc = write_bin(v.path + "/output/proc000000_x.bin", x.data(), x.size());
    if (!rc) rc = write_bin(v.path + "/output/proc000000_z.bin", z.data(), z.size());
    return rc;
}

int gb_export_model(gb_solver *s, int n) {
    if (!s) return GB_ERR_ARG;
    Solver &v = s->s;
    if (v.model_type == 0) {
        const size_t nc = v.ncell();
        float *t;
        GB_CUDA_TRY(cudaMalloc(&t, nc * 3 * 4));
        cudaMemcpyAsync(t, v.lambda, nc * 4, cudaMemcpyDeviceToDevice, v.st);
        cudaMemcpyAsync(t + nc, v.mu, nc * 4, cudaMemcpyDeviceToDevice, v.st);
        cudaMemcpyAsync(t + 2 * nc, v.rho, nc * 4, cudaMemcpyDeviceToDevice, v.st);
        cudaError_t e = launch_lm2vps(t, t + nc, t + 2 * nc, nc, v.st);
        int rc = e == cudaSuccess ? GB_OK : GB_ERR_CUDA;
        if (!rc && v.inv_lambda && v.inv_mu) rc = v.export_data("vp", t, n);
        if (!rc && v.inv_mu) rc = v.export_data("vs", t + nc, n);
        if (!rc && v.inv_rho) rc = v.export_data("rho", t + 2 * nc, n);
        cudaFree(t);
        return rc;
    }
    int rc = GB_OK;
    if (v.inv_lambda) rc = v.export_data("lambda", v.lambda, n);
    if (!rc && v.inv_mu) rc = v.export_data("mu", v.mu, n);
    if (!rc && v.inv_rho) rc = v.export_data("rho", v.rho, n);
    return rc;
}

int gb_export_kernel(gb_solver *s, int n) {
    if (!s) return GB_ERR_ARG;
    Solver &v = s->s;
    if (!v.adj) return GB_OK;
    int rc = GB_OK;
    if (v.inv_lambda) rc = v.export_data("k_lambda", v.k_lambda, n);
    if (!rc && v.inv_mu) rc = v.export_data("k_mu", v.k_mu, n);
    if (!rc && v.inv_rho) rc = v.export_data("k_rho", v.k_rho, n);
    return rc;
}

int gb_export_traces(gb_solver *s, int isrc) {
    if (!s) return GB_ERR_ARG;
    Solver &v = s->s;
    if (v.slots.empty()) {
        set_error("gb_export_traces: no forward run yet");
        return GB_ERR_STATE;
    }
    if (isrc < 0 || isrc >= std::max(v.nsrc, 1)) return GB_ERR_ARG;
    const size_t tr = (size_t)v.nrec * v.nt;
    std::vector<float> h(tr);
    const char *nm[3] = {"x", "y", "z"};
    for (int c : {1, 0, 2}) {
        if (!v.slots[0].out[c]) continue;
        GB_CUDA_TRY(cudaMemcpy(h.data(), v.slots[0].out[c], tr * 4, cudaMemcpyDeviceToHost));
        const std::string file =
            v.path + "/output/" + (v.trace_type ? "u" : "v") + nm[c] + "_" + pad6(isrc) + ".su";
        int rc = write_su(file, h.data(), v.nrec, v.nt, v.dt, v.nsrc ? v.src_x[isrc] : 0.f,
                          v.nsrc ? v.src_z[isrc] : 0.f, v.rec_x.data(), v.rec_z.data());
        if (rc) return rc;
    }
    return GB_OK;
}

int gb_su_write(const char *file, const float *traces, int nrec, int nt, float dt, float xs, float zs,
                const float *rec_x, const float *rec_z) {
    if (!file || !traces || !rec_x || !rec_z || nrec < 1 || nt < 1) {
        set_error("gb_su_write: bad arguments");
        return GB_ERR_ARG;
    }
    return write_su(file, traces, nrec, nt, dt, xs, zs, rec_x, rec_z);
}

int gb_su_read(const char *file, float *traces, int nrec, int nt) {
    if (!file || !traces || nrec < 1 || nt < 1) {
        set_error("gb_su_read: bad arguments");
        return GB_ERR_ARG;
    }
    return read_su(file, traces, nrec, nt);
}

float *gb_slot_ptr(gb_solver *s, int slot, int which) {
    if (!s) return nullptr;
    Solver &v = s->s;
    if (slot < 0 || slot >= (int)v.slots.size()) {
        if (slot == 0 && v.ensure_slots(1) == GB_OK) return gb_slot_ptr(s, slot, which);
        return nullptr;
    }
    if (which >= GB_OUT_X && which <= GB_OUT_Z) return v.slots[slot].out[which - GB_OUT_X];
    if (which >= GB_ADSTF_X && which <= GB_ADSTF_Z) return v.slots[slot].adstf[which - GB_ADSTF_X];
    return nullptr;
}

float *gb_solver_ptr(gb_solver *s, int which) {
    if (!s) return nullptr;
    Solver &v = s->s;
    switch (which) {
        case GB_OUT_X:
        case GB_OUT_Y:
        case GB_OUT_Z:
        case GB_ADSTF_X:
        case GB_ADSTF_Y:
        case GB_ADSTF_Z:
            return gb_slot_ptr(s, 0, which);
        case GB_LAMBDA: return v.lambda;
        case GB_MU: return v.mu;
        case GB_RHO: return v.rho;
        case GB_K_LAMBDA: return v.k_lambda;
        case GB_K_MU: return v.k_mu;
        case GB_K_RHO: return v.k_rho;
        case GB_STF_X: return v.stf[0];
        case GB_STF_Y: return v.stf[1];
        case GB_STF_Z: return v.stf[2];
        default: return nullptr;
    }
}

int gb_solver_dims(const gb_solver *s, int *nx, int *nz, int *nt, int *nsrc, int *nrec) {
    if (!s) return GB_ERR_ARG;
    const Solver &v = s->s;
    if (nx) *nx = v.nx;
    if (nz) *nz = v.nz;
    if (nt) *nt = v.nt;
    if (nsrc) *nsrc = v.nsrc;
    if (nrec) *nrec = v.nrec;
    return GB_OK;
}

int gb_solver_steps(const gb_solver *s, float *dx, float *dz, float *dt) {
    if (!s) return GB_ERR_ARG;
    const Solver &v = s->s;
    if (dx) *dx = v.dx;
    if (dz) *dz = v.dz;
    if (dt) *dt = v.dt;
    return GB_OK;
}

int gb_solver_batch_capacity(gb_solver *s) {
    if (!s) return 0;
    if (s->s.ensure_slots(0)) return 0;
    return s->s.capacity;
}

int gb_solver_set_option(gb_solver *s, const char *key, double value) {
    if (!s || !key) return GB_ERR_ARG;
    Solver &v = s->s;
    const std::string k = key;
    if (k == "batch") {
        if (v.capacity) {
            set_error("option batch: set it before the first run");
            return GB_ERR_STATE;
        }
        v.opt_batch = (int)value;
    } else if (k == "graphs") {
        v.opt_graphs = value != 0;
    } else if (k == "ckpt") {
        const int p = (int)value;
        if (p < CKPT_F32 || p > CKPT_F16) return GB_ERR_ARG;
        v.opt_ckpt = p;
        v.invalidate_graphs();
    } else if (k == "tile") {
        const int t = (int)value;
        if (t < 0 || t > 20) return GB_ERR_ARG;
        v.opt_tile = t;
        if (t == 0) {
            v.tile_id = 0;
            v.tuned = false;
        }
        v.invalidate_graphs();
    } else if (k == "cluster_qm") {
        const int q = (int)value;
        if (q != 0 && q != 4 && q != 8 && q != 10 && q != 12 && q != 16 && q != 20 && q != 24) return GB_ERR_ARG;
        v.opt_cluster_qm = q;
    } else if (k == "cluster_stage") {
        v.opt_stage = value != 0;
    } else if (k == "cluster_kacc") {
        v.opt_kacc = value != 0;
    } else if (k == "cluster_shift") {
        v.opt_shift = value != 0;
    } else if (k == "cluster_snap") {
        v.opt_snap = value != 0;
    } else if (k == "pipeline") {
        v.opt_pipe = value != 0;
    } else if (k == "snap_async") {
        v.opt_snap_async = value != 0;
    } else if (k == "tma") {
        v.opt_tma = value != 0;
        v.invalidate_graphs();
    } else if (k == "cluster") {
        const int c = (int)value;
        if (c < 0 || c > 16) return GB_ERR_ARG;
        v.opt_cluster = c;
    } else if (k == "hbm_budget_gb") {
        if (v.capacity) {
            set_error("option hbm_budget_gb: set it before the first run");
            return GB_ERR_STATE;
        }
        v.opt_budget_gb = value;
    } else {
        set_error("unknown option " + k);
        return GB_ERR_ARG;
    }
    return GB_OK;
}

int gb_solver_timer(gb_solver *s, int begin, double *ms) {
    if (!s) return GB_ERR_ARG;
    Solver &v = s->s;
    if (!v.ev_t0) {
        GB_CUDA_TRY(cudaEventCreate(&v.ev_t0));
        GB_CUDA_TRY(cudaEventCreate(&v.ev_t1));
    }
    if (begin) {
        GB_CUDA_TRY(cudaEventRecord(v.ev_t0, v.st));
        return GB_OK;
    }
    GB_CUDA_TRY(cudaEventRecord(v.ev_t1, v.st));
    GB_CUDA_TRY(cudaEventSynchronize(v.ev_t1));
    float f = 0;
    GB_CUDA_TRY(cudaEventElapsedTime(&f, v.ev_t0, v.ev_t1));
    if (ms) *ms = f;
    return GB_OK;
}

int gb_solver_stats(gb_solver *s, gb_stats *out, int reset) {
    if (!s) return GB_ERR_ARG;
    if (out) *out = s->s.stats;
    if (reset) {
        const int tz = s->s.stats.tile_tz, tx = s->s.stats.tile_tx, cap = s->s.stats.batch_capacity;
        const int bulk = s->s.stats.march_bulk, cadj = s->s.stats.cluster_adj, csh = s->s.stats.cluster_shift;
        s->s.stats = gb_stats{};
        s->s.stats.cluster_adj = cadj;
        s->s.stats.cluster_shift = csh;
        s->s.stats.tile_tz = tz;
        s->s.stats.tile_tx = tx;
        s->s.stats.batch_capacity = cap;
        s->s.stats.march_bulk = bulk;
    }
    return GB_OK;
}

}  // extern "C"
