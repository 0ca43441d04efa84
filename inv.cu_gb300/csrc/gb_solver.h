// Host runtime of the solver: owns device buffers, batch slots, the tile
// tables of sources/receivers, captured CUDA graphs and timing.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "gb_config.h"
#include "gb_internal.h"
#include "gb_snapshot.h"
#include "gbfwi.h"

namespace gb {

struct SlotBuf {
    float *state = nullptr;
    size_t state_floats = 0;
    float *out[3] = {nullptr, nullptr, nullptr};
    float *adstf[3] = {nullptr, nullptr, nullptr};
    void *ckpt = nullptr;
    float *amax = nullptr;
    int ckpt_prec = -1;
    void *tmaps = nullptr;  // TMAP_N tensor maps of this slot's fields and the model (device)
};

struct PointSet {
    std::vector<int> i, j, trace;
};

enum PassKind { PASS_FWD = 0, PASS_FWD_NOCKPT = 1, PASS_ADJ = 2 };

struct GraphInfo {
    cudaGraphExec_t exec = nullptr;
    long long launches = 0;  // kernels one replay runs
    int win_steps = 0;       // steps in its timing window
};

struct Solver {
    // configuration (Solver::init, solver/solver.h:158-224)
    std::string path;
    int nx = 0, nz = 0, nt = 0, sfe = 0, wfe = 0, wae = 0, nsfe = 0;
    float dx = 0, dz = 0, dt = 0, xmax = 0, zmax = 0;
    bool sh = false, psv = false, adj = false;
    int trace_type = 0, model_type = 0, mode = 0;
    int abs_width = 0;
    float abs_alpha = 0;
    bool abs_left = false, abs_right = false, abs_top = false, abs_bottom = false;
    bool inv_lambda = false, inv_mu = false, inv_rho = false;
    int nsrc = 0, nrec = 0;
    int model_npt = 0;
    std::vector<float> src_x, src_z, rec_x, rec_z;
    std::vector<int> src_xi, src_zi, rec_xi, rec_zi;

    // options (no effect on results except ckpt precision)
    int opt_batch = 0;
    bool opt_graphs = true;
    int opt_ckpt = CKPT_F32;
    int opt_tile = 0;  // 0 = autotune
    double opt_budget_gb = 0;
    int num_sms = 152;    // streaming multiprocessors of the device (queried at init)
    int opt_tma = 1;      // marching kernel loads columns with bulk tensor copies when possible
    bool tma_ok = false;  // every slot has its tensor maps (nz % 4 == 0, aligned buffers)
    bool use_tma() const { return opt_tma && tma_ok; }
    int tmaps_T = 0;      // box height the slots' maps are encoded for (0: stale)
    int build_tmaps(SlotBuf &b);
    int refresh_tmaps(int threads);
    int opt_cluster_qm = 0;  // cluster columns per thread (0: chosen with the cluster size)
    int opt_stage = 0;    // cluster adjoint: stage checkpoints in shared memory when they fit
    int opt_kacc = 1;     // cluster adjoint: accumulate the kernels in shared memory when they fit
    int opt_shift = 1;    // cluster passes: row-shifted shared-memory layout (no bank conflicts) when it fits
    int opt_snap = 1;     // cluster adjoint: store the adjoint state, accumulate the kernels after the pass
    int opt_cluster = 1;  // cluster-resident passes: 0 never, 1 automatic R, 2..16 this cluster size
    int opt_snap_async = 1;  // snapshots through the asynchronous writer (0: blocking copy per field)
    SnapWriter snapw;

    // device buffers in the reference layout
    float *lambda = nullptr, *mu = nullptr, *rho = nullptr;
    float *rinv = nullptr;  // 1/rho, refreshed at the start of every pass
    float *k_lambda = nullptr, *k_mu = nullptr, *k_rho = nullptr;
    float *stf[3] = {nullptr, nullptr, nullptr};
    float *ax = nullptr, *az = nullptr;
    int *d_rec_cells = nullptr;   // receiver cells: i[nrec] then j[nrec]
    bool rec_distinct = true;     // no two receivers share a cell
    float *kpart = nullptr;       // per-slot kernel contributions (cluster adjoint)
    size_t kpart_slots = 0;
    float *snapbuf = nullptr;     // cluster adjoint state at each accumulation step
    size_t snap_bytes = 0;

    // batch slots
    std::vector<SlotBuf> slots;
    int capacity = 0;
    Slot *d_slots[3] = {nullptr, nullptr, nullptr};
    Slot *h_slots[3] = {nullptr, nullptr, nullptr};
    Slot *d_tune = nullptr;
    KernelGroup *d_group = nullptr;
    KernelGroup *h_group = nullptr;

    // tile tables
    int tile_id = 0;
    bool tuned = false;  // the autotuner ran for the current options
    TileCfg tile{32, 32};
    int *d_csr = nullptr;
    size_t csr_words = 0;
    std::vector<size_t> src_set;  // per source
    size_t super_set = 0, rec_inj_set = 0, rec_rec_set = 0;

    // graphs, keyed by (pass kind, nslots)
    std::map<std::pair<int, int>, GraphInfo> graphs;
    cudaStream_t st = nullptr;
    // lower-priority stream for work that can fill SMs the main stream's
    // clusters leave free (the kernel accumulation of a finished round)
    cudaStream_t st_side = nullptr;
    cudaEvent_t ev_round = nullptr, ev_side = nullptr;
    cudaEvent_t ev_pass0 = nullptr, ev_pass1 = nullptr, ev_win0 = nullptr, ev_win1 = nullptr;
    cudaEvent_t ev_t0 = nullptr, ev_t1 = nullptr;  // gb_solver_timer
    int win_steps = 0;
    int last_par = 0;
    int last_forward_n = 0;
    gb_stats stats{};

    // --- lifecycle
    int init(const Config &cfg, int nx_, int nz_, float xmax_, float zmax_);
    void release();
    // --- model
    int set_model_points(int npt, const float *x, const float *z, const float *a, const float *b, const float *r);
    int import_model(bool model_true);
    // --- passes
    int ensure_slots(int n);
    int ensure_tables();
    int forward(const int *shots, int n, bool ckpt_on, bool record_u, bool snapshot);
    int adjoint(const int *shots, int n, bool snapshot, int snap_isrc);
    int init_kernels();
    // --- helpers
    size_t ncell() const { return (size_t)nx * nz; }
    // checkpoint fields per snapshot at precision prec (ckpt_nf_sh/psv)
    int nf(int prec) const { return (sh ? ckpt_nf_sh(prec) : 0) + (psv ? ckpt_nf_psv(prec) : 0); }
    size_t slot_bytes(int prec) const;
    int fill_slots(int kind, const int *shots, int n, bool record_u);
    int enqueue_pass(int kind, int n, bool snapshot, int snap_isrc);
    int run_pass(int kind, int n, bool snapshot, int snap_isrc);
    int autotune(int n);
    bool cluster_geometry(bool wave_psv, int n, ClusterGeom *g) const;
    // cluster_geometry results by (wave system, batch size, cluster option)
    mutable std::map<long long, std::pair<bool, ClusterGeom>> cluster_cache;
    bool cluster_ok(const int *shots, int n, bool snapshot) const;
    int run_cluster_pass(int kind, int n);

    // Pipelined gradient of one batch (cluster path, one wave system, more
    // shots than resident clusters): with pipe_on, the forward pass launches
    // one round of pipe_occ shots at a time, records ev_fwd_round[r] after
    // each and returns without waiting; the caller runs round r's misfit on
    // st_side after that event and records ev_mis_round[r]; the adjoint's
    // round r waits for it. The next synchronising pass books the forward's
    // time (ev_fpass0/1).
    int opt_pipe = 1;
    bool pipe_on = false;
    int pipe_rounds = 0, pipe_occ = 0;
    std::vector<cudaEvent_t> ev_fwd_round, ev_mis_round;
    cudaEvent_t ev_fpass0 = nullptr, ev_fpass1 = nullptr;
    bool fpass_pending = false;
    // rounds of a pipelined gradient of these shots (0: not pipelined;
    // never an error code)
    int pipe_plan(const int *shots, int n);
    int book_forward_pass();
    int export_snapshot(int it, int isrc, int par);
    int export_data(const std::string &comp, const float *d_data, int n);
    int export_field(const std::string &comp, const float *d_data, int n);
    void invalidate_graphs();
    cudaError_t record_timing(cudaEvent_t e);
    int max_tiles() const { return ((nz + tile.tz - 1) / tile.tz) * ((nx + tile.tx - 1) / tile.tx); }
};

// Tensor maps of a slot's fields for the marching kernel's bulk loads
// (gb_solver.cu): TMAP_N maps into h, for arrays of nx columns at pitch pz.
bool encode_slot_maps(void *h, const float *state, bool sh, bool psv, const float *rinv, const float *mu,
                      const float *lambda, int nx, int nz, int pz, int rows);

}  // namespace gb

struct gb_solver {
    gb::Solver s;
};
