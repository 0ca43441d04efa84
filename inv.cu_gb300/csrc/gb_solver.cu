// Solver runtime: the GB300 replacement of FdmSolver (solver/fdm.h:222-613)
// and the Solver base class (solver/solver.h:7-268).
//
// Shots are the batching unit. A batch of n shots owns n slots (wavefields,
// traces, adjoint sources, forward checkpoints, all resident in HBM); one
// launch per time step advances all of them. The time loop of a pass is
// captured once into a CUDA graph per (pass kind, n) and replayed; the
// per-slot descriptors live in device memory so a replay can serve another
// set of shots after one small host-to-device copy.
#include <cuda.h>  // CUtensorMap and its enums (the encoder comes from the runtime's driver entry point)
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <map>
#include <vector>

#include "gb_solver.h"

namespace gb {

// Step-kernel configurations: ids 1-5 are 2-D tiles (rows x columns per
// block), ids 6+ the marching kernel (threads per strip, columns per chunk).
static const TileCfg kTiles[] = {
    {32, 32, 0},                                                            // 0: unused
    {32, 32, 0},   {64, 16, 0},   {32, 16, 0},   {16, 32, 0},   {128, 8, 0},  // 1-5
    {56, 32, 64},  {88, 32, 96},  {120, 32, 128}, {120, 64, 128}, {152, 32, 160},  // 6-10
    {152, 64, 160}, {184, 32, 192}, {248, 32, 256}, {248, 64, 256}, {120, 16, 128}, // 11-15
    {56, 16, 64},  {248, 128, 256}, {120, 128, 128}, {152, 128, 160}, {152, 16, 160}, // 16-20
};
static const int kNumTiles = 20;

TileCfg tile_config(int id) { return kTiles[id >= 1 && id <= kNumTiles ? id : 3]; }

// ---------------------------------------------------------------- tables
// Packs a point set into the tile CSR the step kernel reads. For injection
// (inj = true) a point is listed for every tile whose velocity region (tile
// plus 1 cell before and 2 after, in x and z) contains it; for recording it
// is listed once, for the tile that owns its cell. Points sharing a cell form
// one entry whose traces are visited in ascending order.
static std::vector<int> build_csr(const PointSet &p, int nx, int nz, TileCfg tc, bool inj) {
    const int tz = tc.tz, tx = tc.tx;
    const int tiles_z = (nz + tz - 1) / tz, tiles_x = (nx + tx - 1) / tx;
    const int ntiles = tiles_z * tiles_x;
    const int vz = tz + 3;
    std::map<int, std::map<int, std::vector<int>>> per;  // tile -> local -> traces
    for (size_t q = 0; q < p.i.size(); q++) {
        const int i = p.i[q], j = p.j[q];
        if (i < 0 || i >= nx || j < 0 || j >= nz) continue;
        if (inj) {
            for (int txi = std::max(0, (i - tx - 1) / tx - 1); txi <= std::min(tiles_x - 1, (i + 1) / tx); txi++) {
                const int i0 = txi * tx;
                if (i < i0 - 1 || i > i0 + tx + 1) continue;
                for (int tzi = std::max(0, (j - tz - 1) / tz - 1); tzi <= std::min(tiles_z - 1, (j + 1) / tz);
                     tzi++) {
                    const int j0 = tzi * tz;
                    if (j < j0 - 1 || j > j0 + tz + 1) continue;
                    const int local = (i - (i0 - 1)) * vz + (j - (j0 - 1));
                    per[txi * tiles_z + tzi][local].push_back(p.trace[q]);
                }
            }
        } else {
            const int txi = i / tx, tzi = j / tz;
            const int local = (i - txi * tx) * tz + (j - tzi * tz);
            per[txi * tiles_z + tzi][local].push_back(p.trace[q]);
        }
    }
    int nent = 0, ntr = 0;
    for (auto &t : per) {
        nent += (int)t.second.size();
        for (auto &e : t.second) ntr += (int)e.second.size();
    }
    std::vector<int> out(csr_words(ntiles, nent, ntr));
    out[0] = ntiles;
    out[1] = nent;
    out[2] = ntr;
    int *tile_ptr = out.data() + 3;
    int *local = tile_ptr + ntiles + 1;
    int *tptr = local + nent;
    int *traces = tptr + nent + 1;
    int e = 0, t = 0;
    auto it = per.begin();
    for (int tile = 0; tile < ntiles; tile++) {
        tile_ptr[tile] = e;
        if (it != per.end() && it->first == tile) {
            for (auto &ent : it->second) {
                std::vector<int> trs = ent.second;
                std::sort(trs.begin(), trs.end());
                local[e] = ent.first;
                tptr[e] = t;
                for (int v : trs) traces[t++] = v;
                e++;
            }
            ++it;
        }
    }
    tile_ptr[ntiles] = e;
    tptr[nent] = t;
    return out;
}

// ---------------------------------------------------------------- source
// RickerSource::create + Source::init (source/ricker.h:5-21,
// source/source.h:17-37), host float arithmetic.
static void ricker(int nt, float dt, const float *cfg, float *sx, float *sy, float *sz) {
    const float pi = 3.1415927f;
    const float f0 = cfg[0], t0 = cfg[1], angle = cfg[2], amp = cfg[3];
    std::vector<float> s(nt);
    float amax = 0;
    for (int it = 0; it < nt; it++) {
        float t = (float)(size_t)it * dt - t0;
        float pft = pi * f0 * t;
        s[it] = -t * expf(-pft * pft);
        if (fabsf(s[it]) > amax) amax = fabsf(s[it]);
    }
    if (amax > 0)
        for (int it = 0; it < nt; it++) s[it] /= amax;
    for (int it = 0; it < nt; it++) {
        sx[it] = amp * s[it] * cosf(angle);
        sy[it] = amp * s[it];
        sz[it] = amp * s[it] * sinf(angle);
    }
}

// calcIdx (solver/fdm.h:44-47).
static int calc_idx(float c, float L, int n) { return (int)((double)(c / L * (float)(n - 1)) + 0.5); }

// initAbsbound (solver/fdm.h:48-74) as two 1-D profiles: the product over
// the left/right edges depends on i only, bottom/top on j only, and
// ab(i,j) = ax[i] * az[j].
static void absorbing_profiles(int nx, int nz, int w, float alpha, bool l, bool r, bool b, bool t,
                               std::vector<float> &ax, std::vector<float> &az) {
    ax.assign(nx, 1.f);
    az.assign(nz, 1.f);
    for (int i = 0; i < nx; i++) {
        if (l && i + 1 < w) ax[i] *= expf(-powf(alpha * (float)(w - i - 1), 2));
        if (r && i > nx - w) ax[i] *= expf(-powf(alpha * (float)(w + i - nx), 2));
    }
    for (int j = 0; j < nz; j++) {
        if (b && j > nz - w) az[j] *= expf(-powf(alpha * (float)(w + j - nz), 2));
        if (t && j + 1 < w) az[j] *= expf(-powf(alpha * (float)(w - j - 1), 2));
    }
}

// ---------------------------------------------------------------- init
int Solver::init(const Config &cfg, int nx_, int nz_, float xmax_, float zmax_) {
    path = cfg.path;
    dt = cfg.fv("dt");
    nt = cfg.iv("nt");
    sfe = cfg.iv("sfe");
    wfe = cfg.iv("wfe");
    wae = cfg.iv("wae");
    sh = cfg.iv("sh") != 0;
    psv = cfg.iv("psv") != 0;
    mode = cfg.iv("mode");
    adj = mode == 0 || mode == 2;
    trace_type = cfg.iv("trace_type");
    model_type = cfg.iv("model_type");
    abs_alpha = cfg.fv("abs_alpha");
    abs_width = cfg.iv("abs_width");
    abs_left = cfg.iv("abs_left") != 0;
    abs_top = cfg.iv("abs_top") != 0;
    abs_right = cfg.iv("abs_right") != 0;
    abs_bottom = cfg.iv("abs_bottom") != 0;
    inv_lambda = cfg.iv("inv_lambda") != 0;
    inv_mu = cfg.iv("inv_mu") != 0;
    inv_rho = cfg.iv("inv_rho") != 0;
    if (cfg.has("batch")) opt_batch = cfg.iv("batch");
    if (cfg.has("graphs")) opt_graphs = cfg.iv("graphs") != 0;
    if (cfg.has("ckpt_precision")) opt_ckpt = cfg.iv("ckpt_precision");
    if (cfg.has("tile")) opt_tile = cfg.iv("tile");
    if (cfg.has("tma")) opt_tma = cfg.iv("tma") != 0;
    if (cfg.has("cluster_qm")) opt_cluster_qm = cfg.iv("cluster_qm");
    if (cfg.has("cluster_stage")) opt_stage = cfg.iv("cluster_stage") != 0;
    if (cfg.has("cluster_kacc")) opt_kacc = cfg.iv("cluster_kacc") != 0;
    if (cfg.has("cluster_shift")) opt_shift = cfg.iv("cluster_shift") != 0;
    if (cfg.has("cluster_snap")) opt_snap = cfg.iv("cluster_snap") != 0;
    if (cfg.has("pipeline")) opt_pipe = cfg.iv("pipeline") != 0;
    if (cfg.has("snap_async")) opt_snap_async = cfg.iv("snap_async") != 0;
    if (cfg.has("cluster")) opt_cluster = std::max(0, std::min(16, cfg.iv("cluster")));
    nx = nx_;
    nz = nz_;
    xmax = xmax_;
    zmax = zmax_;
    if (nx < 1 || nz < 1 || nt < 1) {
        set_error("solver: grid and nt must be positive (nx=" + std::to_string(nx) + " nz=" + std::to_string(nz) +
                  " nt=" + std::to_string(nt) + ")");
        return GB_ERR_ARG;
    }
    if (!sh && !psv) {
        set_error("solver: neither sh nor psv is enabled");
        return GB_ERR_ARG;
    }
    if ((size_t)nx * nz > (size_t)INT32_MAX / 4) {
        set_error("solver: grid too large");
        return GB_ERR_ARG;
    }
    dx = xmax / (float)(nx - 1);
    dz = zmax / (float)(nz - 1);
    nsfe = sfe > 0 ? nt / sfe : 0;
    if (opt_ckpt < CKPT_F32 || opt_ckpt > CKPT_F16) opt_ckpt = CKPT_F32;
    if (opt_tile < 0 || opt_tile > kNumTiles) opt_tile = 0;

    nsrc = (int)cfg.src.size();
    nrec = (int)cfg.rec.size();
    for (auto &s : cfg.src) {
        src_x.push_back(s[0]);
        src_z.push_back(s[1]);
        src_xi.push_back(calc_idx(s[0], xmax, nx));
        src_zi.push_back(calc_idx(s[1], zmax, nz));
    }
    for (auto &r : cfg.rec) {
        rec_x.push_back(r[0]);
        rec_z.push_back(r[1]);
        rec_xi.push_back(calc_idx(r[0], xmax, nx));
        rec_zi.push_back(calc_idx(r[1], zmax, nz));
    }
    for (int q = 0; q < nsrc; q++)
        if ((int)cfg.src[q][2] != 0) {
            set_error("solver: source type " + std::to_string((int)cfg.src[q][2]) + " (only 0, Ricker)");
            return GB_ERR_ARG;
        }

    {
        int least = 0, greatest = 0;
        GB_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        GB_CUDA_TRY(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, greatest));
        GB_CUDA_TRY(cudaStreamCreateWithPriority(&st_side, cudaStreamNonBlocking, least));
    }
    for (cudaEvent_t *e : {&ev_pass0, &ev_pass1, &ev_win0, &ev_win1}) GB_CUDA_TRY(cudaEventCreate(e));
    for (cudaEvent_t *e : {&ev_round, &ev_side}) GB_CUDA_TRY(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    for (cudaEvent_t *e : {&ev_fpass0, &ev_fpass1}) GB_CUDA_TRY(cudaEventCreate(e));

    const size_t n = ncell();
    {
        int dev = 0, sms = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && sms > 0)
            num_sms = sms;
        (void)cudaGetLastError();
    }
    GB_CUDA_TRY(cudaMalloc(&lambda, n * 4));
    GB_CUDA_TRY(cudaMalloc(&mu, n * 4));
    GB_CUDA_TRY(cudaMalloc(&rho, n * 4));
    GB_CUDA_TRY(cudaMalloc(&rinv, n * 4));
    GB_CUDA_TRY(cudaMemset(lambda, 0, n * 4));
    GB_CUDA_TRY(cudaMemset(mu, 0, n * 4));
    GB_CUDA_TRY(cudaMemset(rho, 0, n * 4));
    if (adj) {
        GB_CUDA_TRY(cudaMalloc(&k_lambda, n * 4));
        GB_CUDA_TRY(cudaMalloc(&k_mu, n * 4));
        GB_CUDA_TRY(cudaMalloc(&k_rho, n * 4));
        GB_CUDA_TRY(cudaMemset(k_lambda, 0, n * 4));
        GB_CUDA_TRY(cudaMemset(k_mu, 0, n * 4));
        GB_CUDA_TRY(cudaMemset(k_rho, 0, n * 4));
    }
    // source time functions
    std::vector<float> hs[3];
    for (int c = 0; c < 3; c++) hs[c].assign((size_t)std::max(nsrc, 1) * nt, 0.f);
    for (int is = 0; is < nsrc; is++)
        ricker(nt, dt, &cfg.src[is][3], &hs[0][(size_t)is * nt], &hs[1][(size_t)is * nt], &hs[2][(size_t)is * nt]);
    for (int c = 0; c < 3; c++) {
        GB_CUDA_TRY(cudaMalloc(&stf[c], hs[c].size() * 4));
        GB_CUDA_TRY(cudaMemcpy(stf[c], hs[c].data(), hs[c].size() * 4, cudaMemcpyHostToDevice));
    }
    std::vector<float> hax, haz;
    absorbing_profiles(nx, nz, abs_width, abs_alpha, abs_left, abs_right, abs_bottom, abs_top, hax, haz);
    GB_CUDA_TRY(cudaMalloc(&ax, nx * 4));
    GB_CUDA_TRY(cudaMalloc(&az, nz * 4));
    GB_CUDA_TRY(cudaMemcpy(ax, hax.data(), nx * 4, cudaMemcpyHostToDevice));
    GB_CUDA_TRY(cudaMemcpy(az, haz.data(), nz * 4, cudaMemcpyHostToDevice));
    {
        std::vector<int> cells(2 * (size_t)std::max(nrec, 1), 0);
        std::vector<long long> keys;
        for (int r = 0; r < nrec; r++) {
            cells[r] = rec_xi[r];
            cells[nrec + r] = rec_zi[r];
            keys.push_back((long long)rec_xi[r] * (nz + 1) + rec_zi[r]);
        }
        std::sort(keys.begin(), keys.end());
        rec_distinct = std::adjacent_find(keys.begin(), keys.end()) == keys.end();
        GB_CUDA_TRY(cudaMalloc(&d_rec_cells, cells.size() * 4));
        GB_CUDA_TRY(cudaMemcpy(d_rec_cells, cells.data(), cells.size() * 4, cudaMemcpyHostToDevice));
    }
    GB_CUDA_TRY(cudaMalloc(&d_group, sizeof(KernelGroup)));
    GB_CUDA_TRY(cudaMallocHost(&h_group, sizeof(KernelGroup)));
    stats = gb_stats{};
    return GB_OK;
}

void Solver::release() {
    if (st) cudaStreamSynchronize(st);
    snapw.close();
    invalidate_graphs();
    for (auto &b : slots) {
        cudaFree(b.state);
        for (int c = 0; c < 3; c++) {
            cudaFree(b.out[c]);
            cudaFree(b.adstf[c]);
        }
        cudaFree(b.ckpt);
        cudaFree(b.amax);
        cudaFree(b.tmaps);
    }
    slots.clear();
    for (float *p : {lambda, mu, rho, rinv, k_lambda, k_mu, k_rho, stf[0], stf[1], stf[2], ax, az}) cudaFree(p);
    for (int q = 0; q < 3; q++) {
        cudaFree(d_slots[q]);
        cudaFreeHost(h_slots[q]);
    }
    cudaFree(d_tune);
    cudaFree(d_group);
    cudaFreeHost(h_group);
    cudaFree(d_csr);
    cudaFree(d_rec_cells);
    cudaFree(kpart);
    cudaFree(snapbuf);
    for (cudaEvent_t e : {ev_pass0, ev_pass1, ev_win0, ev_win1, ev_t0, ev_t1, ev_round, ev_side, ev_fpass0, ev_fpass1})
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : ev_fwd_round) cudaEventDestroy(e);
    for (cudaEvent_t e : ev_mis_round) cudaEventDestroy(e);
    ev_fwd_round.clear();
    ev_mis_round.clear();
    if (st_side) cudaStreamDestroy(st_side);
    st_side = nullptr;
    if (st) cudaStreamDestroy(st);
    st = nullptr;
}

void Solver::invalidate_graphs() {
    for (auto &g : graphs) cudaGraphExecDestroy(g.second.exec);
    graphs.clear();
}

// ---------------------------------------------------------------- model
int Solver::set_model_points(int npt, const float *px, const float *pz, const float *pa, const float *pb,
                             const float *pr) {
    if (npt <= 0 || !px || !pz || !pa || !pb || !pr) {
        set_error("model: empty point set");
        return GB_ERR_ARG;
    }
    const size_t n = ncell();
    // Fast path: when every cell has a model point at distance exactly 0
    // (all shipped examples store the grid itself), the reference's
    // nearest-point search (mesh2grid, solver/fdm.h:4-24) returns the first
    // such point, because 0 is the minimum and the comparison is strict.
    std::vector<int> first(n, -1);
    size_t hit = 0;
    for (int l = 0; l < npt; l++) {
        const long ii = lrintf(px[l] / dx), jj = lrintf(pz[l] / dz);
        for (long i = ii - 1; i <= ii + 1; i++) {
            for (long j = jj - 1; j <= jj + 1; j++) {
                if (i < 0 || j < 0 || i >= nx || j >= nz) continue;
                const float ddx = (float)i * dx - px[l], ddz = (float)j * dz - pz[l];
                if (ddx * ddx + ddz * ddz == 0.f) {
                    int &f = first[(size_t)i * nz + j];
                    if (f < 0) {
                        f = l;
                        hit++;
                    }
                }
            }
        }
    }
    if (hit == n) {
        std::vector<float> h[3];
        for (auto &v : h) v.resize(n);
        for (size_t k = 0; k < n; k++) {
            h[0][k] = pa[first[k]];
            h[1][k] = pb[first[k]];
            h[2][k] = pr[first[k]];
        }
        GB_CUDA_TRY(cudaMemcpyAsync(lambda, h[0].data(), n * 4, cudaMemcpyHostToDevice, st));
        GB_CUDA_TRY(cudaMemcpyAsync(mu, h[1].data(), n * 4, cudaMemcpyHostToDevice, st));
        GB_CUDA_TRY(cudaMemcpyAsync(rho, h[2].data(), n * 4, cudaMemcpyHostToDevice, st));
        GB_CUDA_TRY(cudaStreamSynchronize(st));
    } else {
        float *d[5];
        const float *hsrc[5] = {px, pz, pa, pb, pr};
        for (int q = 0; q < 5; q++) {
            GB_CUDA_TRY(cudaMalloc(&d[q], (size_t)npt * 4));
            GB_CUDA_TRY(cudaMemcpyAsync(d[q], hsrc[q], (size_t)npt * 4, cudaMemcpyHostToDevice, st));
        }
        const float dmax = xmax * xmax + zmax * zmax;
        GB_CUDA_TRY(launch_mesh2grid(lambda, mu, rho, d[0], d[1], d[2], d[3], d[4], npt, dmax, dx, dz, nx, nz, st));
        GB_CUDA_TRY(cudaStreamSynchronize(st));
        for (int q = 0; q < 5; q++) cudaFree(d[q]);
    }
    if (model_type == 0) {
        GB_CUDA_TRY(launch_vps2lm(lambda, mu, rho, n, st));
        GB_CUDA_TRY(cudaStreamSynchronize(st));
    }
    return GB_OK;
}

int Solver::import_model(bool model_true) {
    const std::string dir = path + "/" + (model_true ? "model_true" : "model_init") + "/proc000000_";
    const char *names0[5] = {"x", "z", "vp", "vs", "rho"};
    const char *names1[5] = {"x", "z", "lambda", "mu", "rho"};
    std::vector<float> v[5];
    for (int q = 0; q < 5; q++) {
        int rc = read_bin(dir + (model_type ? names1[q] : names0[q]) + ".bin", v[q]);
        if (rc) return rc;
        if (model_npt && (int)v[q].size() != model_npt) {
            set_error("error: invalid model (" + dir + (model_type ? names1[q] : names0[q]) + ".bin has " +
                      std::to_string(v[q].size()) + " points, expected " + std::to_string(model_npt) + ")");
            return GB_ERR_MODEL;
        }
    }
    return set_model_points((int)v[0].size(), v[0].data(), v[1].data(), v[2].data(), v[3].data(), v[4].data());
}

// ---------------------------------------------------------------- slots
size_t Solver::slot_bytes(int prec) const {
    const size_t n = ncell();
    size_t b = ((sh ? NSH : 0) + (psv ? NPSV : 0)) * n * 4;
    const int ncomp = (sh ? 1 : 0) + (psv ? 2 : 0);
    b += (size_t)ncomp * nrec * nt * 4 * (adj ? 2 : 1);
    if (adj && nsfe) b += (size_t)nsfe * nf(prec) * n * (prec == CKPT_F32 ? 4 : 2) + (size_t)nsfe * nf(prec) * 4;
    return b;
}

// cuTensorMapEncodeTiled through the runtime (no link against the driver
// library); null when the driver does not offer it.
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            (void)cudaGetLastError();
    }
    return fn;
}

// One field float[nx*nz] (k = i*nz + j) as a 2-D tensor {nz, nx}: a box is
// `rows` consecutive rows of TMAP_BOX_COLS consecutive columns, zero outside
// the grid.
static bool encode_field_map(void *out, const float *base, int nx, int nz, int pz, int rows) {
    const auto enc = tensor_map_encoder();
    if (!enc || !base || (reinterpret_cast<uintptr_t>(base) & 15) || pz % 4 || pz < nz || rows < 1 || rows > 256 ||
        rows % 4)
        return false;
    const cuuint64_t dims[2] = {(cuuint64_t)nz, (cuuint64_t)nx};
    const cuuint64_t strides[1] = {(cuuint64_t)pz * 4};
    const cuuint32_t box[2] = {(cuuint32_t)rows, (cuuint32_t)TMAP_BOX_COLS};
    const cuuint32_t estr[2] = {1, 1};
    return enc(static_cast<CUtensorMap *>(out), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(base), dims,
               strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Encodes the TMAP_N maps of a slot's state fields and the model (arrays of
// nx columns at pitch pz) for a box of `rows` rows into h (TMAP_N * TMAP_BYTES
// bytes); false when a field cannot be described. lambda may be null (SH).
bool encode_slot_maps(void *h, const float *state, bool sh, bool psv, const float *rinv, const float *mu,
                      const float *lambda, int nx, int nz, int pz, int rows) {
    static_assert(sizeof(CUtensorMap) == TMAP_BYTES, "tensor map size");
    CUtensorMap *m = static_cast<CUtensorMap *>(h);
    for (int q = 0; q < TMAP_N; q++) m[q] = CUtensorMap{};
    const size_t nc = (size_t)nx * pz;
    bool ok = true;
    const float *p = state;
    if (sh)
        for (int f = 0; f < NSH; f++) ok = ok && encode_field_map(&m[TMAP_SH + f], p + (size_t)f * nc, nx, nz, pz, rows);
    if (sh) p += (size_t)NSH * nc;
    if (psv)
        for (int f = 0; f < NPSV; f++) ok = ok && encode_field_map(&m[f], p + (size_t)f * nc, nx, nz, pz, rows);
    return ok && encode_field_map(&m[TMAP_RINV], rinv, nx, nz, pz, rows) &&
           encode_field_map(&m[TMAP_MU], mu, nx, nz, pz, rows) &&
           (!psv || encode_field_map(&m[TMAP_LAM], lambda, nx, nz, pz, rows));
}

// Space for a slot's tensor maps, for the marching kernel's bulk loads;
// tma_ok records whether its fields can be described (nz % 4 == 0, aligned
// buffers, driver support). The maps are encoded by refresh_tmaps.
int Solver::build_tmaps(SlotBuf &b) {
    std::vector<CUtensorMap> h(TMAP_N);
    if (!(nz % 4 == 0 && encode_slot_maps(h.data(), b.state, sh, psv, rinv, mu, lambda, nx, nz, nz, 32))) {
        tma_ok = false;
        return GB_OK;
    }
    GB_CUDA_TRY(cudaMalloc(&b.tmaps, sizeof(CUtensorMap) * TMAP_N));
    tmaps_T = 0;
    return GB_OK;
}

// Encodes every slot's maps for marching blocks of `threads` rows (the box
// height), ordered on the solver's stream after the kernels that read the
// previous ones. A no-op when they are current or bulk loads are off.
int Solver::refresh_tmaps(int threads) {
    if (!use_tma() || threads <= 0 || threads == tmaps_T) return GB_OK;
    std::vector<CUtensorMap> h(TMAP_N);
    for (auto &b : slots) {
        if (!b.tmaps || !encode_slot_maps(h.data(), b.state, sh, psv, rinv, mu, lambda, nx, nz, nz, threads)) {
            set_error("tensor maps: a field cannot be described for bulk loads");
            return GB_ERR_STATE;
        }
        GB_CUDA_TRY(cudaMemcpyAsync(b.tmaps, h.data(), sizeof(CUtensorMap) * TMAP_N, cudaMemcpyHostToDevice, st));
    }
    tmaps_T = threads;
    return GB_OK;
}

int Solver::ensure_slots(int n) {
    if (capacity == 0) {
        size_t freeb = 0, totalb = 0;
        GB_CUDA_TRY(cudaMemGetInfo(&freeb, &totalb));
        double budget = opt_budget_gb > 0 ? opt_budget_gb * 1e9 : 0.85 * (double)freeb;
        long cap = (long)(budget / (double)slot_bytes(opt_ckpt));
        cap = std::min<long>(cap, std::max(nsrc, 1));
        cap = std::min<long>(cap, 256);
        if (opt_batch > 0) cap = std::min<long>(cap, opt_batch);
        if (cap < 1) {
            set_error("solver: one shot needs " + std::to_string(slot_bytes(opt_ckpt)) +
                      " bytes, more than the HBM budget");
            return GB_ERR_BUDGET;
        }
        // equal batches: as many as the budget needs, as even as possible
        // (64 shots at a budget of 60 run as 32 + 32, not 60 + 4, whose small
        // batch fills the GPU poorly)
        if (cap < nsrc) {
            const long nb = (nsrc + cap - 1) / cap;
            cap = (nsrc + nb - 1) / nb;
        }
        capacity = (int)cap;
        for (int q = 0; q < 3; q++) {
            GB_CUDA_TRY(cudaMalloc(&d_slots[q], sizeof(Slot) * capacity));
            GB_CUDA_TRY(cudaMallocHost(&h_slots[q], sizeof(Slot) * capacity));
            memset(h_slots[q], 0, sizeof(Slot) * capacity);
        }
        GB_CUDA_TRY(cudaMalloc(&d_tune, sizeof(Slot) * capacity));
        stats.batch_capacity = capacity;
    }
    if (n > capacity) {
        set_error("solver: batch of " + std::to_string(n) + " exceeds capacity " + std::to_string(capacity));
        return GB_ERR_BUDGET;
    }
    const size_t nc = ncell();
    while ((int)slots.size() < n) {
        SlotBuf b;
        b.state_floats = ((sh ? NSH : 0) + (psv ? NPSV : 0)) * nc;
        GB_CUDA_TRY(cudaMalloc(&b.state, b.state_floats * 4));
        const size_t tr = (size_t)nrec * nt;
        for (int c = 0; c < 3; c++) {
            const bool used = c == 1 ? sh : psv;
            if (!used || tr == 0) continue;
            GB_CUDA_TRY(cudaMalloc(&b.out[c], tr * 4));
            GB_CUDA_TRY(cudaMemset(b.out[c], 0, tr * 4));
            if (adj) {
                GB_CUDA_TRY(cudaMalloc(&b.adstf[c], tr * 4));
                GB_CUDA_TRY(cudaMemset(b.adstf[c], 0, tr * 4));
            }
        }
        if (slots.empty()) tma_ok = true;  // until a slot's maps fail
        int rc = build_tmaps(b);
        if (rc) return rc;
        slots.push_back(b);
    }
    if (adj && nsfe) {
        for (int q = 0; q < n; q++) {
            SlotBuf &b = slots[q];
            if (b.ckpt_prec == opt_ckpt) continue;
            cudaFree(b.ckpt);
            cudaFree(b.amax);
            const size_t elems = (size_t)nsfe * nf(opt_ckpt) * nc;
            GB_CUDA_TRY(cudaMalloc(&b.ckpt, elems * (opt_ckpt == CKPT_F32 ? 4 : 2)));
            GB_CUDA_TRY(cudaMalloc(&b.amax, (size_t)nsfe * nf(opt_ckpt) * 4));
            b.ckpt_prec = opt_ckpt;
            invalidate_graphs();
        }
    }
    return GB_OK;
}

int Solver::ensure_tables() {
    if (d_csr && tile_id == (opt_tile ? opt_tile : tile_id) && tile_id != 0) return GB_OK;
    if (opt_tile) tile_id = opt_tile;
    if (tile_id == 0) tile_id = 1;
    tile = kTiles[tile_id];
    std::vector<int> all;
    auto add = [&](const std::vector<int> &v) {
        size_t off = all.size();
        all.insert(all.end(), v.begin(), v.end());
        return off;
    };
    src_set.clear();
    PointSet every;
    for (int is = 0; is < nsrc; is++) {
        PointSet one;
        one.i = {src_xi[is]};
        one.j = {src_zi[is]};
        one.trace = {is};
        src_set.push_back(add(build_csr(one, nx, nz, tile, true)));
        every.i.push_back(src_xi[is]);
        every.j.push_back(src_zi[is]);
        every.trace.push_back(is);
    }
    super_set = add(build_csr(every, nx, nz, tile, true));
    PointSet recs;
    recs.i = rec_xi;
    recs.j = rec_zi;
    for (int ir = 0; ir < nrec; ir++) recs.trace.push_back(ir);
    rec_inj_set = add(build_csr(recs, nx, nz, tile, true));
    rec_rec_set = add(build_csr(recs, nx, nz, tile, false));
    if (d_csr) {
        GB_CUDA_TRY(cudaStreamSynchronize(st));
        cudaFree(d_csr);
    }
    csr_words = all.size();
    GB_CUDA_TRY(cudaMalloc(&d_csr, csr_words * 4));
    GB_CUDA_TRY(cudaMemcpy(d_csr, all.data(), csr_words * 4, cudaMemcpyHostToDevice));
    stats.tile_tz = tile.tz;
    stats.tile_tx = tile.tx;
    return GB_OK;
}

int Solver::fill_slots(int kind, const int *shots, int n, bool record_u) {
    Slot *hs = h_slots[kind];
    const size_t nc = ncell();
    for (int b = 0; b < capacity; b++) {
        Slot &S = hs[b];
        memset(&S, 0, sizeof(Slot));
        if (b >= n) continue;
        const SlotBuf &B = slots[b];
        S.nx = nx;
        S.nz = nz;
        S.pz = nz;
        S.nt = nt;
        S.tiles_z = (nz + tile.tz - 1) / tile.tz;
        S.tiles_x = (nx + tile.tx - 1) / tile.tx;
        S.active = 1;
        S.dt = dt;
        S.c9x = 9.f / (8.f * dx);
        S.c24x = 1.f / (24.f * dx);
        S.c9z = 9.f / (8.f * dz);
        S.c24z = 1.f / (24.f * dz);
        S.lambda = lambda;
        S.mu = mu;
        S.rho = rho;
        S.rinv = rinv;
        S.ax = ax;
        S.az = az;
        float *p = B.state;
        if (sh) {
            for (int f = 0; f < NSH; f++) S.sh[f] = p + (size_t)f * nc;
            p += (size_t)NSH * nc;
        }
        if (psv)
            for (int f = 0; f < NPSV; f++) S.psv[f] = p + (size_t)f * nc;
        S.tmap = tma_ok ? B.tmaps : nullptr;
        S.it_base = 0;
        S.par0 = 0;
        S.pts_i = d_rec_cells;
        S.pts_j = d_rec_cells + nrec;
        S.npts = nrec;
        S.src_trace = -1;
        S.sfe = sfe;
        S.ckpt_write = kind == PASS_FWD;
        S.nsfe = nsfe;
        S.ckpt_prec = B.ckpt_prec < 0 ? CKPT_F32 : B.ckpt_prec;
        S.nf = nf(S.ckpt_prec);
        if (kind == PASS_ADJ) {
            S.inj = d_csr + rec_inj_set;
            S.inj_x = B.adstf[0];
            S.inj_y = B.adstf[1];
            S.inj_z = B.adstf[2];
            S.ckpt = B.ckpt;
            S.ckpt_amax = B.amax;
        } else {
            const int is = shots[b];
            S.inj = nsrc ? d_csr + (is >= 0 ? src_set[is] : super_set) : nullptr;
            if (is >= 0 && nsrc) {
                S.src_i = src_xi[is];
                S.src_j = src_zi[is];
                S.src_trace = is;
            }
            S.inj_x = stf[0];
            S.inj_y = stf[1];
            S.inj_z = stf[2];
            S.rec = nrec ? d_csr + rec_rec_set : nullptr;
            S.out_x = B.out[0];
            S.out_y = B.out[1];
            S.out_z = B.out[2];
            S.record_u = record_u;
            if (kind == PASS_FWD) {
                S.ckpt = B.ckpt;
                S.ckpt_amax = B.amax;
            }
        }
    }
    GB_CUDA_TRY(cudaMemcpyAsync(d_slots[kind], hs, sizeof(Slot) * capacity, cudaMemcpyHostToDevice, st));
    return GB_OK;
}

// Records a timing event on st. Inside a stream capture a plain record only
// marks a dependency; the external flag makes it a timestamped event node
// (and is rejected outside a capture).
cudaError_t Solver::record_timing(cudaEvent_t e) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t err = cudaStreamIsCapturing(st, &cs);
    if (err != cudaSuccess) return err;
    return cs == cudaStreamCaptureStatusActive ? cudaEventRecordWithFlags(e, st, cudaEventRecordExternal)
                                               : cudaEventRecord(e, st);
}

// Enqueues one pass on st (also used inside graph capture).
int Solver::enqueue_pass(int kind, int n, bool snapshot, int snap_isrc) {
    const size_t nc = ncell();
    const Slot *ds = d_slots[kind];
    for (int b = 0; b < n; b++) GB_CUDA_TRY(cudaMemsetAsync(slots[b].state, 0, slots[b].state_floats * 4, st));
    const bool ck = kind == PASS_FWD && adj && nsfe > 0;
    const bool q16 = ck && opt_ckpt != CKPT_F32;
    if (q16)
        for (int b = 0; b < n; b++) GB_CUDA_TRY(cudaMemsetAsync(slots[b].amax, 0, (size_t)nsfe * nf(opt_ckpt) * 4, st));
    // timing window: consecutive steps with no other kernel between them
    int w0 = 0, w1 = std::min(nt, 64);
    if (ck) w1 = std::min(w1, sfe - 1);
    if (kind == PASS_ADJ) {
        w0 = std::min(1, nt);
        w1 = std::min(nt, std::min(w0 + 64, sfe > 0 ? sfe : nt));
    }
    if (w1 <= w0) w1 = w0;  // empty window: not timed
    win_steps = w1 - w0;
    const int nwave = (sh ? 1 : 0) + (psv ? 1 : 0);
    int par = 0;
    for (int it = 0; it < nt; it++) {
        int isfe = -1;
        if (ck && (it + 1) % sfe == 0) isfe = nsfe - (it + 1) / sfe;
        if (isfe >= 0) {
            for (int w = 0; w < 2; w++) {
                const bool wp = w == 1;
                if (wp ? !psv : !sh) continue;
                if (q16) GB_CUDA_TRY(launch_ckpt_amax(ds, n, (int)nc, it, 1, wp, st));
                GB_CUDA_TRY(launch_ckpt_store(ds, n, (int)nc, it, 1, wp, st));
                stats.launches += q16 ? 2 : 1;
            }
        }
        if (it == w0 && win_steps > 0) GB_CUDA_TRY(record_timing(ev_win0));
        if (sh) GB_CUDA_TRY(launch_step(false, tile, ds, n, max_tiles(), it, use_tma(), st));
        if (psv) GB_CUDA_TRY(launch_step(true, tile, ds, n, max_tiles(), it, use_tma(), st));
        stats.launches += nwave;
        if (it + 1 == w1 && win_steps > 0) GB_CUDA_TRY(record_timing(ev_win1));
        par ^= 1;
        if (isfe >= 0) {
            for (int w = 0; w < 2; w++) {
                const bool wp = w == 1;
                if (wp ? !psv : !sh) continue;
                if (q16) GB_CUDA_TRY(launch_ckpt_amax(ds, n, (int)nc, it, 0, wp, st));
                GB_CUDA_TRY(launch_ckpt_store(ds, n, (int)nc, it, 0, wp, st));
                stats.launches += q16 ? 2 : 1;
            }
        }
        if (kind == PASS_ADJ && sfe > 0 && it % sfe == 0) {
            if (sh) GB_CUDA_TRY(launch_interaction(false, ds, d_group, 1, (int)nc, it, st));
            if (psv) GB_CUDA_TRY(launch_interaction(true, ds, d_group, 1, (int)nc, it, st));
            stats.launches += nwave;
        }
        if (snapshot) {
            int rc = export_snapshot(it, snap_isrc, par);
            if (rc) return rc;
        }
    }
    last_par = par;
    stats.cell_updates += (long long)nc * nt * n;
    return GB_OK;
}

int Solver::autotune(int n) {
    GB_CUDA_TRY(launch_reciprocal(rinv, rho, ncell(), st));
    // Times every tile shape on the real batch (sources and receivers off,
    // results discarded) and keeps the fastest; the shape does not change
    // any computed value.
    Slot *hs = h_slots[PASS_FWD_NOCKPT];
    std::vector<Slot> tmp(hs, hs + capacity);
    for (int b = 0; b < capacity; b++) {
        tmp[b].inj = nullptr;
        tmp[b].rec = nullptr;
    }
    float best = 1e30f;
    int best_id = 1;
    for (int id = 1; id <= kNumTiles; id++) {
        TileCfg tc = kTiles[id];
        for (int b = 0; b < n; b++) {
            tmp[b].tiles_z = (nz + tc.tz - 1) / tc.tz;
            tmp[b].tiles_x = (nx + tc.tx - 1) / tc.tx;
        }
        GB_CUDA_TRY(cudaMemcpyAsync(d_tune, tmp.data(), sizeof(Slot) * capacity, cudaMemcpyHostToDevice, st));
        if (tc.threads) {
            const int rc = refresh_tmaps(tc.threads);
            if (rc) return rc;
        }
        const int mt = ((nz + tc.tz - 1) / tc.tz) * ((nx + tc.tx - 1) / tc.tx);
        const int reps = 8;
        for (int r = 0; r < 3 + reps; r++) {
            if (r == 3) GB_CUDA_TRY(cudaEventRecord(ev_win0, st));
            if (sh) GB_CUDA_TRY(launch_step(false, tc, d_tune, n, mt, r, use_tma(), st));
            if (psv) GB_CUDA_TRY(launch_step(true, tc, d_tune, n, mt, r, use_tma(), st));
        }
        GB_CUDA_TRY(cudaEventRecord(ev_win1, st));
        GB_CUDA_TRY(cudaEventSynchronize(ev_win1));
        if (tc.threads && use_tma() && march_tma_error()) {
            set_error("marching kernel: a bulk-load wait ran out of iterations while tuning");
            return GB_ERR_CUDA;
        }
        float ms = 0;
        GB_CUDA_TRY(cudaEventElapsedTime(&ms, ev_win0, ev_win1));
        if (ms < best) {
            best = ms;
            best_id = id;
        }
    }
    tile_id = best_id;
    opt_tile = 0;
    return GB_OK;
}

int Solver::run_pass(int kind, int n, bool snapshot, int snap_isrc) {
    if (tile.threads) {
        const int rc = refresh_tmaps(tile.threads);
        if (rc) return rc;
    }
    GB_CUDA_TRY(cudaEventRecord(ev_pass0, st));
    GB_CUDA_TRY(launch_reciprocal(rinv, rho, ncell(), st));
    stats.launches += 1;
    if (opt_graphs && !snapshot) {
        auto key = std::make_pair(kind, n);
        auto g = graphs.find(key);
        if (g == graphs.end()) {
            const long long l0 = stats.launches, c0 = stats.cell_updates;
            GB_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            int rc = enqueue_pass(kind, n, false, -1);
            cudaGraph_t graph = nullptr;
            cudaError_t e = cudaStreamEndCapture(st, &graph);
            GraphInfo info;
            info.launches = stats.launches - l0;
            info.win_steps = win_steps;
            stats.launches = l0;
            stats.cell_updates = c0;
            if (rc) {
                if (graph) cudaGraphDestroy(graph);
                return rc;
            }
            GB_CUDA_TRY(e);
            e = cudaGraphInstantiate(&info.exec, graph, 0);
            cudaGraphDestroy(graph);
            GB_CUDA_TRY(e);
            g = graphs.emplace(key, info).first;
        }
        GB_CUDA_TRY(cudaGraphLaunch(g->second.exec, st));
        stats.launches += g->second.launches;
        stats.cell_updates += (long long)ncell() * nt * n;
        win_steps = g->second.win_steps;
        last_par = nt & 1;
    } else {
        int rc = enqueue_pass(kind, n, snapshot, snap_isrc);
        if (rc) return rc;
    }
    GB_CUDA_TRY(cudaEventRecord(ev_pass1, st));
    GB_CUDA_TRY(cudaStreamSynchronize(st));
    if (snapshot && opt_snap_async) {
        std::string msg;
        const int rc = snapw.drain(&msg);
        if (rc) {
            set_error("snapshot export: " + msg);
            return rc;
        }
    }
    if (tile.threads) stats.march_bulk = use_tma() ? 1 : 0;
    if (use_tma() && tile.threads && march_tma_error()) {
        set_error("marching kernel: a bulk-load wait ran out of iterations; the pass is invalid");
        return GB_ERR_CUDA;
    }
    float ms = 0;
    GB_CUDA_TRY(cudaEventElapsedTime(&ms, ev_pass0, ev_pass1));
    if (kind == PASS_ADJ)
        stats.adjoint_ms += ms;
    else
        stats.forward_ms += ms;
    if (win_steps > 0) {
        float wm = 0;
        if (cudaEventElapsedTime(&wm, ev_win0, ev_win1) == cudaSuccess) {
            stats.step_ms += wm;
            stats.step_launches += win_steps;
        } else {
            (void)cudaGetLastError();  // timing is best effort; clear the error
        }
    }
    return GB_OK;
}

// Cluster geometry for one wave system: R CTAs per shot, each holding
// cols_per columns of the state (plus ghost columns) in shared memory. The
// cost model is the per-SM work of one step (cells per CTA plus a barrier
// allowance) times the number of cluster rounds the batch needs.
bool Solver::cluster_geometry(bool wave_psv, int n, ClusterGeom *out) const {
    if (nx < 2 || nz < 1) return false;
    const long long key =
        ((((long long)n * 32 + opt_cluster) * 32 + opt_cluster_qm) * 2 + (wave_psv ? 1 : 0)) * 2 + (opt_shift ? 1 : 0);
    const auto hit = cluster_cache.find(key);
    if (hit != cluster_cache.end()) {
        if (hit->second.first) *out = hit->second.second;
        return hit->second.first;
    }
    static const bool trace = std::getenv("GBFWI_TRACE") != nullptr;  // print the candidates to stderr
    const size_t limit = 227 * 1024 - 64;  // dynamic shared memory, beside the kernel's static counter
    double best = -1;
    const int rlo = opt_cluster >= 2 ? opt_cluster : 1, rhi = opt_cluster >= 2 ? opt_cluster : 16;
    for (int R = rlo; R <= rhi; R++) {
        for (int qm : {4, 8, 10, 12, 16, 20, 24}) {
            if (opt_cluster_qm && qm != opt_cluster_qm) continue;
            ClusterGeom g{};
            g.R = R;
            g.qmax = qm;
            g.cols_per = ((nx + R - 1) / R + qm - 1) / qm * qm;
            g.G = g.cols_per / qm;
            if (nx - (R - 1) * g.cols_per < 2 || (long)g.G * nz > cluster_max_threads(wave_psv, qm)) continue;
            std::vector<int> per(R, 0);
            for (int r = 0; r < nrec; r++)
                if (rec_xi[r] >= 0 && rec_xi[r] < nx && rec_zi[r] >= 0 && rec_zi[r] < nz)
                    per[rec_xi[r] / g.cols_per]++;
            g.nrec_cta = *std::max_element(per.begin(), per.end());
            // with the row-shifted layout first (conflict-free shared
            // accesses; ties keep it), then without
            for (int shifted = opt_shift ? 1 : 0; shifted >= 0; shifted--) {
                cluster_layout(g, nz, shifted != 0);
                if (cluster_smem_bytes(wave_psv, g, nz) > limit) continue;
                const int occ = cluster_occupancy(wave_psv, g, nz);
                if (occ < 1) {
                    if (trace)
                        std::fprintf(stderr, "gbfwi cluster %s R=%d cols=%d qmax=%d threads=%d shift=%d smem=%zu: no fit\n",
                                     wave_psv ? "psv" : "sh", R, g.cols_per, g.qmax, g.G * nz, g.dshift,
                                     cluster_smem_bytes(wave_psv, g, nz));
                    continue;
                }
                // per-step time ~ cells per SM (CTAs sharing an SM add up) plus a
                // barrier allowance, times the rounds the batch needs
                const int resident = std::min(n, occ);
                const int per_sm = (R * resident + num_sms - 1) / num_sms;
                const double cost =
                    (double)((n + occ - 1) / occ) * ((double)std::max(per_sm, 1) * g.cols_per * nz + 6000.0);
                if (trace)
                    std::fprintf(stderr,
                                 "gbfwi cluster %s R=%d cols=%d qmax=%d threads=%d shift=%d smem=%zu clusters=%d cost=%.0f\n",
                                 wave_psv ? "psv" : "sh", R, g.cols_per, g.qmax, g.G * nz, g.dshift,
                                 cluster_smem_bytes(wave_psv, g, nz), occ, cost);
                if (best < 0 || cost < best) {
                    best = cost;
                    *out = g;
                }
            }
        }
    }
    cluster_cache[key] = {best >= 0, best >= 0 ? *out : ClusterGeom{}};
    return best >= 0;
}

bool Solver::cluster_ok(const int *shots, int n, bool snapshot) const {
    // receiver ids are held as 16-bit values inside the kernel
    if (!opt_cluster || snapshot || !rec_distinct || opt_ckpt != CKPT_F32 || nrec >= 0xffff) return false;
    for (int b = 0; b < n; b++)
        if (shots[b] < 0) return false;
    ClusterGeom g{};
    if (sh && !cluster_geometry(false, n, &g)) return false;
    if (psv && !cluster_geometry(true, n, &g)) return false;
    return true;
}

// One pass with the cluster-resident kernel: one launch per wave system.
int Solver::run_cluster_pass(int kind, int n) {
    const size_t nc = ncell();
    const bool adjp = kind == PASS_ADJ;
    const bool pipe_fwd = pipe_on && !adjp && pipe_rounds > 1;  // returns without waiting
    GB_CUDA_TRY(cudaEventRecord(pipe_fwd ? ev_fpass0 : ev_pass0, st));
    GB_CUDA_TRY(launch_reciprocal(rinv, rho, nc, st));
    stats.launches += 1;
    if (adjp) {
        if (kpart_slots < (size_t)n) {
            GB_CUDA_TRY(cudaStreamSynchronize(st));
            cudaFree(kpart);
            GB_CUDA_TRY(cudaMalloc(&kpart, (size_t)n * 3 * nc * 4));
            kpart_slots = n;
        }
        GB_CUDA_TRY(cudaMemsetAsync(kpart, 0, (size_t)n * 3 * nc * 4, st));
    }
    // adjoint: store the adjoint state at every accumulation step and
    // accumulate the kernels after the pass, in one fully parallel kernel,
    // when the state of every step fits in a quarter of the free device
    // memory (as much memory as the FP32 checkpoints); else accumulate in
    // the pass, where each thread's columns wait on memory one after another
    float *snap = nullptr;
    if (adjp && opt_snap && nsfe > 0) {
        const size_t need = (size_t)n * nsfe * (psv ? 4 : 2) * nc * 4;
        if (need > snap_bytes) {
            size_t free_b = 0, total_b = 0;
            GB_CUDA_TRY(cudaStreamSynchronize(st));
            cudaFree(snapbuf);
            snapbuf = nullptr;
            snap_bytes = 0;
            if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && need <= free_b / 4) {
                if (cudaMalloc(&snapbuf, need) == cudaSuccess)
                    snap_bytes = need;
                else
                    (void)cudaGetLastError();
            }
        }
        if (snap_bytes >= need) snap = snapbuf;
    }
    for (int w = 0; w < 2; w++) {
        const bool wp = w == 1;
        if (wp ? !psv : !sh) continue;
        ClusterGeom g{};
        if (!cluster_geometry(wp, n, &g)) {
            set_error("cluster pass: no geometry fits");
            return GB_ERR_STATE;
        }
        // adjoint: keep the shot's kernels in shared memory for the whole
        // pass, and stage each checkpoint there, when that fits without
        // adding cluster rounds for this batch (the accumulators first). The
        // accumulators are left in HBM when they would take the shared memory
        // past 200 KB: the L1 left beside it no longer holds the lines the
        // accumulation's checkpoint reads share (C2: 13.75 against 13.13 us
        // per adjoint step at 229 KB), and the row-shifted layout is worth
        // more than the accumulators (14.08 us unshifted with them).
        const int occ0 = (adjp && !snap) ? std::max(1, cluster_occupancy(wp, g, nz)) : 1;
        const int rounds = (n + occ0 - 1) / occ0;
        auto fits = [&](const ClusterGeom &h) {
            if (cluster_smem_bytes(wp, h, nz) > 227 * 1024 - 64) return false;
            const int occ = cluster_occupancy(wp, h, nz);
            return occ > 0 && (n + occ - 1) / occ <= rounds;
        };
        if (adjp && !snap && opt_kacc) {
            ClusterGeom gk = g;
            gk.kacc = 1;
            if (cluster_smem_bytes(wp, gk, nz) <= 200 * 1024 && fits(gk)) g.kacc = 1;
        }
        if (adjp && !snap && opt_stage && opt_ckpt == CKPT_F32) {
            ClusterGeom gs = g;
            gs.stage = 1;
            if (fits(gs)) g.stage = 1;
        }
        // the same values as every slot's (fill_slots)
        g.nx = nx;
        g.nz = nz;
        g.nt = nt;
        g.dt = dt;
        g.c9x = 9.f / (8.f * dx);
        g.c24x = 1.f / (24.f * dx);
        g.c9z = 9.f / (8.f * dz);
        g.c24z = 1.f / (24.f * dz);
        if (snap) {
            // one launch per round of resident clusters; the kernel
            // accumulation of a finished round runs on the side stream, on
            // the SMs that the next round's clusters leave free (C2: 96 of
            // 152 in use), so only the last round's waits for it
            const int occ = std::max(1, cluster_occupancy(wp, g, nz));
            const size_t snap_slot = (size_t)nsfe * (wp ? 4 : 2) * nc;
            for (int b0 = 0; b0 < n; b0 += occ) {
                const int nb = std::min(occ, n - b0);
                float *sp = snap + (size_t)b0 * snap_slot, *kp = kpart + (size_t)b0 * 3 * nc;
                // pipelined: this round's shots need their own misfit only
                if (pipe_on && pipe_rounds > 1)
                    for (int r = b0 / pipe_occ; r <= (b0 + nb - 1) / pipe_occ && r < pipe_rounds; r++)
                        GB_CUDA_TRY(cudaStreamWaitEvent(st, ev_mis_round[r], 0));
                GB_CUDA_TRY(launch_cluster(wp, adjp, d_slots[kind] + b0, nb, g, nz, kp, sp, st));
                GB_CUDA_TRY(cudaEventRecord(ev_round, st));
                GB_CUDA_TRY(cudaStreamWaitEvent(st_side, ev_round, 0));
                GB_CUDA_TRY(launch_snap_interaction(wp, d_slots[kind] + b0, nb, sp, g, kp, st_side));
                stats.launches += 2;
            }
            GB_CUDA_TRY(cudaEventRecord(ev_side, st_side));
            GB_CUDA_TRY(cudaStreamWaitEvent(st, ev_side, 0));
        } else if (pipe_fwd) {
            // one launch per round; the caller's misfit of a round starts on
            // the side stream once the round's event has fired
            for (int r = 0, b0 = 0; b0 < n; r++, b0 += pipe_occ) {
                const int nb = std::min(pipe_occ, n - b0);
                GB_CUDA_TRY(launch_cluster(wp, false, d_slots[kind] + b0, nb, g, nz, nullptr, nullptr, st));
                GB_CUDA_TRY(cudaEventRecord(ev_fwd_round[r], st));
                stats.launches += 1;
            }
        } else {
            if (adjp && pipe_on && pipe_rounds > 1)
                for (int r = 0; r < pipe_rounds; r++) GB_CUDA_TRY(cudaStreamWaitEvent(st, ev_mis_round[r], 0));
            GB_CUDA_TRY(launch_cluster(wp, adjp, d_slots[kind], n, g, nz, adjp ? kpart : nullptr, nullptr, st));
            stats.launches += 1;
        }
        if (adjp) {
            GB_CUDA_TRY(launch_cluster_reduce(kpart, n, nc, k_lambda, k_mu, k_rho, wp && inv_lambda, inv_mu, inv_rho,
                                              st));
            GB_CUDA_TRY(cudaMemsetAsync(kpart, 0, (size_t)n * 3 * nc * 4, st));
            stats.launches += 1;
        }
        stats.tile_tz = -g.R;
        stats.tile_tx = g.cols_per;
        if (adjp) stats.cluster_adj = (g.stage ? 1 : 0) | (g.kacc ? 2 : 0) | (snap ? 4 : 0);
        stats.cluster_shift = g.dshift;
    }
    stats.cell_updates += (long long)nc * nt * n;
    last_par = nt & 1;
    if (pipe_fwd) {
        GB_CUDA_TRY(cudaEventRecord(ev_fpass1, st));
        fpass_pending = true;
        return GB_OK;
    }
    GB_CUDA_TRY(cudaEventRecord(ev_pass1, st));
    GB_CUDA_TRY(cudaStreamSynchronize(st));
    if (cluster_wait_error()) {
        set_error("cluster pass: a ghost-column wait ran out of iterations; the pass is invalid");
        return GB_ERR_CUDA;
    }
    float ms = 0;
    GB_CUDA_TRY(cudaEventElapsedTime(&ms, ev_pass0, ev_pass1));
    if (adjp)
        stats.adjoint_ms += ms;
    else
        stats.forward_ms += ms;
    // the whole pass is one kernel per system: book it as nt steps
    stats.step_ms += ms;
    stats.step_launches += nt;
    return book_forward_pass();
}

// the forward pass of a pipelined gradient, booked once it has finished
int Solver::book_forward_pass() {
    if (!fpass_pending) return GB_OK;
    GB_CUDA_TRY(cudaEventSynchronize(ev_fpass1));
    if (cluster_wait_error()) {
        fpass_pending = false;
        set_error("cluster pass: a ghost-column wait ran out of iterations; the pass is invalid");
        return GB_ERR_CUDA;
    }
    float ms = 0;
    GB_CUDA_TRY(cudaEventElapsedTime(&ms, ev_fpass0, ev_fpass1));
    stats.forward_ms += ms;
    stats.step_ms += ms;
    stats.step_launches += nt;
    fpass_pending = false;
    return GB_OK;
}

int Solver::pipe_plan(const int *shots, int n) {
    pipe_rounds = pipe_occ = 0;
    if (!opt_pipe || sh == psv || !adj || nsfe <= 0 || !cluster_ok(shots, n, false)) return 0;
    ClusterGeom g{};
    if (!cluster_geometry(psv, n, &g)) return 0;
    const int occ = cluster_occupancy(psv, g, nz);
    if (occ < 1 || occ >= n) return 0;
    const int rounds = (n + occ - 1) / occ;
    while ((int)ev_fwd_round.size() < rounds) {
        cudaEvent_t a = nullptr, b = nullptr;
        if (cudaEventCreateWithFlags(&a, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&b, cudaEventDisableTiming) != cudaSuccess) {
            (void)cudaGetLastError();  // no pipelining without its events
            if (a) cudaEventDestroy(a);
            return 0;
        }
        ev_fwd_round.push_back(a);
        ev_mis_round.push_back(b);
    }
    pipe_occ = occ;
    pipe_rounds = rounds;
    return rounds;
}

int Solver::forward(const int *shots, int n, bool ckpt_on, bool record_u, bool snapshot) {
    if (n < 1) return GB_OK;
    for (int b = 0; b < n; b++)
        if (shots[b] >= nsrc || (shots[b] < 0 && nsrc == 0)) {
            set_error("forward: shot index " + std::to_string(shots[b]) + " out of range");
            return GB_ERR_ARG;
        }
    int rc = ensure_slots(n);
    if (rc) return rc;
    // the tile configuration is tuned on the first pass that uses the per-step kernels
    if (opt_tile == 0 && !tuned && !cluster_ok(shots, n, snapshot)) {
        rc = ensure_tables();
        if (rc) return rc;
        rc = fill_slots(PASS_FWD_NOCKPT, shots, n, record_u);
        if (rc) return rc;
        rc = autotune(n);
        if (rc) return rc;
        tuned = true;
        cudaFree(d_csr);
        d_csr = nullptr;
        invalidate_graphs();
    }
    if (opt_tile && opt_tile != tile_id) {
        cudaStreamSynchronize(st);
        cudaFree(d_csr);
        d_csr = nullptr;
        invalidate_graphs();
    }
    rc = ensure_tables();
    if (rc) return rc;
    const int kind = (ckpt_on && adj && nsfe) ? PASS_FWD : PASS_FWD_NOCKPT;
    rc = fill_slots(kind, shots, n, record_u);
    if (rc) return rc;
    last_forward_n = n;
    if (cluster_ok(shots, n, snapshot)) return run_cluster_pass(kind, n);
    return run_pass(kind, n, snapshot, -1);
}

int Solver::adjoint(const int *shots, int n, bool snapshot, int snap_isrc) {
    if (n < 1) return GB_OK;
    if (!adj) {
        set_error("adjoint: solver was created for a mode without adjoint (mode 0 or 2 needed)");
        return GB_ERR_STATE;
    }
    if (sfe <= 0 || nt % sfe != 0) {
        set_error("adjoint: nt (" + std::to_string(nt) + ") must be a positive multiple of sfe (" +
                  std::to_string(sfe) + "); the reference reads past its checkpoints otherwise");
        return GB_ERR_ARG;
    }
    int rc = ensure_slots(n);
    if (rc) return rc;
    rc = ensure_tables();
    if (rc) return rc;
    rc = fill_slots(PASS_ADJ, shots, n, false);
    if (rc) return rc;
    KernelGroup &G = *h_group;
    G.k_lambda = k_lambda;
    G.k_mu = k_mu;
    G.k_rho = k_rho;
    G.inv_lambda = inv_lambda;
    G.inv_mu = inv_mu;
    G.inv_rho = inv_rho;
    G.first = 0;
    G.count = n;
    G.nx = nx;
    G.nz = nz;
    GB_CUDA_TRY(cudaMemcpyAsync(d_group, h_group, sizeof(KernelGroup), cudaMemcpyHostToDevice, st));
    if (cluster_ok(shots, n, snapshot)) return run_cluster_pass(PASS_ADJ, n);
    return run_pass(PASS_ADJ, n, snapshot, snap_isrc);
}

int Solver::init_kernels() {
    if (!adj) return GB_OK;
    const size_t n = ncell() * 4;
    GB_CUDA_TRY(cudaMemsetAsync(k_lambda, 0, n, st));
    GB_CUDA_TRY(cudaMemsetAsync(k_mu, 0, n, st));
    GB_CUDA_TRY(cudaMemsetAsync(k_rho, 0, n, st));
    GB_CUDA_TRY(cudaStreamSynchronize(st));
    return GB_OK;
}

// ---------------------------------------------------------------- export
int Solver::export_data(const std::string &comp, const float *d_data, int n) {
    std::vector<float> h(ncell());
    GB_CUDA_TRY(cudaMemcpyAsync(h.data(), d_data, ncell() * 4, cudaMemcpyDeviceToHost, st));
    GB_CUDA_TRY(cudaStreamSynchronize(st));
    return write_bin(path + "/output/proc" + pad6(n) + "_" + comp + ".bin", h.data(), ncell());
}

// One snapshot field: through the asynchronous writer (gb_snapshot.h), or a
// blocking copy and write (opt_snap_async = 0).
int Solver::export_field(const std::string &comp, const float *d_data, int n) {
    if (!opt_snap_async) return export_data(comp, d_data, n);
    GB_CUDA_TRY(snapw.open(ncell()));
    GB_CUDA_TRY(snapw.push(st, d_data, path + "/output/proc" + pad6(n) + "_" + comp + ".bin"));
    return GB_OK;
}

// FdmSolver::exportSnapshot (solver/fdm.h:312-347), slot 0.
int Solver::export_snapshot(int it, int isrc, int par) {
    std::string istr;
    int we = wfe;
    if (isrc >= 0) {
        istr = std::to_string(isrc);
        const size_t digit = std::to_string(nsrc).size();
        while (istr.size() < digit) istr = "0" + istr;
        we = wae;
    }
    if (!we || (it + 1) % we != 0) return GB_OK;
    const size_t nc = ncell();
    float *p = slots[0].state;
    float *shp = sh ? p : nullptr;
    float *psp = sh ? p + (size_t)NSH * nc : p;
    int rc = GB_OK;
    if (trace_type == 0) {
        if (sh && !rc) rc = export_field("vy" + istr, shp + (size_t)(VY0 + par) * nc, it + 1);
        if (psv && !rc) rc = export_field("vx" + istr, psp + (size_t)(VX0 + par) * nc, it + 1);
        if (psv && !rc) rc = export_field("vz" + istr, psp + (size_t)(VZ0 + par) * nc, it + 1);
    } else if (trace_type == 1) {
        if (sh && !rc) rc = export_field("uy" + istr, shp + (size_t)UY * nc, it + 1);
        if (psv && !rc) rc = export_field("ux" + istr, psp + (size_t)UX * nc, it + 1);
        if (psv && !rc) rc = export_field("uz" + istr, psp + (size_t)UZ * nc, it + 1);
    }
    return rc;
}

}  // namespace gb
