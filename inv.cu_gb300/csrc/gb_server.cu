// Serving engine: continuous batching of forward+adjoint shot requests.
//
// Each request is one shot on its own model and grid (its own nx, nz, nt,
// wave system, sources and receivers): forward with checkpoints, waveform
// misfit against its observed traces, adjoint with kernel accumulation. The
// engine replays a stream of requests with arrival times. Before every round
// it admits the requests that have arrived, in arrival order, while their
// device footprint (model, wavefields, traces, checkpoints, kernels) fits the
// HBM budget and a slot is free. A round advances every admitted request by
// `sfe` steps: each wave system's requests form one or two groups, and one
// step launch per group covers all of its requests, whatever their grid size
// or phase (forward or adjoint), because every request keeps its own time
// base in its slot descriptor; the groups' launch chains run on streams of
// their own. Requests that finish their forward get their misfit and
// adjoint sources and start the adjoint in the next round; requests that
// finish their adjoint return their kernels and leave, freeing memory for
// waiting requests. The host never waits for the GPU inside a run.
//
// Every request computes exactly the operations of a lone solve, in the
// same order, so its result does not depend on what else is in flight.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "gb_solver.h"

namespace gb {

// kernels of gb_misfit.cu used per request
cudaError_t launch_taper(float *tw, float dt, int nt, cudaStream_t st);
struct TraceRefS {
    const float *syn;
    const float *obs;
    float *adstf;
};
cudaError_t launch_waveform_refs(const void *refs, const float *tw, int ntr, int nt, float sqrt_dt, double *val,
                                 cudaStream_t st);

namespace {

// Default step kernel configuration: marching strips of 120 rows, chunks of
// 64 columns, the fastest of the marching configurations on a mixed batch of
// the serving workload (64 requests with sides of 128-1024 cells: 24.3
// requests/s against 22.2 with 152-row strips); option "tile" selects any of
// the solver's 1..20.
constexpr int kServerTile = 9;

struct Req {
    long long id = 0;
    gb_request_desc d{};
    // device block and views
    char *blk = nullptr;
    size_t bytes = 0;
    float *lam = nullptr, *mu = nullptr, *rho = nullptr, *rinv = nullptr, *ax = nullptr, *az = nullptr;
    float *stf = nullptr, *state = nullptr, *out[3] = {}, *adstf[3] = {}, *obs[3] = {}, *k[3] = {};
    float *tw = nullptr, *amax = nullptr;
    void *ckpt = nullptr;
    double *val = nullptr;
    TraceRefS *refs = nullptr;
    int *csr_src = nullptr, *csr_rin = nullptr, *csr_rec = nullptr;
    int nsfe = 0, nf = 0, ncomp = 0;
    int pz = 0;              // address pitch of the state and model arrays
    void *tmaps = nullptr;   // tensor maps of the fields (bulk loads), or null
    // host data the admission's uploads read; kept until the request leaves,
    // so the admission does not wait for its copies
    std::vector<float> h_ax, h_az, h_stf;
    std::vector<int> h_csr;
    std::vector<char> h_maps;
    std::vector<TraceRefS> h_refs;
    // progress
    int phase = 0;  // 0 waiting, 1 forward, 2 adjoint, 4 results being copied out, 3 done
    int it = 0;
    int pin = -1;  // pinned result buffer while phase is 4
    double t_admit = 0, t_done = 0;
    double misfit = 0;
    std::vector<float> res[3];
};

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace

struct Server {
    int sfe = 10, prec = CKPT_F32, max_slots = 64;
    TileCfg tile = {0, 0, 0};  // step kernel configuration (set at creation)
    // bulk tensor loads in the marching kernel: requested (option "tma"), and
    // still possible (every admitted request's maps could be encoded)
    bool opt_tma = true, tma_ok = true;
    bool use_tma() const { return opt_tma && tma_ok && tile.threads > 0; }
    double budget = 0;
    size_t used = 0;
    cudaStream_t st = nullptr;
    // Chains of a round on several streams (option "streams"): 2 runs the SH
    // requests' steps on a side stream beside the P-SV ones on st, 4 splits
    // each system's requests into two groups, each on its own stream. The
    // requests are independent within a round, so each chain fills the
    // others' launch tails. Side streams start after the round's table copy
    // (ev_fork) and st waits for each (ev_join) at the round's end.
    int streams = 4;  // 512-request capacity: 38.2-39.1 requests/s against 37.6-38.5 with 2 (one box)
    static constexpr int kSide = 3;
    cudaStream_t side[kSide] = {};
    cudaEvent_t ev_fork = nullptr, ev_join[kSide] = {};
    std::vector<Req> reqs;
    // Slot and group tables: one device copy, and a ring of pinned host
    // staging buffers; a staging buffer is refilled only after the event
    // recorded behind its previous copy has completed.
    static constexpr int kStage = 4;
    Slot *d_tab = nullptr, *h_tab[kStage] = {};
    KernelGroup *d_grp = nullptr, *h_grp[kStage] = {};
    cudaEvent_t copied[kStage] = {};
    int tab_cap = 0;
    // Block maps of the round's marching launches (option "compact", on by
    // default): one entry per tile of every request, (slot << 16) | tile,
    // one range per launch chain, staged like the tables. Without them a
    // launch runs max_tiles blocks for every request and the blocks past a
    // smaller request's tiles exit at once.
    bool compact = true;
    unsigned *d_map = nullptr, *h_map[kStage] = {};
    size_t map_cap = 0;
    // Pinned result buffers. A request that finishes its adjoint has its
    // kernels and per-trace misfit values copied into one, behind the
    // buffer's event, and frees its device block; it is finalised (results
    // into its host vectors, misfit summed, completion time read from the
    // event) once that event has completed. Admissions, phase changes and
    // completions thus never wait for the stream, and the host prepares the
    // next rounds while the GPU runs.
    static constexpr int kPins = 8;
    struct Pin {
        char *buf = nullptr;
        cudaEvent_t ev = nullptr;
        Req *owner = nullptr;
    };
    Pin pins[kPins];
    size_t pin_bytes = 0;
    cudaEvent_t ev_t0 = nullptr;  // recorded when a run starts: the origin of the completion times
    // statistics
    int max_active = 0;
    long long rounds = 0, launches = 0;
    double run_s = 0;

    // State and model arrays are allocated at a pitch of nz rounded up to a
    // multiple of 4 (the most admit() uses).
    size_t footprint(const gb_request_desc &d, int nf, int nsfe, int ncomp) const {
        const size_t n = (size_t)d.nx * d.nz, np = (size_t)d.nx * ((d.nz + 3) & ~3);
        const size_t tr = (size_t)d.nrec * d.nt;
        const int nfield = d.psv ? NPSV : NSH;
        size_t b = 0;
        b += align256(4 * np * 4);                                 // lam mu rho rinv
        b += align256((size_t)(d.nx + d.nz) * 4);                  // ax az
        b += align256((size_t)3 * d.nt * 4);                       // stf
        b += align256((size_t)nfield * np * 4);                    // state
        b += align256((size_t)TMAP_N * TMAP_BYTES);                // tensor maps
        b += 3 * align256((size_t)ncomp * tr * 4);                 // out, adstf, obs
        b += align256(3 * n * 4);                                  // kernels
        b += align256((size_t)d.nt * 4);                           // taper
        b += align256((size_t)nsfe * nf * 4);                      // amax
        b += align256((size_t)nsfe * nf * n * (prec == CKPT_F32 ? 4 : 2));
        b += align256((size_t)ncomp * d.nrec * 8);                 // misfit values
        b += align256((size_t)ncomp * d.nrec * sizeof(TraceRefS));
        return b;
    }
};

}  // namespace gb

using namespace gb;

struct gb_server {
    gb::Server s;
};

namespace {

std::vector<int> csr_for(TileCfg tc, int nx, int nz, const std::vector<int> &ii, const std::vector<int> &jj,
                         bool inj) {
    // same packing as the solver's tables
    const int tz = tc.tz, tx = tc.tx;
    const int tiles_z = (nz + tz - 1) / tz, tiles_x = (nx + tx - 1) / tx, ntiles = tiles_z * tiles_x;
    const int vz = tz + 3;
    std::map<int, std::map<int, std::vector<int>>> per;
    for (size_t q = 0; q < ii.size(); q++) {
        const int i = ii[q], j = jj[q];
        if (i < 0 || i >= nx || j < 0 || j >= nz) continue;
        if (inj) {
            for (int txi = std::max(0, (i - tx - 1) / tx - 1); txi <= std::min(tiles_x - 1, (i + 1) / tx); txi++) {
                const int i0 = txi * tx;
                if (i < i0 - 1 || i > i0 + tx + 1) continue;
                for (int tzi = std::max(0, (j - tz - 1) / tz - 1); tzi <= std::min(tiles_z - 1, (j + 1) / tz); tzi++) {
                    const int j0 = tzi * tz;
                    if (j < j0 - 1 || j > j0 + tz + 1) continue;
                    per[txi * tiles_z + tzi][(i - (i0 - 1)) * vz + (j - (j0 - 1))].push_back((int)q);
                }
            }
        } else {
            const int txi = i / tx, tzi = j / tz;
            per[txi * tiles_z + tzi][(i - txi * tx) * tz + (j - tzi * tz)].push_back((int)q);
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
    int *tile_ptr = out.data() + 3, *local = tile_ptr + ntiles + 1, *tptr = local + nent, *traces = tptr + nent + 1;
    int e = 0, t = 0;
    auto itp = per.begin();
    for (int tile = 0; tile < ntiles; tile++) {
        tile_ptr[tile] = e;
        if (itp != per.end() && itp->first == tile) {
            for (auto &ent : itp->second) {
                local[e] = ent.first;
                tptr[e] = t;
                for (int v : ent.second) traces[t++] = v;
                e++;
            }
            ++itp;
        }
    }
    tile_ptr[ntiles] = e;
    tptr[nent] = t;
    return out;
}

int calc_idx(float c, float L, int n) { return (int)((double)(c / L * (float)(n - 1)) + 0.5); }

void ricker1(int nt, float dt, const float *cfg, float *sx, float *sy, float *sz) {
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

// Uploads a request into its device block (model, profiles, source, obs,
// tables) and zeroes state, kernels and checkpoint scales.
int admit(Server &S, Req &r) {
    const gb_request_desc &d = r.d;
    const size_t n = (size_t)d.nx * d.nz, tr = (size_t)d.nrec * d.nt;
    // the marching kernel reads columns that start on 16-byte boundaries: a
    // pitch of nz rounded up to a multiple of 4 (the 2-D tile kernel uses nz)
    r.pz = S.tile.threads > 0 ? (d.nz + 3) & ~3 : d.nz;
    const size_t np = (size_t)d.nx * r.pz;
    GB_CUDA_TRY(cudaMallocAsync((void **)&r.blk, r.bytes, S.st));
    char *p = r.blk;
    auto take = [&](size_t b) {
        char *q = p;
        p += align256(b);
        return q;
    };
    r.lam = (float *)take(4 * np * 4);
    r.mu = r.lam + np;
    r.rho = r.lam + 2 * np;
    r.rinv = r.lam + 3 * np;
    r.ax = (float *)take((size_t)(d.nx + d.nz) * 4);
    r.az = r.ax + d.nx;
    r.stf = (float *)take((size_t)3 * d.nt * 4);
    const int nfield = d.psv ? NPSV : NSH;
    r.state = (float *)take((size_t)nfield * np * 4);
    void *maps = take((size_t)TMAP_N * TMAP_BYTES);
    const int comps_psv[2] = {0, 2}, comps_sh[1] = {1};
    const int *cs = d.psv ? comps_psv : comps_sh;
    float *outb = (float *)take((size_t)r.ncomp * tr * 4);
    float *adb = (float *)take((size_t)r.ncomp * tr * 4);
    float *obb = (float *)take((size_t)r.ncomp * tr * 4);
    for (int q = 0; q < r.ncomp; q++) {
        r.out[cs[q]] = outb + q * tr;
        r.adstf[cs[q]] = adb + q * tr;
        r.obs[cs[q]] = obb + q * tr;
    }
    float *kb = (float *)take(3 * n * 4);
    for (int q = 0; q < 3; q++) r.k[q] = kb + q * n;
    r.tw = (float *)take((size_t)d.nt * 4);
    r.amax = (float *)take((size_t)r.nsfe * r.nf * 4);
    r.ckpt = take((size_t)r.nsfe * r.nf * n * (S.prec == CKPT_F32 ? 4 : 2));
    r.val = (double *)take((size_t)r.ncomp * d.nrec * 8);
    r.refs = (TraceRefS *)take((size_t)r.ncomp * d.nrec * sizeof(TraceRefS));

    // host-side preparation
    const float xmax = d.dx * (d.nx - 1), zmax = d.dz * (d.nz - 1);
    std::vector<float> &hax = r.h_ax, &haz = r.h_az;
    hax.assign(d.nx, 1.f);
    haz.assign(d.nz, 1.f);
    const int w = d.abs_width;
    const float a = d.abs_alpha;
    for (int i = 0; i < d.nx; i++) {
        if (d.abs_left && i + 1 < w) hax[i] *= expf(-powf(a * (float)(w - i - 1), 2));
        if (d.abs_right && i > d.nx - w) hax[i] *= expf(-powf(a * (float)(w + i - d.nx), 2));
    }
    for (int j = 0; j < d.nz; j++) {
        if (d.abs_bottom && j > d.nz - w) haz[j] *= expf(-powf(a * (float)(w + j - d.nz), 2));
        if (d.abs_top && j + 1 < w) haz[j] *= expf(-powf(a * (float)(w - j - 1), 2));
    }
    std::vector<float> &hstf = r.h_stf;
    hstf.assign(3 * (size_t)d.nt, 0.f);
    ricker1(d.nt, d.dt, d.src + 3, hstf.data(), hstf.data() + d.nt, hstf.data() + 2 * d.nt);
    const std::vector<int> si = {calc_idx(d.src[0], xmax, d.nx)}, sj = {calc_idx(d.src[1], zmax, d.nz)};
    std::vector<int> ri(d.nrec), rj(d.nrec);
    for (int q = 0; q < d.nrec; q++) {
        ri[q] = calc_idx(d.rec[2 * q], xmax, d.nx);
        rj[q] = calc_idx(d.rec[2 * q + 1], zmax, d.nz);
    }
    const std::vector<int> c1 = csr_for(S.tile, d.nx, d.nz, si, sj, true);
    const std::vector<int> c2 = csr_for(S.tile, d.nx, d.nz, ri, rj, true);
    const std::vector<int> c3 = csr_for(S.tile, d.nx, d.nz, ri, rj, false);
    r.h_csr.clear();
    r.h_csr.insert(r.h_csr.end(), c1.begin(), c1.end());
    r.h_csr.insert(r.h_csr.end(), c2.begin(), c2.end());
    r.h_csr.insert(r.h_csr.end(), c3.begin(), c3.end());
    GB_CUDA_TRY(cudaMallocAsync((void **)&r.csr_src, r.h_csr.size() * 4, S.st));
    r.csr_rin = r.csr_src + c1.size();
    r.csr_rec = r.csr_rin + c2.size();

    // uploads (pageable sources are staged by the runtime; they stay valid
    // until the request completes, by the API contract)
    // model columns at the pitch; rows nz .. pz-1 are never read (the step
    // kernels stop at row nz, the bulk loads' tensors end there)
    if (r.pz != d.nz) GB_CUDA_TRY(cudaMemsetAsync(r.lam, 0, 4 * np * 4, S.st));
    const float *src[3] = {d.lambda, d.mu, d.rho};
    float *dst[3] = {r.lam, r.mu, r.rho};
    for (int q = 0; q < 3; q++)
        GB_CUDA_TRY(cudaMemcpy2DAsync(dst[q], (size_t)r.pz * 4, src[q], (size_t)d.nz * 4, (size_t)d.nz * 4, d.nx,
                                      cudaMemcpyHostToDevice, S.st));
    GB_CUDA_TRY(launch_reciprocal(r.rinv, r.rho, np, S.st));
    // tensor maps of the state and model fields for the marching kernel's
    // bulk loads, for its strips of S.tile.threads rows
    r.tmaps = nullptr;
    std::vector<char> &hmaps = r.h_maps;
    hmaps.assign((size_t)TMAP_N * TMAP_BYTES, 0);
    if (S.use_tma()) {
        const float *sh_state = d.psv ? nullptr : r.state, *psv_state = d.psv ? r.state : nullptr;
        if (encode_slot_maps(hmaps.data(), d.psv ? psv_state : sh_state, !d.psv, d.psv != 0, r.rinv, r.mu, r.lam,
                             d.nx, d.nz, r.pz, S.tile.threads)) {
            GB_CUDA_TRY(cudaMemcpyAsync(maps, hmaps.data(), hmaps.size(), cudaMemcpyHostToDevice, S.st));
            r.tmaps = maps;
        } else {
            S.tma_ok = false;  // this request's fields cannot be described: per-row loads from now on
        }
    }
    GB_CUDA_TRY(cudaMemcpyAsync(r.ax, hax.data(), d.nx * 4, cudaMemcpyHostToDevice, S.st));
    GB_CUDA_TRY(cudaMemcpyAsync(r.az, haz.data(), d.nz * 4, cudaMemcpyHostToDevice, S.st));
    GB_CUDA_TRY(cudaMemcpyAsync(r.stf, hstf.data(), hstf.size() * 4, cudaMemcpyHostToDevice, S.st));
    GB_CUDA_TRY(cudaMemcpyAsync(r.csr_src, r.h_csr.data(), r.h_csr.size() * 4, cudaMemcpyHostToDevice, S.st));
    if (d.obs)
        GB_CUDA_TRY(cudaMemcpyAsync(obb, d.obs, (size_t)r.ncomp * tr * 4, cudaMemcpyHostToDevice, S.st));
    else
        GB_CUDA_TRY(cudaMemsetAsync(obb, 0, (size_t)r.ncomp * tr * 4, S.st));
    GB_CUDA_TRY(cudaMemsetAsync(r.state, 0, (size_t)nfield * np * 4, S.st));
    GB_CUDA_TRY(cudaMemsetAsync(kb, 0, 3 * n * 4, S.st));
    GB_CUDA_TRY(cudaMemsetAsync(r.amax, 0, (size_t)r.nsfe * r.nf * 4, S.st));
    GB_CUDA_TRY(cudaMemsetAsync(outb, 0, (size_t)r.ncomp * tr * 4, S.st));
    GB_CUDA_TRY(launch_taper(r.tw, d.dt, d.nt, S.st));
    std::vector<TraceRefS> &refs = r.h_refs;
    refs.resize((size_t)r.ncomp * d.nrec);
    for (int ir = 0; ir < d.nrec; ir++)
        for (int q = 0; q < r.ncomp; q++) {
            const size_t off = (size_t)ir * d.nt;
            refs[(size_t)ir * r.ncomp + q] = {outb + q * tr + off, obb + q * tr + off, adb + q * tr + off};
        }
    GB_CUDA_TRY(cudaMemcpyAsync(r.refs, refs.data(), refs.size() * sizeof(TraceRefS), cudaMemcpyHostToDevice, S.st));
    // no wait: the host data stays with the request until it leaves
    r.phase = 1;
    r.it = 0;
    S.used += r.bytes;
    return GB_OK;
}

void fill_slot(const Server &S, const Req &r, Slot &s) {
    memset(&s, 0, sizeof s);
    const gb_request_desc &d = r.d;
    s.nx = d.nx;
    s.nz = d.nz;
    s.pz = r.pz;
    s.tmap = r.tmaps;
    s.nt = d.nt;
    s.tiles_z = (d.nz + S.tile.tz - 1) / S.tile.tz;
    s.tiles_x = (d.nx + S.tile.tx - 1) / S.tile.tx;
    s.active = 1;
    s.it_base = r.it;
    s.par0 = r.it & 1;
    s.sfe = S.sfe;
    s.dt = d.dt;
    s.c9x = 9.f / (8.f * d.dx);
    s.c24x = 1.f / (24.f * d.dx);
    s.c9z = 9.f / (8.f * d.dz);
    s.c24z = 1.f / (24.f * d.dz);
    s.lambda = r.lam;
    s.mu = r.mu;
    s.rho = r.rho;
    s.rinv = r.rinv;
    s.ax = r.ax;
    s.az = r.az;
    const size_t np = (size_t)d.nx * r.pz;
    if (d.psv)
        for (int f = 0; f < NPSV; f++) s.psv[f] = r.state + f * np;
    else
        for (int f = 0; f < NSH; f++) s.sh[f] = r.state + f * np;
    s.nsfe = r.nsfe;
    s.nf = r.nf;
    s.ckpt_prec = S.prec;
    s.ckpt = r.ckpt;
    s.ckpt_amax = r.amax;
    if (r.phase == 1) {
        s.inj = r.csr_src;
        s.inj_x = r.stf;
        s.inj_y = r.stf + d.nt;
        s.inj_z = r.stf + 2 * d.nt;
        s.rec = r.csr_rec;
        s.out_x = r.out[0];
        s.out_y = r.out[1];
        s.out_z = r.out[2];
        s.record_u = 1;
        s.ckpt_write = 1;
    } else {
        s.inj = r.csr_rin;
        s.inj_x = r.adstf[0];
        s.inj_y = r.adstf[1];
        s.inj_z = r.adstf[2];
        s.ckpt_write = 0;
    }
}

double now_s(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// One round: every active request advances sfe steps.
int round_once(Server &S, std::vector<Req *> &act) {
    // Chains: a wave system's requests split into G groups (G = 2 with four
    // streams, else 1), each group's steps of the round one chain of
    // launches. Table order: for P-SV then SH, for each group, its adjoint
    // requests then its forward ones; a request's group is its position
    // among the admitted requests of its system, modulo G.
    const int G = S.streams >= 4 ? 2 : 1;
    std::vector<Req *> order;
    int counts[2][2][2] = {};  // [psv][group][phase-1]
    std::vector<int> grp(act.size());
    {
        int seen[2] = {0, 0};
        for (size_t q = 0; q < act.size(); q++) grp[q] = seen[act[q]->d.psv]++ % G;
    }
    for (int w = 1; w >= 0; w--)
        for (int g = 0; g < G; g++)
            for (int ph = 2; ph >= 1; ph--)
                for (size_t q = 0; q < act.size(); q++) {
                    Req *r = act[q];
                    if (r->d.psv == w && r->phase == ph && grp[q] == g) {
                        order.push_back(r);
                        counts[w][g][ph - 1]++;
                    }
                }
    const int n = (int)order.size();
    if (n > S.tab_cap) {
        GB_CUDA_TRY(cudaStreamSynchronize(S.st));
        cudaFree(S.d_tab);
        cudaFree(S.d_grp);
        for (int b = 0; b < Server::kStage; b++) {
            cudaFreeHost(S.h_tab[b]);
            cudaFreeHost(S.h_grp[b]);
        }
        S.tab_cap = std::max(n, 2 * S.tab_cap);
        GB_CUDA_TRY(cudaMalloc(&S.d_tab, sizeof(Slot) * S.tab_cap));
        GB_CUDA_TRY(cudaMalloc(&S.d_grp, sizeof(KernelGroup) * S.tab_cap));
        for (int b = 0; b < Server::kStage; b++) {
            GB_CUDA_TRY(cudaMallocHost(&S.h_tab[b], sizeof(Slot) * S.tab_cap));
            GB_CUDA_TRY(cudaMallocHost(&S.h_grp[b], sizeof(KernelGroup) * S.tab_cap));
        }
    }
    const int b = (int)(S.rounds % Server::kStage);
    if (!S.copied[b]) GB_CUDA_TRY(cudaEventCreateWithFlags(&S.copied[b], cudaEventDisableTiming));
    GB_CUDA_TRY(cudaEventSynchronize(S.copied[b]));  // its previous copy has been consumed
    Slot *h_tab = S.h_tab[b];
    KernelGroup *h_grp = S.h_grp[b];
    int max_tiles[2] = {0, 0}, max_cells[2] = {0, 0};
    size_t max_n_fwd[2] = {0, 0};
    for (int q = 0; q < n; q++) {
        fill_slot(S, *order[q], h_tab[q]);
        const int w = order[q]->d.psv;
        max_tiles[w] = std::max(max_tiles[w], h_tab[q].tiles_z * h_tab[q].tiles_x);
        const size_t cells = (size_t)order[q]->d.nx * order[q]->d.nz;
        if (order[q]->phase == 2) max_cells[w] = std::max(max_cells[w], (int)cells);
        if (order[q]->phase == 1) max_n_fwd[w] = std::max(max_n_fwd[w], cells);
        KernelGroup &g = h_grp[q];
        g.k_lambda = order[q]->k[0];
        g.k_mu = order[q]->k[1];
        g.k_rho = order[q]->k[2];
        g.inv_lambda = order[q]->d.inv_lambda;
        g.inv_mu = order[q]->d.inv_mu;
        g.inv_rho = order[q]->d.inv_rho;
        g.first = q;
        g.count = 1;
        g.nx = order[q]->d.nx;
        g.nz = order[q]->d.nz;
    }
    // the chains, in table order: system w, group g, first table entry,
    // entry count, adjoint entries (first in the chain), stream
    struct Chain {
        int w, base, cnt, nadj;
        cudaStream_t st;
        size_t map_off, map_n;
    };
    std::vector<Chain> chains;
    {
        int base = 0;
        for (int w = 1; w >= 0; w--)
            for (int g = 0; g < G; g++) {
                const int cnt = counts[w][g][0] + counts[w][g][1];
                if (cnt) chains.push_back({w, base, cnt, counts[w][g][1], nullptr, 0, 0});
                base += cnt;
            }
    }
    // block maps, one range per chain, slots numbered within their chain
    // (16 bits each for the slot and the tile; a round beyond that launches
    // max_tiles blocks per request instead)
    bool use_map = S.compact && S.tile.threads > 0 && n <= 65536;
    size_t total = 0;
    for (int q = 0; use_map && q < n; q++) {
        const size_t t = (size_t)h_tab[q].tiles_z * h_tab[q].tiles_x;
        use_map = t <= 65536;
        total += t;
    }
    if (use_map) {
        if (total > S.map_cap) {
            GB_CUDA_TRY(cudaStreamSynchronize(S.st));  // every staged map has been consumed
            cudaFree(S.d_map);
            for (int r = 0; r < Server::kStage; r++) cudaFreeHost(S.h_map[r]);
            S.map_cap = std::max(total, 2 * S.map_cap);
            GB_CUDA_TRY(cudaMalloc(&S.d_map, sizeof(unsigned) * S.map_cap));
            for (int r = 0; r < Server::kStage; r++)
                GB_CUDA_TRY(cudaMallocHost(&S.h_map[r], sizeof(unsigned) * S.map_cap));
        }
        unsigned *hm = S.h_map[b];
        size_t e = 0;
        for (Chain &c : chains) {
            c.map_off = e;
            for (int q = 0; q < c.cnt; q++) {
                const unsigned t = (unsigned)(h_tab[c.base + q].tiles_z * h_tab[c.base + q].tiles_x);
                for (unsigned tile = 0; tile < t; tile++) hm[e++] = ((unsigned)q << 16) | tile;
            }
            c.map_n = e - c.map_off;
        }
        if (e) GB_CUDA_TRY(cudaMemcpyAsync(S.d_map, hm, sizeof(unsigned) * e, cudaMemcpyHostToDevice, S.st));
    }
    GB_CUDA_TRY(cudaMemcpyAsync(S.d_tab, h_tab, sizeof(Slot) * n, cudaMemcpyHostToDevice, S.st));
    GB_CUDA_TRY(cudaMemcpyAsync(S.d_grp, h_grp, sizeof(KernelGroup) * n, cudaMemcpyHostToDevice, S.st));
    GB_CUDA_TRY(cudaEventRecord(S.copied[b], S.st));
    const bool q16 = S.prec != CKPT_F32;
    // streams: one chain on S.st with one stream; with two, the P-SV chain
    // on S.st and the SH chain on the side stream; with four, every chain on
    // its own stream. The side streams start after the round's table copy
    // (ev_fork) and S.st waits for them at the round's end (ev_join).
    int nside = 0;
    for (size_t c = 0; c < chains.size(); c++) {
        int sidx = 0;  // 0: S.st, k > 0: S.side[k - 1]
        if (S.streams >= 4)
            sidx = (int)c;
        else if (S.streams == 2)
            sidx = chains[c].w ? 0 : 1;
        if (sidx > 0 && chains.size() == 1) sidx = 0;
        if (sidx > 0) {
            if (!S.side[sidx - 1]) {
                GB_CUDA_TRY(cudaStreamCreateWithFlags(&S.side[sidx - 1], cudaStreamNonBlocking));
                GB_CUDA_TRY(cudaEventCreateWithFlags(&S.ev_join[sidx - 1], cudaEventDisableTiming));
            }
            nside = std::max(nside, sidx);
        }
        chains[c].st = sidx ? S.side[sidx - 1] : S.st;
    }
    if (nside) {
        if (!S.ev_fork) GB_CUDA_TRY(cudaEventCreateWithFlags(&S.ev_fork, cudaEventDisableTiming));
        GB_CUDA_TRY(cudaEventRecord(S.ev_fork, S.st));
        for (int k = 0; k < nside; k++) GB_CUDA_TRY(cudaStreamWaitEvent(S.side[k], S.ev_fork, 0));
    }
    for (int k = 0; k < S.sfe; k++) {
        for (const Chain &c : chains) {
            const int w = c.w;
            const Slot *tab = S.d_tab + c.base;
            const cudaStream_t sw = c.st;
            // forward checkpoints of u before the step (the kernels select
            // the forward slots whose step is a checkpoint step)
            if (k == S.sfe - 1 && c.cnt > c.nadj) {
                if (q16) GB_CUDA_TRY(launch_ckpt_amax(tab, c.cnt, (int)max_n_fwd[w], k, 1, w, sw));
                GB_CUDA_TRY(launch_ckpt_store(tab, c.cnt, (int)max_n_fwd[w], k, 1, w, sw));
                S.launches += q16 ? 2 : 1;
            }
            if (use_map)
                GB_CUDA_TRY(launch_step(w, S.tile, tab, c.cnt, max_tiles[w], k, S.use_tma(), sw, S.d_map + c.map_off,
                                        (int)c.map_n));
            else
                GB_CUDA_TRY(launch_step(w, S.tile, tab, c.cnt, max_tiles[w], k, S.use_tma(), sw));
            S.launches++;
            if (k == S.sfe - 1 && c.cnt > c.nadj) {
                if (q16) GB_CUDA_TRY(launch_ckpt_amax(tab, c.cnt, (int)max_n_fwd[w], k, 0, w, sw));
                GB_CUDA_TRY(launch_ckpt_store(tab, c.cnt, (int)max_n_fwd[w], k, 0, w, sw));
                S.launches += q16 ? 2 : 1;
            }
            if (k == 0 && c.nadj) {
                GB_CUDA_TRY(launch_interaction(w, S.d_tab, S.d_grp + c.base, c.nadj, max_cells[w], k, sw));
                S.launches++;
            }
        }
    }
    for (int k = 0; k < nside; k++) {
        GB_CUDA_TRY(cudaEventRecord(S.ev_join[k], S.side[k]));
        GB_CUDA_TRY(cudaStreamWaitEvent(S.st, S.ev_join[k], 0));
    }
    for (Req *r : act) r->it += S.sfe;
    S.rounds++;
    return GB_OK;
}

size_t pin_need(const Req &r) {
    return align256((size_t)3 * r.d.nx * r.d.nz * 4) + (size_t)r.ncomp * r.d.nrec * 8;
}

// Results of the request in pin p (its event has completed) into its host
// vectors; its completion time is the event's time since the run began.
int finalize(Server &S, int p, size_t &done) {
    Server::Pin &P = S.pins[p];
    Req &r = *P.owner;
    const size_t n = (size_t)r.d.nx * r.d.nz;
    const float *k = reinterpret_cast<const float *>(P.buf);
    for (int q = 0; q < 3; q++) r.res[q].assign(k + q * n, k + (q + 1) * n);
    const double *v = reinterpret_cast<const double *>(P.buf + align256(3 * n * 4));
    r.misfit = 0;
    for (int t = 0; t < r.ncomp * r.d.nrec; t++) r.misfit += v[t];
    float ms = 0;
    GB_CUDA_TRY(cudaEventElapsedTime(&ms, S.ev_t0, P.ev));
    r.t_done = ms * 1e-3;
    r.phase = 3;
    r.pin = -1;
    r.h_ax = {};
    r.h_az = {};
    r.h_stf = {};
    r.h_csr = {};
    r.h_maps = {};
    r.h_refs = {};
    P.owner = nullptr;
    done++;
    return GB_OK;
}

// Finalises every pinned result whose copies have completed (wait = true:
// every one, waiting for them).
int reap(Server &S, size_t &done, bool wait) {
    for (int p = 0; p < Server::kPins; p++) {
        if (!S.pins[p].owner) continue;
        if (wait) {
            GB_CUDA_TRY(cudaEventSynchronize(S.pins[p].ev));
        } else {
            const cudaError_t q = cudaEventQuery(S.pins[p].ev);
            if (q == cudaErrorNotReady) {
                if (cudaPeekAtLastError() == cudaErrorNotReady) (void)cudaGetLastError();
                continue;
            }
            GB_CUDA_TRY(q);
        }
        const int rc = finalize(S, p, done);
        if (rc) return rc;
    }
    return GB_OK;
}

// Copies a finished request's kernels and misfit values into a free pinned
// buffer (waiting for the oldest one if none is free) and frees its block.
int retire(Server &S, Req &r, size_t &done) {
    int p = -1;
    for (int q = 0; q < Server::kPins && p < 0; q++)
        if (!S.pins[q].owner) p = q;
    if (p < 0) {
        GB_CUDA_TRY(cudaEventSynchronize(S.pins[0].ev));
        const int rc = finalize(S, 0, done);
        if (rc) return rc;
        p = 0;
    }
    Server::Pin &P = S.pins[p];
    const size_t n = (size_t)r.d.nx * r.d.nz;
    for (int q = 0; q < 3; q++)
        GB_CUDA_TRY(cudaMemcpyAsync(P.buf + q * n * 4, r.k[q], n * 4, cudaMemcpyDeviceToHost, S.st));
    const int ntr = r.ncomp * r.d.nrec;
    if (ntr)
        GB_CUDA_TRY(cudaMemcpyAsync(P.buf + align256(3 * n * 4), r.val, (size_t)ntr * 8, cudaMemcpyDeviceToHost, S.st));
    GB_CUDA_TRY(cudaEventRecord(P.ev, S.st));
    GB_CUDA_TRY(cudaFreeAsync(r.blk, S.st));
    GB_CUDA_TRY(cudaFreeAsync(r.csr_src, S.st));
    r.blk = nullptr;
    r.csr_src = nullptr;
    r.phase = 4;
    r.pin = p;
    P.owner = &r;
    S.used -= r.bytes;  // stream-ordered: a later admission's allocation follows the free
    return GB_OK;
}

}  // namespace

extern "C" {

gb_server *gb_server_create(int sfe, int ckpt_precision, double hbm_budget_gb, int max_slots) {
    if (sfe < 1 || ckpt_precision < 0 || ckpt_precision > 2) {
        set_error("gb_server_create: sfe must be >= 1 and ckpt_precision 0, 1 or 2");
        return nullptr;
    }
    gb_server *h = new gb_server();
    Server &S = h->s;
    S.sfe = sfe;
    S.prec = ckpt_precision;
    S.max_slots = max_slots > 0 ? max_slots : 1 << 20;
    size_t freeb = 0, total = 0;
    if (cudaStreamCreateWithFlags(&S.st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMemGetInfo(&freeb, &total) != cudaSuccess) {
        set_error("gb_server_create: no CUDA device");
        delete h;
        return nullptr;
    }
    S.budget = hbm_budget_gb > 0 ? hbm_budget_gb * 1e9 : 0.8 * (double)freeb;
    S.tile = tile_config(kServerTile);
    return h;
}

int gb_server_set_option(gb_server *h, const char *key, double value) {
    if (!h || !key) return GB_ERR_ARG;
    const std::string k = key;
    if (k == "tile") {
        const int t = (int)value;
        if (t < 1 || t > 20) {
            set_error("gb_server_set_option: tile must be 1..20");
            return GB_ERR_ARG;
        }
        h->s.tile = tile_config(t);
        return GB_OK;
    }
    if (k == "tma") {
        h->s.opt_tma = value != 0;
        return GB_OK;
    }
    if (k == "compact") {
        h->s.compact = value != 0;
        return GB_OK;
    }
    if (k == "streams") {
        if (value != 1 && value != 2 && value != 4) {
            set_error("gb_server_set_option: streams must be 1, 2 or 4");
            return GB_ERR_ARG;
        }
        h->s.streams = (int)value;
        return GB_OK;
    }
    set_error("gb_server_set_option: unknown option " + k);
    return GB_ERR_ARG;
}

long long gb_server_submit(gb_server *h, const gb_request_desc *d) {
    if (!h || !d || d->nx < 8 || d->nz < 8 || d->nt < 1 || !d->lambda || !d->mu || !d->rho || d->nrec < 0 ||
        (d->nrec && !d->rec)) {
        set_error("gb_server_submit: invalid request");
        return -1;
    }
    Server &S = h->s;
    if (d->nt % S.sfe) {
        set_error("gb_server_submit: nt must be a multiple of the server's sfe");
        return -1;
    }
    if (!(d->dx > 0) || !(d->dz > 0) || !(d->dt > 0)) {
        set_error("gb_server_submit: dx, dz, dt must be positive");
        return -1;
    }
    Req r;
    r.id = (long long)S.reqs.size();
    r.d = *d;
    r.ncomp = d->psv ? 2 : 1;
    r.nf = d->psv ? ckpt_nf_psv(S.prec) : ckpt_nf_sh(S.prec);
    r.nsfe = d->nt / S.sfe;
    r.bytes = S.footprint(*d, r.nf, r.nsfe, r.ncomp);
    if ((double)r.bytes > S.budget) {
        set_error("gb_server_submit: request needs " + std::to_string(r.bytes) + " bytes, more than the budget");
        return -1;
    }
    S.reqs.push_back(r);
    return r.id;
}

int gb_server_run(gb_server *h) {
    if (!h) return GB_ERR_ARG;
    Server &S = h->s;
    std::vector<size_t> order(S.reqs.size());
    for (size_t q = 0; q < order.size(); q++) order[q] = q;
    std::stable_sort(order.begin(), order.end(),
                     [&](size_t a, size_t b) { return S.reqs[a].d.arrival < S.reqs[b].d.arrival; });
    std::deque<size_t> waiting(order.begin(), order.end());
    for (size_t q : order) {
        S.reqs[q].phase = 0;
        S.reqs[q].blk = nullptr;
    }
    // pinned result buffers for the largest request
    size_t need = 0;
    for (const Req &r : S.reqs) need = std::max(need, pin_need(r));
    if (need > S.pin_bytes) {
        GB_CUDA_TRY(cudaStreamSynchronize(S.st));
        for (auto &P : S.pins) {
            cudaFreeHost(P.buf);
            P.buf = nullptr;
        }
        for (auto &P : S.pins) GB_CUDA_TRY(cudaMallocHost((void **)&P.buf, need));
        S.pin_bytes = need;
    }
    for (auto &P : S.pins)
        if (!P.ev) GB_CUDA_TRY(cudaEventCreate(&P.ev));
    if (!S.ev_t0) GB_CUDA_TRY(cudaEventCreate(&S.ev_t0));
    std::vector<Req *> act;
    const auto t0 = std::chrono::steady_clock::now();
    GB_CUDA_TRY(cudaEventRecord(S.ev_t0, S.st));
    size_t done = 0;
    while (done < S.reqs.size()) {
        // admission in arrival order, by HBM budget and free slots
        while (!waiting.empty()) {
            Req &r = S.reqs[waiting.front()];
            if (r.d.arrival > now_s(t0)) break;
            if ((int)act.size() >= S.max_slots || (double)(S.used + r.bytes) > S.budget) break;
            int rc = admit(S, r);
            if (rc) return rc;
            r.t_admit = now_s(t0);
            act.push_back(&r);
            waiting.pop_front();
        }
        S.max_active = std::max(S.max_active, (int)act.size());
        if (act.empty()) {
            // nothing on the GPU but results being copied out: wait for them
            const int rc = reap(S, done, true);
            if (rc) return rc;
            if (waiting.empty()) break;
            const double wait = S.reqs[waiting.front()].d.arrival - now_s(t0);
            if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.01)));
            continue;
        }
        int rc = round_once(S, act);
        if (rc) return rc;
        // phase changes
        std::vector<Req *> still;
        for (Req *r : act) {
            if (r->it < r->d.nt) {
                still.push_back(r);
                continue;
            }
            const gb_request_desc &d = r->d;
            if (r->phase == 1) {
                // waveform misfit and adjoint sources (misfit/waveform.h:4-40)
                const int ntr = r->ncomp * d.nrec;
                if (ntr) GB_CUDA_TRY(launch_waveform_refs(r->refs, r->tw, ntr, d.nt, std::sqrt(d.dt), r->val, S.st));
                S.launches++;
                // (the per-trace values stay on the device until the
                // request leaves; its misfit is their sum, formed then)
                GB_CUDA_TRY(cudaMemsetAsync(r->state, 0, (size_t)(d.psv ? NPSV : NSH) * d.nx * r->pz * 4, S.st));
                r->phase = 2;
                r->it = 0;
                still.push_back(r);
            } else {
                const int rc2 = retire(S, *r, done);
                if (rc2) return rc2;
            }
        }
        act.swap(still);
        rc = reap(S, done, false);
        if (rc) return rc;
    }
    {
        const int rc = reap(S, done, true);
        if (rc) return rc;
    }
    GB_CUDA_TRY(cudaStreamSynchronize(S.st));
    S.run_s = now_s(t0);
    if (S.opt_tma && S.tile.threads > 0 && march_tma_error()) {
        set_error("server: a bulk-load wait of the marching kernel ran out of iterations; results are invalid");
        return GB_ERR_CUDA;
    }
    return GB_OK;
}

int gb_server_result(gb_server *h, long long id, float *k_lambda, float *k_mu, float *k_rho, double *misfit,
                     double *latency_s) {
    if (!h || id < 0 || id >= (long long)h->s.reqs.size()) return GB_ERR_ARG;
    Req &r = h->s.reqs[id];
    if (r.phase != 3) {
        set_error("gb_server_result: request not finished");
        return GB_ERR_STATE;
    }
    float *outs[3] = {k_lambda, k_mu, k_rho};
    for (int q = 0; q < 3; q++)
        if (outs[q]) std::copy(r.res[q].begin(), r.res[q].end(), outs[q]);
    if (misfit) *misfit = r.misfit;
    if (latency_s) *latency_s = r.t_done - r.d.arrival;
    return GB_OK;
}

int gb_server_report(gb_server *h, gb_server_stats *out) {
    if (!h || !out) return GB_ERR_ARG;
    Server &S = h->s;
    std::vector<double> lat;
    long long cells = 0;
    for (auto &r : S.reqs)
        if (r.phase == 3) {
            lat.push_back(r.t_done - r.d.arrival);
            cells += 2LL * r.d.nx * r.d.nz * r.d.nt;
        }
    std::sort(lat.begin(), lat.end());
    auto pct = [&](double p) {
        if (lat.empty()) return 0.0;
        const size_t i = (size_t)std::min<double>(lat.size() - 1, std::ceil(p * lat.size()) - 1);
        return lat[i];
    };
    memset(out, 0, sizeof *out);
    out->completed = (int)lat.size();
    out->wall_s = S.run_s;
    out->p50_s = pct(0.50);
    out->p99_s = pct(0.99);
    out->max_concurrent = S.max_active;
    out->rounds = S.rounds;
    out->launches = S.launches;
    out->cell_updates = cells;
    return GB_OK;
}

void gb_server_destroy(gb_server *h) {
    if (!h) return;
    Server &S = h->s;
    if (S.st) cudaStreamSynchronize(S.st);
    for (auto &r : S.reqs) {
        if (r.blk) cudaFree(r.blk);
        if (r.csr_src) cudaFree(r.csr_src);
    }
    cudaFree(S.d_tab);
    cudaFree(S.d_grp);
    cudaFree(S.d_map);
    for (auto &P : S.pins) {
        cudaFreeHost(P.buf);
        if (P.ev) cudaEventDestroy(P.ev);
    }
    if (S.ev_t0) cudaEventDestroy(S.ev_t0);
    for (int b = 0; b < Server::kStage; b++) {
        cudaFreeHost(S.h_tab[b]);
        cudaFreeHost(S.h_grp[b]);
        cudaFreeHost(S.h_map[b]);
        if (S.copied[b]) cudaEventDestroy(S.copied[b]);
    }
    for (int k = 0; k < Server::kSide; k++)
        if (S.side[k]) cudaStreamSynchronize(S.side[k]);
    if (S.ev_fork) cudaEventDestroy(S.ev_fork);
    for (int k = 0; k < Server::kSide; k++) {
        if (S.ev_join[k]) cudaEventDestroy(S.ev_join[k]);
        if (S.side[k]) cudaStreamDestroy(S.side[k]);
    }
    if (S.st) cudaStreamDestroy(S.st);
    delete h;
}

}  // extern "C"
