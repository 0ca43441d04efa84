// Misfits and the shot loop: the GB300 replacement of Misfit
// (misfit/misfit.h:3-153), WaveformMisfit (misfit/waveform.h) and
// EnvelopeMisfit (misfit/envelope.h).
//
// The reference runs one shot at a time and, per trace, one launch plus one
// cuBLAS round trip. Here a whole batch of shots is forwarded together, the
// misfit of every trace of the batch is one launch (one block per trace,
// FP64 sums), and the adjoint batch follows. Per-trace values are summed on
// the host in the reference's order (shot, receiver, component).
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <iostream>
#include <vector>

#include "gb_solver.h"

namespace gb {

// taper (misfit/waveform.h:9-27): 10% cosine taper at both ends.
__global__ void k_taper(float *tw, float dt, int nt) {
    const int it = blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= nt) return;
    const float pi = 3.1415927f;
    float t_end = (nt - 1) * dt;
    float taper_width = t_end / 10;
    float t_min = taper_width;
    float t_max = t_end - taper_width;
    float t = it * dt;
    if (t <= t_min)
        tw[it] = 0.5 + 0.5 * cosf(pi * (t_min - t) / (taper_width));
    else if (t >= t_max)
        tw[it] = 0.5 + 0.5 * cosf(pi * (t_max - t) / (taper_width));
    else
        tw[it] = 1;
}

cudaError_t launch_taper(float *tw, float dt, int nt, cudaStream_t st) {
    k_taper<<<(nt + 255) / 256, 256, 0, st>>>(tw, dt, nt);
    return cudaGetLastError();
}

// One batch trace: synthetic, observed and adjoint-source rows.
struct TraceRef {
    const float *syn;
    const float *obs;
    float *adstf;
};

__device__ __forceinline__ double block_sum(double v, double *red) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    __syncthreads();
    return t;  // valid in thread 0
}

__device__ __forceinline__ float block_max(float v, float *red) {
    for (int o = 16; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    float t = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
    for (int o = 16; o; o >>= 1) t = fmaxf(t, __shfl_xor_sync(0xffffffffu, t, o));
    __syncthreads();
    return t;  // valid in every thread of warp 0; broadcast below
}

// WaveformMisfit::run per trace (misfit/waveform.h:4-8,35-40):
// r = (syn - obs) * tw, adstf[nt-1-it] = 2 * r * tw, value ||r|| * sqrt(dt).
__global__ void k_waveform(const TraceRef *__restrict__ tr, const float *__restrict__ tw, int nt, float sqrt_dt,
                           double *val) {
    __shared__ double red[32];
    const TraceRef T = tr[blockIdx.x];
    double acc = 0.0;
    for (int it = threadIdx.x; it < nt; it += blockDim.x) {
        const float w = tw[it];
        const float r = (T.syn[it] - T.obs[it]) * w;
        T.adstf[nt - it - 1] = r * w * 2;
        acc += (double)r * (double)r;
    }
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) val[blockIdx.x] = sqrt(acc) * (double)sqrt_dt;
}

// Waveform misfit over an arbitrary table of trace references (used by the
// serving engine, one request at a time).
cudaError_t launch_waveform_refs(const void *refs, const float *tw, int ntr, int nt, float sqrt_dt, double *val,
                                 cudaStream_t st) {
    if (ntr <= 0) return cudaSuccess;
    k_waveform<<<ntr, 256, 0, st>>>(static_cast<const TraceRef *>(refs), tw, nt, sqrt_dt, val);
    return cudaGetLastError();
}

// ---- envelope (misfit/envelope.h:4-90)
// Rows of n complex samples; row < nrow_a come from `a` rows, the rest from
// `b` rows (real part, imaginary 0).
__global__ void k_env_load(cufftComplex *c, const TraceRef *__restrict__ tr, int first, int ntr, int nt) {
    const int row = blockIdx.x;
    const int q = row < ntr ? row : row - ntr;
    const float *src = row < ntr ? tr[first + q].syn : tr[first + q].obs;
    cufftComplex *dst = c + (size_t)row * nt;
    for (int it = threadIdx.x; it < nt; it += blockDim.x) dst[it] = make_cuComplex(src[it], 0.f);
}

// _hilbert mask (misfit/envelope.h:4-28): for even n, bins 1..n/2 doubled
// (Nyquist included), bin n/2+1 kept, higher bins zeroed; for odd n, bins
// 1..(n-1)/2 doubled and the rest zeroed. Bin 0 is kept.
__global__ void k_env_mask(cufftComplex *c, int nt) {
    cufftComplex *h = c + (size_t)blockIdx.x * nt;
    for (int i = threadIdx.x; i < nt; i += blockDim.x) {
        if (i == 0) continue;
        float f;
        if (nt % 2 == 0)
            f = i < nt / 2 + 1 ? 2.f : (i > nt / 2 + 1 ? 0.f : 1.f);
        else
            f = i < (nt + 1) / 2 ? 2.f : 0.f;
        if (f != 1.f) {
            h[i].x *= f;
            h[i].y *= f;
        }
    }
}

// After the first Hilbert pair: envelopes, etmp, the second Hilbert input
// (written over the obs row) and the misfit value ||esyn - eobs|| sqrt(dt).
__global__ void k_env_mid(cufftComplex *c, float *etmp, int ntr, int nt, float sqrt_dt, double *val) {
    __shared__ double red[32];
    __shared__ float redf[32];
    __shared__ float s_max;
    const int q = blockIdx.x;
    cufftComplex *cs = c + (size_t)q * nt;
    cufftComplex *co = c + (size_t)(ntr + q) * nt;
    float *et = etmp + (size_t)q * nt;
    const float inv_n = (float)nt;
    float m = 0.f;
    for (int it = threadIdx.x; it < nt; it += blockDim.x) {
        const float es = sqrtf(cs[it].x * cs[it].x + cs[it].y * cs[it].y) / inv_n;
        m = fmaxf(m, fabsf(es));
    }
    m = block_max(m, redf);
    if (threadIdx.x == 0) {
        float mx = m * 0.05;
        if (mx < 0.05) mx = 0.05;
        s_max = mx;
    }
    __syncthreads();
    const float mx = s_max;
    double acc = 0.0;
    for (int it = threadIdx.x; it < nt; it += blockDim.x) {
        const float es = sqrtf(cs[it].x * cs[it].x + cs[it].y * cs[it].y) / inv_n;
        const float eo = sqrtf(co[it].x * co[it].x + co[it].y * co[it].y) / inv_n;
        const float e = (es - eo) / (es + mx);
        et[it] = e;
        const float ersd = cs[it].y / inv_n * e;
        co[it] = make_cuComplex(ersd, 0.f);
        const double d = (double)es - (double)eo;
        acc += d * d;
    }
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) val[q] = sqrt(acc) * (double)sqrt_dt;
}

// prepareEnvelopeSTF (misfit/envelope.h:46-49): adstf[nt-1-it] = etmp*syn - H.
__global__ void k_env_final(const cufftComplex *c, const float *etmp, const TraceRef *__restrict__ tr, int first,
                            int ntr, int nt) {
    const int q = blockIdx.x;
    const TraceRef T = tr[first + q];
    const cufftComplex *co = c + (size_t)(ntr + q) * nt;
    const float *et = etmp + (size_t)q * nt;
    for (int it = threadIdx.x; it < nt; it += blockDim.x)
        T.adstf[nt - it - 1] = et[it] * T.syn[it] - co[it].y / (float)nt;
}

}  // namespace gb

// ------------------------------------------------------------ Misfit object
using namespace gb;

struct gb_misfit {
    Solver *s = nullptr;
    gb_filter *filter = nullptr;
    bool own_filter = false;
    int type = 0;
    float *obs[3] = {nullptr, nullptr, nullptr};  // [nsrc][nrec*nt]
    float *tw = nullptr;
    TraceRef *d_tr = nullptr;
    std::vector<TraceRef> h_tr;
    double *d_val = nullptr;
    std::vector<double> h_val;  // [nsrc][nrec][ncomp]
    double ref = 1.0;
    // envelope
    cufftHandle plan2 = 0, plan1 = 0;
    int rows = 0;
    cufftComplex *cbuf = nullptr;
    float *etmp = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    long long launches = 0;
    // pipelined batches: per-round timing events, per-trace values in pinned memory
    std::vector<cudaEvent_t> ev_r0, ev_r1;
    double *h_pin = nullptr;
    size_t h_pin_n = 0;
    // observed traces queued by gb_misfit_set_obs_async: the upload stream,
    // the event behind its copies, and whether the next run must wait for it
    cudaStream_t st_up = nullptr;
    cudaEvent_t ev_obs = nullptr;
    bool obs_pending = false;

    int comps(int *c) const {
        int n = 0;
        if (s->sh) c[n++] = 1;
        if (s->psv) {
            c[n++] = 0;
            c[n++] = 2;
        }
        return n;
    }
};

static int misfit_alloc(gb_misfit *m) {
    Solver &s = *m->s;
    const size_t tr = (size_t)s.nrec * s.nt;
    for (int c = 0; c < 3; c++) {
        const bool used = c == 1 ? s.sh : s.psv;
        if (!used) continue;
        GB_CUDA_TRY(cudaMalloc(&m->obs[c], std::max<size_t>(tr * s.nsrc, 1) * 4));
        GB_CUDA_TRY(cudaMemset(m->obs[c], 0, std::max<size_t>(tr * s.nsrc, 1) * 4));
    }
    GB_CUDA_TRY(cudaMalloc(&m->tw, (size_t)s.nt * 4));
    GB_CUDA_TRY(launch_taper(m->tw, s.dt, s.nt, s.st));
    GB_CUDA_TRY(cudaStreamSynchronize(s.st));
    GB_CUDA_TRY(cudaEventCreate(&m->e0));
    GB_CUDA_TRY(cudaEventCreate(&m->e1));
    int cs[3];
    const int nc = m->comps(cs);
    m->h_val.assign((size_t)s.nsrc * s.nrec * nc, 0.0);
    return GB_OK;
}

static int misfit_tables(gb_misfit *m, const int *shots, int n, cudaStream_t st = nullptr) {
    Solver &s = *m->s;
    if (!st) st = s.st;
    int cs[3];
    const int nc = m->comps(cs);
    const size_t ntr = (size_t)n * nc * s.nrec;
    if (m->h_tr.size() < ntr || !m->d_tr) {
        cudaFree(m->d_tr);
        cudaFree(m->d_val);
        const size_t cap = (size_t)s.capacity * nc * std::max(s.nrec, 1);
        GB_CUDA_TRY(cudaMalloc(&m->d_tr, cap * sizeof(TraceRef)));
        GB_CUDA_TRY(cudaMalloc(&m->d_val, cap * sizeof(double)));
        m->h_tr.resize(cap);
    }
    // order: slot, receiver, component (the reference's summation order)
    size_t q = 0;
    for (int b = 0; b < n; b++)
        for (int ir = 0; ir < s.nrec; ir++)
            for (int k = 0; k < nc; k++) {
                const int c = cs[k];
                const size_t off = (size_t)ir * s.nt;
                m->h_tr[q].syn = s.slots[b].out[c] + off;
                m->h_tr[q].obs = m->obs[c] + (size_t)shots[b] * s.nrec * s.nt + off;
                m->h_tr[q].adstf = s.slots[b].adstf[c] + off;
                q++;
            }
    GB_CUDA_TRY(cudaMemcpyAsync(m->d_tr, m->h_tr.data(), ntr * sizeof(TraceRef), cudaMemcpyHostToDevice, st));
    return GB_OK;
}

static int envelope_plans(gb_misfit *m, int rows) {
    Solver &s = *m->s;
    if (m->rows >= rows && m->cbuf) return GB_OK;
    if (m->plan2) cufftDestroy(m->plan2);
    if (m->plan1) cufftDestroy(m->plan1);
    cudaFree(m->cbuf);
    cudaFree(m->etmp);
    m->plan1 = m->plan2 = 0;
    int n[1] = {s.nt};
    if (cufftPlanMany(&m->plan2, 1, n, nullptr, 1, s.nt, nullptr, 1, s.nt, CUFFT_C2C, 2 * rows) != CUFFT_SUCCESS ||
        cufftPlanMany(&m->plan1, 1, n, nullptr, 1, s.nt, nullptr, 1, s.nt, CUFFT_C2C, rows) != CUFFT_SUCCESS) {
        set_error("envelope misfit: cuFFT plan creation failed");
        return GB_ERR_CUDA;
    }
    cufftSetStream(m->plan2, s.st);
    cufftSetStream(m->plan1, s.st);
    GB_CUDA_TRY(cudaMalloc(&m->cbuf, (size_t)2 * rows * s.nt * sizeof(cufftComplex)));
    GB_CUDA_TRY(cudaMalloc(&m->etmp, (size_t)rows * s.nt * 4));
    m->rows = rows;
    return GB_OK;
}

static int fft_error() {
    set_error("envelope misfit: cuFFT execution failed");
    return GB_ERR_CUDA;
}

// traces [tr0, tr0 + ntr) of the table, on stream st
static int envelope_run(gb_misfit *m, int ntr, int tr0 = 0, cudaStream_t st = nullptr) {
    Solver &s = *m->s;
    if (!st) st = s.st;
    const int rows = std::min(ntr, 4096);
    int rc = envelope_plans(m, rows);
    if (rc) return rc;
    cufftSetStream(m->plan2, st);
    cufftSetStream(m->plan1, st);
    const float sq = std::sqrt(s.dt);
    for (int first = tr0; first < tr0 + ntr; first += rows) {
        const int r = std::min(rows, tr0 + ntr - first);
        k_env_load<<<2 * r, 256, 0, st>>>(m->cbuf, m->d_tr, first, r, s.nt);
        GB_CUDA_TRY(cudaGetLastError());
        // rows [0, r) hold synthetics and [r, 2r) observations; a short tail
        // still runs the full plan, the rows past 2r are never read
        if (cufftExecC2C(m->plan2, m->cbuf, m->cbuf, CUFFT_FORWARD) != CUFFT_SUCCESS) return fft_error();
        k_env_mask<<<2 * r, 256, 0, st>>>(m->cbuf, s.nt);
        GB_CUDA_TRY(cudaGetLastError());
        if (cufftExecC2C(m->plan2, m->cbuf, m->cbuf, CUFFT_INVERSE) != CUFFT_SUCCESS) return fft_error();
        k_env_mid<<<r, 256, 0, st>>>(m->cbuf, m->etmp, r, s.nt, sq, m->d_val + first);
        GB_CUDA_TRY(cudaGetLastError());
        cufftComplex *co = m->cbuf + (size_t)r * s.nt;
        if (cufftExecC2C(m->plan1, co, co, CUFFT_FORWARD) != CUFFT_SUCCESS) return fft_error();
        k_env_mask<<<r, 256, 0, st>>>(co, s.nt);
        GB_CUDA_TRY(cudaGetLastError());
        if (cufftExecC2C(m->plan1, co, co, CUFFT_INVERSE) != CUFFT_SUCCESS) return fft_error();
        k_env_final<<<r, 256, 0, st>>>(m->cbuf, m->etmp, m->d_tr, first, r, s.nt);
        GB_CUDA_TRY(cudaGetLastError());
        m->launches += 5;
    }
    cufftSetStream(m->plan2, s.st);
    cufftSetStream(m->plan1, s.st);
    return GB_OK;
}

// Misfit of one forward batch: adjoint sources into the slots, per-trace
// values into h_val.
static int misfit_batch(gb_misfit *m, const int *shots, int n) {
    Solver &s = *m->s;
    int rc = misfit_tables(m, shots, n);
    if (rc) return rc;
    int cs[3];
    const int nc = m->comps(cs);
    const int ntr = n * nc * s.nrec;
    if (ntr == 0) return GB_OK;
    if (m->obs_pending) GB_CUDA_TRY(cudaStreamWaitEvent(s.st, m->ev_obs, 0));
    GB_CUDA_TRY(cudaEventRecord(m->e0, s.st));
    if (m->type == 0) {
        k_waveform<<<ntr, 256, 0, s.st>>>(m->d_tr, m->tw, s.nt, std::sqrt(s.dt), m->d_val);
        GB_CUDA_TRY(cudaGetLastError());
        m->launches += 1;
    } else {
        rc = envelope_run(m, ntr);
        if (rc) return rc;
    }
    GB_CUDA_TRY(cudaEventRecord(m->e1, s.st));
    std::vector<double> v(ntr);
    GB_CUDA_TRY(cudaMemcpyAsync(v.data(), m->d_val, ntr * sizeof(double), cudaMemcpyDeviceToHost, s.st));
    GB_CUDA_TRY(cudaStreamSynchronize(s.st));
    float ms = 0;
    if (cudaEventElapsedTime(&ms, m->e0, m->e1) == cudaSuccess)
        s.stats.misfit_ms += ms;
    else
        (void)cudaGetLastError();
    for (int b = 0; b < n; b++)
        std::copy(v.begin() + (size_t)b * nc * s.nrec, v.begin() + (size_t)(b + 1) * nc * s.nrec,
                  m->h_val.begin() + (size_t)shots[b] * nc * s.nrec);
    return GB_OK;
}

// Pipelined misfit of a batch whose forward pass runs as rounds (the
// solver's pipe_plan): round r's traces are processed on the side stream as
// soon as that round's forward has finished, overlapping the next round on
// the SMs its clusters leave free, and each round signals the adjoint round
// that needs it. Per-trace values land in pinned memory; misfit_pipe_finish
// books them once the adjoint pass has synchronised.
static int misfit_batch_pipe(gb_misfit *m, const int *shots, int n) {
    Solver &s = *m->s;
    int cs[3];
    const int nc = m->comps(cs);
    const int per_shot = nc * s.nrec;
    const int ntr = n * per_shot;
    if (ntr == 0) return GB_OK;
    // the trace table of the batch, uploaded on the side stream ahead of its
    // first wait (the main stream is still running the forward rounds)
    int rc = misfit_tables(m, shots, n, s.st_side);
    if (rc) return rc;
    if (m->h_pin_n < (size_t)ntr) {
        if (m->h_pin) cudaFreeHost(m->h_pin);
        m->h_pin = nullptr;
        m->h_pin_n = 0;
        GB_CUDA_TRY(cudaMallocHost(&m->h_pin, (size_t)ntr * sizeof(double)));
        m->h_pin_n = ntr;
    }
    while ((int)m->ev_r0.size() < s.pipe_rounds) {
        cudaEvent_t a = nullptr, b = nullptr;
        GB_CUDA_TRY(cudaEventCreate(&a));
        GB_CUDA_TRY(cudaEventCreate(&b));
        m->ev_r0.push_back(a);
        m->ev_r1.push_back(b);
    }
    cudaStream_t side = s.st_side;
    if (m->obs_pending) GB_CUDA_TRY(cudaStreamWaitEvent(side, m->ev_obs, 0));
    for (int r = 0; r < s.pipe_rounds; r++) {
        const int b0 = r * s.pipe_occ, nb = std::min(s.pipe_occ, n - b0);
        const int tr0 = b0 * per_shot, ntr_r = nb * per_shot;
        GB_CUDA_TRY(cudaStreamWaitEvent(side, s.ev_fwd_round[r], 0));
        GB_CUDA_TRY(cudaEventRecord(m->ev_r0[r], side));
        if (m->type == 0) {
            k_waveform<<<ntr_r, 256, 0, side>>>(m->d_tr + tr0, m->tw, s.nt, std::sqrt(s.dt), m->d_val + tr0);
            GB_CUDA_TRY(cudaGetLastError());
            m->launches += 1;
        } else {
            rc = envelope_run(m, ntr_r, tr0, side);
            if (rc) return rc;
        }
        GB_CUDA_TRY(cudaEventRecord(m->ev_r1[r], side));
        GB_CUDA_TRY(cudaEventRecord(s.ev_mis_round[r], side));
    }
    GB_CUDA_TRY(cudaMemcpyAsync(m->h_pin, m->d_val, (size_t)ntr * sizeof(double), cudaMemcpyDeviceToHost, side));
    return GB_OK;
}

// After the pipelined batch's adjoint (or a synchronisation of both streams):
// per-trace values into h_val, misfit time booked.
static int misfit_pipe_finish(gb_misfit *m, const int *shots, int n) {
    Solver &s = *m->s;
    GB_CUDA_TRY(cudaStreamSynchronize(s.st_side));
    int cs[3];
    const int per_shot = m->comps(cs) * s.nrec;
    for (int r = 0; r < s.pipe_rounds; r++) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, m->ev_r0[r], m->ev_r1[r]) == cudaSuccess)
            s.stats.misfit_ms += ms;
        else
            (void)cudaGetLastError();
    }
    for (int b = 0; b < n; b++)
        std::copy(m->h_pin + (size_t)b * per_shot, m->h_pin + (size_t)(b + 1) * per_shot,
                  m->h_val.begin() + (size_t)shots[b] * per_shot);
    return GB_OK;
}

static int misfit_run(gb_misfit *m, bool kernel, bool snapshot, double *value) {
    Solver &s = *m->s;
    if (kernel) {
        int rc = s.init_kernels();
        if (rc) return rc;
    }
    int rc = s.ensure_slots(1);
    if (rc) return rc;
    const int bsz = snapshot ? 1 : s.capacity;
    std::vector<int> shots;
    for (int first = 0; first < s.nsrc; first += bsz) {
        shots.clear();
        for (int is = first; is < std::min(s.nsrc, first + bsz); is++) shots.push_back(is);
        const int n = (int)shots.size();
        // a gradient whose forward runs in rounds of resident clusters: the
        // misfit of each round overlaps the next round of the forward and the
        // adjoint of the previous one
        if (kernel && !snapshot && s.pipe_plan(shots.data(), n) > 1) {
            s.pipe_on = true;
            rc = s.forward(shots.data(), n, true, true, false);
            if (!rc) rc = misfit_batch_pipe(m, shots.data(), n);
            if (!rc) rc = s.adjoint(shots.data(), n, false, shots[0]);
            s.pipe_on = false;
            if (!rc) rc = misfit_pipe_finish(m, shots.data(), n);
            if (rc) {
                cudaStreamSynchronize(s.st_side);
                (void)s.book_forward_pass();
                return rc;
            }
            continue;
        }
        rc = s.forward(shots.data(), n, kernel, s.adj || s.trace_type == 1, false);
        if (rc) return rc;
        rc = misfit_batch(m, shots.data(), n);
        if (rc) return rc;
        if (kernel) {
            rc = s.adjoint(shots.data(), n, snapshot, shots[0]);
            if (rc) return rc;
        }
    }
    if (kernel && m->filter) {
        GB_CUDA_TRY(cudaEventRecord(m->e0, s.st));
        for (float *k : {s.k_lambda, s.k_mu, s.k_rho}) {
            rc = gb_filter_apply(m->filter, k);
            if (rc) return rc;
        }
        GB_CUDA_TRY(cudaEventRecord(m->e1, s.st));
        GB_CUDA_TRY(cudaEventSynchronize(m->e1));
        float ms = 0;
        if (cudaEventElapsedTime(&ms, m->e0, m->e1) == cudaSuccess)
            s.stats.filter_ms += ms;
        else
            (void)cudaGetLastError();
        m->launches += 6;
    }
    double total = 0.0;
    for (double v : m->h_val) total += v;
    if (value) *value = total;
    s.stats.launches += m->launches;
    m->launches = 0;
    return GB_OK;
}

// ------------------------------------------------------------ C ABI
extern "C" {

static gb_misfit *misfit_new(int type, gb_solver *sol, gb_filter *f, int sigma, bool make_filter) {
    if (!sol) {
        set_error("misfit: null solver");
        return nullptr;
    }
    if (type != 0 && type != 1) {
        set_error("misfit: type must be 0 (waveform) or 1 (envelope)");
        return nullptr;
    }
    gb_misfit *m = new gb_misfit();
    m->s = &sol->s;
    m->type = type;
    m->filter = f;
    if (!f && make_filter) {
        m->filter = gb_filter_create(sol->s.nx, sol->s.nz, sigma);
        if (!m->filter) {
            delete m;
            return nullptr;
        }
        m->own_filter = true;
    }
    if (misfit_alloc(m)) {
        gb_misfit_destroy(m);
        return nullptr;
    }
    return m;
}

gb_misfit *gb_misfit_create(const gb_config *cfg, gb_solver *sol, gb_filter *f) {
    if (!cfg || !sol) {
        set_error("gb_misfit_create: null argument");
        return nullptr;
    }
    const Config &c = *reinterpret_cast<const Config *>(cfg);
    // filter = 0 is the Gaussian filter; the reference dereferences a null
    // filter for any other value (misfit/misfit.h:96), here it means none.
    const bool want = c.iv("filter") == 0;
    gb_misfit *m = misfit_new(c.iv("misfit"), sol, want ? f : nullptr, c.iv("filter_sigma"), want && !f);
    if (!m) return nullptr;
    Solver &s = sol->s;
    const size_t tr = (size_t)s.nrec * s.nt;
    int rc = GB_OK;
    if (c.iv("trace_file")) {
        std::vector<float> buf(tr);
        for (int is = 0; is < s.nsrc && !rc; is++) {
            for (int comp = 0; comp < 3 && !rc; comp++) {
                if (!m->obs[comp]) continue;
                const char *nm[3] = {"x", "y", "z"};
                const std::string file = s.path + "/traces/" + (s.trace_type ? "u" : "v") + nm[comp] + "_" + pad6(is) + ".su";
                rc = read_su(file, buf.data(), s.nrec, s.nt);
                if (rc) break;
                if (s.trace_type == 0) {
                    // v -> u (misfit/misfit.h:110-120)
                    for (int ir = 0; ir < s.nrec; ir++) {
                        float *b = buf.data() + (size_t)ir * s.nt;
                        b[0] *= s.dt;
                        for (int it = 1; it < s.nt; it++) b[it] = b[it - 1] + b[it] * s.dt;
                    }
                }
                if (cudaMemcpy(m->obs[comp] + (size_t)is * tr, buf.data(), tr * 4, cudaMemcpyHostToDevice) != cudaSuccess)
                    rc = GB_ERR_CUDA;
            }
        }
    } else {
        std::cout << "Generating traces" << std::endl;
        rc = s.import_model(true);
        if (!rc) rc = s.ensure_slots(1);
        std::vector<int> shots;
        for (int first = 0; first < s.nsrc && !rc; first += s.capacity) {
            const int b = std::min(s.capacity, s.nsrc - first);
            shots.clear();
            for (int q = 0; q < b; q++) shots.push_back(first + q);
            rc = s.forward(shots.data(), b, false, s.adj || s.trace_type == 1, false);
            for (int q = 0; q < b && !rc; q++)
                for (int comp = 0; comp < 3; comp++)
                    if (m->obs[comp] &&
                        cudaMemcpy(m->obs[comp] + (size_t)(first + q) * tr, s.slots[q].out[comp], tr * 4,
                                   cudaMemcpyDeviceToDevice) != cudaSuccess)
                        rc = GB_ERR_CUDA;
        }
    }
    if (!rc) rc = s.import_model(false);
    if (rc) {
        gb_misfit_destroy(m);
        return nullptr;
    }
    return m;
}

gb_misfit *gb_misfit_create_obs(int type, gb_solver *sol, gb_filter *f, const float *ox, const float *oy,
                                const float *oz) {
    gb_misfit *m = misfit_new(type, sol, f, 0, false);
    if (!m) return nullptr;
    if (gb_misfit_set_obs(m, ox, oy, oz)) {
        gb_misfit_destroy(m);
        return nullptr;
    }
    return m;
}

int gb_misfit_set_obs(gb_misfit *m, const float *ox, const float *oy, const float *oz) {
    if (!m) return GB_ERR_ARG;
    Solver &s = *m->s;
    const float *h[3] = {ox, oy, oz};
    const size_t bytes = (size_t)s.nsrc * s.nrec * s.nt * 4;
    if (m->obs_pending) {  // queued copies of gb_misfit_set_obs_async land first
        GB_CUDA_TRY(cudaEventSynchronize(m->ev_obs));
        m->obs_pending = false;
    }
    for (int c = 0; c < 3; c++) {
        if (!m->obs[c]) continue;
        if (!h[c]) {
            set_error("gb_misfit_set_obs: component " + std::to_string(c) + " is used but was not given");
            return GB_ERR_ARG;
        }
        GB_CUDA_TRY(cudaMemcpyAsync(m->obs[c], h[c], bytes, cudaMemcpyHostToDevice, s.st));
    }
    GB_CUDA_TRY(cudaStreamSynchronize(s.st));
    return GB_OK;
}

int gb_misfit_set_obs_async(gb_misfit *m, const float *ox, const float *oy, const float *oz) {
    if (!m) return GB_ERR_ARG;
    Solver &s = *m->s;
    const float *h[3] = {ox, oy, oz};
    for (int c = 0; c < 3; c++)
        if (m->obs[c] && !h[c]) {
            set_error("gb_misfit_set_obs_async: component " + std::to_string(c) + " is used but was not given");
            return GB_ERR_ARG;
        }
    if (!m->st_up) {
        GB_CUDA_TRY(cudaStreamCreateWithFlags(&m->st_up, cudaStreamNonBlocking));
        GB_CUDA_TRY(cudaEventCreateWithFlags(&m->ev_obs, cudaEventDisableTiming));
    }
    // (the solver's stream is idle between calls: no kernel of an earlier
    // run still reads the observed traces)
    const size_t bytes = (size_t)s.nsrc * s.nrec * s.nt * 4;
    for (int c = 0; c < 3; c++)
        if (m->obs[c]) GB_CUDA_TRY(cudaMemcpyAsync(m->obs[c], h[c], bytes, cudaMemcpyHostToDevice, m->st_up));
    GB_CUDA_TRY(cudaEventRecord(m->ev_obs, m->st_up));
    m->obs_pending = true;
    return GB_OK;
}

int gb_misfit_run(gb_misfit *m, int kernel, int snapshot, double *value) {
    if (!m) return GB_ERR_ARG;
    const int rc = misfit_run(m, kernel != 0, snapshot != 0, value);
    if (m->obs_pending) {
        // the copies are complete once the run's misfit stages have run; an
        // early error return waits for them here
        GB_CUDA_TRY(cudaEventSynchronize(m->ev_obs));
        m->obs_pending = false;
    }
    return rc;
}

int gb_misfit_trace_values(gb_misfit *m, double *out, size_t n) {
    if (!m || !out) return GB_ERR_ARG;
    if (n > m->h_val.size()) n = m->h_val.size();
    std::copy(m->h_val.begin(), m->h_val.begin() + n, out);
    return GB_OK;
}

void gb_misfit_destroy(gb_misfit *m) {
    if (!m) return;
    // the solver may already be destroyed: wait for the device instead of its stream
    cudaDeviceSynchronize();
    for (int c = 0; c < 3; c++) cudaFree(m->obs[c]);
    cudaFree(m->tw);
    cudaFree(m->d_tr);
    cudaFree(m->d_val);
    cudaFree(m->cbuf);
    cudaFree(m->etmp);
    if (m->plan1) cufftDestroy(m->plan1);
    if (m->plan2) cufftDestroy(m->plan2);
    if (m->e0) cudaEventDestroy(m->e0);
    if (m->e1) cudaEventDestroy(m->e1);
    if (m->own_filter) gb_filter_destroy(m->filter);
    for (cudaEvent_t e : m->ev_r0) cudaEventDestroy(e);
    for (cudaEvent_t e : m->ev_r1) cudaEventDestroy(e);
    if (m->h_pin) cudaFreeHost(m->h_pin);
    if (m->ev_obs) cudaEventDestroy(m->ev_obs);
    if (m->st_up) cudaStreamDestroy(m->st_up);
    delete m;
}

}  // extern "C"
