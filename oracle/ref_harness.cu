// Reference-kernel harness: TEST INFRASTRUCTURE ONLY (only tests/ load it).
//
// Runs the reference's own device code under a restatement of its host loops,
// so that the GB300 path can be compared with the reference's FP32 arithmetic
// as nvcc compiles it, not only with the C restatement in fdm_oracle.c. The
// kernels are the reference's, compiled from its sources into
// oracle/_ref/inv_ref.cubin by oracle/Makefile (target `ref`, only where the
// reference sources are present); this file holds no reference code. It loads
// the cubin with the runtime's library API, looks the kernels up by their
// mangled names (as nvcc reports them) and launches them in the order of:
//   FdmSolver::runForward  solver/fdm.h:515-570 (divS, addSTF, divV, saveRec,
//                          checkpoints before/after the step: fdm.h:521-560)
//   FdmSolver::runAdjoint  solver/fdm.h:571-612
//   divS / divV            solver/fdm.h:273-294
//   initAbsbound           solver/fdm.h:48-74 (launched as in fdm.h:453-456)
//   GaussianFilter         filter/gaussian.h:37-61
//   WaveformMisfit::run    misfit/waveform.h:35-40 (taper: waveform.h:44-51)
//   EnvelopeMisfit::run    misfit/envelope.h:58-90 (hilbert: envelope.h:91-98)
//   Optimizer primitives   optimizer/optimizer.h:49-107 (p_calc, p_dot, p_amax
//                          over one parameter: device::calc/dot/amax,
//                          lib/device.h:157-192) and polyfit/solveQR
//                          (optimizer.h:108-178, cuSOLVER QR, reduceSystem,
//                          cuBLAS triangular solve)
// (the misfits with cuFFT and cuBLAS as the reference calls them, one trace
// at a time, device::amax/norm from lib/device.h:170-180)
// with the reference's launch shapes (Dim::init, lib/device.h:46-57, with
// device::nthread = 0: nx blocks of nz threads).
//
// Checkpoint layout (the C oracle's): ckpt[(isfe * nf + q) * n], q over
// (uy, vy) for SH or (ux, uz, vx, vz) for P-SV; one wave system per call.
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <cufft.h>
#include <cusolverDn.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

// the C oracle's parameter block (oracle.py OrcParams); outside the anonymous
// namespace so that the extern "C" entry points taking it keep external linkage
struct RefParams {
    int nx, nz, nt, sfe, sh, psv, nsrc, nrec;
    double dx, dz, dt;
    int record_u, adj, inv_lambda, inv_mu, inv_rho;
};

namespace {

// member layout of the reference's Dim (lib/device.h:7-13), passed by value
struct Dim {
    int nx, nz, dg, db, size;
};

Dim make_dim(int nx, int nz) { return Dim{nx, nz, nx, nz, nx * nz}; }

enum K {
    K_DIVSY, K_DIVSXZ, K_DIVVY, K_DIVVXZ, K_UPDSY, K_UPDSXZ, K_UPDVY, K_UPDVXZ, K_ADDSTF, K_SAVEREC,
    K_IRHOY, K_IRHOXZ, K_IMUY, K_IMUXZ, K_ILAMXZ, K_ABS, K_GINIT, K_GX, K_GZ,
    K_TAPER, K_DIFF, K_HILB, K_R2C, K_C2IMAG, K_C2ABS, K_ETMP, K_ESTF, K_MUL, K_AXPBY, K_SCALE, K_REDSYS, K_N
};
// names as nvcc reports them for the reference's kernels
const char *kNames[K_N] = {
    "_ZN10_FdmSolver5divSYEPfS0_S0_ff3Dim",
    "_ZN10_FdmSolver6divSXZEPfS0_S0_S0_S0_ff3Dim",
    "_ZN10_FdmSolver5divVYEPfS0_S0_ff3Dim",
    "_ZN10_FdmSolver6divVXZEPfS0_S0_S0_S0_S0_ff3Dim",
    "_ZN10_FdmSolver8updateSYEPfS0_S0_S0_S0_f3Dim",
    "_ZN10_FdmSolver9updateSXZEPfS0_S0_S0_S0_S0_S0_S0_S0_f3Dim",
    "_ZN10_FdmSolver8updateVYEPfS0_S0_S0_S0_f3Dim",
    "_ZN10_FdmSolver9updateVXZEPfS0_S0_S0_S0_S0_S0_S0_f3Dim",
    "_ZN10_FdmSolver6addSTFEPfS0_S0_S0_S0_S0_PmS1_ibbmm3Dim",
    "_ZN10_FdmSolver7saveRecEPfS0_S0_S0_S0_S0_PmS1_bbmm3Dim",
    "_ZN10_FdmSolver15interactionRhoYEPfS0_S0_f3Dim",
    "_ZN10_FdmSolver16interactionRhoXZEPfS0_S0_S0_S0_f3Dim",
    "_ZN10_FdmSolver14interactionMuYEPfS0_S0_S0_S0_f3Dim",
    "_ZN10_FdmSolver15interactionMuXZEPfS0_S0_S0_S0_S0_S0_S0_S0_f3Dim",
    "_ZN10_FdmSolver19interactionLambdaXZEPfS0_S0_S0_S0_f3Dim",
    "_ZN10_FdmSolver12initAbsboundEPfmfbbbb3Dim",
    "_ZN15_GaussianFilter18initialiseGaussianEPfm3Dim",
    "_ZN15_GaussianFilter13filterKernelXEPfS0_m3Dim",
    "_ZN15_GaussianFilter13filterKernelZEPfS0_S0_m3Dim",
    "_ZN15_WaveformMisfit5taperEPffi",
    "_ZN15_WaveformMisfit4diffEPfS0_S0_S0_S0_m",
    "_ZN15_EnvelopeMisfit8_hilbertEP6float2m",
    "_ZN15_EnvelopeMisfit7copyR2CEP6float2Pf",
    "_ZN15_EnvelopeMisfit10copyC2ImagEPfP6float2i",
    "_ZN15_EnvelopeMisfit9copyC2AbsEPfP6float2i",
    "_ZN15_EnvelopeMisfit11envelopeTmpEPfS0_S0_f",
    "_ZN15_EnvelopeMisfit18prepareEnvelopeSTFEPfS0_S0_S0_m",
    "_ZN6device5_calcEPfS0_S0_3Dim",
    "_ZN6device5_calcEPffS0_fS0_3Dim",
    "_ZN6device5_calcEPffS0_3Dim",
    "_ZN10_Optimizer12reduceSystemEPKdPdS1_S2_ii",
};

cudaLibrary_t g_lib = nullptr;
cudaKernel_t g_k[K_N] = {};
std::string g_err;
cublasHandle_t g_cb = nullptr;  // device::cublas_handle of the optimizer primitives

int fail(const std::string &what, cudaError_t e) {
    g_err = what + ": " + cudaGetErrorString(e);
    return 1;
}
#define REF_TRY(x)                                   \
    do {                                             \
        cudaError_t e_ = (x);                        \
        if (e_ != cudaSuccess) return fail(#x, e_);  \
    } while (0)

int launch(K k, unsigned grid, unsigned block, void **args) {
    REF_TRY(cudaLaunchKernel((const void *)g_k[k], dim3(grid), dim3(block), args, 0, nullptr));
    return 0;
}

// device buffers of one call, freed on scope exit
struct Bufs {
    std::vector<void *> p;
    ~Bufs() {
        for (void *q : p) cudaFree(q);
    }
    template <typename T>
    T *alloc(size_t n) {
        void *q = nullptr;
        if (cudaMalloc(&q, (n ? n : 1) * sizeof(T)) != cudaSuccess) return nullptr;
        cudaMemset(q, 0, (n ? n : 1) * sizeof(T));
        p.push_back(q);
        return static_cast<T *>(q);
    }
};

struct Fields {
    float *vy, *uy, *sxy, *szy, *dsy, *dvydx, *dvydz, *dvydx_fw, *dvydz_fw;
    float *vx, *vz, *ux, *uz, *sxx, *szz, *sxz, *dsx, *dsz, *dvxdx, *dvxdz, *dvzdx, *dvzdz;
    float *dvxdx_fw, *dvxdz_fw, *dvzdx_fw, *dvzdz_fw;
    float *lam, *mu, *rho, *ab;
};

bool alloc_fields(Bufs &b, Fields &f, size_t n) {
    float **all[] = {&f.vy, &f.uy, &f.sxy, &f.szy, &f.dsy, &f.dvydx, &f.dvydz, &f.dvydx_fw, &f.dvydz_fw,
                     &f.vx, &f.vz, &f.ux, &f.uz, &f.sxx, &f.szz, &f.sxz, &f.dsx, &f.dsz, &f.dvxdx, &f.dvxdz,
                     &f.dvzdx, &f.dvzdz, &f.dvxdx_fw, &f.dvxdz_fw, &f.dvzdx_fw, &f.dvzdz_fw,
                     &f.lam, &f.mu, &f.rho, &f.ab};
    for (float **q : all)
        if (!(*q = b.alloc<float>(n))) return false;
    return true;
}

int upload_model(const Fields &f, size_t n, const float *lam, const float *mu, const float *rho, const float *ab) {
    REF_TRY(cudaMemcpy(f.lam, lam, n * 4, cudaMemcpyHostToDevice));
    REF_TRY(cudaMemcpy(f.mu, mu, n * 4, cudaMemcpyHostToDevice));
    REF_TRY(cudaMemcpy(f.rho, rho, n * 4, cudaMemcpyHostToDevice));
    REF_TRY(cudaMemcpy(f.ab, ab, n * 4, cudaMemcpyHostToDevice));
    return 0;
}

size_t *upload_ids(Bufs &b, const int *ids, int n) {
    std::vector<size_t> h(n > 0 ? n : 1, 0);
    for (int q = 0; q < n; q++) h[q] = (size_t)ids[q];
    size_t *d = b.alloc<size_t>(h.size());
    if (d) cudaMemcpy(d, h.data(), h.size() * sizeof(size_t), cudaMemcpyHostToDevice);
    return d;
}

// divS (solver/fdm.h:273-281)
int div_s(const RefParams &p, Fields &f, Dim &dim) {
    float dx = (float)p.dx, dz = (float)p.dz;
    if (p.sh) {
        void *a[] = {&f.dsy, &f.sxy, &f.szy, &dx, &dz, &dim};
        if (launch(K_DIVSY, dim.dg, dim.db, a)) return 1;
    }
    if (p.psv) {
        void *a[] = {&f.dsx, &f.dsz, &f.sxx, &f.szz, &f.sxz, &dx, &dz, &dim};
        if (launch(K_DIVSXZ, dim.dg, dim.db, a)) return 1;
    }
    return 0;
}

// divV (solver/fdm.h:282-294)
int div_v(const RefParams &p, Fields &f, Dim &dim) {
    float dx = (float)p.dx, dz = (float)p.dz, dt = (float)p.dt;
    if (p.sh) {
        void *a1[] = {&f.vy, &f.uy, &f.dsy, &f.rho, &f.ab, &dt, &dim};
        void *a2[] = {&f.dvydx, &f.dvydz, &f.vy, &dx, &dz, &dim};
        void *a3[] = {&f.sxy, &f.szy, &f.dvydx, &f.dvydz, &f.mu, &dt, &dim};
        if (launch(K_UPDVY, dim.dg, dim.db, a1) || launch(K_DIVVY, dim.dg, dim.db, a2) ||
            launch(K_UPDSY, dim.dg, dim.db, a3))
            return 1;
    }
    if (p.psv) {
        void *a1[] = {&f.vx, &f.vz, &f.ux, &f.uz, &f.dsx, &f.dsz, &f.rho, &f.ab, &dt, &dim};
        void *a2[] = {&f.dvxdx, &f.dvxdz, &f.dvzdx, &f.dvzdz, &f.vx, &f.vz, &dx, &dz, &dim};
        void *a3[] = {&f.sxx, &f.szz, &f.sxz, &f.dvxdx, &f.dvxdz, &f.dvzdx, &f.dvzdz, &f.lam, &f.mu, &dt, &dim};
        if (launch(K_UPDVXZ, dim.dg, dim.db, a1) || launch(K_DIVVXZ, dim.dg, dim.db, a2) ||
            launch(K_UPDSXZ, dim.dg, dim.db, a3))
            return 1;
    }
    return 0;
}

int to_host(float *dst, const float *src, size_t n) {
    REF_TRY(cudaMemcpy(dst, src, n * 4, cudaMemcpyDeviceToHost));
    return 0;
}
int to_dev(float *dst, const float *src, size_t n) {
    REF_TRY(cudaMemcpy(dst, src, n * 4, cudaMemcpyHostToDevice));
    return 0;
}

bool valid(const RefParams *p) {
    return g_lib && p && p->nx > 4 && p->nz > 4 && p->nz <= 1024 && p->nt > 0 && (p->sh != 0) != (p->psv != 0);
}

}  // namespace

extern "C" {

const char *ref_last_error() { return g_err.c_str(); }

// Loads the cubin and looks up every kernel; 0 on success.
int ref_open(const char *cubin) {
    if (g_lib) return 0;
    REF_TRY(cudaFree(nullptr));
    REF_TRY(cudaLibraryLoadFromFile(&g_lib, cubin, nullptr, nullptr, 0, nullptr, nullptr, 0));
    for (int k = 0; k < K_N; k++) {
        const cudaError_t e = cudaLibraryGetKernel(&g_k[k], g_lib, kNames[k]);
        if (e != cudaSuccess) {
            cudaLibraryUnload(g_lib);
            g_lib = nullptr;
            return fail(std::string("kernel ") + kNames[k], e);
        }
    }
    return 0;
}

// initAbsbound into out[nx*nz] (solver/fdm.h:48-74).
int ref_absbound(int nx, int nz, int width, float alpha, int left, int right, int bottom, int top, float *out) {
    if (!g_lib || nx < 1 || nz < 1 || nz > 1024) return 1;
    Bufs b;
    float *d = b.alloc<float>((size_t)nx * nz);
    if (!d) return 1;
    Dim dim = make_dim(nx, nz);
    size_t w = (size_t)width;
    bool l = left, r = right, bo = bottom, t = top;
    void *a[] = {&d, &w, &alpha, &l, &r, &bo, &t, &dim};
    if (launch(K_ABS, dim.dg, dim.db, a)) return 1;
    return to_host(out, d, (size_t)nx * nz);
}

// FdmSolver::runForward for one wave system. Traces out_* [nrec*nt] (the
// unused components untouched); ckpt [nsfe*nf*n] when p->adj and p->sfe.
int ref_forward(const RefParams *p, const float *lam, const float *mu, const float *rho, const float *ab,
                const float *stf_x, const float *stf_y, const float *stf_z, const int *src_x, const int *src_z,
                const int *rec_x, const int *rec_z, int isrc, float *out_x, float *out_y, float *out_z,
                float *ckpt) {
    if (!valid(p)) return 1;
    const size_t n = (size_t)p->nx * p->nz, nt = (size_t)p->nt;
    Bufs b;
    Fields f{};
    if (!alloc_fields(b, f, n) || upload_model(f, n, lam, mu, rho, ab)) return 1;
    float *stf[3], *out[3];
    const float *hs[3] = {stf_x, stf_y, stf_z};
    for (int c = 0; c < 3; c++) {
        stf[c] = b.alloc<float>((size_t)p->nsrc * nt);
        out[c] = b.alloc<float>((size_t)p->nrec * nt);
        if (!stf[c] || !out[c]) return 1;
        if (hs[c] && to_dev(stf[c], hs[c], (size_t)p->nsrc * nt)) return 1;
    }
    size_t *sx = upload_ids(b, src_x, p->nsrc), *sz = upload_ids(b, src_z, p->nsrc);
    size_t *rx = upload_ids(b, rec_x, p->nrec), *rz = upload_ids(b, rec_z, p->nrec);
    if (!sx || !sz || !rx || !rz) return 1;
    Dim dim = make_dim(p->nx, p->nz);
    const int nsfe = p->sfe ? p->nt / p->sfe : 0;
    const int nf = p->sh ? 2 : 4;
    bool sh = p->sh, psv = p->psv;
    for (size_t it = 0; it < nt; it++) {
        int isfe = -1;
        if (p->sfe && p->adj && (it + 1) % p->sfe == 0) isfe = nsfe - (int)((it + 1) / p->sfe);
        if (isfe >= 0 && ckpt) {
            float *c0 = ckpt + (size_t)isfe * nf * n;
            if (p->sh ? to_host(c0, f.uy, n) : (to_host(c0, f.ux, n) || to_host(c0 + n, f.uz, n))) return 1;
        }
        if (div_s(*p, f, dim)) return 1;
        {
            int is = isrc;
            size_t itv = it, ntv = nt;
            void *a[] = {&f.dsx, &f.dsy, &f.dsz, &stf[0], &stf[1], &stf[2], &sx, &sz, &is, &sh, &psv, &itv, &ntv, &dim};
            if (p->nsrc > 0 && launch(K_ADDSTF, p->nsrc, 1, a)) return 1;
        }
        if (div_v(*p, f, dim)) return 1;
        {
            float *wx = p->record_u ? f.ux : f.vx, *wy = p->record_u ? f.uy : f.vy, *wz = p->record_u ? f.uz : f.vz;
            size_t itv = it, ntv = nt;
            void *a[] = {&out[0], &out[1], &out[2], &wx, &wy, &wz, &rx, &rz, &sh, &psv, &itv, &ntv, &dim};
            if (p->nrec > 0 && launch(K_SAVEREC, p->nrec, 1, a)) return 1;
        }
        if (isfe >= 0 && ckpt) {
            float *c0 = ckpt + (size_t)isfe * nf * n;
            if (p->sh ? to_host(c0 + n, f.vy, n) : (to_host(c0 + 2 * n, f.vx, n) || to_host(c0 + 3 * n, f.vz, n)))
                return 1;
        }
    }
    REF_TRY(cudaDeviceSynchronize());
    float *ho[3] = {out_x, out_y, out_z};
    for (int c = 0; c < 3; c++)
        if (ho[c] && to_host(ho[c], out[c], (size_t)p->nrec * nt)) return 1;
    return 0;
}

// FdmSolver::runAdjoint for one wave system: adds this shot's contribution to
// the host kernels k_* [n] (the ones p->inv_* select).
int ref_adjoint(const RefParams *p, const float *lam, const float *mu, const float *rho, const float *ab,
                const float *ad_x, const float *ad_y, const float *ad_z, const int *rec_x, const int *rec_z,
                const float *ckpt, float *k_lambda, float *k_mu, float *k_rho) {
    if (!valid(p) || p->sfe <= 0 || !ckpt) return 1;
    const size_t n = (size_t)p->nx * p->nz, nt = (size_t)p->nt;
    Bufs b;
    Fields f{};
    if (!alloc_fields(b, f, n) || upload_model(f, n, lam, mu, rho, ab)) return 1;
    float *ad[3];
    const float *ha[3] = {ad_x, ad_y, ad_z};
    for (int c = 0; c < 3; c++) {
        ad[c] = b.alloc<float>((size_t)p->nrec * nt);
        if (!ad[c]) return 1;
        if (ha[c] && to_dev(ad[c], ha[c], (size_t)p->nrec * nt)) return 1;
    }
    float *kl = b.alloc<float>(n), *km = b.alloc<float>(n), *kr = b.alloc<float>(n);
    if (!kl || !km || !kr || to_dev(kl, k_lambda, n) || to_dev(km, k_mu, n) || to_dev(kr, k_rho, n)) return 1;
    size_t *rx = upload_ids(b, rec_x, p->nrec), *rz = upload_ids(b, rec_z, p->nrec);
    if (!rx || !rz) return 1;
    Dim dim = make_dim(p->nx, p->nz);
    const int nf = p->sh ? 2 : 4;
    const size_t sfe = (size_t)p->sfe;
    float dx = (float)p->dx, dz = (float)p->dz;
    bool sh = p->sh, psv = p->psv;
    for (size_t it = 0; it < nt; it++) {
        if (div_s(*p, f, dim)) return 1;
        {
            int is = -1;
            size_t itv = it, ntv = nt;
            void *a[] = {&f.dsx, &f.dsy, &f.dsz, &ad[0], &ad[1], &ad[2], &rx, &rz, &is, &sh, &psv, &itv, &ntv, &dim};
            if (p->nrec > 0 && launch(K_ADDSTF, p->nrec, 1, a)) return 1;
        }
        if (div_v(*p, f, dim)) return 1;
        if ((it + sfe) % sfe == 0) {
            const size_t isfe = (it + sfe) / sfe - 1;
            float ndt = (float)sfe * (float)p->dt;
            const float *c0 = ckpt + isfe * nf * n;
            if (p->sh) {
                if (to_dev(f.dsy, c0, n)) return 1;
                void *g1[] = {&f.dvydx, &f.dvydz, &f.uy, &dx, &dz, &dim};
                void *g2[] = {&f.dvydx_fw, &f.dvydz_fw, &f.dsy, &dx, &dz, &dim};
                if (launch(K_DIVVY, dim.dg, dim.db, g1) || launch(K_DIVVY, dim.dg, dim.db, g2)) return 1;
                if (to_dev(f.dsy, c0 + n, n)) return 1;
                void *ar[] = {&kr, &f.vy, &f.dsy, &ndt, &dim};
                void *am[] = {&km, &f.dvydx, &f.dvydx_fw, &f.dvydz, &f.dvydz_fw, &ndt, &dim};
                if (p->inv_rho && launch(K_IRHOY, dim.dg, dim.db, ar)) return 1;
                if (p->inv_mu && launch(K_IMUY, dim.dg, dim.db, am)) return 1;
            } else {
                if (to_dev(f.dsx, c0, n) || to_dev(f.dsz, c0 + n, n)) return 1;
                void *g1[] = {&f.dvxdx, &f.dvxdz, &f.dvzdx, &f.dvzdz, &f.ux, &f.uz, &dx, &dz, &dim};
                void *g2[] = {&f.dvxdx_fw, &f.dvxdz_fw, &f.dvzdx_fw, &f.dvzdz_fw, &f.dsx, &f.dsz, &dx, &dz, &dim};
                if (launch(K_DIVVXZ, dim.dg, dim.db, g1) || launch(K_DIVVXZ, dim.dg, dim.db, g2)) return 1;
                if (to_dev(f.dsx, c0 + 2 * n, n) || to_dev(f.dsz, c0 + 3 * n, n)) return 1;
                void *ar[] = {&kr, &f.vx, &f.dsx, &f.vz, &f.dsz, &ndt, &dim};
                void *am[] = {&km, &f.dvxdx, &f.dvxdx_fw, &f.dvxdz, &f.dvxdz_fw, &f.dvzdx, &f.dvzdx_fw,
                              &f.dvzdz, &f.dvzdz_fw, &ndt, &dim};
                void *al[] = {&kl, &f.dvxdx, &f.dvxdx_fw, &f.dvzdz, &f.dvzdz_fw, &ndt, &dim};
                if (p->inv_rho && launch(K_IRHOXZ, dim.dg, dim.db, ar)) return 1;
                if (p->inv_mu && launch(K_IMUXZ, dim.dg, dim.db, am)) return 1;
                if (p->inv_lambda && launch(K_ILAMXZ, dim.dg, dim.db, al)) return 1;
            }
        }
    }
    REF_TRY(cudaDeviceSynchronize());
    return to_host(k_lambda, kl, n) || to_host(k_mu, km, n) || to_host(k_rho, kr, n);
}

// GaussianFilter::init + apply on data[nx*nz] (filter/gaussian.h:37-61).
int ref_gaussian(int nx, int nz, int sigma, float *data) {
    if (!g_lib || nx < 1 || nz < 1 || nz > 1024) return 1;
    const size_t n = (size_t)nx * nz;
    Bufs b;
    float *d = b.alloc<float>(n), *gsum = b.alloc<float>(n), *gtmp = b.alloc<float>(n);
    if (!d || !gsum || !gtmp || to_dev(d, data, n)) return 1;
    Dim dim = make_dim(nx, nz);
    size_t s = (size_t)sigma;
    void *a0[] = {&gsum, &s, &dim};
    void *a1[] = {&d, &gtmp, &s, &dim};
    void *a2[] = {&d, &gtmp, &gsum, &s, &dim};
    if (launch(K_GINIT, dim.dg, dim.db, a0) || launch(K_GX, dim.dg, dim.db, a1) || launch(K_GZ, dim.dg, dim.db, a2))
        return 1;
    REF_TRY(cudaDeviceSynchronize());
    return to_host(data, d, n);
}

// Misfit::run's per-trace misfit (misfit/misfit.h:29-41) for ntr traces of
// nt samples: type 0 waveform, 1 envelope. Writes each trace's adjoint source
// (adstf [ntr*nt]) and value (values [ntr], as the reference returns it).
int ref_misfit(int type, int ntr, int nt, double dt_in, const float *syn, const float *obs, float *adstf,
               float *values) {
    if (!g_lib || ntr < 1 || nt < 2 || (type != 0 && type != 1)) return 1;
    const size_t n = (size_t)ntr * nt;
    Bufs b;
    float *ds = b.alloc<float>(n), *dob = b.alloc<float>(n), *dad = b.alloc<float>(n);
    float *misfit = b.alloc<float>(nt), *tw = b.alloc<float>(nt);
    float *esyn = b.alloc<float>(nt), *eobs = b.alloc<float>(nt), *ersd = b.alloc<float>(nt),
          *etmp = b.alloc<float>(nt);
    float2 *csyn = b.alloc<float2>(nt), *cobs = b.alloc<float2>(nt);
    if (!ds || !dob || !dad || !misfit || !tw || !esyn || !eobs || !ersd || !etmp || !csyn || !cobs) return 1;
    if (to_dev(ds, syn, n) || to_dev(dob, obs, n)) return 1;
    cublasHandle_t cb = nullptr;
    if (cublasCreate(&cb) != CUBLAS_STATUS_SUCCESS) {
        g_err = "cublasCreate";
        return 1;
    }
    cufftHandle plan = 0;
    if (type == 1 && cufftPlan1d(&plan, nt, CUFFT_C2C, 1) != CUFFT_SUCCESS) {
        cublasDestroy(cb);
        g_err = "cufftPlan1d";
        return 1;
    }
    const float dt = (float)dt_in;
    size_t ntv = (size_t)nt;
    int nti = nt;
    Dim dim = make_dim(nt, 1);  // Dim(nt, 1): nt blocks of one thread
    int rc = 0;
    auto hilbert = [&](float *x, float2 *data) -> int {
        void *a0[] = {&data, &x};
        void *a1[] = {&data, &ntv};
        if (launch(K_R2C, nt, 1, a0)) return 1;
        if (cufftExecC2C(plan, data, data, CUFFT_FORWARD) != CUFFT_SUCCESS) return 1;
        if (launch(K_HILB, nt, 1, a1)) return 1;
        return cufftExecC2C(plan, data, data, CUFFT_INVERSE) != CUFFT_SUCCESS;
    };
    if (type == 0) {
        void *a[] = {&tw, (void *)&dt, &nti};
        rc = launch(K_TAPER, nt, 1, a);
    }
    for (int r = 0; r < ntr && !rc; r++) {
        float *sy = ds + (size_t)r * nt, *ob = dob + (size_t)r * nt, *ad = dad + (size_t)r * nt;
        float v = 0.f;
        if (type == 0) {
            void *a[] = {&sy, &ob, &ad, &misfit, &tw, &ntv};
            if (launch(K_DIFF, nt, 1, a) || cublasSnrm2(cb, nt, misfit, 1, &v) != CUBLAS_STATUS_SUCCESS) {
                rc = 1;
                break;
            }
        } else {
            if (hilbert(sy, csyn) || hilbert(ob, cobs)) {
                rc = 1;
                break;
            }
            void *a0[] = {&esyn, &csyn, &nti};
            void *a1[] = {&eobs, &cobs, &nti};
            if (launch(K_C2ABS, nt, 1, a0) || launch(K_C2ABS, nt, 1, a1)) {
                rc = 1;
                break;
            }
            int idx = 0;
            float e = 0.f;
            if (cublasIsamax(cb, nt, esyn, 1, &idx) != CUBLAS_STATUS_SUCCESS ||
                cudaMemcpy(&e, esyn + idx - 1, 4, cudaMemcpyDeviceToHost) != cudaSuccess) {
                rc = 1;
                break;
            }
            float mx = std::fabs(e) * 0.05;  // device::amax(...) * 0.05 into a float
            if (mx < 0.05) mx = 0.05;
            void *a2[] = {&etmp, &esyn, &eobs, &mx};
            void *a3[] = {&ersd, &csyn, &nti};
            void *a4[] = {&ersd, &ersd, &etmp, &dim};
            void *a5[] = {&ersd, &cobs, &nti};
            void *a6[] = {&ad, &etmp, &sy, &ersd, &ntv};
            float one = 1.f, mone = -1.f;
            void *a7[] = {&ersd, &one, &esyn, &mone, &eobs, &dim};
            if (launch(K_ETMP, nt, 1, a2) || launch(K_C2IMAG, nt, 1, a3) || launch(K_MUL, dim.dg, dim.db, a4) ||
                hilbert(ersd, cobs) || launch(K_C2IMAG, nt, 1, a5) || launch(K_ESTF, nt, 1, a6) ||
                launch(K_AXPBY, dim.dg, dim.db, a7) || cublasSnrm2(cb, nt, ersd, 1, &v) != CUBLAS_STATUS_SUCCESS) {
                rc = 1;
                break;
            }
        }
        values[r] = v * std::sqrt(dt);
    }
    if (plan) cufftDestroy(plan);
    cublasDestroy(cb);
    if (rc) {
        if (g_err.empty()) g_err = "ref_misfit";
        return 1;
    }
    REF_TRY(cudaDeviceSynchronize());
    return to_host(adstf, dad, n);
}

// device::calc (lib/device.h:157-176) on host arrays of one nx*nz grid,
// launched as solver->dim (nx blocks of nz threads): c = ka*a + kb*b, or
// c = ka*a when b is null. c may be a or b (the kernels are elementwise).
int ref_calc(float *c, float ka, const float *a, float kb, const float *b, int nx, int nz) {
    if (!g_lib || nx < 1 || nz < 1 || nz > 1024) return 1;
    const size_t n = (size_t)nx * nz;
    Bufs bf;
    float *dc = bf.alloc<float>(n), *da = bf.alloc<float>(n), *db = bf.alloc<float>(n);
    if (!dc || !da || !db || to_dev(da, a, n) || (b && to_dev(db, b, n))) return 1;
    Dim dim = make_dim(nx, nz);
    if (b) {
        void *args[] = {&dc, &ka, &da, &kb, &db, &dim};
        if (launch(K_AXPBY, dim.dg, dim.db, args)) return 1;
    } else {
        void *args[] = {&dc, &ka, &da, &dim};
        if (launch(K_SCALE, dim.dg, dim.db, args)) return 1;
    }
    REF_TRY(cudaDeviceSynchronize());
    return to_host(c, dc, n);
}

// device::dot (lib/device.h:188-192): cublasSdot, FP32 result.
int ref_dot(const float *a, const float *b, int n, float *out) {
    if (!g_lib || n < 1) return 1;
    if (!g_cb && cublasCreate(&g_cb) != CUBLAS_STATUS_SUCCESS) {
        g_err = "cublasCreate";
        return 1;
    }
    Bufs bf;
    float *da = bf.alloc<float>(n), *db = bf.alloc<float>(n);
    if (!da || !db || to_dev(da, a, n) || to_dev(db, b, n)) return 1;
    if (cublasSdot(g_cb, n, da, 1, db, 1, out) != CUBLAS_STATUS_SUCCESS) {
        g_err = "cublasSdot";
        return 1;
    }
    return 0;
}

// device::amax (lib/device.h:178-182): cublasIsamax, then |a[index - 1]|.
int ref_amax(const float *a, int n, float *out) {
    if (!g_lib || n < 1) return 1;
    if (!g_cb && cublasCreate(&g_cb) != CUBLAS_STATUS_SUCCESS) {
        g_err = "cublasCreate";
        return 1;
    }
    Bufs bf;
    float *da = bf.alloc<float>(n);
    int index = 0;
    float v = 0.f;
    if (!da || to_dev(da, a, n)) return 1;
    if (cublasIsamax(g_cb, n, da, 1, &index) != CUBLAS_STATUS_SUCCESS || index < 1 || index > n) {
        g_err = "cublasIsamax";
        return 1;
    }
    REF_TRY(cudaMemcpy(&v, da + index - 1, 4, cudaMemcpyDeviceToHost));
    *out = std::fabs(v);
    return 0;
}

// Optimizer::polyfit(double*) + solveQR (optimizer/optimizer.h:108-172): the
// least-squares quadratic p[0] x^2 + p[1] x + p[2] through n points, by
// cuSOLVER's QR of the n x 3 system, Q^T y, the reference's reduceSystem
// kernel and cublasDtrsm, with the geqrf workspace size for both cuSOLVER
// calls as the reference passes it. The reference also multiplies Q into an
// unused, uninitialised matrix (optimizer.h:126-127); that product is not
// formed here. *ormqr_status: what cusolverDnDormqr returned (the reference
// does not look).
int ref_polyfit(const double *x, const double *y, int n, double *p, int *ormqr_status) {
    // n >= 3: reduceSystem reads the top 3 x 3 block of the n-row factor
    if (!g_lib || n < 3 || n > 1024) {
        g_err = "ref_polyfit: 3 to 1024 points";
        return 1;
    }
    if (!g_cb && cublasCreate(&g_cb) != CUBLAS_STATUS_SUCCESS) {
        g_err = "cublasCreate";
        return 1;
    }
    const int nrows = n, ncols = 3, k = std::min(nrows, ncols);
    std::vector<double> A(3 * (size_t)n);
    for (int i = 0; i < n; i++) {
        A[i] = x[i] * x[i];
        A[i + n] = x[i];
        A[i + 2 * n] = 1;
    }
    cusolverDnHandle_t sh = nullptr;
    if (cusolverDnCreate(&sh) != CUSOLVER_STATUS_SUCCESS) {
        g_err = "cusolverDnCreate";
        return 1;
    }
    int rc = 1;
    Bufs bf;
    int *info = bf.alloc<int>(1);
    double *dA = bf.alloc<double>((size_t)nrows * ncols), *dTAU = bf.alloc<double>(k);
    double *dC = bf.alloc<double>((size_t)nrows * nrows);  // zeroed, as device::init(d_C, 0.0, dim)
    double *dR = bf.alloc<double>(ncols * ncols), *dB = bf.alloc<double>(ncols * ncols);
    int work_size = 0;
    double *work = nullptr;
    if (info && dA && dTAU && dC && dR && dB &&
        cudaMemcpy(dA, A.data(), A.size() * 8, cudaMemcpyHostToDevice) == cudaSuccess &&
        cusolverDnDgeqrf_bufferSize(sh, nrows, ncols, dA, nrows, &work_size) == CUSOLVER_STATUS_SUCCESS &&
        (work = bf.alloc<double>(work_size > 0 ? work_size : 1)) != nullptr &&
        cusolverDnDgeqrf(sh, nrows, ncols, dA, nrows, dTAU, work, work_size, info) == CUSOLVER_STATUS_SUCCESS &&
        cudaMemcpy(dC, y, (size_t)nrows * 8, cudaMemcpyHostToDevice) == cudaSuccess) {
        *ormqr_status = (int)cusolverDnDormqr(sh, CUBLAS_SIDE_LEFT, CUBLAS_OP_T, nrows, ncols, k, dA, nrows, dTAU,
                                              dC, nrows, work, work_size, info);
        int M = nrows, N = ncols;
        void *args[] = {&dA, &dR, &dC, &dB, &M, &N};
        const double one = 1.;
        if (!launch(K_REDSYS, ncols, ncols, args) &&
            cublasDtrsm(g_cb, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, ncols,
                        ncols, &one, dR, ncols, dB, ncols) == CUBLAS_STATUS_SUCCESS &&
            cudaMemcpy(p, dB, ncols * 8, cudaMemcpyDeviceToHost) == cudaSuccess)
            rc = 0;
    }
    cusolverDnDestroy(sh);
    if (rc && g_err.empty()) g_err = "ref_polyfit";
    return rc;
}

}  // extern "C"
