/*
 * Body of the CPU oracle for the staggered-grid solver. Test infrastructure
 * only: it is compiled twice by fdm_oracle.c, once with REAL=float (the FP32
 * oracle that restates the reference arithmetic operation by operation) and
 * once with REAL=double (the FP64 oracle used for error reports).
 *
 * Every loop below restates one kernel of the reference solver:
 *   solver/fdm.h:76-87    divSY          solver/fdm.h:88-102  divSXZ
 *   solver/fdm.h:103-117  divVY          solver/fdm.h:118-136 divVXZ
 *   solver/fdm.h:138-142  updateSY       solver/fdm.h:143-149 updateSXZ
 *   solver/fdm.h:150-154  updateVY       solver/fdm.h:155-161 updateVXZ
 *   solver/fdm.h:163-180  addSTF         solver/fdm.h:181-196 saveRec
 *   solver/fdm.h:198-219  interaction*   solver/fdm.h:515-612 time loops
 * Layout: float[nx*nz], k = i*nz + j (lib/device.h:38-40).
 */

#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)
#define FN(name) CAT(name, SUFFIX)

/* One 4th-order staggered difference, written exactly as the reference:
 * 9 * (a - b) / (8 * h) - (c - d) / (24 * h). */
static inline REAL FN(d4)(REAL a, REAL b, REAL c, REAL d, REAL h) {
    return (REAL)9 * (a - b) / ((REAL)8 * h) - (c - d) / ((REAL)24 * h);
}

typedef struct {
    REAL *vx, *vy, *vz, *ux, *uy, *uz, *sxx, *szz, *sxz, *sxy, *szy;
    REAL *dsx, *dsy, *dsz;
    REAL *dvxdx, *dvxdz, *dvzdx, *dvzdz, *dvydx, *dvydz;
    REAL *dvxdx_fw, *dvxdz_fw, *dvzdx_fw, *dvzdz_fw, *dvydx_fw, *dvydz_fw;
} FN(fields);

static REAL *FN(zalloc)(size_t n) { return (REAL *)calloc(n ? n : 1, sizeof(REAL)); }

static void FN(fields_alloc)(FN(fields) * f, size_t n) {
    REAL **p = (REAL **)f;
    for (size_t q = 0; q < sizeof(FN(fields)) / sizeof(REAL *); q++) p[q] = FN(zalloc)(n);
}
static void FN(fields_free)(FN(fields) * f) {
    REAL **p = (REAL **)f;
    for (size_t q = 0; q < sizeof(FN(fields)) / sizeof(REAL *); q++) free(p[q]);
}
static void FN(fields_zero)(FN(fields) * f, size_t n) {
    /* initWavefields, solver/fdm.h:295-311 */
    REAL *z[] = {f->vx, f->vy, f->vz, f->ux, f->uy, f->uz, f->sxx, f->szz, f->sxz, f->sxy, f->szy};
    for (size_t q = 0; q < sizeof(z) / sizeof(z[0]); q++) memset(z[q], 0, n * sizeof(REAL));
}

/* divSY / divSXZ (solver/fdm.h:76-102): backward-staggered stress divergence.
 * x part only for 2 <= i < nx-2 (else 0); z part added only for 2 <= j < nz-2. */
static void FN(divS)(const orc_params *p, FN(fields) * f) {
    const int nx = p->nx, nz = p->nz;
    const REAL dx = (REAL)p->dx, dz = (REAL)p->dz;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; i++) {
        for (int j = 0; j < nz; j++) {
            size_t k = (size_t)i * nz + j;
            if (p->sh) {
                const REAL *a = f->sxy, *b = f->szy;
                if (i >= 2 && i < nx - 2)
                    f->dsy[k] = FN(d4)(a[k], a[k - nz], a[k + nz], a[k - 2 * nz], dx);
                else
                    f->dsy[k] = 0;
                if (j >= 2 && j < nz - 2) f->dsy[k] += FN(d4)(b[k], b[k - 1], b[k + 1], b[k - 2], dz);
            }
            if (p->psv) {
                const REAL *xx = f->sxx, *xz = f->sxz, *zz = f->szz;
                if (i >= 2 && i < nx - 2) {
                    f->dsx[k] = FN(d4)(xx[k], xx[k - nz], xx[k + nz], xx[k - 2 * nz], dx);
                    f->dsz[k] = FN(d4)(xz[k], xz[k - nz], xz[k + nz], xz[k - 2 * nz], dx);
                } else {
                    f->dsx[k] = 0;
                    f->dsz[k] = 0;
                }
                if (j >= 2 && j < nz - 2) {
                    f->dsx[k] += FN(d4)(xz[k], xz[k - 1], xz[k + 1], xz[k - 2], dz);
                    f->dsz[k] += FN(d4)(zz[k], zz[k - 1], zz[k + 1], zz[k - 2], dz);
                }
            }
        }
    }
}

/* divVY / divVXZ (solver/fdm.h:103-136): forward-staggered gradients of
 * (vx, vy, vz) written to the given outputs; 0 outside 1 <= i < nx-2,
 * 1 <= j < nz-2. Also used on displacement at adjoint interaction steps. */
static void FN(divV_sh)(const orc_params *p, REAL *ddx, REAL *ddz, const REAL *w) {
    const int nx = p->nx, nz = p->nz;
    const REAL dx = (REAL)p->dx, dz = (REAL)p->dz;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; i++) {
        for (int j = 0; j < nz; j++) {
            size_t k = (size_t)i * nz + j;
            ddx[k] = (i >= 1 && i < nx - 2) ? FN(d4)(w[k + nz], w[k], w[k + 2 * nz], w[k - nz], dx) : 0;
            ddz[k] = (j >= 1 && j < nz - 2) ? FN(d4)(w[k + 1], w[k], w[k + 2], w[k - 1], dz) : 0;
        }
    }
}
static void FN(divV_psv)(const orc_params *p, REAL *dxdx, REAL *dxdz, REAL *dzdx, REAL *dzdz,
                         const REAL *wx, const REAL *wz) {
    const int nx = p->nx, nz = p->nz;
    const REAL dx = (REAL)p->dx, dz = (REAL)p->dz;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; i++) {
        for (int j = 0; j < nz; j++) {
            size_t k = (size_t)i * nz + j;
            if (i >= 1 && i < nx - 2) {
                dxdx[k] = FN(d4)(wx[k + nz], wx[k], wx[k + 2 * nz], wx[k - nz], dx);
                dzdx[k] = FN(d4)(wz[k + nz], wz[k], wz[k + 2 * nz], wz[k - nz], dx);
            } else {
                dxdx[k] = 0;
                dzdx[k] = 0;
            }
            if (j >= 1 && j < nz - 2) {
                dxdz[k] = FN(d4)(wx[k + 1], wx[k], wx[k + 2], wx[k - 1], dz);
                dzdz[k] = FN(d4)(wz[k + 1], wz[k], wz[k + 2], wz[k - 1], dz);
            } else {
                dxdz[k] = 0;
                dzdz[k] = 0;
            }
        }
    }
}

/* addSTF (solver/fdm.h:163-180): stf[is*nt + it] added to ds at the source
 * cell, for is == isrc or every is when isrc < 0. Sources are visited in
 * index order, which is the race-free reading of the reference's "+=". */
static void FN(addSTF)(const orc_params *p, FN(fields) * f, const REAL *sx, const REAL *sy,
                       const REAL *sz, const int *xid, const int *zid, int n, int isrc, int it) {
    for (int is = 0; is < n; is++) {
        if (isrc < 0 || isrc == is) {
            size_t km = (size_t)xid[is] * p->nz + zid[is];
            size_t ks = (size_t)is * p->nt + it;
            if (p->sh) f->dsy[km] += sy[ks];
            if (p->psv) {
                f->dsx[km] += sx[ks];
                f->dsz[km] += sz[ks];
            }
        }
    }
}

/* divV (solver/fdm.h:282-294): updateV*, divV*, updateS* in that order. */
static void FN(divV)(const orc_params *p, FN(fields) * f, const REAL *lambda, const REAL *mu,
                     const REAL *rho, const REAL *ab) {
    const size_t n = (size_t)p->nx * p->nz;
    const REAL dt = (REAL)p->dt;
    if (p->sh) {
#pragma omp parallel for schedule(static)
        for (size_t k = 0; k < n; k++) {
            f->vy[k] = ab[k] * (f->vy[k] + dt * f->dsy[k] / rho[k]);
            f->uy[k] += f->vy[k] * dt;
        }
        FN(divV_sh)(p, f->dvydx, f->dvydz, f->vy);
#pragma omp parallel for schedule(static)
        for (size_t k = 0; k < n; k++) {
            f->sxy[k] += dt * mu[k] * f->dvydx[k];
            f->szy[k] += dt * mu[k] * f->dvydz[k];
        }
    }
    if (p->psv) {
#pragma omp parallel for schedule(static)
        for (size_t k = 0; k < n; k++) {
            f->vx[k] = ab[k] * (f->vx[k] + dt * f->dsx[k] / rho[k]);
            f->vz[k] = ab[k] * (f->vz[k] + dt * f->dsz[k] / rho[k]);
            f->ux[k] += f->vx[k] * dt;
            f->uz[k] += f->vz[k] * dt;
        }
        FN(divV_psv)(p, f->dvxdx, f->dvxdz, f->dvzdx, f->dvzdz, f->vx, f->vz);
#pragma omp parallel for schedule(static)
        for (size_t k = 0; k < n; k++) {
            f->sxx[k] += dt * ((lambda[k] + 2 * mu[k]) * f->dvxdx[k] + lambda[k] * f->dvzdz[k]);
            f->szz[k] += dt * ((lambda[k] + 2 * mu[k]) * f->dvzdz[k] + lambda[k] * f->dvxdx[k]);
            f->sxz[k] += dt * (mu[k] * (f->dvxdz[k] + f->dvzdx[k]));
        }
    }
}

/* saveRec (solver/fdm.h:181-196). */
static void FN(saveRec)(const orc_params *p, const REAL *wx, const REAL *wy, const REAL *wz,
                        REAL *ox, REAL *oy, REAL *oz, const int *xid, const int *zid, int it) {
    for (int ir = 0; ir < p->nrec; ir++) {
        size_t km = (size_t)xid[ir] * p->nz + zid[ir];
        size_t kr = (size_t)ir * p->nt + it;
        if (p->sh) oy[kr] = wy[km];
        if (p->psv) {
            ox[kr] = wx[km];
            oz[kr] = wz[km];
        }
    }
}

/* Checkpoint slot layout used by the oracle: ckpt[(isfe * nf + q) * N], with
 * q = 0..nf-1 over (uy, vy) for SH then (ux, uz, vx, vz) for P-SV. */
static int FN(nckpt)(const orc_params *p) { return (p->sh ? 2 : 0) + (p->psv ? 4 : 0); }

/* FdmSolver::runForward (solver/fdm.h:515-570). u is stored before the step
 * and v after it, at slot isfe = nsfe - (it+1)/sfe (the one-step offset of the
 * reference). record_u selects displacement recording (adj || trace_type==1). */
void FN(orc_forward)(const orc_params *p, const REAL *lambda, const REAL *mu, const REAL *rho,
                     const REAL *ab, const REAL *stf_x, const REAL *stf_y, const REAL *stf_z,
                     const int *src_x, const int *src_z, const int *rec_x, const int *rec_z, int isrc,
                     REAL *out_x, REAL *out_y, REAL *out_z, REAL *ckpt) {
    const size_t n = (size_t)p->nx * p->nz;
    const int nsfe = p->sfe ? p->nt / p->sfe : 0;
    const int nf = FN(nckpt)(p);
    FN(fields) f;
    FN(fields_alloc)(&f, n);
    FN(fields_zero)(&f, n);
    for (int it = 0; it < p->nt; it++) {
        int isfe = -1;
        if (p->sfe && p->adj && (it + 1) % p->sfe == 0) isfe = nsfe - (it + 1) / p->sfe;
        if (isfe >= 0 && ckpt) {
            int q = 0;
            if (p->sh) memcpy(ckpt + ((size_t)isfe * nf + q++) * n, f.uy, n * sizeof(REAL));
            if (p->psv) {
                memcpy(ckpt + ((size_t)isfe * nf + q++) * n, f.ux, n * sizeof(REAL));
                memcpy(ckpt + ((size_t)isfe * nf + q++) * n, f.uz, n * sizeof(REAL));
            }
        }
        FN(divS)(p, &f);
        FN(addSTF)(p, &f, stf_x, stf_y, stf_z, src_x, src_z, p->nsrc, isrc, it);
        FN(divV)(p, &f, lambda, mu, rho, ab);
        if (p->record_u)
            FN(saveRec)(p, f.ux, f.uy, f.uz, out_x, out_y, out_z, rec_x, rec_z, it);
        else
            FN(saveRec)(p, f.vx, f.vy, f.vz, out_x, out_y, out_z, rec_x, rec_z, it);
        if (isfe >= 0 && ckpt) {
            int q = (p->sh ? 1 : 0) + (p->psv ? 2 : 0);
            if (p->sh) memcpy(ckpt + ((size_t)isfe * nf + q++) * n, f.vy, n * sizeof(REAL));
            if (p->psv) {
                memcpy(ckpt + ((size_t)isfe * nf + q++) * n, f.vx, n * sizeof(REAL));
                memcpy(ckpt + ((size_t)isfe * nf + q++) * n, f.vz, n * sizeof(REAL));
            }
        }
    }
    FN(fields_free)(&f);
}

/* FdmSolver::runAdjoint (solver/fdm.h:571-612): same operator driven by the
 * adjoint sources at every receiver; every sfe steps (it % sfe == 0) the
 * checkpoint isfe = it/sfe is paired with the adjoint state and the kernels
 * are updated with ndt = sfe*dt (interaction*, solver/fdm.h:198-219). */
void FN(orc_adjoint)(const orc_params *p, const REAL *lambda, const REAL *mu, const REAL *rho,
                     const REAL *ab, const REAL *adstf_x, const REAL *adstf_y, const REAL *adstf_z,
                     const int *rec_x, const int *rec_z, const REAL *ckpt, REAL *k_lambda, REAL *k_mu,
                     REAL *k_rho) {
    const size_t n = (size_t)p->nx * p->nz;
    const int nf = FN(nckpt)(p);
    FN(fields) f;
    FN(fields_alloc)(&f, n);
    FN(fields_zero)(&f, n);
    for (int it = 0; it < p->nt; it++) {
        FN(divS)(p, &f);
        FN(addSTF)(p, &f, adstf_x, adstf_y, adstf_z, rec_x, rec_z, p->nrec, -1, it);
        FN(divV)(p, &f, lambda, mu, rho, ab);
        if ((it + p->sfe) % p->sfe == 0) {
            size_t isfe = (size_t)((it + p->sfe) / p->sfe - 1);
            const REAL ndt = (REAL)p->sfe * (REAL)p->dt;
            int q = 0;
            if (p->sh) {
                const REAL *uy_fw = ckpt + (isfe * nf + q++) * n;
                const REAL *vy_fw = ckpt + (isfe * nf + q++) * n;
                FN(divV_sh)(p, f.dvydx, f.dvydz, f.uy);
                FN(divV_sh)(p, f.dvydx_fw, f.dvydz_fw, uy_fw);
#pragma omp parallel for schedule(static)
                for (size_t k = 0; k < n; k++) {
                    if (p->inv_rho) k_rho[k] -= vy_fw[k] * f.vy[k] * ndt;
                    if (p->inv_mu)
                        k_mu[k] -= (f.dvydx[k] * f.dvydx_fw[k] + f.dvydz[k] * f.dvydz_fw[k]) * ndt;
                }
            }
            if (p->psv) {
                const REAL *ux_fw = ckpt + (isfe * nf + q++) * n;
                const REAL *uz_fw = ckpt + (isfe * nf + q++) * n;
                const REAL *vx_fw = ckpt + (isfe * nf + q++) * n;
                const REAL *vz_fw = ckpt + (isfe * nf + q++) * n;
                FN(divV_psv)(p, f.dvxdx, f.dvxdz, f.dvzdx, f.dvzdz, f.ux, f.uz);
                FN(divV_psv)(p, f.dvxdx_fw, f.dvxdz_fw, f.dvzdx_fw, f.dvzdz_fw, ux_fw, uz_fw);
#pragma omp parallel for schedule(static)
                for (size_t k = 0; k < n; k++) {
                    if (p->inv_rho) k_rho[k] -= (vx_fw[k] * f.vx[k] + vz_fw[k] * f.vz[k]) * ndt;
                    if (p->inv_mu)
                        k_mu[k] -= (2 * f.dvxdx[k] * f.dvxdx_fw[k] + 2 * f.dvzdz[k] * f.dvzdz_fw[k] +
                                    (f.dvxdz[k] + f.dvzdx[k]) * (f.dvzdx_fw[k] + f.dvxdz_fw[k])) *
                                   ndt;
                    if (p->inv_lambda)
                        k_lambda[k] -= ((f.dvxdx[k] + f.dvzdz[k]) * (f.dvxdx_fw[k] + f.dvzdz_fw[k])) * ndt;
                }
            }
        }
    }
    FN(fields_free)(&f);
}

#undef FN
#undef CAT
#undef CAT2
