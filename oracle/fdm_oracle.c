/*
 * CPU oracle for the inv.cu hot path — TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain-C restatement of the reference's algorithm, used by the
 * tests, by the smoke check and by the benchmark's CPU-baseline leg as the
 * thing results are checked against (or timed beside). The product never
 * links or calls it.
 *
 * Pinning: the forward SH path (stencils, guards, absorbing boundary, Ricker
 * source, receivers, grid inference, mesh2grid) is pinned against the
 * reference's golden seismograms example/checker/traces/vy_0000NN.su. The
 * P-SV, adjoint/kernel and Gaussian-filter restatements have no golden
 * vectors in the reference (it ships no tests); they follow the cited source
 * lines operation by operation and are cross-checked by property tests.
 *
 * Build: oracle/Makefile (gcc -O2 -fopenmp -ffp-contract=off). Contraction is
 * off so the FP32 oracle rounds the same way on x86-64 and aarch64.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    int nx, nz, nt, sfe;
    int sh, psv;
    int nsrc, nrec;
    double dx, dz, dt;
    int record_u; /* adj || trace_type == 1 (solver/fdm.h:540-551) */
    int adj;      /* mode 0 or 2: checkpoints are taken (solver/solver.h:166) */
    int inv_lambda, inv_mu, inv_rho;
} orc_params;

#define REAL float
#define SUFFIX _f32
#include "fdm_oracle_body.h"
#undef REAL
#undef SUFFIX

#define REAL double
#define SUFFIX _f64
#include "fdm_oracle_body.h"
#undef REAL
#undef SUFFIX

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* calcIdx (solver/fdm.h:44-47): id = (int)(coord / L * (n - 1) + 0.5), all in
 * float as on the device. */
void orc_calc_idx(int n, const float *coord, float L, float ngrid, int *id) {
    /* the 0.5 literal is a double, so the last addition is in double */
    for (int i = 0; i < n; i++) id[i] = (int)((double)(coord[i] / L * (ngrid - 1)) + 0.5);
}

/* RickerSource::create (source/ricker.h:5-21) and Source::init
 * (source/source.h:17-37): s(t) = -t * exp(-(pi f0 t)^2), t = it*dt - t0,
 * normalised by max|s|, then x/y/z components amp*s*cos(angle), amp*s,
 * amp*s*sin(angle). Host float arithmetic with host::pi = 3.1415927f. */
void orc_ricker(int nt, float dt, float f0, float t0, float angle, float amp, float *sx, float *sy,
                float *sz) {
    const float pi = 3.1415927f;
    float *stf = (float *)malloc((size_t)(nt > 0 ? nt : 1) * sizeof(float));
    float amax = 0;
    for (int it = 0; it < nt; it++) {
        float t = (float)(size_t)it * dt - t0;
        float pft = pi * f0 * t;
        stf[it] = -t * expf(-pft * pft);
        if (fabsf(stf[it]) > amax) amax = fabsf(stf[it]);
    }
    if (amax > 0)
        for (int it = 0; it < nt; it++) stf[it] /= amax;
    for (int it = 0; it < nt; it++) {
        sx[it] = amp * stf[it] * cosf(angle);
        sy[it] = amp * stf[it];
        sz[it] = amp * stf[it] * sinf(angle);
    }
    free(stf);
}

/* taper (misfit/waveform.h:9-27): 10% cosine taper at both ends; float with
 * device::pi and double 0.5 literals. */
void orc_taper(int nt, float dt, float *tw) {
    const float pi = 3.1415927f;
    float t_end = (nt - 1) * dt;
    float taper_width = t_end / 10;
    float t_min = taper_width;
    float t_max = t_end - taper_width;
    for (int it = 0; it < nt; it++) {
        float t = it * dt;
        if (t <= t_min)
            tw[it] = (float)(0.5 + 0.5 * cosf(pi * (t_min - t) / (taper_width)));
        else if (t >= t_max)
            tw[it] = (float)(0.5 + 0.5 * cosf(pi * (t_max - t) / (taper_width)));
        else
            tw[it] = 1;
    }
}

/* initAbsbound (solver/fdm.h:48-74): product of exp(-(alpha*d)^2) over the
 * enabled edges, in the order left, right, bottom, top, in float. */
void orc_absbound(int nx, int nz, int width, float alpha, int left, int right, int bottom, int top,
                  float *ab) {
    for (int i = 0; i < nx; i++) {
        for (int j = 0; j < nz; j++) {
            size_t k = (size_t)i * nz + j;
            float a = 1;
            if (left && i + 1 < width) {
                float t = alpha * (float)(width - i - 1);
                a *= expf(-powf(t, 2));
            }
            if (right && i > nx - width) {
                float t = alpha * (float)(width + i - nx);
                a *= expf(-powf(t, 2));
            }
            if (bottom && j > nz - width) {
                float t = alpha * (float)(width + j - nz);
                a *= expf(-powf(t, 2));
            }
            if (top && j + 1 < width) {
                float t = alpha * (float)(width - j - 1);
                a *= expf(-powf(t, 2));
            }
            ab[k] = a;
        }
    }
}

/* mesh2grid (solver/fdm.h:4-24): brute-force nearest model point per cell,
 * strict "<" so the first point wins ties; dmax = xmax^2 + zmax^2. Cells with
 * no point closer than dmax keep the initial values in (lambda, mu, rho). */
void orc_mesh2grid(int nx, int nz, float dx, float dz, int npt, const float *px, const float *pz,
                   const float *pvp, const float *pvs, const float *prho, float dmax, float *lambda,
                   float *mu, float *rho) {
#pragma omp parallel for schedule(dynamic, 4)
    for (int i = 0; i < nx; i++) {
        for (int j = 0; j < nz; j++) {
            size_t k = (size_t)i * nz + j;
            float x = i * dx, z = j * dz, dmin = dmax;
            for (int l = 0; l < npt; l++) {
                float ddx = x - px[l], ddz = z - pz[l];
                float d = ddx * ddx + ddz * ddz;
                if (d < dmin) {
                    dmin = d;
                    lambda[k] = pvp[l];
                    mu[k] = pvs[l];
                    rho[k] = prho[l];
                }
            }
        }
    }
}

/* vps2lm (solver/fdm.h:25-36), in place. */
void orc_vps2lm(size_t n, float *lambda, float *mu, const float *rho) {
    for (size_t k = 0; k < n; k++) {
        float vp = lambda[k], vs = mu[k];
        lambda[k] = (vp > vs) ? rho[k] * (vp * vp - 2 * vs * vs) : 0;
        mu[k] = rho[k] * vs * vs;
    }
}

/* gaussian (filter/gaussian.h:4-8). The argument is a size_t built from
 * (int i) - (size_t n): for n > i it wraps to ~1.8e19, whose square is +inf in
 * float, so the weight is exactly 0 and the filter is one-sided. The
 * conversion is restated literally. */
static float orc_gauss(size_t x, size_t sigma) {
    const float pi = 3.1415927f; /* device::pi, lib/device.h:96 */
    float xf = (float)x;
    float sigmaf = (float)sigma;
    return (1 / (sqrtf(2 * pi) * sigmaf)) * expf(-xf * xf / (2 * sigmaf * sigmaf));
}

/* GaussianFilter::init + apply (filter/gaussian.h:9-36,45-56), FP32. */
void orc_gaussian(int nx, int nz, int sigma, float *data) {
    size_t n = (size_t)nx * nz;
    float *gtmp = (float *)malloc(n * sizeof(float));
    float *gsum = (float *)malloc(n * sizeof(float));
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; i++) {
        for (int j = 0; j < nz; j++) {
            float sumx = 0, sumz = 0;
            for (size_t m = 0; m < (size_t)nx; m++) sumx += orc_gauss((size_t)(i - (long long)m), sigma);
            for (size_t m = 0; m < (size_t)nz; m++) sumz += orc_gauss((size_t)(j - (long long)m), sigma);
            gsum[(size_t)i * nz + j] = sumx * sumz;
        }
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; i++) {
        for (int j = 0; j < nz; j++) {
            float s = 0;
            for (size_t m = 0; m < (size_t)nx; m++)
                s += orc_gauss((size_t)(i - (long long)m), sigma) * data[m * nz + j];
            gtmp[(size_t)i * nz + j] = s;
        }
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; i++) {
        for (int j = 0; j < nz; j++) {
            size_t k = (size_t)i * nz + j;
            float s = 0;
            for (size_t m = 0; m < (size_t)nz; m++)
                s += orc_gauss((size_t)(j - (long long)m), sigma) * gtmp[(size_t)i * nz + m];
            data[k] = s / gsum[k];
        }
    }
    free(gtmp);
    free(gsum);
}

/* One gaussian weight, exported for the quirk test. */
float orc_gauss_weight(long long i, long long n, int sigma) {
    return orc_gauss((size_t)(i - n), (size_t)sigma);
}
