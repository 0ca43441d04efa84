// Per-cell arithmetic of the time step, shared by every step kernel (2-D
// tile, marching strip, cluster-resident) so that they compute bit-identical
// results. Every multiply-add is an explicit fmaf: the result does not depend
// on how the compiler would contract a plain expression in each kernel.
//
// The operations follow the reference (solver/fdm.h:76-161); its divisions by
// 8h, 24h and rho are multiplications by 9/(8h), 1/(24h) and 1/rho here.
#pragma once

namespace gb {

// Backward-staggered difference at k: 9(a0 - am1)/(8h) - (ap1 - am2)/(24h).
__device__ __forceinline__ float st_dminus(float a0, float am1, float ap1, float am2, float c9, float c24) {
    return fmaf(a0 - am1, c9, -((ap1 - am2) * c24));
}
// Forward-staggered difference at k: 9(ap1 - a0)/(8h) - (ap2 - am1)/(24h).
__device__ __forceinline__ float st_dplus(float ap1, float a0, float ap2, float am1, float c9, float c24) {
    return fmaf(ap1 - a0, c9, -((ap2 - am1) * c24));
}
// v' = ab (v + dt ds / rho)   (updateV*, solver/fdm.h:150-161)
__device__ __forceinline__ float st_velocity(float ab, float dt, float ds, float rinv, float v) {
    return ab * fmaf(dt * ds, rinv, v);
}
// u' = u + v' dt
__device__ __forceinline__ float st_displacement(float u, float vn, float dt) { return fmaf(vn, dt, u); }
// P-SV stress update (updateSXZ, solver/fdm.h:143-149).
__device__ __forceinline__ void st_stress_psv(float &sxx, float &szz, float &sxz, float l, float m, float dt,
                                              float dvxdx, float dvxdz, float dvzdx, float dvzdz) {
    const float l2m = fmaf(2.f, m, l);
    sxx = fmaf(dt, fmaf(l2m, dvxdx, l * dvzdz), sxx);
    szz = fmaf(dt, fmaf(l2m, dvzdz, l * dvxdx), szz);
    sxz = fmaf(dt, m * (dvxdz + dvzdx), sxz);
}
// SH stress update (updateSY, solver/fdm.h:138-142).
__device__ __forceinline__ void st_stress_sh(float &sxy, float &szy, float m, float dt, float dvydx, float dvydz) {
    const float dtm = dt * m;
    sxy = fmaf(dtm, dvydx, sxy);
    szy = fmaf(dtm, dvydz, szy);
}

// Kernel accumulation (interaction*, solver/fdm.h:198-219): k - c ndt, the
// contribution c formed in a fixed order (products feeding a sum are
// __fmul_rn, which the compiler never fuses), so the in-pass, after-pass
// and per-step forms give the same bits.
// SH: k_rho -= v_fw v ndt
__device__ __forceinline__ float st_krho_sh(float k, float vf, float va, float ndt) {
    return fmaf(-__fmul_rn(vf, va), ndt, k);
}
// SH: k_mu -= (dx u dx u_fw + dz u dz u_fw) ndt
__device__ __forceinline__ float st_kmu_sh(float k, float ux, float fx, float uz, float fz, float ndt) {
    return fmaf(-fmaf(ux, fx, __fmul_rn(uz, fz)), ndt, k);
}
// P-SV: k_rho -= (vx vx_fw + vz vz_fw) ndt
__device__ __forceinline__ float st_krho_psv(float k, float vf0, float va0, float vf1, float va1, float ndt) {
    return fmaf(-fmaf(vf0, va0, __fmul_rn(vf1, va1)), ndt, k);
}
// P-SV: k_mu -= (2 dxux dxux_fw + 2 dzuz dzuz_fw + (dzux + dxuz)(dxuz_fw + dzux_fw)) ndt
__device__ __forceinline__ float st_kmu_psv(float k, float dvxdx, float dvxdz, float dvzdx, float dvzdz, float fxdx,
                                            float fxdz, float fzdx, float fzdz, float ndt) {
    const float shear = __fmul_rn(dvxdz + dvzdx, fzdx + fxdz);
    return fmaf(-fmaf(2.f * dvxdx, fxdx, fmaf(2.f * dvzdz, fzdz, shear)), ndt, k);
}
// The P-SV kernels from the forward strains of a 16-bit checkpoint: the
// divergence dv = dxux_fw + dzuz_fw, the difference dd = dxux_fw - dzuz_fw
// and the shear sum sh = dxuz_fw + dzux_fw. 2 a x + 2 b z with x = (dv + dd)/2,
// z = (dv - dd)/2 is (a + b) dv + (a - b) dd, so
//   k_mu     -= ((dxux + dzuz) dv + (dxux - dzuz) dd + (dzux + dxuz) sh) ndt
//   k_lambda -= (dxux + dzuz) dv ndt
__device__ __forceinline__ float st_kmu_psv_strain(float k, float dvxdx, float dvxdz, float dvzdx, float dvzdz,
                                                   float fdv, float fdd, float fsh, float ndt) {
    const float c = fmaf(dvxdx + dvzdz, fdv, fmaf(dvxdx - dvzdz, fdd, __fmul_rn(dvxdz + dvzdx, fsh)));
    return fmaf(-c, ndt, k);
}
__device__ __forceinline__ float st_klambda_psv_strain(float k, float dvxdx, float dvzdz, float fdv, float ndt) {
    return fmaf(-__fmul_rn(dvxdx + dvzdz, fdv), ndt, k);
}
// P-SV: k_lambda -= (dxux + dzuz)(dxux_fw + dzuz_fw) ndt
__device__ __forceinline__ float st_klambda_psv(float k, float dvxdx, float dvzdz, float fxdx, float fzdz, float ndt) {
    return fmaf(-__fmul_rn(dvxdx + dvzdz, fxdx + fzdz), ndt, k);
}

}  // namespace gb
