// Fused time-step kernels of the staggered-grid velocity-stress solver.
//
// One launch advances every slot (shot) of a batch by one time step: the
// reference's six launches per step (divS, addSTF, updateV, divV, updateS,
// saveRec; solver/fdm.h:273-294,534-551) become one kernel per wave system.
//
// A thread block owns a TZ x TX tile (z contiguous). It
//   1. stages stress at time n on the tile plus a 3-cell halo in shared memory,
//   2. computes the stress divergence on the tile plus the velocity halo
//      (1 cell before, 2 after), adds the source or adjoint-source samples that
//      fall there, and updates velocity (absorbing factor applied to v only,
//      solver/fdm.h:150-161) and, on owned cells, displacement,
//   3. records the receivers it owns, then
//   4. updates stress on the owned cells from the velocity in shared memory.
// The velocity halo is recomputed by each neighbouring tile, so one launch
// needs no grid-wide synchronisation; stress and velocity are ping-ponged
// between two buffers so no tile reads a neighbour's half-updated values.
//
// Derivative guards follow the reference exactly (solver/fdm.h:76-136): the
// x part of the stress divergence is 0 outside 2 <= i < nx-2, the z part is
// added only for 2 <= j < nz-2, velocity gradients are 0 outside
// 1 <= i < nx-2 / 1 <= j < nz-2. The reference's divisions are replaced by
// multiplications with 9/(8h), 1/(24h) and the reciprocal density; the
// difference is FP32 round-off (about 1e-6 relative on the golden traces).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>

#include "gb_internal.h"
#include "gb_stencil.h"

namespace gb {

constexpr int kThreads = 256;

__device__ __forceinline__ float dminus(float a0, float am1, float ap1, float am2, float c9, float c24) {
    return st_dminus(a0, am1, ap1, am2, c9, c24);
}
__device__ __forceinline__ float dplus(float ap1, float a0, float ap2, float am1, float c9, float c24) {
    return st_dplus(ap1, a0, ap2, am1, c9, c24);
}

struct Csr {
    const int *tile_ptr, *local, *tptr, *traces;
    __device__ Csr(const int *p) {
        const int ntiles = p[0], nent = p[1];
        tile_ptr = p + 3;
        local = tile_ptr + ntiles + 1;
        tptr = local + nent;
        traces = tptr + nent + 1;
    }
};

// Asynchronous 4-byte global->shared copy; with pred == false nothing is
// read and the shared word is zero-filled (src must still be a valid address).
__device__ __forceinline__ void cp_async4(float *dst, const float *src, bool pred) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    const int n = pred ? 4 : 0;
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

constexpr int kMaxInjTraces = 128;  // source samples staged in shared memory per tile

template <bool PSV, int TZ, int TX>
__global__ void __launch_bounds__(kThreads) k_step(const Slot *__restrict__ slots, int kstep) {
    constexpr int NS = PSV ? 3 : 2;  // stress components held in shared memory
    constexpr int NV = PSV ? 2 : 1;  // velocity components
    constexpr int RZ = TZ + 6, RX = TX + 6;
    constexpr int VZ = TZ + 3, VX = TX + 3;
    constexpr int NR = RX * RZ, NVR = VX * VZ, NO = TX * TZ;
    constexpr int QS = (NR + kThreads - 1) / kThreads;
    constexpr int QV = (NVR + kThreads - 1) / kThreads;
    constexpr int QO = (NO + kThreads - 1) / kThreads;
    __shared__ float s_sig[NS][NR];
    __shared__ float s_v[NV][NVR];  // velocity at time n, then n+1 (same cell, same thread)
    __shared__ float s_rho[NVR];  // reciprocal density
    __shared__ float s_inj[NV][kMaxInjTraces];

    // Blocks run shot-minor (block b: shot b % nslots, tile b / nslots): the
    // same tile of every shot runs close together, so the model, shared by
    // the shots, is read from HBM once and from L2 after.
    const unsigned blk = blockIdx.y * gridDim.x + blockIdx.x;
    const Slot &S = slots[blk % gridDim.y];
    if (!S.active) return;
    const int it = S.it_base + kstep;
    if (it < 0 || it >= S.nt) return;
    const int par = (S.par0 + kstep) & 1;
    const int nx = S.nx, nz = S.nz;
    const int tile = (int)(blk / gridDim.y);
    if (tile >= S.tiles_z * S.tiles_x) return;
    const int tzi = tile % S.tiles_z, txi = tile / S.tiles_z;
    const int j0 = tzi * TZ, i0 = txi * TX;
    const int tid = threadIdx.x;

    const float *sig_in[NS];
    float *sig_out[NS];
    const float *v_in[NV];
    float *v_out[NV];
    float *u[NV];
    if (PSV) {
#pragma unroll
        for (int f = 0; f < NS; f++) {
            sig_in[f] = S.psv[SXX0 + 2 * f + par];
            sig_out[f] = S.psv[SXX0 + 2 * f + (par ^ 1)];
        }
#pragma unroll
        for (int f = 0; f < NV; f++) {
            v_in[f] = S.psv[VX0 + 2 * f + par];
            v_out[f] = S.psv[VX0 + 2 * f + (par ^ 1)];
            u[f] = S.psv[UX + f];
        }
    } else {
#pragma unroll
        for (int f = 0; f < NS; f++) {
            sig_in[f] = S.sh[SXY0 + 2 * f + par];
            sig_out[f] = S.sh[SXY0 + 2 * f + (par ^ 1)];
        }
        v_in[0] = S.sh[VY0 + par];
        v_out[0] = S.sh[VY0 + (par ^ 1)];
        u[0] = S.sh[UY];
    }
    const float dt = S.dt, c9x = S.c9x, c24x = S.c24x, c9z = S.c9z, c24z = S.c24z;
    const float *rho = S.rinv;  // reciprocal density, precomputed per pass

    // ---- 0. issue every load of the tile before waiting for any.
    // Stress at time n on the tile + 3-cell halo (zero outside the grid;
    // those values only feed results the guards discard).
#pragma unroll
    for (int q = 0; q < QS; q++) {
        const int e = tid + q * kThreads;
        if (e < NR) {
            const int c = e / RZ, r = e - c * RZ;
            const int i = i0 - 3 + c, j = j0 - 3 + r;
            const bool in = (unsigned)i < (unsigned)nx && (unsigned)j < (unsigned)nz;
            const size_t k = in ? (size_t)i * nz + j : 0;
#pragma unroll
            for (int f = 0; f < NS; f++) cp_async4(&s_sig[f][e], sig_in[f] + k, in);
        }
    }
    // Velocity at time n and density on the velocity region (tile + 1 cell
    // before, 2 after).
#pragma unroll
    for (int q = 0; q < QV; q++) {
        const int e = tid + q * kThreads;
        if (e < NVR) {
            const int c = e / VZ, r = e - c * VZ;
            const int i = i0 - 1 + c, j = j0 - 1 + r;
            const bool in = (unsigned)i < (unsigned)nx && (unsigned)j < (unsigned)nz;
            const size_t k = in ? (size_t)i * nz + j : 0;
#pragma unroll
            for (int f = 0; f < NV; f++) cp_async4(&s_v[f][e], v_in[f] + k, in);
            cp_async4(&s_rho[e], rho + k, in);
        }
    }
    // Displacement of owned cells (velocity-region numbering) and the moduli
    // of owned cells (tile numbering) go to registers.
    float u_reg[QV][NV];
#pragma unroll
    for (int q = 0; q < QV; q++) {
        const int e = tid + q * kThreads;
        const int c = e / VZ, r = e - c * VZ;
        const int i = i0 - 1 + c, j = j0 - 1 + r;
        const bool own = e < NVR && c >= 1 && c <= TX && r >= 1 && r <= TZ && i < nx && j < nz;
#pragma unroll
        for (int f = 0; f < NV; f++) u_reg[q][f] = own ? u[f][(size_t)i * nz + j] : 0.f;
    }
    float mu_reg[QO], lam_reg[QO];
#pragma unroll
    for (int q = 0; q < QO; q++) {
        const int e = tid + q * kThreads;
        const int c = e / TZ, r = e - c * TZ;
        const int i = i0 + c, j = j0 + r;
        const bool in = e < NO && i < nx && j < nz;
        const size_t k = in ? (size_t)i * nz + j : 0;
        mu_reg[q] = in ? __ldg(S.mu + k) : 0.f;
        lam_reg[q] = (PSV && in) ? __ldg(S.lambda + k) : 0.f;
    }
    // Source (or adjoint-source) samples falling in the velocity region.
    int ninj = 0, inj_first = 0, tr_first = 0, ntr = 0;
    const int *inj_local = nullptr, *inj_tptr = nullptr;
    if (S.inj) {
        const Csr cs(S.inj);
        inj_first = cs.tile_ptr[tile];
        ninj = cs.tile_ptr[tile + 1] - inj_first;
        if (ninj) {
            inj_local = cs.local;
            inj_tptr = cs.tptr;
            tr_first = cs.tptr[inj_first];
            ntr = cs.tptr[inj_first + ninj] - tr_first;
            if (ntr <= kMaxInjTraces) {
                const int nt = S.nt;
                for (int t = tid; t < ntr; t += kThreads) {
                    const size_t ks = (size_t)cs.traces[tr_first + t] * nt + it;
                    if (PSV) {
                        s_inj[0][t] = __ldg(S.inj_x + ks);
                        s_inj[NV - 1][t] = __ldg(S.inj_z + ks);
                    } else {
                        s_inj[0][t] = __ldg(S.inj_y + ks);
                    }
                }
            }
        }
    }
    cp_async_wait_all();
    __syncthreads();

    // ---- 1. stress divergence, source samples (added in trace order,
    //         solver/fdm.h:163-180), velocity and displacement updates.
#pragma unroll
    for (int q = 0; q < QV; q++) {
        const int e = tid + q * kThreads;
        if (e >= NVR) continue;
        const int c = e / VZ, r = e - c * VZ;
        const int i = i0 - 1 + c, j = j0 - 1 + r;
        if (!((unsigned)i < (unsigned)nx && (unsigned)j < (unsigned)nz)) {
#pragma unroll
            for (int f = 0; f < NV; f++) s_v[f][e] = 0.f;
            continue;
        }
        const int cc = c + 2, rr = r + 2;
#define SG(f, dc, dr) s_sig[f][(cc + (dc)) * RZ + rr + (dr)]
        float ds[NV];
        if (PSV) {
            float dsx = 0.f, dsz = 0.f;
            if (i >= 2 && i < nx - 2) {
                dsx = dminus(SG(0, 0, 0), SG(0, -1, 0), SG(0, 1, 0), SG(0, -2, 0), c9x, c24x);
                dsz = dminus(SG(2, 0, 0), SG(2, -1, 0), SG(2, 1, 0), SG(2, -2, 0), c9x, c24x);
            }
            if (j >= 2 && j < nz - 2) {
                dsx += dminus(SG(2, 0, 0), SG(2, 0, -1), SG(2, 0, 1), SG(2, 0, -2), c9z, c24z);
                dsz += dminus(SG(1, 0, 0), SG(1, 0, -1), SG(1, 0, 1), SG(1, 0, -2), c9z, c24z);
            }
            ds[0] = dsx;
            ds[NV - 1] = dsz;
        } else {
            float dsy = 0.f;
            if (i >= 2 && i < nx - 2) dsy = dminus(SG(0, 0, 0), SG(0, -1, 0), SG(0, 1, 0), SG(0, -2, 0), c9x, c24x);
            if (j >= 2 && j < nz - 2) dsy += dminus(SG(1, 0, 0), SG(1, 0, -1), SG(1, 0, 1), SG(1, 0, -2), c9z, c24z);
            ds[0] = dsy;
        }
#undef SG
        if (ninj) {
            for (int p = 0; p < ninj; p++) {
                if (inj_local[inj_first + p] != e) continue;
                for (int t = inj_tptr[inj_first + p]; t < inj_tptr[inj_first + p + 1]; t++) {
                    if (ntr <= kMaxInjTraces) {
#pragma unroll
                        for (int f = 0; f < NV; f++) ds[f] += s_inj[f][t - tr_first];
                    } else {
                        const Csr cs(S.inj);
                        const size_t ks = (size_t)cs.traces[t] * S.nt + it;
                        if (PSV) {
                            ds[0] += __ldg(S.inj_x + ks);
                            ds[NV - 1] += __ldg(S.inj_z + ks);
                        } else {
                            ds[0] += __ldg(S.inj_y + ks);
                        }
                    }
                }
            }
        }
        const size_t k = (size_t)i * nz + j;
        const float ab = __ldg(S.ax + i) * __ldg(S.az + j);
        const float rinv = s_rho[e];
        const bool own = c >= 1 && c <= TX && r >= 1 && r <= TZ;
#pragma unroll
        for (int f = 0; f < NV; f++) {
            const float vn = st_velocity(ab, dt, ds[f], rinv, s_v[f][e]);
            s_v[f][e] = vn;
            if (own) {
                v_out[f][k] = vn;
                u[f][k] = st_displacement(u_reg[q][f], vn, dt);
            }
        }
    }
    __syncthreads();

    // ---- 2. receivers owned by this tile (solver/fdm.h:181-196): u when
    //         record_u (adjoint-capable runs or trace_type 1), else v.
    if (S.rec) {
        const Csr cs(S.rec);
        const int first = cs.tile_ptr[tile], nrec = cs.tile_ptr[tile + 1] - first;
        const int nt = S.nt;
        for (int q = tid; q < nrec; q += kThreads) {
            const int ent = first + q;
            const int e = cs.local[ent];  // c * TZ + r within the owned tile
            const int c = e / TZ, r = e - c * TZ;
            const size_t k = (size_t)(i0 + c) * nz + (j0 + r);
            const int ev = (c + 1) * VZ + (r + 1);
            for (int t = cs.tptr[ent]; t < cs.tptr[ent + 1]; t++) {
                const size_t kr = (size_t)cs.traces[t] * nt + it;
                if (PSV) {
                    S.out_x[kr] = S.record_u ? u[0][k] : s_v[0][ev];
                    S.out_z[kr] = S.record_u ? u[NV - 1][k] : s_v[NV - 1][ev];
                } else {
                    S.out_y[kr] = S.record_u ? u[0][k] : s_v[0][ev];
                }
            }
        }
    }

    // ---- 3. stress update on owned cells (solver/fdm.h:138-149).
#pragma unroll
    for (int q = 0; q < QO; q++) {
        const int e = tid + q * kThreads;
        if (e >= NO) continue;
        const int c = e / TZ, r = e - c * TZ;
        const int i = i0 + c, j = j0 + r;
        if (i >= nx || j >= nz) continue;
        const size_t k = (size_t)i * nz + j;
        const int vc = c + 1, vr = r + 1;
        const int se = (c + 3) * RZ + (r + 3);
#define VV(f, dc, dr) s_v[f][(vc + (dc)) * VZ + vr + (dr)]
        const float m = mu_reg[q];
        if (PSV) {
            float dvxdx = 0.f, dvzdx = 0.f, dvxdz = 0.f, dvzdz = 0.f;
            if (i >= 1 && i < nx - 2) {
                dvxdx = dplus(VV(0, 1, 0), VV(0, 0, 0), VV(0, 2, 0), VV(0, -1, 0), c9x, c24x);
                dvzdx = dplus(VV(1, 1, 0), VV(1, 0, 0), VV(1, 2, 0), VV(1, -1, 0), c9x, c24x);
            }
            if (j >= 1 && j < nz - 2) {
                dvxdz = dplus(VV(0, 0, 1), VV(0, 0, 0), VV(0, 0, 2), VV(0, 0, -1), c9z, c24z);
                dvzdz = dplus(VV(1, 0, 1), VV(1, 0, 0), VV(1, 0, 2), VV(1, 0, -1), c9z, c24z);
            }
            float sxx = s_sig[0][se], szz = s_sig[1][se], sxz = s_sig[2][se];
            st_stress_psv(sxx, szz, sxz, lam_reg[q], m, dt, dvxdx, dvxdz, dvzdx, dvzdz);
            sig_out[0][k] = sxx;
            sig_out[1][k] = szz;
            sig_out[2][k] = sxz;
        } else {
            float dvydx = 0.f, dvydz = 0.f;
            if (i >= 1 && i < nx - 2) dvydx = dplus(VV(0, 1, 0), VV(0, 0, 0), VV(0, 2, 0), VV(0, -1, 0), c9x, c24x);
            if (j >= 1 && j < nz - 2) dvydz = dplus(VV(0, 0, 1), VV(0, 0, 0), VV(0, 0, 2), VV(0, 0, -1), c9z, c24z);
            float sxy = s_sig[0][se], szy = s_sig[1][se];
            st_stress_sh(sxy, szy, m, dt, dvydx, dvydz);
            sig_out[0][k] = sxy;
            sig_out[1][k] = szy;
        }
#undef VV
    }
}

template <bool PSV>
static cudaError_t launch_step_t(TileCfg tc, const Slot *d_slots, int nslots, int max_tiles, int k,
                                 cudaStream_t st) {
    dim3 grid(max_tiles, nslots);
    if (tc.tz == 32 && tc.tx == 32)
        k_step<PSV, 32, 32><<<grid, kThreads, 0, st>>>(d_slots, k);
    else if (tc.tz == 64 && tc.tx == 16)
        k_step<PSV, 64, 16><<<grid, kThreads, 0, st>>>(d_slots, k);
    else if (tc.tz == 32 && tc.tx == 16)
        k_step<PSV, 32, 16><<<grid, kThreads, 0, st>>>(d_slots, k);
    else if (tc.tz == 16 && tc.tx == 32)
        k_step<PSV, 16, 32><<<grid, kThreads, 0, st>>>(d_slots, k);
    else if (tc.tz == 128 && tc.tx == 8)
        k_step<PSV, 128, 8><<<grid, kThreads, 0, st>>>(d_slots, k);
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}

cudaError_t launch_step(bool psv, TileCfg tc, const Slot *d_slots, int nslots, int max_tiles, int k, bool tma,
                        cudaStream_t st, const unsigned *block_map, int nmap) {
    if (tc.threads) return launch_march(psv, tma, tc.threads, tc.tx, d_slots, nslots, max_tiles, k, st, block_map, nmap);
    if (block_map) return cudaErrorInvalidValue;
    if (nslots <= 0 || max_tiles <= 0) return cudaSuccess;
    return psv ? launch_step_t<true>(tc, d_slots, nslots, max_tiles, k, st)
               : launch_step_t<false>(tc, d_slots, nslots, max_tiles, k, st);
}

// ------------------------------------------------------------ checkpoints
// Forward checkpoints (solver/fdm.h:521-533,552-560): at the step with
// (it+1) % sfe == 0, displacement is saved before the step and velocity after
// it, into slot isfe = nsfe - (it+1)/sfe. Storage is FP32, BF16 or FP16; the
// 16-bit forms store the displacement's differences that the kernel
// accumulation reads instead of the displacement (ckpt_nf_sh/psv), and use
// one power-of-two scale per snapshot and field, derived from the field's
// max |value|, so the scaling itself adds no rounding.
__device__ __forceinline__ float ckpt_scale(float amax, int prec) { return ckpt_scale_of(amax, prec); }

// The fields of one checkpoint group (displacement before the step,
// which_u = 1, or velocity after it, which_u = 0) of one wave system: their
// index in the slot's checkpoint and how each is formed from the state.
struct CkGroup {
    int nfld;
    int q[3];
    int kind;  // 0: copies of a, b; 1: SH d/dx, d/dz of a; 2: P-SV strains of a = ux, b = uz
    const float *a, *b;
};

__device__ __forceinline__ CkGroup ckpt_group(const Slot &S, bool psv, int which_u, int par) {
    CkGroup g;
    const bool q16 = S.ckpt_prec != CKPT_F32;
    if (!psv) {
        g.kind = (which_u && q16) ? 1 : 0;
        g.a = which_u ? S.sh[UY] : S.sh[VY0 + par];
        g.b = nullptr;
        if (q16) {
            g.nfld = which_u ? 2 : 1;
            g.q[0] = which_u ? 0 : 2;
            g.q[1] = 1;
        } else {
            g.nfld = 1;
            g.q[0] = which_u ? 0 : 1;
        }
        return g;
    }
    const int base = S.sh[0] != nullptr ? ckpt_nf_sh(S.ckpt_prec) : 0;
    g.a = which_u ? S.psv[UX] : S.psv[VX0 + par];
    g.b = which_u ? S.psv[UZ] : S.psv[VZ0 + par];
    g.kind = (which_u && q16) ? 2 : 0;
    if (q16) {
        g.nfld = which_u ? 3 : 2;
        for (int f = 0; f < g.nfld; f++) g.q[f] = base + (which_u ? 0 : 3) + f;
    } else {
        g.nfld = 2;
        for (int f = 0; f < 2; f++) g.q[f] = base + (which_u ? 0 : 2) + f;
    }
    return g;
}

// Field f of group g at cell k, in FP32: a copy, or the forward-staggered
// differences of the kernel accumulation (the guards and arithmetic of
// k_interaction's FP32 path: 0 where the reference skips a difference).
// Column i = k / nz and row j of reference-layout cell k among n cells: a
// 32-bit division below 2^31 cells (the 64-bit one takes several times the
// instructions, and these kernels divide once per cell).
__device__ __forceinline__ void cell_ij(size_t k, int nz, size_t n, int &i, int &j) {
    if (n < ((size_t)1 << 31)) {
        const unsigned u = (unsigned)k, q = u / (unsigned)nz;
        i = (int)q;
        j = (int)(u - q * (unsigned)nz);
    } else {
        i = (int)(k / nz);
        j = (int)(k - (size_t)i * nz);
    }
}

// Every field of group g at cell k, in FP32: copies, or the forward-staggered
// differences of the kernel accumulation (the guards and arithmetic of
// k_interaction's FP32 path: 0 where the reference skips a difference), each
// neighbour loaded once for all the group's fields.
__device__ __forceinline__ void ckpt_values(const Slot &S, const CkGroup &g, size_t k, float *out) {
    const int nx = S.nx, nz = S.nz, pz = S.pz;
    int i, j;
    cell_ij(k, nz, (size_t)nx * nz, i, j);
    const size_t a = (size_t)i * pz + j;  // the state address at the slot's pitch
    if (g.kind == 0) {
        out[0] = __ldg(g.a + a);
        if (g.nfld > 1) out[1] = __ldg(g.b + a);
        return;
    }
    const bool gx = i >= 1 && i < nx - 2, gz = j >= 1 && j < nz - 2;
    auto ddx = [&](const float *w) {
        return gx ? dplus(__ldg(w + a + pz), __ldg(w + a), __ldg(w + a + 2 * pz), __ldg(w + a - pz), S.c9x, S.c24x)
                  : 0.f;
    };
    auto ddz = [&](const float *w) {
        return gz ? dplus(__ldg(w + a + 1), __ldg(w + a), __ldg(w + a + 2), __ldg(w + a - 1), S.c9z, S.c24z) : 0.f;
    };
    if (g.kind == 1) {
        out[0] = ddx(g.a);
        out[1] = ddz(g.a);
        return;
    }
    const float exx = ddx(g.a), ezz = ddz(g.b);
    out[0] = exx + ezz;              // divergence
    out[1] = exx - ezz;              // normal-strain difference
    out[2] = ddx(g.b) + ddz(g.a);    // d(uz)/dx + d(ux)/dz, summed as st_kmu_psv sums them
}

// Checkpoint slot of step index k for slot S, or -1 when k is not a
// checkpoint step of S; *par receives the parity of the velocity written by
// that step.
__device__ __forceinline__ int ckpt_slot(const Slot &S, int k, int *par) {
    if (!S.active || !S.ckpt || !S.ckpt_write || S.sfe <= 0) return -1;
    const int it = S.it_base + k;
    if (it < 0 || it >= S.nt || (it + 1) % S.sfe != 0) return -1;
    const int isfe = S.nsfe - (it + 1) / S.sfe;
    *par = (S.par0 + k + 1) & 1;
    return (isfe >= 0 && isfe < S.nsfe) ? isfe : -1;
}

__global__ void k_ckpt_amax(const Slot *__restrict__ slots, int kstep, int which_u, bool psv) {
    const Slot &S = slots[blockIdx.y];
    int par = 0;
    const int isfe = ckpt_slot(S, kstep, &par);
    if (isfe < 0) return;
    if (psv ? S.psv[0] == nullptr : S.sh[0] == nullptr) return;
    const CkGroup g = ckpt_group(S, psv, which_u, par);
    const size_t n = (size_t)S.nx * S.nz;
    __shared__ float red[3][32];
    float m[3] = {0.f, 0.f, 0.f};
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        float v[3];
        ckpt_values(S, g, k, v);
#pragma unroll
        for (int f = 0; f < 3; f++)
            if (f < g.nfld) m[f] = fmaxf(m[f], fabsf(v[f]));
    }
#pragma unroll
    for (int f = 0; f < 3; f++) {
        if (f >= g.nfld) break;
        float x = m[f];
        for (int o = 16; o; o >>= 1) x = fmaxf(x, __shfl_xor_sync(0xffffffffu, x, o));
        if ((threadIdx.x & 31) == 0) red[f][threadIdx.x >> 5] = x;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        for (int f = 0; f < g.nfld; f++) {
            float x = threadIdx.x < (blockDim.x >> 5) ? red[f][threadIdx.x] : 0.f;
            for (int o = 16; o; o >>= 1) x = fmaxf(x, __shfl_xor_sync(0xffffffffu, x, o));
            // non-negative floats order like their bit patterns
            if (threadIdx.x == 0)
                atomicMax(reinterpret_cast<unsigned *>(S.ckpt_amax) + (size_t)isfe * S.nf + g.q[f], __float_as_uint(x));
        }
    }
}

__global__ void k_ckpt_store(const Slot *__restrict__ slots, int kstep, int which_u, bool psv) {
    const Slot &S = slots[blockIdx.y];
    int par = 0;
    const int isfe = ckpt_slot(S, kstep, &par);
    if (isfe < 0) return;
    if (psv ? S.psv[0] == nullptr : S.sh[0] == nullptr) return;
    const CkGroup g = ckpt_group(S, psv, which_u, par);
    const size_t n = (size_t)S.nx * S.nz;
    size_t off[3];
#pragma unroll
    for (int f = 0; f < 3; f++) off[f] = ((size_t)isfe * S.nf + g.q[f < g.nfld ? f : 0]) * n;
    // the fields' scales, formed once per block (a division and an exponent
    // split each; on small grids a thread stores only a cell or two)
    __shared__ float s_sc[3];
    if ((int)threadIdx.x < g.nfld)
        s_sc[threadIdx.x] = S.ckpt_prec != CKPT_F32
                                ? ckpt_scale(S.ckpt_amax[(size_t)isfe * S.nf + g.q[threadIdx.x]], S.ckpt_prec)
                                : 1.f;
    __syncthreads();
    float sc[3];
#pragma unroll
    for (int f = 0; f < 3; f++) sc[f] = f < g.nfld ? s_sc[f] : 1.f;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        float v[3];
        ckpt_values(S, g, k, v);
#pragma unroll
        for (int f = 0; f < 3; f++) {
            if (f >= g.nfld) break;
            if (S.ckpt_prec == CKPT_F32)
                static_cast<float *>(S.ckpt)[off[f] + k] = v[f];
            else if (S.ckpt_prec == CKPT_BF16)
                static_cast<__nv_bfloat16 *>(S.ckpt)[off[f] + k] = __float2bfloat16_rn(v[f] * sc[f]);
            else
                static_cast<__half *>(S.ckpt)[off[f] + k] = __float2half_rn(v[f] * sc[f]);
        }
    }
}

// Blocks per slot (or group) for the grid-stride cell loops: about 2432
// blocks in all, so that batches of many small grids (serving) do not launch
// tens of thousands of blocks that find no work, at least 8 per slot, and no
// more than the slot's cells need.
static int cell_blocks(size_t n, int nslots) {
    const int need = (int)std::min<size_t>((n + 255) / 256, 1 << 20);
    const int share = std::max(8, 2432 / std::max(nslots, 1));
    return std::max(1, std::min(need, share));
}

cudaError_t launch_ckpt_amax(const Slot *d_slots, int nslots, int n, int k, int which_u, bool psv,
                             cudaStream_t st) {
    if (nslots <= 0) return cudaSuccess;
    k_ckpt_amax<<<dim3(cell_blocks((size_t)n, nslots), nslots), 256, 0, st>>>(d_slots, k, which_u, psv);
    return cudaGetLastError();
}

cudaError_t launch_ckpt_store(const Slot *d_slots, int nslots, int n, int k, int which_u, bool psv,
                              cudaStream_t st) {
    if (nslots <= 0) return cudaSuccess;
    k_ckpt_store<<<dim3(cell_blocks((size_t)n, nslots), nslots), 256, 0, st>>>(d_slots, k, which_u, psv);
    return cudaGetLastError();
}

// ------------------------------------------------------------ interaction
// Sensitivity-kernel accumulation at adjoint steps with it % sfe == 0
// (solver/fdm.h:583-606, interaction*: solver/fdm.h:198-219): gradients of the
// adjoint displacement and of the checkpointed forward displacement, the
// checkpointed forward velocity and the adjoint velocity, scaled by
// ndt = sfe*dt. Each thread owns one cell and walks the group's slots in
// order, so shots accumulate without atomics and deterministically.
__device__ __forceinline__ float ck_load(const Slot &S, int isfe, int q, size_t k, size_t n, float inv) {
    const size_t off = ((size_t)isfe * S.nf + q) * n + k;
    if (S.ckpt_prec == CKPT_F32) return __ldg(static_cast<const float *>(S.ckpt) + off);
    if (S.ckpt_prec == CKPT_BF16) return __bfloat162float(static_cast<const __nv_bfloat16 *>(S.ckpt)[off]) * inv;
    return __half2float(static_cast<const __half *>(S.ckpt)[off]) * inv;
}

template <bool PSV>
__global__ void k_interaction(const Slot *__restrict__ slots, const KernelGroup *__restrict__ groups, int kstep) {
    const KernelGroup &G = groups[blockIdx.y];
    const int nx = G.nx, nz = G.nz;
    const size_t n = (size_t)nx * nz;
    __shared__ float s_inv[5];
    // the block's cells, blockDim.x at a time (the loop bound is the same for
    // every thread; threads past the grid work on the last cell and store
    // nothing, so that every thread reaches the block barriers below)
    for (size_t kb = blockIdx.x * (size_t)blockDim.x; kb < n; kb += (size_t)gridDim.x * blockDim.x) {
        const size_t k0 = kb + threadIdx.x;
        const bool live = k0 < n;
        const size_t k = live ? k0 : n - 1;
        int i, j;
        cell_ij(k, nz, n, i, j);
        const bool gx = i >= 1 && i < nx - 2, gz = j >= 1 && j < nz - 2;
        float kl = G.inv_lambda ? G.k_lambda[k] : 0.f;
        float km = G.inv_mu ? G.k_mu[k] : 0.f;
        float kr = G.inv_rho ? G.k_rho[k] : 0.f;
        for (int s = G.first; s < G.first + G.count; s++) {
            const Slot &S = slots[s];
            if (!S.active || !S.ckpt || S.sfe <= 0) continue;
            const int it = S.it_base + kstep;
            if (it < 0 || it >= S.nt || it % S.sfe != 0) continue;
            const int isfe = it / S.sfe;
            if (isfe >= S.nsfe) continue;
            const int par = (S.par0 + kstep + 1) & 1;  // velocity written by this step
            const float ndt = (float)S.sfe * S.dt;
            const float c9x = S.c9x, c24x = S.c24x, c9z = S.c9z, c24z = S.c24z;
            const bool q16 = S.ckpt_prec != CKPT_F32;
            const int base = (PSV && S.sh[0] != nullptr) ? ckpt_nf_sh(S.ckpt_prec) : 0;
            const int nfs = PSV ? ckpt_nf_psv(S.ckpt_prec) : ckpt_nf_sh(S.ckpt_prec);
            // the inverse scales of the slot's checkpoint fields, formed once per
            // block (a division and an exponent split each); the slot conditions
            // above are the same for every thread of the block
            __syncthreads();  // every thread has read the previous slot's
            if ((int)threadIdx.x < nfs) {
                const float a = S.ckpt_amax ? S.ckpt_amax[(size_t)isfe * S.nf + base + threadIdx.x] : 0.f;
                s_inv[threadIdx.x] = 1.f / ckpt_scale(a, S.ckpt_prec);
            }
            __syncthreads();
            float inv[5];
            for (int q = 0; q < nfs; q++) inv[q] = s_inv[q];
            // the slot's state at its pitch; checkpoints and kernels in the reference layout
            const int pz = S.pz;
            const size_t a = (size_t)i * pz + j;
            auto grad = [&](const float *w, float &ddx, float &ddz) {
                ddx = gx ? dplus(__ldg(w + a + pz), __ldg(w + a), __ldg(w + a + 2 * pz), __ldg(w + a - pz), c9x, c24x) : 0.f;
                ddz = gz ? dplus(__ldg(w + a + 1), __ldg(w + a), __ldg(w + a + 2), __ldg(w + a - 1), c9z, c24z) : 0.f;
            };
            auto grad_ck = [&](int q, float &ddx, float &ddz) {
                const float iv = inv[q];
                ddx = gx ? dplus(ck_load(S, isfe, base + q, k + nz, n, iv), ck_load(S, isfe, base + q, k, n, iv),
                                 ck_load(S, isfe, base + q, k + 2 * nz, n, iv), ck_load(S, isfe, base + q, k - nz, n, iv),
                                 c9x, c24x)
                         : 0.f;
                ddz = gz ? dplus(ck_load(S, isfe, base + q, k + 1, n, iv), ck_load(S, isfe, base + q, k, n, iv),
                                 ck_load(S, isfe, base + q, k + 2, n, iv), ck_load(S, isfe, base + q, k - 1, n, iv),
                                 c9z, c24z)
                         : 0.f;
            };
            auto ck = [&](int q) { return ck_load(S, isfe, base + q, k, n, inv[q]); };
            if (PSV) {
                float dvxdx, dvxdz, dvzdx, dvzdz;
                grad(S.psv[UX], dvxdx, dvxdz);
                grad(S.psv[UZ], dvzdx, dvzdz);
                // forward: FP32 displacement (differences taken here), or the
                // stored strains: divergence, normal-strain difference, shear sum (16-bit)
                float fxdx = 0.f, fxdz = 0.f, fzdx = 0.f, fzdz = 0.f, fdv = 0.f, fdd = 0.f, fsh = 0.f;
                if (q16) {
                    fdv = ck(0);
                    fdd = ck(1);
                    fsh = ck(2);
                } else {
                    grad_ck(0, fxdx, fxdz);
                    grad_ck(1, fzdx, fzdz);
                }
                if (G.inv_rho) {
                    const float vx_fw = ck(q16 ? 3 : 2);
                    const float vz_fw = ck(q16 ? 4 : 3);
                    kr = st_krho_psv(kr, vx_fw, __ldg(S.psv[VX0 + par] + a), vz_fw, __ldg(S.psv[VZ0 + par] + a), ndt);
                }
                if (G.inv_mu)
                    km = q16 ? st_kmu_psv_strain(km, dvxdx, dvxdz, dvzdx, dvzdz, fdv, fdd, fsh, ndt)
                             : st_kmu_psv(km, dvxdx, dvxdz, dvzdx, dvzdz, fxdx, fxdz, fzdx, fzdz, ndt);
                if (G.inv_lambda)
                    kl = q16 ? st_klambda_psv_strain(kl, dvxdx, dvzdz, fdv, ndt)
                             : st_klambda_psv(kl, dvxdx, dvzdz, fxdx, fzdz, ndt);
            } else {
                float dvydx, dvydz, fdx, fdz;
                grad(S.sh[UY], dvydx, dvydz);
                if (q16) {
                    fdx = ck(0);
                    fdz = ck(1);
                } else {
                    grad_ck(0, fdx, fdz);
                }
                if (G.inv_rho) {
                    const float vy_fw = ck(q16 ? 2 : 1);
                    kr = st_krho_sh(kr, vy_fw, __ldg(S.sh[VY0 + par] + a), ndt);
                }
                if (G.inv_mu) km = st_kmu_sh(km, dvydx, fdx, dvydz, fdz, ndt);
            }
        }
        if (live) {
            if (G.inv_lambda) G.k_lambda[k] = kl;
            if (G.inv_mu) G.k_mu[k] = km;
            if (G.inv_rho) G.k_rho[k] = kr;
        }
    }
}

cudaError_t launch_interaction(bool psv, const Slot *d_slots, const KernelGroup *d_groups, int ngroups,
                               int max_cells, int k, cudaStream_t st) {
    if (ngroups <= 0) return cudaSuccess;
    const dim3 grid(cell_blocks((size_t)max_cells, ngroups), ngroups);
    if (psv)
        k_interaction<true><<<grid, 256, 0, st>>>(d_slots, d_groups, k);
    else
        k_interaction<false><<<grid, 256, 0, st>>>(d_slots, d_groups, k);
    return cudaGetLastError();
}

}  // namespace gb
