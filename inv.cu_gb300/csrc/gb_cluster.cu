// Cluster-resident solver: a whole forward or adjoint pass of one shot in one
// thread-block cluster, with the wavefield kept in distributed shared memory.
//
// When a shot's state (P-SV 7 fields, SH 4 fields, FP32) fits in the shared
// memory of R CTAs (R <= 16), the time loop runs inside one persistent
// kernel: CTA r of a cluster owns the grid columns [r*cp, (r+1)*cp) and keeps
// their state in its shared memory; the x-neighbours of its first and last
// columns are read from the neighbouring CTAs' shared memory through the
// cluster (distributed shared memory). Each time step is
//   phase A  stress divergence, sources, velocity and displacement update
//   barrier  (all velocities written, all stresses of step n still in place)
//   phase B  velocity gradients and stress update
//   barrier  (all stresses written before the next phase A reads them)
// plus, in the adjoint, the kernel accumulation every sfe steps (one more
// barrier). Only receivers, checkpoints and the model (read from L2) touch
// memory outside the SM, so the per-step cost is the stencil arithmetic and
// shared-memory traffic instead of DRAM/L2 round trips and kernel launches.
//
// Every cell is computed with the operations, in the order, of the fused
// step kernels (gb_step.cu): forward traces and checkpoints are bit-identical
// to theirs. The adjoint accumulates each shot's kernel contribution in a
// per-shot buffer that is added to the kernels after the pass, in shot order.
#include <cooperative_groups.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>

#include "gb_internal.h"
#include "gb_stencil.h"

namespace cg = cooperative_groups;

namespace gb {

__device__ __forceinline__ float cdm(float a0, float am1, float ap1, float am2, float c9, float c24) {
    return st_dminus(a0, am1, ap1, am2, c9, c24);
}
__device__ __forceinline__ float cdp(float ap1, float a0, float ap2, float am1, float c9, float c24) {
    return st_dplus(ap1, a0, ap2, am1, c9, c24);
}

__device__ __forceinline__ float ck_get(const Slot &S, int isfe, int q, size_t k, size_t n, float inv) {
    const size_t off = ((size_t)isfe * S.nf + q) * n + k;
    if (S.ckpt_prec == CKPT_F32) return __ldg(static_cast<const float *>(S.ckpt) + off);
    if (S.ckpt_prec == CKPT_BF16) return __bfloat162float(static_cast<const __nv_bfloat16 *>(S.ckpt)[off]) * inv;
    return __half2float(static_cast<const __half *>(S.ckpt)[off]) * inv;
}

// Shared-memory field order. P-SV: vx vz ux uz sxx szz sxz; SH: vy uy sxy szy.
template <bool PSV, bool ADJ>
__global__ void __launch_bounds__(1024, 1) k_cluster(const Slot *__restrict__ slots, ClusterGeom g,
                                                     float *__restrict__ kpart) {
    constexpr int NF = PSV ? 7 : 4;
    constexpr int NV = PSV ? 2 : 1;
    constexpr int FV = 0, FU = NV, FS = 2 * NV;  // first velocity, displacement, stress field
    extern __shared__ float sm[];
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const int slot = blockIdx.x / g.R;
    const Slot &S = slots[slot];
    if (!S.active) return;  // uniform over the cluster: one slot per cluster
    const int nx = S.nx, nz = S.nz, nt = S.nt, cp = g.cols_per;
    const size_t ncell = (size_t)nx * nz;
    const int x0 = rank * cp, x1 = min(x0 + cp, nx);
    const int t = threadIdx.x, row = t % g.rows_pad, grp = t / g.rows_pad;
    const bool act = row < nz && grp < g.G;
    const int ncol = (act && x1 - x0 > grp) ? (x1 - x0 - grp + g.G - 1) / g.G : 0;

    // shared memory: NF fields [cp][nz], then the receiver map [cp][nz] (the
    // receiver, or adjoint source, at each owned cell; -1 for none)
    int *recmap = reinterpret_cast<int *>(sm + (size_t)NF * cp * nz);
    for (int e = t; e < NF * cp * nz; e += blockDim.x) sm[e] = 0.f;
    for (int e = t; e < cp * nz; e += blockDim.x) recmap[e] = -1;
    __syncthreads();
    for (int r = t; r < S.npts; r += blockDim.x) {
        const int i = S.pts_i[r], j = S.pts_j[r];
        if (i >= x0 && i < x1 && j >= 0 && j < nz) recmap[(i - x0) * nz + j] = r;  // cells are distinct
    }
    const int src_k = (!ADJ && S.src_trace >= 0) ? S.src_i * nz + S.src_j : -1;  // forward source cell

    const float dt = S.dt, c9x = S.c9x, c24x = S.c24x, c9z = S.c9z, c24z = S.c24z;
    const float azj = act ? __ldg(S.az + row) : 0.f;
    const bool zS = row >= 2 && row < nz - 2, zV = row >= 1 && row < nz - 2;
    const int base_ck = (PSV && S.sh[0] != nullptr) ? 2 : 0;  // checkpoint field offset of this system
    cl.sync();

    // column i of field f: own shared memory or a neighbour's, by rank
    auto col = [&](int f, int i) -> const float * {
        const int owner = i / cp;
        float *p = sm + ((size_t)f * cp + (i - owner * cp)) * nz;
        return owner == rank ? p : cl.map_shared_rank(p, owner);
    };
    auto own = [&](int f, int i) -> float * { return sm + ((size_t)f * cp + (i - x0)) * nz; };

    for (int it = 0; it < nt; it++) {
        // forward checkpoint of displacement before the step
        int isfe = -1;
        if (!ADJ && S.ckpt && S.sfe > 0 && (it + 1) % S.sfe == 0) isfe = S.nsfe - (it + 1) / S.sfe;
        if (isfe >= 0) {
            for (int q = 0; q < ncol; q++) {
                const int i = x0 + grp + q * g.G;
                const size_t k = (size_t)i * nz + row;
#pragma unroll
                for (int f = 0; f < NV; f++)
                    static_cast<float *>(S.ckpt)[((size_t)isfe * S.nf + base_ck + f) * ncell + k] = own(FU + f, i)[row];
            }
        }
        // ---- phase A: divergence, sources, velocity, displacement
        for (int q = 0; q < ncol; q++) {
            const int i = x0 + grp + q * g.G;
            const size_t k = (size_t)i * nz + row;
            const bool xS = i >= 2 && i < nx - 2;
            float ds[NV];
            const bool inner = i - 2 >= x0 && i + 1 < x1;
            if (PSV) {
                // sxx (x), sxz (x and z), szz (z)
                const float *a0 = own(FS + 0, i), *c0 = own(FS + 2, i), *b0 = own(FS + 1, i);
                float dsx = 0.f, dsz = 0.f;
                if (xS) {
                    const float *am1 = inner ? a0 - nz : col(FS + 0, i - 1), *ap1 = inner ? a0 + nz : col(FS + 0, i + 1),
                                *am2 = inner ? a0 - 2 * nz : col(FS + 0, i - 2);
                    const float *cm1 = inner ? c0 - nz : col(FS + 2, i - 1), *cp1 = inner ? c0 + nz : col(FS + 2, i + 1),
                                *cm2 = inner ? c0 - 2 * nz : col(FS + 2, i - 2);
                    dsx = cdm(a0[row], am1[row], ap1[row], am2[row], c9x, c24x);
                    dsz = cdm(c0[row], cm1[row], cp1[row], cm2[row], c9x, c24x);
                }
                if (zS) {
                    dsx += cdm(c0[row], c0[row - 1], c0[row + 1], c0[row - 2], c9z, c24z);
                    dsz += cdm(b0[row], b0[row - 1], b0[row + 1], b0[row - 2], c9z, c24z);
                }
                ds[0] = dsx;
                ds[NV - 1] = dsz;
            } else {
                const float *a0 = own(FS + 0, i), *b0 = own(FS + 1, i);
                float dsy = 0.f;
                if (xS) {
                    const float *am1 = inner ? a0 - nz : col(FS + 0, i - 1), *ap1 = inner ? a0 + nz : col(FS + 0, i + 1),
                                *am2 = inner ? a0 - 2 * nz : col(FS + 0, i - 2);
                    dsy = cdm(a0[row], am1[row], ap1[row], am2[row], c9x, c24x);
                }
                if (zS) dsy += cdm(b0[row], b0[row - 1], b0[row + 1], b0[row - 2], c9z, c24z);
                ds[0] = dsy;
            }
            const int rq = recmap[(i - x0) * nz + row];
            if (!ADJ && (int)k == src_k) {
                const size_t ks = (size_t)S.src_trace * nt + it;
                if (PSV) {
                    ds[0] += __ldg(S.inj_x + ks);
                    ds[NV - 1] += __ldg(S.inj_z + ks);
                } else {
                    ds[0] += __ldg(S.inj_y + ks);
                }
            }
            if (ADJ && rq >= 0) {
                const size_t ks = (size_t)rq * nt + it;
                if (PSV) {
                    ds[0] += __ldg(S.inj_x + ks);
                    ds[NV - 1] += __ldg(S.inj_z + ks);
                } else {
                    ds[0] += __ldg(S.inj_y + ks);
                }
            }
            const float ab = __ldg(S.ax + i) * azj;
            const float rinv = __ldg(S.rinv + k);
            float vn[NV], un[NV];
#pragma unroll
            for (int f = 0; f < NV; f++) {
                float *pv = own(FV + f, i), *pu = own(FU + f, i);
                vn[f] = st_velocity(ab, dt, ds[f], rinv, pv[row]);
                un[f] = st_displacement(pu[row], vn[f], dt);
                pv[row] = vn[f];
                pu[row] = un[f];
            }
            if (!ADJ && rq >= 0) {
                const size_t kr = (size_t)rq * nt + it;
                if (PSV) {
                    S.out_x[kr] = S.record_u ? un[0] : vn[0];
                    S.out_z[kr] = S.record_u ? un[NV - 1] : vn[NV - 1];
                } else {
                    S.out_y[kr] = S.record_u ? un[0] : vn[0];
                }
            }
            if (isfe >= 0) {
#pragma unroll
                for (int f = 0; f < NV; f++)
                    static_cast<float *>(S.ckpt)[((size_t)isfe * S.nf + base_ck + NV + f) * ncell + k] = vn[f];
            }
        }
        cl.sync();
        // ---- phase B: velocity gradients and stress update
        for (int q = 0; q < ncol; q++) {
            const int i = x0 + grp + q * g.G;
            const size_t k = (size_t)i * nz + row;
            const bool xV = i >= 1 && i < nx - 2;
            const bool inner = i - 1 >= x0 && i + 2 < x1;
            float dxv[NV], dzv[NV];
#pragma unroll
            for (int f = 0; f < NV; f++) {
                const float *v0 = own(FV + f, i);
                dxv[f] = 0.f;
                if (xV) {
                    const float *vp1 = inner ? v0 + nz : col(FV + f, i + 1), *vp2 = inner ? v0 + 2 * nz : col(FV + f, i + 2),
                                *vm1 = inner ? v0 - nz : col(FV + f, i - 1);
                    dxv[f] = cdp(vp1[row], v0[row], vp2[row], vm1[row], c9x, c24x);
                }
                dzv[f] = zV ? cdp(v0[row + 1], v0[row], v0[row + 2], v0[row - 1], c9z, c24z) : 0.f;
            }
            const float m = __ldg(S.mu + k);
            if (PSV) {
                const float l = __ldg(S.lambda + k);
                float *sxx = own(FS + 0, i), *szz = own(FS + 1, i), *sxz = own(FS + 2, i);
                float a = sxx[row], b = szz[row], c = sxz[row];
                st_stress_psv(a, b, c, l, m, dt, dxv[0], dzv[0], dxv[1], dzv[1]);
                sxx[row] = a;
                szz[row] = b;
                sxz[row] = c;
            } else {
                float *sxy = own(FS + 0, i), *szy = own(FS + 1, i);
                float a = sxy[row], b = szy[row];
                st_stress_sh(a, b, m, dt, dxv[0], dzv[0]);
                sxy[row] = a;
                szy[row] = b;
            }
        }
        cl.sync();
        // ---- adjoint: kernel accumulation every sfe steps (solver/fdm.h:583-606)
        if (ADJ && S.ckpt && S.sfe > 0 && it % S.sfe == 0 && it / S.sfe < S.nsfe) {
            const int isfe_a = it / S.sfe;
            const float ndt = (float)S.sfe * dt;
            const int nfu = NV;
            float inv[4];
            for (int q = 0; q < 2 * nfu; q++) {
                const float a = S.ckpt_amax ? S.ckpt_amax[(size_t)isfe_a * S.nf + base_ck + q] : 0.f;
                inv[q] = 1.f / ckpt_scale_of(a, S.ckpt_prec);
            }
            float *kl = kpart + ((size_t)slot * 3 + 0) * ncell;
            float *km = kpart + ((size_t)slot * 3 + 1) * ncell;
            float *kr = kpart + ((size_t)slot * 3 + 2) * ncell;
            for (int q = 0; q < ncol; q++) {
                const int i = x0 + grp + q * g.G;
                const size_t k = (size_t)i * nz + row;
                const bool gx = i >= 1 && i < nx - 2;
                const bool inner = i - 1 >= x0 && i + 2 < x1;
                float ux[NV], uzz[NV], fx[NV], fz[NV];
#pragma unroll
                for (int f = 0; f < NV; f++) {
                    const float *u0 = own(FU + f, i);
                    ux[f] = 0.f;
                    if (gx) {
                        const float *up1 = inner ? u0 + nz : col(FU + f, i + 1), *up2 = inner ? u0 + 2 * nz : col(FU + f, i + 2),
                                    *um1 = inner ? u0 - nz : col(FU + f, i - 1);
                        ux[f] = cdp(up1[row], u0[row], up2[row], um1[row], c9x, c24x);
                    }
                    uzz[f] = zV ? cdp(u0[row + 1], u0[row], u0[row + 2], u0[row - 1], c9z, c24z) : 0.f;
                    const int qc = base_ck + f;
                    const float iv = inv[f];
                    fx[f] = gx ? cdp(ck_get(S, isfe_a, qc, k + nz, ncell, iv), ck_get(S, isfe_a, qc, k, ncell, iv),
                                     ck_get(S, isfe_a, qc, k + 2 * nz, ncell, iv),
                                     ck_get(S, isfe_a, qc, k - nz, ncell, iv), c9x, c24x)
                               : 0.f;
                    fz[f] = zV ? cdp(ck_get(S, isfe_a, qc, k + 1, ncell, iv), ck_get(S, isfe_a, qc, k, ncell, iv),
                                     ck_get(S, isfe_a, qc, k + 2, ncell, iv), ck_get(S, isfe_a, qc, k - 1, ncell, iv),
                                     c9z, c24z)
                               : 0.f;
                }
                if (PSV) {
                    const float dvxdx = ux[0], dvxdz = uzz[0], dvzdx = ux[1], dvzdz = uzz[1];
                    const float fxdx = fx[0], fxdz = fz[0], fzdx = fx[1], fzdz = fz[1];
                    const float vx_fw = ck_get(S, isfe_a, base_ck + 2, k, ncell, inv[2]);
                    const float vz_fw = ck_get(S, isfe_a, base_ck + 3, k, ncell, inv[3]);
                    kr[k] -= (vx_fw * own(FV + 0, i)[row] + vz_fw * own(FV + 1, i)[row]) * ndt;
                    km[k] -= (2.f * dvxdx * fxdx + 2.f * dvzdz * fzdz + (dvxdz + dvzdx) * (fzdx + fxdz)) * ndt;
                    kl[k] -= ((dvxdx + dvzdz) * (fxdx + fzdz)) * ndt;
                } else {
                    const float vy_fw = ck_get(S, isfe_a, 1, k, ncell, inv[1]);
                    kr[k] -= vy_fw * own(FV, i)[row] * ndt;
                    km[k] -= (ux[0] * fx[0] + uzz[0] * fz[0]) * ndt;
                }
            }
            cl.sync();
        }
    }
}

// k_c += sum over slots of kpart[slot][c], in slot order, for the inverted
// parameters.
__global__ void k_cluster_reduce(const float *__restrict__ kpart, int nslots, size_t ncell, float *kl, float *km,
                                 float *kr, int inv_l, int inv_m, int inv_r) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < ncell; k += (size_t)gridDim.x * blockDim.x) {
        float a = inv_l ? kl[k] : 0.f, b = inv_m ? km[k] : 0.f, c = inv_r ? kr[k] : 0.f;
        for (int s = 0; s < nslots; s++) {
            a += kpart[((size_t)s * 3 + 0) * ncell + k];
            b += kpart[((size_t)s * 3 + 1) * ncell + k];
            c += kpart[((size_t)s * 3 + 2) * ncell + k];
        }
        if (inv_l) kl[k] = a;
        if (inv_m) km[k] = b;
        if (inv_r) kr[k] = c;
    }
}

size_t cluster_smem_bytes(bool psv, const ClusterGeom &g, int nz) {
    return (size_t)((psv ? 7 : 4) + 1) * g.cols_per * nz * 4;
}

template <bool PSV, bool ADJ>
static cudaError_t launch_cluster_t(const Slot *d_slots, int nslots, ClusterGeom g, int nz, float *kpart,
                                    cudaStream_t st) {
    const size_t smem = cluster_smem_bytes(PSV, g, nz);
    cudaError_t e = cudaFuncSetAttribute(k_cluster<PSV, ADJ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (g.R > 8) {
        e = cudaFuncSetAttribute(k_cluster<PSV, ADJ>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return e;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(g.R * nslots);
    cfg.blockDim = dim3(g.rows_pad * g.G);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = g.R;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_cluster<PSV, ADJ>, d_slots, g, kpart);
}

cudaError_t launch_cluster(bool psv, bool adj, const Slot *d_slots, int nslots, ClusterGeom g, int nz, float *kpart,
                           cudaStream_t st) {
    if (nslots <= 0) return cudaSuccess;
    if (psv)
        return adj ? launch_cluster_t<true, true>(d_slots, nslots, g, nz, kpart, st)
                   : launch_cluster_t<true, false>(d_slots, nslots, g, nz, kpart, st);
    return adj ? launch_cluster_t<false, true>(d_slots, nslots, g, nz, kpart, st)
               : launch_cluster_t<false, false>(d_slots, nslots, g, nz, kpart, st);
}

cudaError_t launch_cluster_reduce(const float *kpart, int nslots, size_t ncell, float *kl, float *km, float *kr,
                                  int inv_l, int inv_m, int inv_r, cudaStream_t st) {
    const unsigned blocks = (unsigned)std::min<size_t>((ncell + 255) / 256, 4096);
    k_cluster_reduce<<<blocks, 256, 0, st>>>(kpart, nslots, ncell, kl, km, kr, inv_l, inv_m, inv_r);
    return cudaGetLastError();
}

// Largest number of clusters of this geometry that can be resident at once
// (0 when the geometry cannot launch).
int cluster_occupancy(bool psv, ClusterGeom g, int nz) {
    const size_t smem = cluster_smem_bytes(psv, g, nz);
    auto kern = psv ? (void *)k_cluster<true, false> : (void *)k_cluster<false, false>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
        (void)cudaGetLastError();
        return 0;
    }
    if (g.R > 8 && cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
        (void)cudaGetLastError();
        return 0;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(g.R * 4);
    cfg.blockDim = dim3(g.rows_pad * g.G);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = g.R;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) != cudaSuccess) {
        (void)cudaGetLastError();
        return 0;
    }
    return n;
}

}  // namespace gb
