// Cluster-resident solver: a whole forward or adjoint pass of one shot in one
// thread-block cluster, with the wavefield kept in shared memory.
//
// When a shot's state (P-SV 7 fields, SH 4 fields, FP32) fits in the shared
// memory of R CTAs (R <= 16), the time loop runs inside one persistent
// kernel. CTA r of a cluster owns the grid columns [r*cp, r*cp + ncols) and
// keeps them in its shared memory, with two ghost columns on either side.
// Each thread owns one grid row of up to QM consecutive columns and keeps the
// model of those cells (1/rho, mu, lambda) in registers for the whole pass;
// the x damping profile and the CTA's receiver ids sit in small shared
// tables behind the fields. Each time step is
//   phase A  stress divergence, sources, velocity and displacement update
//   barrier  (all velocities written, all stresses of step n still in place)
//   phase B  velocity gradients and stress update
//   barrier  (all stresses written before the next phase A reads them)
// plus, in the adjoint, every sfe steps either a store of the adjoint state
// of the CTA's cells for the kernel accumulation after the pass
// (k_snap_interaction), or the accumulation itself (one cluster barrier
// more; the shot's kernels stay in shared memory for the whole pass when
// the CTA has room, and the checkpoint can be staged there during phase B).
// A thread that updates one of the CTA's edge columns also writes the new
// value into the neighbouring CTA's ghost column, with an asynchronous
// store that completes on that CTA's mbarrier of the phase, so the stencils
// only ever read the CTA's own shared memory. The barriers between the
// phases are CTA barriers, followed, in the threads that read ghost columns,
// by a wait on the phase's mbarrier: neighbours synchronise point to point,
// without a cluster-wide barrier per step. The x-differences walk the
// thread's columns with a sliding window: one new shared-memory load per
// field per cell.
//
// Every cell is computed with the operations, in the order, of the fused
// step kernels (gb_stencil.h): forward traces and checkpoints are
// bit-identical to theirs. Each shot's kernel contribution goes to a
// per-shot buffer (from k_snap_interaction, directly from the in-pass
// accumulation, or from its shared-memory accumulators at the end of the
// pass) that is added to the kernels after the pass, in shot order.
#include <cooperative_groups.h>

#include <algorithm>

#include "gb_internal.h"
#include "gb_stencil.h"

namespace cg = cooperative_groups;

namespace gb {

// Threads per CTA for QM columns per thread: the model registers (2 per
// owned cell for SH, 3 for P-SV) plus about 56 (SH) or 64 (P-SV) registers of
// per-thread state must fit in the 65536-register file of the SM.
__host__ __device__ constexpr int cluster_threads_for(bool psv, int qm) {
    return psv ? (qm <= 4 ? 800 : qm <= 8 ? 736 : qm <= 10 ? 640 : qm <= 12 ? 608 : qm <= 16 ? 576 : qm <= 20 ? 512 : 480)
               : (qm <= 4 ? 1024 : qm <= 10 ? 896 : qm <= 12 ? 800 : qm <= 16 ? 736 : qm <= 20 ? 640 : 608);
}

int cluster_max_threads(bool psv, int qm) { return cluster_threads_for(psv, qm); }

// Shared-memory layout of the fields (see k_cluster): the row stride rs and
// the row shift dshift between the column blocks of consecutive thread
// groups. A warp whose lanes span two groups (rows a .. nz-1 of group g, rows
// 0 .. of group g+1, QM columns further right) hits 32 distinct banks when,
// with r = rs mod 32 odd, dshift = nz - QM * r^-1 (mod 32); among the odd rs
// in [cp+4, cp+35] the one with the smallest field size is taken. Without
// the shift (shift false, nz a multiple of 32, nz < 32 or a single group)
// rs = (cp+4) | 1 and the straddling warps see two-way conflicts.
void cluster_layout(ClusterGeom &g, int nz, bool shift) {
    const int cp = g.cols_per, G = g.G;
    g.rs = (cp + 4) | 1;
    g.dshift = 0;
    if (!shift || G < 2 || nz < 32 || nz % 32 == 0) return;
    long best = -1;
    for (int rs = cp + 4; rs < cp + 36; rs++) {
        if (rs % 2 == 0) continue;
        int rinv = 1;  // inverse of rs mod 32 (odd numbers are units)
        while ((rinv * (rs % 32)) % 32 != 1) rinv += 2;
        int d = ((nz - g.qmax * rinv) % 32 + 32) % 32;
        if (d > 16) d -= 32;
        const long size = (long)(nz + 4 + (G - 1) * std::abs(d)) * rs;
        if (best < 0 || size < best) {
            best = size;
            g.rs = rs;
            g.dshift = d;
        }
    }
}

// rows of one shared-memory field: nz + 4 plus the groups' row shifts
__host__ __device__ inline int cluster_field_rows(int nz, int G, int dshift) {
    return nz + 4 + (G - 1) * (dshift < 0 ? -dshift : dshift);
}

__device__ __forceinline__ uint32_t cl_mapa(uint32_t addr, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
    return r;
}
// Ghost pushes: an asynchronous store into a neighbour's shared memory that
// completes `bytes` on that CTA's mbarrier (cluster addresses).
__device__ __forceinline__ void cl_push(uint32_t addr, float v, uint32_t bar) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b32 [%0], %1, [%2];" ::"r"(addr),
                 "r"(__float_as_uint(v)), "r"(bar)
                 : "memory");
}
__device__ __forceinline__ void cl_mbar_init(uint32_t bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void cl_mbar_expect(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// Waits (acquire, cluster scope) for phase `parity` of the mbarrier, at most
// kClusterWaitIters tries; false when they ran out.
constexpr int kClusterWaitIters = 1 << 20;
__device__ __forceinline__ bool cl_mbar_wait(uint32_t bar, uint32_t parity) {
    for (int i = 0; i < kClusterWaitIters; i++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, "
            "p;\n}"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}
__device__ int g_cluster_wait_error;  // set when a ghost-column wait ran out of iterations

// 4-byte asynchronous copy global -> shared (completed by cp_async_wait_all)
__device__ __forceinline__ void cp_async4(float *dst, const float *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
// as cp_async4, zero-filling dst without reading when pred is false (src stays valid)
__device__ __forceinline__ void cp_async4_zf(float *dst, const float *src, bool pred) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
                 "l"(src), "r"(pred ? 4 : 0)
                 : "memory");
}

// Shared-memory field order. P-SV: vx vz ux uz sxx szz sxz; SH: vy uy sxy szy.
// Each field is stored by rows (x fastest) with two zero pad rows above and
// below it: field f, row j (-2 .. nz+1), local column c (-2 .. cp+1) of
// thread group h (c / QM; the ghost columns go with the group beside them) at
// sm[f*fs + (j + 2 + sigma_h)*rs + c + 2], sigma_h = sigma_0 + h*dshift >= 0,
// fs = cluster_field_rows(nz, G, dshift)*rs. The row stride rs >= cp + 4 is
// odd, so that a warp of consecutive rows of one group hits 32 distinct
// banks, and a thread's consecutive columns are immediate offsets from one
// address; the row shift makes warps that span two groups conflict-free too
// (cluster_layout). Reads of the two columns on either side of a thread's
// block add the row offset between the groups.
//
// cp is a multiple of QM and every thread updates QM columns; in the last CTA
// the columns past the grid are updated too (never read by a grid column:
// the x differences of the last two grid columns are masked off).
template <bool PSV, bool ADJ, int QM>
__global__ void __launch_bounds__(cluster_threads_for(PSV, QM), 1)
    k_cluster(const Slot *__restrict__ slots, ClusterGeom g, float *__restrict__ kpart, float *__restrict__ snap) {
    constexpr int NV = PSV ? 2 : 1;
    constexpr int NF = PSV ? 7 : 4;
    constexpr int NSF = NF - 2 * NV;             // stress fields
    constexpr int FV = 0, FU = NV, FS = 2 * NV;  // first velocity, displacement, stress field
    constexpr int NWA = PSV ? 2 : 1;             // stresses differentiated in x in phase A
    extern __shared__ float sm[];
    cg::cluster_group cl = cg::this_cluster();
    const int R = g.R;
    const int rank = (int)cl.block_rank();
    const int slot = blockIdx.x / R;
    const Slot &S = slots[slot];
    if (!S.active) return;  // uniform over the cluster: one slot per cluster
    const int nx = g.nx, nz = g.nz, nt = g.nt, cp = g.cols_per;
    const size_t ncell = (size_t)nx * nz;
    const int x0 = rank * cp;
    const int ncols = min(cp, nx - x0);  // grid columns of this CTA, >= 2
    const int rs = g.rs, G = g.G, dsh = g.dshift;
    const int fs = cluster_field_rows(nz, G, dsh) * rs;  // one field
    const int sig0 = dsh < 0 ? -(G - 1) * dsh : 0;        // row shift of group 0
    const int t = threadIdx.x, j = t % nz, grp = t / nz;
    const int cb = grp * QM;                     // first local column of this thread
    const int nq = max(0, min(QM, ncols - cb));  // of which grid columns
    const int i0 = x0 + cb;                      // its global column

    // receiver (or adjoint source) of each owned cell, through a map built in
    // the still unused field memory; the ids of the thread's receivers go to
    // rtab[rbase ...] in column order
    float *s_ax = sm + NF * fs;                          // ax of columns -2 .. cp+1
    int *rtab = reinterpret_cast<int *>(s_ax + cp + 4);  // g.nrec_cta entries
    // per receiver entry NV values: the next step's adjoint source (adjoint)
    // or, as an int, the receiver cell's field-0 offset in shared memory
    // (forward); then NV values of the next step's forward source
    float *rbuf = reinterpret_cast<float *>(rtab + g.nrec_cta);
    float *sbuf = rbuf + (size_t)g.nrec_cta * NV;
    // adjoint with g.stage: the checkpoint the next kernel accumulation reads,
    // NV displacement fields over columns -1 .. cp+1 and NV velocity fields
    // over columns 0 .. cp-1, stored by columns ([field][column][row])
    float *ckst = sbuf + NV;
    // adjoint with g.kacc: the shot's kernels of the CTA's columns (P-SV lambda,
    // mu, rho; SH mu, rho), [kernel][column][row], zero at the start of the pass
    constexpr int NKA = PSV ? 3 : 2;
    float *kacc = ckst + (g.stage ? (size_t)NV * (2 * cp + 3) * nz : 0);
    __shared__ int s_count;
    // ghost columns of phase A (velocity; displacement too for an in-pass
    // accumulation) and of phase B (stresses) landed from the neighbours
    __shared__ __align__(8) unsigned long long s_gbar[2];
    __shared__ int s_cdead;  // a ghost wait ran out: no mbarrier operation after it
    const uint32_t gbar = (uint32_t)__cvta_generic_to_shared(s_gbar);
    int *map = reinterpret_cast<int *>(sm);
    for (int e = t; e < cp * nz; e += blockDim.x) map[e] = -1;
    if (t == 0) {
        s_count = 0;
        s_cdead = 0;
        cl_mbar_init(gbar);
        cl_mbar_init(gbar + 8u);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    for (int r = t; r < S.npts; r += blockDim.x) {
        const int i = S.pts_i[r] - x0, jj = S.pts_j[r];
        if (i >= 0 && i < ncols && jj >= 0 && jj < nz) map[i * nz + jj] = r;  // cells are distinct
    }
    __syncthreads();
    unsigned rmask = 0, xs_mask = 0, xv_mask = 0;
#pragma unroll
    for (int q = 0; q < QM; q++) {
        if (q < nq && map[(cb + q) * nz + j] >= 0) rmask |= 1u << q;
        const int i = i0 + q;
        if (i >= 2 && i < nx - 2) xs_mask |= 1u << q;
        if (i >= 1 && i < nx - 2) xv_mask |= 1u << q;
    }
    const int rbase = rmask ? atomicAdd(&s_count, __popc(rmask)) : 0;
    if (rbase + __popc(rmask) > g.nrec_cta) rmask = 0;  // not reached: the host sizes the table
    {
        int n = 0;
#pragma unroll
        for (int q = 0; q < QM; q++)
            if ((rmask >> q) & 1) {
                rtab[rbase + n] = map[(cb + q) * nz + j];
                // forward: the cell's field-0 offset in shared memory, from
                // which the thread that writes the sample out reads it
                if (!ADJ) reinterpret_cast<int *>(rbuf)[rbase + n] = (j + 2 + sig0 + grp * dsh) * rs + cb + q + 2;
                n++;
            }
    }
    int srcq = -1;  // owned column of the forward source
    if (!ADJ && S.src_trace >= 0 && S.src_j == j && S.src_i - i0 >= 0 && S.src_i - i0 < nq) srcq = S.src_i - i0;
    // the forward source's cell (adjoint sources: see the warp flag below)
    const unsigned spmask = srcq >= 0 ? 1u << srcq : 0u;
    __syncthreads();
    for (int e = t; e < NF * fs; e += blockDim.x) sm[e] = 0.f;
    if (ADJ && g.kacc)
        for (int e = t; e < NKA * cp * nz; e += blockDim.x) kacc[e] = 0.f;
    for (int c = t - 2; c < cp + 2; c += blockDim.x) s_ax[c + 2] = __ldg(S.ax + min(max(x0 + c, 0), nx - 1));

    // model of the owned cells
    float p_ri[QM], p_mu[QM], p_la[PSV ? QM : 1];
    const float azj = __ldg(S.az + j);
#pragma unroll
    for (int q = 0; q < QM; q++) {
        const int i = min(i0 + q, nx - 1);  // columns past the grid use the last one's
        const size_t k = (size_t)i * nz + j;
        p_ri[q] = __ldg(S.rinv + k);
        p_mu[q] = __ldg(S.mu + k);
        if (PSV) p_la[q] = __ldg(S.lambda + k);
    }

    const float dt = g.dt, c9x = g.c9x, c24x = g.c24x, c9z = g.c9z, c24z = g.c24z;
    const bool zS = j >= 2 && j < nz - 2, zV = j >= 1 && j < nz - 2;
    const int base_ck = (PSV && S.sh[0] != nullptr) ? 2 : 0;  // checkpoint field offset of this system
    float *const P = sm + (j + 2 + sig0 + grp * dsh) * rs + cb + 2;  // field 0, row j, column cb
    // neighbours' shared memory: cluster address of their field 0, row j,
    // column -2, in the rows of their last group (left neighbour, whose
    // columns cp, cp+1 this CTA writes) or first group (right neighbour)
    const uint32_t lf =
        rank > 0 ? cl_mapa((uint32_t)__cvta_generic_to_shared(sm + (j + 2 + sig0 + (G - 1) * dsh) * rs), rank - 1)
                 : 0u;
    const uint32_t rt =
        rank < R - 1 ? cl_mapa((uint32_t)__cvta_generic_to_shared(sm + (j + 2 + sig0) * rs), rank + 1) : 0u;
    // the thread owning columns 0, 1 sends them left; the one owning columns
    // cp-2, cp-1 sends them right (a CTA with a right neighbour holds cp columns)
    const bool edge_l = rank > 0 && grp == 0, edge_r = rank < R - 1 && cb + QM == cp;
    // Ghost exchange. The edge threads push their new values into the
    // neighbours' ghost columns with asynchronous stores that complete bytes
    // on the receiving CTA's mbarrier of the phase (s_gbar[0]: phase A,
    // s_gbar[1]: phase B); thread 0 arms it with the bytes this CTA receives
    // (left neighbour's last column / right neighbour's first two in phase A,
    // the left's last two / the right's first in phase B), and after the
    // phase's CTA barrier the threads that read ghost columns (the edge
    // groups) wait for it. No cluster-wide barrier per step: a neighbour can
    // overwrite a ghost column only after it received this CTA's pushes of
    // the phase that follows the reads of that column, and a thread pushes
    // a column only after reading its own ghosts for it. (A cluster barrier
    // with a cluster-scope release by every thread cost about a tenth of the
    // step: the release waits for the thread's outstanding global stores.)
    // the neighbours' mbarriers (formed where an edge thread pushes: held
    // through the loop they would take registers from every thread)
    auto gbar_l = [&]() { return cl_mapa(gbar, rank - 1); };
    auto gbar_r = [&]() { return cl_mapa(gbar, rank + 1); };
    auto ghost_expect = [&](int b) {
        if (t == 0 && !*(volatile int *)&s_cdead) {
            const uint32_t has_l = rank > 0 ? 1u : 0u, has_r = rank < R - 1 ? 1u : 0u;
            const uint32_t bytes = b ? 4u * NSF * (uint32_t)nz * (2u * has_l + has_r)
                                     : 4u * NV * ((ADJ && !snap) ? 2u : 1u) * (uint32_t)nz * (has_l + 2u * has_r);
            cl_mbar_expect(gbar + 8u * b, bytes);
        }
    };
    auto ghost_wait = [&](bool reader, int b, int it) {
        if (reader && !*(volatile int *)&s_cdead && !cl_mbar_wait(gbar + 8u * b, (uint32_t)(it & 1))) {
            s_cdead = 1;
            atomicOr(&g_cluster_wait_error, 1);
        }
    };

    // Steps are counted as it = blk * sfe + ph (sfe > 0), kept by increments
    // instead of an integer division per step. Checkpoint index written after
    // the step with counters (ph, blk) (-1: none).
    const int sfe = S.sfe > 0 ? S.sfe : 1;
    auto ckpt_at = [&](int ph, int blk) -> int {
        if (ADJ || !S.ckpt || S.sfe <= 0 || ph != sfe - 1) return -1;
        return S.nsfe - (blk + 1);
    };
    // owned grid cells of NV fields from field f0 to checkpoint field q0
    auto store_ckpt = [&](int isfe, int f0, int q0) {
        float *ck = static_cast<float *>(S.ckpt) + ((size_t)isfe * S.nf + base_ck + q0) * ncell + (size_t)i0 * nz + j;
#pragma unroll 1
        for (int q = 0; q < nq; q++)
#pragma unroll
            for (int f = 0; f < NV; f++) ck[f * ncell + (size_t)q * nz] = P[(f0 + f) * fs + q];
    };
    auto inj_of = [&](int f) -> const float * { return PSV ? (f == 0 ? S.inj_x : S.inj_z) : S.inj_y; };
    // injection of step `step` into shared memory, read after cp_async_wait_all
    auto prefetch = [&](int step) {
        if (step >= nt) return;
        if (!ADJ && srcq >= 0) {
#pragma unroll
            for (int f = 0; f < NV; f++) cp_async4(sbuf + f, inj_of(f) + (size_t)S.src_trace * nt + step);
        }
        // adjoint sources: entry e by thread e (not by the entry's owner, whose
        // row may own every surface receiver of its columns); the issuing
        // threads wait for their copies before the barrier that precedes the
        // owners' reads
        if (ADJ) {
            const int ncr = min(*(volatile int *)&s_count, g.nrec_cta);
#pragma unroll 1
            for (int e = t; e < ncr; e += blockDim.x) {
                const size_t ks = (size_t)rtab[e] * nt + step;
#pragma unroll
                for (int f = 0; f < NV; f++) cp_async4(rbuf + e * NV + f, inj_of(f) + ks);
            }
        }
    };
    // copies checkpoint isfe into ckst (this thread: row j of the columns
    // grp, grp + G, ...); completed by cp_async_wait_all
    auto stage_ckpt = [&](int isfe) {
        const float *ckb = static_cast<const float *>(S.ckpt) + ((size_t)isfe * S.nf + base_ck) * ncell + j;
#pragma unroll
        for (int f = 0; f < NV; f++) {
            for (int col = grp; col < cp + 3; col += g.G) {
                const int gc = x0 - 1 + col;
                const bool ok = gc >= 0 && gc < nx;
                cp_async4_zf(ckst + ((size_t)f * (cp + 3) + col) * nz + j, ckb + (size_t)f * ncell + (size_t)(ok ? gc : 0) * nz,
                             ok);
            }
            for (int col = grp; col < cp; col += g.G) {
                const int gc = x0 + col;
                const bool ok = gc < nx;
                cp_async4_zf(ckst + ((size_t)NV * (cp + 3) + (size_t)f * cp + col) * nz + j,
                             ckb + (size_t)(NV + f) * ncell + (size_t)(ok ? gc : 0) * nz, ok);
            }
        }
    };
    cl.sync();
    if (ckpt_at(0, 0) >= 0) store_ckpt(ckpt_at(0, 0), FU, 0);  // displacement before step 0
    prefetch(0);
    if (ADJ) {
        cp_async_wait_all();
        __syncthreads();
    }

    unsigned rb = (unsigned)rbase, sq = (unsigned)srcq, qn = (unsigned)nq;
    // per-thread flags: 1 / 2 pushes to the left / right neighbour, 4 / 8 z
    // parts of the stress divergence / velocity gradient, 16 / 32 a thread
    // group to the left / right, 64 record displacement, 128 push displacement
    // ghosts (in-pass accumulation), 256 the warp holds receivers
    unsigned fl = (edge_l ? 1u : 0u) | (edge_r ? 2u : 0u) | (zS ? 4u : 0u) | (zV ? 8u : 0u) | (grp > 0 ? 16u : 0u) |
                  (grp < G - 1 ? 32u : 0u) | (S.record_u ? 64u : 0u) | ((ADJ && !snap) ? 128u : 0u) |
                  (__any_sync(__activemask(), rmask != 0u) ? 256u : 0u);
    unsigned spm = spmask;
    int ph = 0, blk = 0;  // it = blk * sfe + ph
    for (int it = 0; it < nt; it++) {
        // The per-column conditions below are invariant over the time loop;
        // hoisting them out of it would hold registers per owned column.
        // Redefining their inputs each step keeps them local.
        asm volatile("" : "+r"(xs_mask), "+r"(xv_mask), "+r"(rmask), "+r"(rb));
        asm volatile("" : "+r"(sq), "+r"(qn), "+r"(fl), "+r"(spm));
        const int nq = (int)qn, srcq = (int)sq, rbase = (int)rb;
        const bool eL = fl & 1u, eR = fl & 2u, zs = fl & 4u, zv = fl & 8u;
        // offsets (elements) from P's row to row j of the columns left of cb
        // (group grp-1) and right of cb+QM-1 (group grp+1); ghost columns
        // share the row shift of the group beside them
        const int dl = (fl & 16u) ? -g.dshift * g.rs : 0, dr = (fl & 32u) ? g.dshift * g.rs : 0;
        if (spm) cp_async_wait_all();  // this step's injection
        ghost_expect(0);
        // ---- phase A: divergence, sources, velocity, displacement
        {
            float wa[NWA][4];  // x-window: columns c-2, c-1, c, c+1
#pragma unroll
            for (int w = 0; w < NWA; w++) {
                const float *p = P + (FS + 2 * w) * fs;
                wa[w][0] = p[dl - 2];
                wa[w][1] = p[dl - 1];
                wa[w][2] = p[0];
            }
#pragma unroll
            for (int q = 0; q < QM; q++) {
#pragma unroll
                for (int w = 0; w < NWA; w++) wa[w][3] = P[(FS + 2 * w) * fs + q + 1 + (q == QM - 1 ? dr : 0)];
                const bool xS = (xs_mask >> q) & 1;
                // ds = 0; ds = (x part) where xS; ds += (z part) where zS  (gb_stencil.h order)
                float ds[NV];
                if (PSV) {
                    // sxx (x), sxz (x and z), szz (z)
                    const float *c0 = P + (FS + 2) * fs + q, *b0 = P + (FS + 1) * fs + q;
                    const float ax_ = st_dminus(wa[0][2], wa[0][1], wa[0][3], wa[0][0], c9x, c24x);
                    const float az_ = st_dminus(wa[NWA - 1][2], wa[NWA - 1][1], wa[NWA - 1][3], wa[NWA - 1][0], c9x, c24x);
                    const float bx_ = st_dminus(wa[NWA - 1][2], c0[-rs], c0[rs], c0[-2 * rs], c9z, c24z);
                    const float bz_ = st_dminus(b0[0], b0[-rs], b0[rs], b0[-2 * rs], c9z, c24z);
                    const float dsx = xS ? ax_ : 0.f, dsz = xS ? az_ : 0.f;
                    ds[0] = zs ? dsx + bx_ : dsx;
                    ds[NV - 1] = zs ? dsz + bz_ : dsz;
                } else {
                    const float *b0 = P + (FS + 1) * fs + q;
                    const float ax_ = st_dminus(wa[0][2], wa[0][1], wa[0][3], wa[0][0], c9x, c24x);
                    const float bz_ = st_dminus(b0[0], b0[-rs], b0[rs], b0[-2 * rs], c9z, c24z);
                    const float dsy = xS ? ax_ : 0.f;
                    ds[0] = zs ? dsy + bz_ : dsy;
                }
                // forward source: a branch around its one cell
                if (!ADJ && ((spm >> q) & 1) && q == srcq) {
#pragma unroll
                    for (int f = 0; f < NV; f++) ds[f] += sbuf[f];
                }
                // adjoint sources: in a warp that holds receivers (a uniform
                // branch) every lane reads its entry (entry 0 where it has
                // none: in bounds) and keeps the sum where the cell is one
                if (ADJ && (fl & 256u)) {
                    const bool hit = (rmask >> q) & 1;
                    const int e = rbase + __popc(rmask & ((1u << q) - 1u));
#pragma unroll
                    for (int f = 0; f < NV; f++) {
                        const float a = rbuf[e * NV + f];
                        ds[f] = hit ? ds[f] + a : ds[f];
                    }
                }
                const float ab = s_ax[cb + q + 2] * azj;
                float vn[NV], un[NV];
#pragma unroll
                for (int f = 0; f < NV; f++) {
                    float *pv = P + (FV + f) * fs + q, *pu = P + (FU + f) * fs + q;
                    vn[f] = st_velocity(ab, dt, ds[f], p_ri[q], *pv);
                    un[f] = st_displacement(*pu, vn[f], dt);
                    *pv = vn[f];
                    *pu = un[f];
                }
                // ghosts: the left neighbour reads columns 0, 1, the right one column cp-1
                // (displacement too for an in-pass kernel accumulation)
                if (q < 2 && eL) {
                    const uint32_t a = lf + 4u * (uint32_t)(cp + q + 2);
#pragma unroll
                    for (int f = 0; f < NV; f++) {
                        cl_push(a + 4u * (uint32_t)((FV + f) * fs), vn[f], gbar_l());
                        if (ADJ && (fl & 128u)) cl_push(a + 4u * (uint32_t)((FU + f) * fs), un[f], gbar_l());
                    }
                }
                if (q == QM - 1 && eR) {
                    const uint32_t a = rt + 4u;
#pragma unroll
                    for (int f = 0; f < NV; f++) {
                        cl_push(a + 4u * (uint32_t)((FV + f) * fs), vn[f], gbar_r());
                        if (ADJ && (fl & 128u)) cl_push(a + 4u * (uint32_t)((FU + f) * fs), un[f], gbar_r());
                    }
                }
#pragma unroll
                for (int w = 0; w < NWA; w++) {
                    wa[w][0] = wa[w][1];
                    wa[w][1] = wa[w][2];
                    wa[w][2] = wa[w][3];
                }
            }
        }
        __syncthreads();
        ghost_wait(eL || eR, 0, it);
        // Global traffic of the step, issued here so that phase B's work hides
        // its latency before the next barrier: recorded samples, checkpoints
        // of velocity (after this step's update) and displacement (before the
        // next step; phase B changes neither), the next step's injection.
        if (!ADJ) {
            // recorded samples, u when record_u else v (solver/fdm.h:181-196):
            // entry e by thread e, read from the cell's place in shared memory
            // (updated in phase A, before the barrier above; phase B leaves it)
            const int ncr = min(*(volatile int *)&s_count, g.nrec_cta);
            const int *roff = reinterpret_cast<const int *>(rbuf);
            const int fo = ((fl & 64u) ? FU : FV) * fs;
#pragma unroll 1
            for (int e = t; e < ncr; e += blockDim.x) {
                const size_t kr = (size_t)rtab[e] * nt + it;
                const float *pc = sm + roff[e] + fo;
                if (PSV) {
                    S.out_x[kr] = pc[0];
                    S.out_z[kr] = pc[(NV - 1) * fs];
                } else {
                    S.out_y[kr] = pc[0];
                }
            }
            const int isfe = ckpt_at(ph, blk);
            if (isfe >= 0) store_ckpt(isfe, FV, NV);
            const bool wrap = ph + 1 == sfe;
            const int isfe_n = it + 1 < nt ? ckpt_at(wrap ? 0 : ph + 1, wrap ? blk + 1 : blk) : -1;
            if (isfe_n >= 0) store_ckpt(isfe_n, FU, 0);
        }
        prefetch(it + 1);
        if (ADJ && g.stage && S.ckpt && S.sfe > 0 && ph == 0 && blk < S.nsfe) stage_ckpt(blk);
        ghost_expect(1);
        // ---- phase B: velocity gradients and stress update
        {
            float wb[NV][4];  // x-window: columns c-1, c, c+1, c+2
#pragma unroll
            for (int f = 0; f < NV; f++) {
                const float *p = P + (FV + f) * fs;
                wb[f][0] = p[dl - 1];
                wb[f][1] = p[0];
                wb[f][2] = p[1];
            }
#pragma unroll
            for (int q = 0; q < QM; q++) {
                const bool xV = (xv_mask >> q) & 1;
                float dxv[NV], dzv[NV];
#pragma unroll
                for (int f = 0; f < NV; f++) {
                    const float *v0 = P + (FV + f) * fs + q;
                    wb[f][3] = v0[2 + (q >= QM - 2 ? dr : 0)];
                    const float gx = st_dplus(wb[f][2], wb[f][1], wb[f][3], wb[f][0], c9x, c24x);
                    const float gz = st_dplus(v0[rs], wb[f][1], v0[2 * rs], v0[-rs], c9z, c24z);
                    dxv[f] = xV ? gx : 0.f;
                    dzv[f] = zv ? gz : 0.f;
                }
                float *ps = P + FS * fs + q;
                float sv[NSF];
#pragma unroll
                for (int f = 0; f < NSF; f++) sv[f] = ps[f * fs];
                if (PSV)
                    st_stress_psv(sv[0], sv[1], sv[NSF - 1], p_la[q], p_mu[q], dt, dxv[0], dzv[0], dxv[NV - 1],
                                  dzv[NV - 1]);
                else
                    st_stress_sh(sv[0], sv[1], p_mu[q], dt, dxv[0], dzv[0]);
#pragma unroll
                for (int f = 0; f < NSF; f++) ps[f * fs] = sv[f];
                // ghosts: the left neighbour reads column 0, the right one columns cp-2, cp-1
                if (q == 0 && eL) {
                    const uint32_t a = lf + 4u * (uint32_t)(cp + 2);
#pragma unroll
                    for (int f = 0; f < NSF; f++) cl_push(a + 4u * (uint32_t)((FS + f) * fs), sv[f], gbar_l() + 8u);
                }
                if (q >= QM - 2 && eR) {
                    const uint32_t a = rt + 4u * (uint32_t)(q - QM + 2);
#pragma unroll
                    for (int f = 0; f < NSF; f++) cl_push(a + 4u * (uint32_t)((FS + f) * fs), sv[f], gbar_r() + 8u);
                }
#pragma unroll
                for (int f = 0; f < NV; f++) {
                    wb[f][0] = wb[f][1];
                    wb[f][1] = wb[f][2];
                    wb[f][2] = wb[f][3];
                }
            }
        }
        if (ADJ) cp_async_wait_all();  // this thread's copies of the next step's adjoint sources
        __syncthreads();
        ghost_wait(eL || eR, 1, it);
        // ---- adjoint with snap: the adjoint state of the owned grid cells at
        // each accumulation step, [slot][step][u fields, v fields][cell], for
        // the kernel accumulation after the pass (k_snap_interaction). Own
        // cells only, read before this thread's next write: no barrier.
        if (ADJ && snap && S.ckpt && S.sfe > 0 && ph == 0 && blk < S.nsfe) {
            float *sp = snap + ((size_t)slot * S.nsfe + blk) * (2 * NV) * ncell + (size_t)i0 * nz + j;
#pragma unroll 1
            for (int q = 0; q < nq; q++)
#pragma unroll
                for (int f = 0; f < NV; f++) {
                    sp[(size_t)f * ncell + (size_t)q * nz] = P[(FU + f) * fs + q];
                    sp[(size_t)(NV + f) * ncell + (size_t)q * nz] = P[(FV + f) * fs + q];
                }
        }
        // ---- adjoint: kernel accumulation every sfe steps (solver/fdm.h:583-606)
        // FP32 checkpoints (the only precision this path takes), copied into
        // shared memory at the start of phase B when g.stage, else read from
        // HBM: the x-differences walk the thread's columns with a window over
        // the checkpointed displacement, so each column adds one load per
        // field; rows and columns are clamped to the grid (HBM) or zero-filled
        // (staged), and a cell's differences are masked where the reference
        // skips them. The shared accumulators (g.kacc) or the per-shot kernel
        // buffer take the `-=`.
        if (ADJ && !snap && S.ckpt && S.sfe > 0 && ph == 0 && blk < S.nsfe) {
            const int isfe_a = blk;
            const float ndt = (float)S.sfe * dt;
            const float *ckb = static_cast<const float *>(S.ckpt) + ((size_t)isfe_a * S.nf + base_ck) * ncell;
            const size_t kc = (size_t)i0 * nz + j;  // this thread's first cell
            const int zm = zv ? -1 : 0, zp = zv ? 1 : 0, zp2 = zv ? 2 : 0;
            auto colk = [&](int q) -> size_t { return (size_t)min(max(i0 + q, 0), nx - 1) * nz + j; };
            float cw[NV][4];  // checkpointed displacement f at columns c-1, c, c+1, c+2
            if (g.stage) {
                cp_async_wait_all();
                __syncthreads();
            }
#pragma unroll
            for (int f = 0; f < NV; f++) {
                if (g.stage) {
                    const float *us = ckst + ((size_t)f * (cp + 3) + cb + 1) * nz + j;
                    cw[f][0] = us[-(int)nz];
                    cw[f][1] = us[0];
                    cw[f][2] = us[nz];
                } else {
                    const float *u = ckb + (size_t)f * ncell;
                    cw[f][0] = __ldg(u + colk(-1));
                    cw[f][1] = __ldg(u + colk(0));
                    cw[f][2] = __ldg(u + colk(1));
                }
            }
            float *kl = kpart + ((size_t)slot * 3 + 0) * ncell + kc;
            float *km = kpart + ((size_t)slot * 3 + 1) * ncell + kc;
            float *kr = kpart + ((size_t)slot * 3 + 2) * ncell + kc;
            // or the shared accumulators of the thread's first cell
            const bool kin = g.kacc != 0;
            float *al = kacc + (size_t)cb * nz + j;
            float *am = al + (PSV ? (size_t)cp * nz : 0);
            float *ar = am + (size_t)cp * nz;
            const bool staged = g.stage != 0;  // staging copies waited for above
            // staged checkpoint: displacement f at local column c + o (o >= -1), velocity f at c
            const float *su = ckst + (size_t)(cb + 1) * nz + j;
            const float *sv = ckst + ((size_t)NV * (cp + 3) + cb) * nz + j;
            // The kernel buffer is read one column ahead of its update: the
            // compiler cannot tell that columns q and q+1 are distinct
            // addresses, so an in-place `-=` would wait for each store before
            // the next load.
            float nk[3] = {0.f, 0.f, 0.f};  // kernel buffer (lambda, mu, rho) at the next column
            if (nq > 0 && !kin) {
                if (PSV) nk[0] = kl[0];
                nk[1] = km[0];
                nk[2] = kr[0];
            }
#pragma unroll 2
            for (int q = 0; q < QM; q++) {
                if (q < nq) {
                    const size_t o = (size_t)q * nz;
                    float ok[3] = {nk[0], nk[1], nk[2]};
                    if (kin) {
                        ok[0] = PSV ? al[o] : 0.f;
                        ok[1] = am[o];
                        ok[2] = ar[o];
                    } else if (q + 1 < nq) {
                        const size_t o1 = (size_t)(q + 1) * nz;
                        if (PSV) nk[0] = kl[o1];
                        nk[1] = km[o1];
                        nk[2] = kr[o1];
                    }
                    const bool gx = (xv_mask >> q) & 1;
                    float ux[NV], uzz[NV], fx[NV], fz[NV], vf[NV];
#pragma unroll
                    for (int f = 0; f < NV; f++) {
                        const float *u = ckb + (size_t)f * ncell;
                        const float *uc = u + kc + (size_t)q * nz;
                        const float *us = su + ((size_t)f * (cp + 3) + q) * nz;
                        float z1, z2, zm1;
                        if (staged) {
                            cw[f][3] = us[2 * nz];
                            vf[f] = sv[((size_t)f * cp + q) * nz];
                            z1 = us[zp];
                            z2 = us[zp2];
                            zm1 = us[zm];
                        } else {
                            cw[f][3] = __ldg(u + colk(q + 2));
                            vf[f] = __ldg(uc + (size_t)NV * ncell);  // checkpointed velocity f
                            z1 = __ldg(uc + zp);
                            z2 = __ldg(uc + zp2);
                            zm1 = __ldg(uc + zm);
                        }
                        const float *u0 = P + (FU + f) * fs + q;
                        const float um1 = u0[(q == 0 ? dl : 0) - 1];
                        const float up1 = u0[(q == QM - 1 ? dr : 0) + 1];
                        const float up2 = u0[(q >= QM - 2 ? dr : 0) + 2];
                        ux[f] = gx ? st_dplus(up1, u0[0], up2, um1, c9x, c24x) : 0.f;
                        uzz[f] = zv ? st_dplus(u0[rs], u0[0], u0[2 * rs], u0[-rs], c9z, c24z) : 0.f;
                        fx[f] = gx ? st_dplus(cw[f][2], cw[f][1], cw[f][3], cw[f][0], c9x, c24x) : 0.f;
                        fz[f] = zv ? st_dplus(z1, cw[f][1], z2, zm1, c9z, c24z) : 0.f;
                        cw[f][0] = cw[f][1];
                        cw[f][1] = cw[f][2];
                        cw[f][2] = cw[f][3];
                    }
                    const float *v0 = P + FV * fs + q;
                    float nl = 0.f, nm, nr;
                    if (PSV) {
                        const float dvxdx = ux[0], dvxdz = uzz[0], dvzdx = ux[NV - 1], dvzdz = uzz[NV - 1];
                        const float fxdx = fx[0], fxdz = fz[0], fzdx = fx[NV - 1], fzdz = fz[NV - 1];
                        nr = st_krho_psv(ok[2], vf[0], v0[0], vf[NV - 1], v0[fs], ndt);
                        nm = st_kmu_psv(ok[1], dvxdx, dvxdz, dvzdx, dvzdz, fxdx, fxdz, fzdx, fzdz, ndt);
                        nl = st_klambda_psv(ok[0], dvxdx, dvzdz, fxdx, fzdz, ndt);
                    } else {
                        nr = st_krho_sh(ok[2], vf[0], v0[0], ndt);
                        nm = st_kmu_sh(ok[1], ux[0], fx[0], uzz[0], fz[0], ndt);
                    }
                    if (kin) {
                        ar[o] = nr;
                        am[o] = nm;
                        if (PSV) al[o] = nl;
                    } else {
                        kr[o] = nr;
                        km[o] = nm;
                        if (PSV) kl[o] = nl;
                    }
                }
            }
            cl.sync();
        }
        if (++ph == sfe) {
            ph = 0;
            blk++;
        }
    }
    // every push into this CTA has landed (the waits above); the barrier
    // keeps each CTA's shared memory until the whole cluster is done
    cl.sync();
    // the shared accumulators (written by this thread only) go to the shot's buffer
    if (ADJ && g.kacc) {
        const size_t kc = (size_t)i0 * nz + j;
#pragma unroll 1
        for (int q = 0; q < nq; q++)
#pragma unroll
            for (int k = 0; k < NKA; k++)
                kpart[((size_t)slot * 3 + (PSV ? k : k + 1)) * ncell + kc + (size_t)q * nz] = kacc[((size_t)k * cp + cb + q) * nz + j];
    }
}

// Kernel accumulation of a cluster-resident adjoint pass from the adjoint
// state it stored at every accumulation step (snap) and the forward
// checkpoints (solver/fdm.h:583-606): for each cell, the differences and the
// accumulation helpers (gb_stencil.h) of the in-pass accumulation, over the
// accumulation steps in step order, so the per-shot kernels are
// bit-identical to it. A thread owns one row of kSnapCols consecutive
// columns of one shot (blockIdx.y = slot; consecutive threads take
// consecutive rows, so every load is coalesced): per step it loads the
// displacement of columns c0-1 .. c0+kSnapCols+1 once into an x-window (the
// x-differences of all its cells) plus each cell's z-neighbours and
// velocities, instead of four loads per x-difference. Where the reference
// skips a difference the neighbour offsets are 0 and the window's columns
// are clamped to the grid, so no read leaves it; such differences are masked.
constexpr int kSnapCols = 4;
template <bool PSV>
__global__ void k_snap_interaction(const Slot *__restrict__ slots, const float *__restrict__ snap, ClusterGeom g,
                                   float *__restrict__ kpart) {
    constexpr int NV = PSV ? 2 : 1, C = kSnapCols;
    const int slot = blockIdx.y;
    const Slot &S = slots[slot];
    if (!S.active || !S.ckpt || S.sfe <= 0) return;
    const int nx = g.nx, nz = g.nz;
    const size_t ncell = (size_t)nx * nz;
    const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned strip = tid / (unsigned)nz, j = tid - strip * (unsigned)nz;
    const int c0 = (int)strip * C;  // first column of this thread
    if (c0 >= nx) return;
    const int nc = min(C, nx - c0);
    const bool zv = j >= 1 && (int)j < nz - 2;
    const long oz = zv ? 1 : 0;
    // window column w (0 .. C+2) is grid column c0 - 1 + w, clamped
    long wcol[C + 3];
#pragma unroll
    for (int w = 0; w < C + 3; w++) wcol[w] = (long)min(max(c0 - 1 + w, 0), nx - 1) * nz + j;
    const float ndt = (float)S.sfe * g.dt, c9x = g.c9x, c24x = g.c24x, c9z = g.c9z, c24z = g.c24z;
    const int base_ck = (PSV && S.sh[0] != nullptr) ? 2 : 0;
    const int nacc = min(S.nsfe, (g.nt - 1) / S.sfe + 1);
    float kl[C], km[C], kr[C];
#pragma unroll
    for (int c = 0; c < C; c++) kl[c] = km[c] = kr[c] = 0.f;
#pragma unroll 1
    for (int a = 0; a < nacc; a++) {
        const float *ua = snap + ((size_t)slot * S.nsfe + a) * (2 * NV) * ncell;
        const float *uf = static_cast<const float *>(S.ckpt) + ((size_t)a * S.nf + base_ck) * ncell;
        float ux[NV][C], uzz[NV][C], fx[NV][C], fz[NV][C], vf[NV][C], va[NV][C];
#pragma unroll
        for (int f = 0; f < NV; f++) {
            const float *u0 = ua + (size_t)f * ncell, *w0 = uf + (size_t)f * ncell;
            float wa_[C + 3], wf_[C + 3];
#pragma unroll
            for (int w = 0; w < C + 3; w++) {
                wa_[w] = u0[wcol[w]];
                wf_[w] = __ldg(w0 + wcol[w]);
            }
#pragma unroll
            for (int c = 0; c < C; c++) {
                const int i = c0 + c;
                const bool gx = i >= 1 && i < nx - 2;
                const long k = wcol[c + 1];  // this cell
                // (a cell whose x-difference is masked may see clamped
                // copies in the window: the value is discarded)
                ux[f][c] = gx ? st_dplus(wa_[c + 2], wa_[c + 1], wa_[c + 3], wa_[c], c9x, c24x) : 0.f;
                fx[f][c] = gx ? st_dplus(wf_[c + 2], wf_[c + 1], wf_[c + 3], wf_[c], c9x, c24x) : 0.f;
                const float a0 = wa_[c + 1], b0 = wf_[c + 1];
                uzz[f][c] = zv ? st_dplus(u0[k + oz], a0, u0[k + 2 * oz], u0[k - oz], c9z, c24z) : 0.f;
                fz[f][c] = zv ? st_dplus(__ldg(w0 + k + oz), b0, __ldg(w0 + k + 2 * oz), __ldg(w0 + k - oz), c9z, c24z)
                              : 0.f;
                vf[f][c] = __ldg(uf + (size_t)(NV + f) * ncell + k);
                va[f][c] = ua[(size_t)(NV + f) * ncell + k];
            }
        }
#pragma unroll
        for (int c = 0; c < C; c++) {
            if (PSV) {
                const float dvxdx = ux[0][c], dvxdz = uzz[0][c], dvzdx = ux[NV - 1][c], dvzdz = uzz[NV - 1][c];
                const float fxdx = fx[0][c], fxdz = fz[0][c], fzdx = fx[NV - 1][c], fzdz = fz[NV - 1][c];
                kr[c] = st_krho_psv(kr[c], vf[0][c], va[0][c], vf[NV - 1][c], va[NV - 1][c], ndt);
                km[c] = st_kmu_psv(km[c], dvxdx, dvxdz, dvzdx, dvzdz, fxdx, fxdz, fzdx, fzdz, ndt);
                kl[c] = st_klambda_psv(kl[c], dvxdx, dvzdz, fxdx, fzdz, ndt);
            } else {
                kr[c] = st_krho_sh(kr[c], vf[0][c], va[0][c], ndt);
                km[c] = st_kmu_sh(km[c], ux[0][c], fx[0][c], uzz[0][c], fz[0][c], ndt);
            }
        }
    }
#pragma unroll
    for (int c = 0; c < C; c++) {
        if (c >= nc) break;
        const size_t k = (size_t)(c0 + c) * nz + j;
        if (PSV) kpart[((size_t)slot * 3 + 0) * ncell + k] = kl[c];
        kpart[((size_t)slot * 3 + 1) * ncell + k] = km[c];
        kpart[((size_t)slot * 3 + 2) * ncell + k] = kr[c];
    }
}

cudaError_t launch_snap_interaction(bool psv, const Slot *d_slots, int nslots, const float *snap, ClusterGeom g,
                                    float *kpart, cudaStream_t st) {
    const size_t threads = (size_t)((g.nx + kSnapCols - 1) / kSnapCols) * g.nz;
    const dim3 grid((unsigned)((threads + 255) / 256), nslots);
    if (psv)
        k_snap_interaction<true><<<grid, 256, 0, st>>>(d_slots, snap, g, kpart);
    else
        k_snap_interaction<false><<<grid, 256, 0, st>>>(d_slots, snap, g, kpart);
    return cudaGetLastError();
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
    const int nv = psv ? 2 : 1;
    const size_t stage = g.stage ? (size_t)nv * (2 * g.cols_per + 3) * nz : 0;
    const size_t kacc = g.kacc ? (size_t)(psv ? 3 : 2) * g.cols_per * nz : 0;
    return ((size_t)(psv ? 7 : 4) * g.rs * cluster_field_rows(nz, g.G, g.dshift) + (g.cols_per + 4) + g.nrec_cta +
            (size_t)(g.nrec_cta + 1) * nv + stage + kacc) *
           4;
}

template <bool PSV, bool ADJ>
static void *cluster_kernel_q(int qm) {
    switch (qm) {
    case 4: return (void *)k_cluster<PSV, ADJ, 4>;
    case 8: return (void *)k_cluster<PSV, ADJ, 8>;
    case 12: return (void *)k_cluster<PSV, ADJ, 12>;
    case 16: return (void *)k_cluster<PSV, ADJ, 16>;
    case 10: return (void *)k_cluster<PSV, ADJ, 10>;
    case 20: return (void *)k_cluster<PSV, ADJ, 20>;
    case 24: return (void *)k_cluster<PSV, ADJ, 24>;
    default: return nullptr;
    }
}

static void *cluster_kernel(bool psv, bool adj, int qm) {
    if (psv) return adj ? cluster_kernel_q<true, true>(qm) : cluster_kernel_q<true, false>(qm);
    return adj ? cluster_kernel_q<false, true>(qm) : cluster_kernel_q<false, false>(qm);
}

static cudaError_t cluster_attrs(const void *kern, size_t smem, int R) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess && R > 8) e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    return e;
}

static cudaLaunchConfig_t cluster_config(ClusterGeom g, int nz, int nslots, size_t smem, cudaStream_t st,
                                         cudaLaunchAttribute *attr) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(g.R * nslots);
    cfg.blockDim = dim3(g.G * nz);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = g.R;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cfg;
}

int cluster_wait_error() {
    int e = 0;
    if (cudaMemcpyFromSymbol(&e, g_cluster_wait_error, sizeof(int)) != cudaSuccess) {
        (void)cudaGetLastError();
        return 1;
    }
    if (e) {
        const int z = 0;
        (void)cudaMemcpyToSymbol(g_cluster_wait_error, &z, sizeof(int));
    }
    return e;
}

cudaError_t launch_cluster(bool psv, bool adj, const Slot *d_slots, int nslots, ClusterGeom g, int nz, float *kpart,
                           float *snap, cudaStream_t st) {
    if (nslots <= 0) return cudaSuccess;
    void *kern = cluster_kernel(psv, adj, g.qmax);
    if (!kern) return cudaErrorInvalidValue;
    const size_t smem = cluster_smem_bytes(psv, g, nz);
    cudaError_t e = cluster_attrs(kern, smem, g.R);
    if (e != cudaSuccess) return e;
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = cluster_config(g, nz, nslots, smem, st, attr);
    void *args[] = {(void *)&d_slots, (void *)&g, (void *)&kpart, (void *)&snap};
    return cudaLaunchKernelExC(&cfg, kern, args);
}

cudaError_t launch_cluster_reduce(const float *kpart, int nslots, size_t ncell, float *kl, float *km, float *kr,
                                  int inv_l, int inv_m, int inv_r, cudaStream_t st) {
    const unsigned blocks = (unsigned)std::min<size_t>((ncell + 255) / 256, 4096);
    k_cluster_reduce<<<blocks, 256, 0, st>>>(kpart, nslots, ncell, kl, km, kr, inv_l, inv_m, inv_r);
    return cudaGetLastError();
}

// Largest number of clusters of this geometry that can be resident at once,
// for both passes (0 when the geometry cannot launch).
int cluster_occupancy(bool psv, ClusterGeom g, int nz) {
    const size_t smem = cluster_smem_bytes(psv, g, nz);
    int best = -1;
    for (int adj = 0; adj < 2; adj++) {
        void *kern = cluster_kernel(psv, adj != 0, g.qmax);
        if (!kern || cluster_attrs(kern, smem, g.R) != cudaSuccess) {
            (void)cudaGetLastError();
            return 0;
        }
        cudaLaunchAttribute attr[1];
        cudaLaunchConfig_t cfg = cluster_config(g, nz, 4, smem, nullptr, attr);
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) != cudaSuccess) {
            (void)cudaGetLastError();
            return 0;
        }
        best = best < 0 ? n : std::min(best, n);
    }
    return std::max(best, 0);
}

}  // namespace gb
