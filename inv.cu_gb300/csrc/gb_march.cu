// Marching step kernel: the production form of the fused time step.
//
// A block of T threads owns a z-strip (one grid row per thread) and marches
// along x over a chunk of C columns. Window rows are [w0, w0 + T) with
// w0 = strip * (T - 8) - 4, a multiple of 4 (16-byte aligned rows for bulk
// copies); rows [w0 + 4, w0 + T - 4) are owned, the stencil reads three rows
// of halo on either side (the window holds four). At column step p the
// block
//   * loads stress at column p (the x-neighbours of earlier columns stay in a
//     4-deep register queue per thread),
//   * computes the stress divergence and the new velocity and displacement at
//     column p-1 (z-neighbours of stress come from shared memory, written at
//     the previous step), adds the sources falling there, records receivers,
//   * exchanges the new velocity of column p-1 through shared memory (the only
//     barrier of the step; buffers are double-buffered by column parity),
//   * updates stress at column p-3 from the velocity register queue
//     (x-gradient) and the queued z-gradients.
// Each field element is read once per step except the 3-column and 3-row
// halos of a chunk, so the DRAM traffic stays near the algorithmic bytes and
// the work per cell is a few dozen instructions. Loads for column p+1 are
// issued before the arithmetic of column p.
//
// Arithmetic, guards and update order are those of the 2-D tile kernel
// (solver/fdm.h:76-161): results do not depend on T, C or batching.
#include <type_traits>

#include "gb_internal.h"
#include "gb_stencil.h"

namespace gb {

__device__ __forceinline__ float dminus_m(float a0, float am1, float ap1, float am2, float c9, float c24) {
    return st_dminus(a0, am1, ap1, am2, c9, c24);
}
__device__ __forceinline__ float dplus_m(float ap1, float a0, float ap2, float am1, float c9, float c24) {
    return st_dplus(ap1, a0, ap2, am1, c9, c24);
}

struct CsrM {
    const int *tile_ptr, *local, *tptr, *traces;
    __device__ CsrM(const int *p) {
        const int ntiles = p[0], nent = p[1];
        tile_ptr = p + 3;
        local = tile_ptr + ntiles + 1;
        tptr = local + nent;
        traces = tptr + nent + 1;
    }
};

constexpr int kMaxMarchThreads = 256;
constexpr int kRing = 8;  // ring slots per thread: column p is read while p+1..p+7 are in flight
// Bulk loads fill the same ring as kStages stages of kStageCols columns: one
// tensor copy per field and stage ({T rows, kStageCols columns} box).
constexpr int kStageCols = 4, kStages = kRing / kStageCols;
// A tile's source and receiver lists (cells, trace ranges, receiver traces)
// and this step's injection values are copied into shared memory before the
// march when they hold at most kCsrStage entries and kInjStage / kCsrStage
// traces; a tile with more walks the lists in global memory.
constexpr int kInjStage = 256, kCsrStage = 256;
constexpr int kCsrStageWords = 5 * kCsrStage + 2;
// The x-absorbing factor of the chunk's velocity columns (c0-1 .. c1+1) is
// staged in shared memory before the march (chunks of at most kAxStage - 3
// columns), so the per-column velocity update reads it there instead of
// waiting on a global load.
constexpr int kAxStage = 264;
static_assert(kStageCols == TMAP_BOX_COLS, "bulk-load box width");

// 4-byte async copy to shared address `d` (a 32-bit shared-window address);
// pred == false zero-fills without reading (src stays a valid address).
__device__ __forceinline__ void cpa4(unsigned d, const float *src, bool pred) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(pred ? 4 : 0) : "memory");
}
__device__ __forceinline__ void cpa_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cpa_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// ---- bulk tensor loads (TMA) completed on an mbarrier per ring slot
__device__ int g_march_tma_error;  // set when a bulk-load wait ran out of iterations

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0;
}
// Waits for phase `parity` of the barrier, at most kWaitIters tries.
constexpr int kWaitIters = 1 << 20;
__device__ __forceinline__ bool mbar_wait_bounded(unsigned bar, unsigned parity) {
    for (int i = 0; i < kWaitIters; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// One box ({T rows, kStageCols columns}, as encoded in the map) of a 2-D
// tensor {nz, nx} into shared memory, columns consecutive; row z0 must be a
// multiple of 4 (16-byte aligned); coordinates outside the tensor read as zero.
__device__ __forceinline__ void tma_col(unsigned dst, const void *tmap, int z0, int col, unsigned bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];" ::"r"(dst),
        "l"(tmap), "r"(z0), "r"(col), "r"(bar)
        : "memory");
}

// Words staged per column step: stress at p (NS), velocity, displacement and
// reciprocal density at p-1 (2 NV + 1), moduli at p-3 (the x-absorbing
// factor comes from the chunk's staged copy).
template <bool PSV>
struct MarchWords {
    static constexpr int NS = PSV ? 3 : 2, NV = PSV ? 2 : 1;
    static constexpr int SG = 0, V = NS, U = NS + NV, RHO = NS + 2 * NV, MU = RHO + 1, LAM = MU + 1,
                         N = PSV ? LAM + 1 : MU + 1;
};

template <bool PSV>
__host__ __device__ constexpr int march_smem_words(int threads) {
    return (kRing * MarchWords<PSV>::N + 2 * ((PSV ? 2 : 1) + (PSV ? 2 : 1))) * threads + 2 * 2 * (2 + 2) * 2 +
           (PSV ? 2 : 1) * kInjStage + kCsrStageWords + kAxStage;
}

// TMA = false: each thread stages its own row with 4-byte cp.async.
// TMA = true: warp 0 loads whole strip columns with bulk tensor copies (one
// per field and 32 rows) that complete on the ring slot's mbarrier; needs
// nz % 4 == 0 and the slots' tensor maps. Both read the same values for
// every cell they use, so results are identical.
// Registers are capped per wave system (SH 96, P-SV 128, no spills): left to
// itself ptxas settled the SH form at 64-80 registers with spills, and the
// 16-shot 4096 x 1024 steps ran fastest with these caps (higher ones leave
// fewer blocks resident).
template <bool PSV, bool TMA, bool MAP>
__global__ void __maxnreg__(PSV ? 128 : 96) k_march(const Slot *__restrict__ slots, int kstep,
                                                            int chunk, const unsigned *__restrict__ block_map) {
    using W = MarchWords<PSV>;
    constexpr int NS = W::NS, NV = W::NV;
    constexpr int NZS = PSV ? 2 : 1;  // stress components with a z-derivative (sxz, szz | szy)
    extern __shared__ __align__(128) float smem[];
    __shared__ __align__(8) unsigned long long s_bar[kStages];
    __shared__ int s_dead;
    __shared__ int s_inj_meta[2];  // first trace entry and count of the staged injection values
    const int T = blockDim.x, O = T - 8;
    const int TP = T + 4;  // exchange rows padded by 2 on both sides
    float *ring = smem;                                  // [kRing][W::N][T]
    float *s_sz = ring + kRing * W::N * T;               // [2][NZS][TP]
    float *s_vz = s_sz + 2 * NZS * TP;                   // [2][NV][TP]
    // [NV][kInjStage] behind s_vz (its address is recomputed where it is read)
    auto inj_stage = [&]() { return smem + kRing * W::N * blockDim.x + 2 * (NZS + NV) * (blockDim.x + 4); };
    // [kAxStage] behind the staged lists: ax of columns c0-1 .. c1+1
    auto ax_stage = [&]() { return inj_stage() + NV * kInjStage + kCsrStageWords; };

    // Blocks run shot-minor (block b: shot b % nslots, tile b / nslots): the
    // same strip of every shot runs close together, so the model columns,
    // shared by the shots, are read from HBM once and from L2 after. With a
    // block map (requests of different sizes, each with its own model) block
    // b takes the slot and tile of entry b, so no block is launched for a
    // tile a slot does not have.
    // (a form of its own: a run-time choice between the two pushed the SH
    // bulk-load form past its register cap)
    unsigned sidx, tile_u;
    if constexpr (MAP) {
        const unsigned e = __ldg(block_map + blockIdx.x);
        sidx = e >> 16;
        tile_u = e & 0xffffu;
    } else {
        const unsigned blk = blockIdx.y * gridDim.x + blockIdx.x;
        sidx = blk % gridDim.y;
        tile_u = blk / gridDim.y;
    }
    const Slot &S = slots[sidx];
    if (!S.active) return;
    const int it = S.it_base + kstep;
    if (it < 0 || it >= S.nt) return;
    const int par = (S.par0 + kstep) & 1;
    const int nx = S.nx, nz = S.nz, nt = S.nt, pz = S.pz;  // pz: address pitch of the grid arrays
    const int tile = (int)tile_u;
    if (tile >= S.tiles_z * S.tiles_x) return;
    const int strip = tile % S.tiles_z, ck = tile / S.tiles_z;
    const int t = threadIdx.x;
    const int j = strip * O - 4 + t;          // grid row of this thread
    const int c0 = ck * chunk;                 // first owned column
    const int c1 = min(c0 + chunk, nx);        // one past the last owned column
    const bool rowin = (unsigned)j < (unsigned)nz;
    const bool rowown = t >= 4 && t < T - 4 && rowin;
    const bool zS = j >= 2 && j < nz - 2;      // z part of the stress divergence
    const bool zV = j >= 1 && j < nz - 2;      // z part of the velocity gradient
    const float dt = S.dt, c9x = S.c9x, c24x = S.c24x, c9z = S.c9z, c24z = S.c24z;
    const float azj = rowin ? __ldg(S.az + j) : 0.f;
    const int st = t + 2;                      // padded exchange index
    const int record_u = S.record_u;

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
    const float *lam = S.lambda, *mu = S.mu, *rinv_g = S.rinv;

    // Sources in the velocity region of this window and receivers of its
    // owned cells, both sorted by column then row. The next entry's cell is
    // kept in a register so the per-column test needs no memory access.
    const int VZ = O + 3;
    int inj_ptr = 0, inj_end = 0, rec_ptr = 0, rec_end = 0;
    const int *inj_local = nullptr, *inj_tptr = nullptr, *inj_traces = nullptr;
    const int *rec_local = nullptr, *rec_tptr = nullptr, *rec_traces = nullptr;
    if (S.inj) {
        const CsrM c(S.inj);
        inj_ptr = c.tile_ptr[tile];
        inj_end = c.tile_ptr[tile + 1];
        inj_local = c.local;
        inj_tptr = c.tptr;
        inj_traces = c.traces;
    }
    if (S.rec) {
        const CsrM c(S.rec);
        rec_ptr = c.tile_ptr[tile];
        rec_end = c.tile_ptr[tile + 1];
        rec_local = c.local;
        rec_tptr = c.tptr;
        rec_traces = c.traces;
    }
    // The tile's lists and this step's injection values go to shared memory
    // (one round of loads now instead of dependent global loads at every
    // column step that has a source or receiver: an adjoint with a receiver
    // in every surface column waited on memory at each of them). When they
    // fit, the list pointers below point at the copies, with entry and trace
    // indices rebased to 0, so the march walks them unchanged.
    {
        float *s_inj = inj_stage();
        int *si_loc = reinterpret_cast<int *>(s_inj + NV * kInjStage);
        int *si_tp = si_loc + kCsrStage, *sr_loc = si_tp + kCsrStage + 1;
        int *sr_tp = sr_loc + kCsrStage, *sr_tr = sr_tp + kCsrStage + 1;
        const int ni = inj_end - inj_ptr, nr = rec_end - rec_ptr;
        const int i0 = ni > 0 ? inj_tptr[inj_ptr] : 0, ti = ni > 0 ? inj_tptr[inj_end] - i0 : 0;
        const int r0 = nr > 0 ? rec_tptr[rec_ptr] : 0, tr = nr > 0 ? rec_tptr[rec_end] - r0 : 0;
        const bool stage_i = ni > 0 && ni <= kCsrStage && ti <= kInjStage;  // uniform over the block
        const bool stage_r = nr > 0 && nr <= kCsrStage && tr <= kCsrStage;
        if (stage_i) {
            for (int k = t; k < ni; k += T) si_loc[k] = inj_local[inj_ptr + k];
            for (int k = t; k <= ni; k += T) si_tp[k] = inj_tptr[inj_ptr + k] - i0;
            for (int e = t; e < ti; e += T) {
                const int ks = inj_traces[i0 + e] * nt + it;
                if (PSV) {
                    s_inj[e] = __ldg(S.inj_x + ks);
                    s_inj[kInjStage + e] = __ldg(S.inj_z + ks);
                } else {
                    s_inj[e] = __ldg(S.inj_y + ks);
                }
            }
        }
        if (stage_r) {
            for (int k = t; k < nr; k += T) sr_loc[k] = rec_local[rec_ptr + k];
            for (int k = t; k <= nr; k += T) sr_tp[k] = rec_tptr[rec_ptr + k] - r0;
            for (int e = t; e < tr; e += T) sr_tr[e] = rec_traces[r0 + e];
        }
        {
            float *s_axc = ax_stage();
            for (int k = t; k < c1 - c0 + 3; k += T) s_axc[k] = __ldg(S.ax + min(max(c0 - 1 + k, 0), nx - 1));
        }
        if (t == 0) {
            s_inj_meta[0] = stage_i ? 0 : i0;  // trace index of s_inj[0]
            s_inj_meta[1] = stage_i ? ti : 0;  // staged values
        }
        __syncthreads();
        if (stage_i) {
            inj_local = si_loc;
            inj_tptr = si_tp;
            inj_ptr = 0;
            inj_end = ni;
        }
        if (stage_r) {
            rec_local = sr_loc;
            rec_tptr = sr_tp;
            rec_traces = sr_tr;
            rec_ptr = 0;
            rec_end = nr;
        }
    }
    int inj_next = inj_ptr < inj_end ? inj_local[inj_ptr] : 0x7fffffff;
    int rec_next = rec_ptr < rec_end ? rec_local[rec_ptr] : 0x7fffffff;

    // Issues the loads of column step p into ring slot `slot` (own row only).
    // Offsets are 32-bit (grids are limited to 2^29 cells); the shared
    // address of this thread's ring row is computed once.
    const unsigned ring_row = (unsigned)__cvta_generic_to_shared(ring + t);
    const int jj = rowin ? j : 0;
    auto issue = [&](int p, int slot) {
        const unsigned rs = ring_row + (unsigned)(slot * W::N * T) * 4u;
        const bool cs = (unsigned)p < (unsigned)nx && rowin;
        const int ks = cs ? p * pz + jj : 0;
#pragma unroll
        for (int f = 0; f < NS; f++) cpa4(rs + (W::SG + f) * T * 4, sig_in[f] + ks, cs);
        const int pv = p - 1;
        const bool cv = (unsigned)pv < (unsigned)nx && rowin && pv >= c0 - 1;
        const int kv = cv ? pv * pz + jj : 0;
        const bool uo = cv && rowown && pv >= c0 && pv < c1;
#pragma unroll
        for (int f = 0; f < NV; f++) {
            cpa4(rs + (W::V + f) * T * 4, v_in[f] + kv, cv);
            cpa4(rs + (W::U + f) * T * 4, u[f] + kv, uo);
        }
        cpa4(rs + W::RHO * T * 4, rinv_g + kv, cv);
        const int pm = p - 3;
        const bool cm = pm >= c0 && pm < c1 && rowown;
        const int km = cm ? pm * pz + jj : 0;
        cpa4(rs + W::MU * T * 4, mu + km, cm);
        if (PSV) cpa4(rs + W::LAM * T * 4, lam + km, cm);
    };

    const int p_first = c0 - 3, p_last = c1 + 2;
    const int nstep = p_last - p_first + 1;
    const int nstage = (nstep + kStageCols - 1) / kStageCols;
    // bulk loads (warp 0; lane 0 arms the stage's barrier with the byte count first)
    const char *tm = static_cast<const char *>(S.tmap);
    const int w0 = strip * O - 4;
    const unsigned bar0 = (unsigned)__cvta_generic_to_shared(s_bar);
    const unsigned ring0 = (unsigned)__cvta_generic_to_shared(ring);
    constexpr int NTF = NS + 2 * NV + 2 + (PSV ? 1 : 0);  // fields per column step
    // lane f < NTF of warp 0 loads field f: its ring word, tensor map and
    // column offset from the step's column p (stress p, velocity,
    // displacement and 1/rho p-1, moduli p-3)
    int lw = 0, lcol = 0;
    const void *lmap = tm;
    if (TMA && t < NTF) {
        int map;
        if (t < NS) {
            lw = W::SG + t;
            map = PSV ? SXX0 + 2 * t + par : TMAP_SH + SXY0 + 2 * t + par;
        } else if (t < NS + NV) {
            lw = W::V + (t - NS);
            map = PSV ? VX0 + 2 * (t - NS) + par : TMAP_SH + VY0 + par;
            lcol = -1;
        } else if (t < NS + 2 * NV) {
            lw = W::U + (t - NS - NV);
            map = PSV ? UX + (t - NS - NV) : TMAP_SH + UY;
            lcol = -1;
        } else if (t == NS + 2 * NV) {
            lw = W::RHO;
            map = TMAP_RINV;
            lcol = -1;
        } else if (t == NS + 2 * NV + 1) {
            lw = W::MU;
            map = TMAP_MU;
            lcol = -3;
        } else {
            lw = PSV ? W::LAM : W::MU;
            map = TMAP_LAM;
            lcol = -3;
        }
        lmap = tm + (size_t)map * TMAP_BYTES;
    }
    // stage m = column steps [kStageCols*m, kStageCols*(m+1)) into ring stage m % kStages
    auto issue_tma = [&](int m) {
        if (t >= 32) return;
        const int slot = m % kStages;
        const unsigned bar = bar0 + 8u * (unsigned)slot;
        if (t == 0) mbar_expect_tx(bar, (unsigned)(NTF * T * kStageCols * 4));
        __syncwarp();
        if (t < NTF) {
            // the stage was last read by ordinary loads (before a block barrier)
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            const unsigned dst = ring0 + 4u * (unsigned)((slot * W::N + lw) * kStageCols * T);
            tma_col(dst, lmap, w0, p_first + kStageCols * m + lcol, bar);
        }
    };
    bool dead = false;  // a bulk-load wait ran out of iterations (never in a correct run)
    if (TMA) {
        if (t == 0) {
            for (int sl = 0; sl < kStages; sl++) mbar_init(bar0 + 8u * (unsigned)sl, 1);
            s_dead = 0;
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncthreads();
    }

    float sq[4][NS], vq[4][NV], dzq[3][NV];
#pragma unroll
    for (int a = 0; a < 4; a++) {
#pragma unroll
        for (int f = 0; f < NS; f++) sq[a][f] = 0.f;
#pragma unroll
        for (int f = 0; f < NV; f++) vq[a][f] = 0.f;
    }
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int f = 0; f < NV; f++) dzq[a][f] = 0.f;

    int issued = 0, sdone = 0;  // stages issued / waited for (bulk loads)
    // prologue: kRing - 1 column steps (cp.async) or kStages stages (bulk) in flight
    if (TMA) {
        for (int m = 0; m < kStages && m < nstage; m++) {
            issue_tma(m);
            issued = m + 1;
        }
    } else {
#pragma unroll
        for (int q = 0; q < kRing - 1; q++) {
            if (q < nstep) issue(p_first + q, q);
            cpa_commit();
        }
    }
    // bulk loads: waits for stage m (whole strip, kStageCols columns; phase
    // m / kStages of its barrier) and refills the ring stage consumed in
    // stage m-1 (every thread finished reading it before the previous column
    // step's barrier); returns the stage's ring row of this thread
    auto stage_start = [&](int m) -> const float * {
        if (!dead && !mbar_wait_bounded(bar0 + 8u * (unsigned)(m % kStages), (unsigned)((m / kStages) & 1))) {
            dead = true;
            s_dead = 1;
            atomicOr(&g_march_tma_error, 1);
        }
        sdone = m + 1;
        if (m >= 1 && m + 1 < nstage && !dead) {
            issue_tma(m + 1);
            issued = m + 2;
        }
        return ring + (m % kStages) * W::N * kStageCols * T + t;
    };
    // word stride of a column step in the ring
    const int ws = TMA ? kStageCols * T : T;

    // Column step q: the stress of column p = p_first + q arrives (ring row
    // rs), the velocity and displacement of column p - 1 and the stress of
    // column p - 3 are updated. STEADY: a step whose velocity column is
    // stored and whose stress column is updated, in a chunk at least two
    // columns away from the grid's x edges, where every column test below
    // holds and is left out. CHK: read the block's bulk-load failure flag
    // after the barrier (it can only be set at a stage's first step).
    // Returns false when the march must stop (a bulk-load wait failed).
    auto step = [&](const int q, const float *rs, auto steady, const bool chk) __attribute__((always_inline)) {
        constexpr bool STEADY = decltype(steady)::value;
        const int p = p_first + q;
        float cur[W::N];
#pragma unroll
        for (int w = 0; w < W::N; w++) cur[w] = rs[w * ws];
        const int buf = q & 1;
#pragma unroll
        for (int f = 0; f < NS; f++) {
            sq[0][f] = sq[1][f];
            sq[1][f] = sq[2][f];
            sq[2][f] = sq[3][f];
            sq[3][f] = cur[W::SG + f];
        }
        float *sz_w = s_sz + buf * NZS * TP;
        if (PSV) {
            sz_w[st] = cur[W::SG + 2];       // sxz
            sz_w[TP + st] = cur[W::SG + 1];  // szz
        } else {
            sz_w[st] = cur[W::SG + 1];  // szy
        }
        const int pv = p - 1;  // velocity column of this step
        const bool vcol = STEADY || pv >= c0 - 1;
        float vn[NV];
#pragma unroll
        for (int f = 0; f < NV; f++) vn[f] = 0.f;
        if (vcol) {
            const float *sz_r = s_sz + (buf ^ 1) * NZS * TP;
            float ds[NV];
            const bool xS = STEADY || (pv >= 2 && pv < nx - 2);
            if (PSV) {
                float dsx = xS ? dminus_m(sq[2][0], sq[1][0], sq[3][0], sq[0][0], c9x, c24x) : 0.f;
                float dsz = xS ? dminus_m(sq[2][2], sq[1][2], sq[3][2], sq[0][2], c9x, c24x) : 0.f;
                if (zS) {
                    const float *a = sz_r, *b = sz_r + TP;
                    dsx += dminus_m(a[st], a[st - 1], a[st + 1], a[st - 2], c9z, c24z);
                    dsz += dminus_m(b[st], b[st - 1], b[st + 1], b[st - 2], c9z, c24z);
                }
                ds[0] = dsx;
                ds[NV - 1] = dsz;
            } else {
                float dsy = xS ? dminus_m(sq[2][0], sq[1][0], sq[3][0], sq[0][0], c9x, c24x) : 0.f;
                if (zS) dsy += dminus_m(sz_r[st], sz_r[st - 1], sz_r[st + 1], sz_r[st - 2], c9z, c24z);
                ds[0] = dsy;
            }
            // sources at this column, in trace order (solver/fdm.h:163-180)
            const int cl = pv - (c0 - 1);
            while (inj_next < (cl + 1) * VZ) {
                if (t == inj_next - cl * VZ + 3) {
                    // read back here (volatile) rather than held in registers
                    // through the march: sources are rare cells
                    const int e0 = *(volatile int *)&s_inj_meta[0], n = *(volatile int *)&s_inj_meta[1];
                    const float *s_inj = inj_stage();
                    for (int e = inj_tptr[inj_ptr]; e < inj_tptr[inj_ptr + 1]; e++) {
                        const int o = e - e0;
                        if (o < n) {
                            ds[0] += s_inj[o];
                            if (PSV) ds[NV - 1] += s_inj[kInjStage + o];
                        } else {
                            const int ks = inj_traces[e] * nt + it;
                            if (PSV) {
                                ds[0] += __ldg(S.inj_x + ks);
                                ds[NV - 1] += __ldg(S.inj_z + ks);
                            } else {
                                ds[0] += __ldg(S.inj_y + ks);
                            }
                        }
                    }
                }
                inj_ptr++;
                inj_next = inj_ptr < inj_end ? inj_local[inj_ptr] : 0x7fffffff;
            }
            if (STEADY || ((unsigned)pv < (unsigned)nx && rowin)) {
                const float ab = ax_stage()[pv - (c0 - 1)] * azj;
                const float rinv = cur[W::RHO];
#pragma unroll
                for (int f = 0; f < NV; f++) {
                    vn[f] = st_velocity(ab, dt, ds[f], rinv, cur[W::V + f]);
                    // rows outside the grid keep 0, as in the other steps
                    if (STEADY) vn[f] = rowin ? vn[f] : 0.f;
                }
            }
            if (STEADY || (pv >= c0 && pv < c1)) {
                const int oc = pv - c0;
                float un[NV];
#pragma unroll
                for (int f = 0; f < NV; f++) un[f] = st_displacement(cur[W::U + f], vn[f], dt);
                if (rowown) {
                    const int kv = pv * pz + j;
#pragma unroll
                    for (int f = 0; f < NV; f++) {
                        v_out[f][kv] = vn[f];
                        u[f][kv] = un[f];
                    }
                }
                // receivers (solver/fdm.h:181-196): u when record_u, else v
                while (rec_next < (oc + 1) * O) {
                    if (rowown && t == rec_next - oc * O + 4) {
                        for (int e = rec_tptr[rec_ptr]; e < rec_tptr[rec_ptr + 1]; e++) {
                            const int kr = rec_traces[e] * nt + it;
                            if (PSV) {
                                S.out_x[kr] = record_u ? un[0] : vn[0];
                                S.out_z[kr] = record_u ? un[NV - 1] : vn[NV - 1];
                            } else {
                                S.out_y[kr] = record_u ? un[0] : vn[0];
                            }
                        }
                    }
                    rec_ptr++;
                    rec_next = rec_ptr < rec_end ? rec_local[rec_ptr] : 0x7fffffff;
                }
            }
        }
        float *vz_w = s_vz + buf * NV * TP;
#pragma unroll
        for (int f = 0; f < NV; f++) {
            vq[0][f] = vq[1][f];
            vq[1][f] = vq[2][f];
            vq[2][f] = vq[3][f];
            vq[3][f] = vn[f];
            vz_w[f * TP + st] = vn[f];
        }
        __syncthreads();
        if (TMA && chk && s_dead) return false;  // uniform: s_dead is read after the barrier
        // z-gradient of the new velocity at column pv
#pragma unroll
        for (int f = 0; f < NV; f++) {
            dzq[0][f] = dzq[1][f];
            dzq[1][f] = dzq[2][f];
            const float *a = vz_w + f * TP;
            dzq[2][f] = (vcol && zV) ? dplus_m(a[st + 1], a[st], a[st + 2], a[st - 1], c9z, c24z) : 0.f;
        }
        // stress update at column pm = p - 3 (solver/fdm.h:138-149)
        const int pm = p - 3;
        if ((STEADY || (pm >= c0 && pm < c1)) && rowown) {
            const bool xV = STEADY || (pm >= 1 && pm < nx - 2);
            const int km = pm * pz + j;
            const float m = cur[W::MU];
            if (PSV) {
                const float dvxdx = xV ? dplus_m(vq[2][0], vq[1][0], vq[3][0], vq[0][0], c9x, c24x) : 0.f;
                const float dvzdx = xV ? dplus_m(vq[2][1], vq[1][1], vq[3][1], vq[0][1], c9x, c24x) : 0.f;
                const float dvxdz = dzq[0][0], dvzdz = dzq[0][1];
                float sxx = sq[0][0], szz = sq[0][1], sxz = sq[0][2];
                st_stress_psv(sxx, szz, sxz, cur[W::LAM], m, dt, dvxdx, dvxdz, dvzdx, dvzdz);
                sig_out[0][km] = sxx;
                sig_out[1][km] = szz;
                sig_out[2][km] = sxz;
            } else {
                const float dvydx = xV ? dplus_m(vq[2][0], vq[1][0], vq[3][0], vq[0][0], c9x, c24x) : 0.f;
                const float dvydz = dzq[0][0];
                float sxy = sq[0][0], szy = sq[0][1];
                st_stress_sh(sxy, szy, m, dt, dvydx, dvydz);
                sig_out[0][km] = sxy;
                sig_out[1][km] = szy;
            }
        }
        return true;
    };
    // any column step, with its ring handling
    auto any_step = [&](const int q) -> bool {
        const float *rs;
        bool chk = false;
        if (TMA) {
            const int m = q / kStageCols, qc = q - m * kStageCols;
            if (qc == 0) {
                rs = stage_start(m);
                chk = true;
            } else {
                rs = ring + (m % kStages) * W::N * kStageCols * T + t;
            }
            rs += qc * T;
        } else {
            cpa_wait<kRing - 2>();  // column step q has landed (own row)
            rs = ring + (q % kRing) * W::N * T + t;
            // refill the slot read at the previous step (every thread
            // finished reading it before the previous step's barrier)
            if (q + kRing - 1 < nstep) issue(p_first + q + kRing - 1, (q + kRing - 1) % kRing);
            cpa_commit();
        }
        return step(q, rs, std::false_type{}, chk);
    };

    // Steps 0..7 (the velocity and stress columns start at steps 3 and 6),
    // then, with bulk loads in a chunk away from the grid's x edges, whole
    // stages of steady steps while the stage's last step stores its velocity
    // column (q < cc + 4), then the remaining steps.
    const int cc = c1 - c0;
    const bool interior = c0 >= 2 && c1 <= nx - 2;
    constexpr int kSteadyStage = 2;  // first stage whose steps are all past step 6
    const int m_end = (TMA && interior) ? cc / kStageCols + 1 : 0;
    bool run = true;
    int q = 0;
    for (; q < nstep && q < kSteadyStage * kStageCols && run; q++) run = any_step(q);
    if (run && m_end > kSteadyStage) {
        for (int m = kSteadyStage; m < m_end; m++) {
            const float *rs = stage_start(m);
            const int q0 = m * kStageCols;
            if (!step(q0, rs, std::true_type{}, true)) {
                run = false;
                break;
            }
#pragma unroll
            for (int qc = 1; qc < kStageCols; qc++) step(q0 + qc, rs + qc * T, std::true_type{}, false);
        }
        q = m_end * kStageCols;
    }
    for (; q < nstep && run; q++) run = any_step(q);
    if (!TMA) cpa_wait<0>();
    if (TMA && s_dead) {
        // leave no bulk copy in flight into this block's shared memory
        for (int mm = sdone; mm < issued; mm++)
            (void)mbar_wait_bounded(bar0 + 8u * (unsigned)(mm % kStages), (unsigned)((mm / kStages) & 1));
    }
}

int march_tma_error() {
    int e = 0;
    if (cudaMemcpyFromSymbol(&e, g_march_tma_error, sizeof(int)) != cudaSuccess) {
        (void)cudaGetLastError();
        return 1;
    }
    if (e) {
        const int z = 0;
        (void)cudaMemcpyToSymbol(g_march_tma_error, &z, sizeof(int));
    }
    return e;
}

template <bool PSV, bool TMA, bool MAP>
static cudaError_t launch_march_t(dim3 grid, int threads, size_t smem, const Slot *d_slots, int k, int chunk,
                                  cudaStream_t st, const unsigned *block_map) {
    static bool attr_set = false;
    if (!attr_set) {
        const cudaError_t e = cudaFuncSetAttribute(k_march<PSV, TMA, MAP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   march_smem_words<PSV>(kMaxMarchThreads) * 4);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    k_march<PSV, TMA, MAP><<<grid, threads, smem, st>>>(d_slots, k, chunk, block_map);
    return cudaGetLastError();
}

template <bool PSV, bool TMA>
static cudaError_t launch_march_m(dim3 grid, int threads, size_t smem, const Slot *d_slots, int k, int chunk,
                                  cudaStream_t st, const unsigned *block_map) {
    return block_map ? launch_march_t<PSV, TMA, true>(grid, threads, smem, d_slots, k, chunk, st, block_map)
                     : launch_march_t<PSV, TMA, false>(grid, threads, smem, d_slots, k, chunk, st, nullptr);
}

cudaError_t launch_march(bool psv, bool tma, int threads, int chunk, const Slot *d_slots, int nslots, int max_tiles,
                         int k, cudaStream_t st, const unsigned *block_map, int nmap) {
    if (block_map ? nmap <= 0 : (nslots <= 0 || max_tiles <= 0)) return cudaSuccess;
    if (threads < 32 || threads > kMaxMarchThreads || threads % 32 || chunk < 1 || chunk + 3 > kAxStage)
        return cudaErrorInvalidValue;
    const dim3 grid = block_map ? dim3((unsigned)nmap, 1) : dim3(max_tiles, nslots);
    const size_t smem = (size_t)(psv ? march_smem_words<true>(threads) : march_smem_words<false>(threads)) * 4;
    if (psv)
        return tma ? launch_march_m<true, true>(grid, threads, smem, d_slots, k, chunk, st, block_map)
                   : launch_march_m<true, false>(grid, threads, smem, d_slots, k, chunk, st, block_map);
    return tma ? launch_march_m<false, true>(grid, threads, smem, d_slots, k, chunk, st, block_map)
               : launch_march_m<false, false>(grid, threads, smem, d_slots, k, chunk, st, block_map);
}

}  // namespace gb
