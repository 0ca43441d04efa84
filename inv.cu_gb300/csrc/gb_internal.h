// Internal types shared by the CUDA kernels and the host runtime of libgbfwi.
//
// Grid layout everywhere is the reference's: float[nx*nz], k = i*nz + j, z
// (depth) contiguous (lib/device.h:38-40). Wavefields use the same layout so
// the model, kernel and trace buffers can be handed to callers unchanged.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <string>

namespace gb {

// Number of state arrays per wave system in one slot. Stress and velocity are
// ping-ponged (the fused step reads time level n and writes n+1 into the
// other buffer, so neighbouring tiles never see a half-updated field);
// displacement is updated in place (it is only read at its own cell).
enum FieldPsv { VX0, VX1, VZ0, VZ1, SXX0, SXX1, SZZ0, SZZ1, SXZ0, SXZ1, UX, UZ, NPSV };
enum FieldSh { VY0, VY1, SXY0, SXY1, SZY0, SZY1, UY, NSH };

// Checkpoint storage precision.
enum CkptPrec { CKPT_F32 = 0, CKPT_BF16 = 1, CKPT_F16 = 2 };

// One shot being propagated: everything a step kernel needs, in device
// memory. A batch is an array of slots; blockIdx.y selects the slot.
struct Slot {
    int nx, nz, nt;
    // address pitch of the slot's state and model arrays: cell (i, j) lies at
    // i*pz + j; pz == nz is the reference layout (the solver), a larger pz
    // (rows nz .. pz-1 unused) lets a served request of any nz use tensor maps
    // (column starts on 16-byte boundaries). Checkpoints, traces and kernels
    // keep the reference layout.
    int pz;
    int tiles_z, tiles_x;
    int active;
    // Time base: a launch with step index k advances this slot from step
    // it = it_base + k, reading the ping-pong buffers of parity
    // (par0 + k) & 1. Lockstep batches use it_base = par0 = 0 and k = it;
    // served requests each keep their own base.
    int it_base, par0;
    int sfe;         // checkpoint spacing (steps)
    int ckpt_write;  // 1: forward pass stores checkpoints; 0: adjoint reads them
    // cluster-resident path: forward source cell and trace (src_trace < 0:
    // none), receiver cells (distinct)
    int src_i, src_j, src_trace;
    const int *pts_i, *pts_j;
    int npts;
    float dt;
    float c9x, c24x, c9z, c24z;  // 9/(8h) and 1/(24h) for h = dx, dz
    const float *lambda, *mu, *rho;
    const float *rinv;     // 1/rho rounded to nearest, refreshed at each pass
    const float *ax, *az;  // absorbing profiles: ab(i,j) = ax[i] * az[j]
    float *psv[NPSV];      // P-SV state (null when the slot has no P-SV)
    float *sh[NSH];        // SH state (null when the slot has no SH)
    // injection (forward sources or adjoint receivers): packed tile CSR
    const int *inj;
    const float *inj_x, *inj_y, *inj_z;  // trace data, value = inj_c[trace*nt + it]
    // recording (receivers): packed tile CSR over owned cells
    const int *rec;
    float *out_x, *out_y, *out_z;
    int record_u;
    // checkpoints: [nsfe][nf][nx*nz] elements of ckpt_prec, scale [nsfe][nf]
    void *ckpt;
    float *ckpt_amax;
    int nsfe, nf, ckpt_prec;
    // tensor maps (128-byte CUtensorMap each) of this slot's fields for the
    // marching kernel's bulk loads, indexed by TMAP_*; null when unused
    const void *tmap;
};

// Tensor map index of a P-SV field f (FieldPsv), an SH field (TMAP_SH + FieldSh)
// and the model fields. Each map covers one field as a 2-D tensor {nz, nx}
// with a box of {marching threads, TMAP_BOX_COLS} (rows, columns).
constexpr int TMAP_SH = NPSV, TMAP_RINV = NPSV + NSH, TMAP_MU = TMAP_RINV + 1, TMAP_LAM = TMAP_RINV + 2,
              TMAP_N = TMAP_RINV + 3, TMAP_BYTES = 128, TMAP_BOX_COLS = 4;

// A group of slots that accumulate into the same sensitivity kernels.
struct KernelGroup {
    float *k_lambda, *k_mu, *k_rho;
    int inv_lambda, inv_mu, inv_rho;
    int first, count;  // slot range
    int nx, nz;
};

// Configuration of the fused step kernel. threads == 0: 2-D tile kernel
// owning tz x tx cells per block. threads > 0: marching kernel, one grid row
// per thread, tz = threads - 8 owned rows per strip, tx = columns per chunk.
struct TileCfg {
    int tz, tx, threads;
};
// The step kernel configurations 1..20 (1-5: 2-D tiles, 6-20: marching strips).
TileCfg tile_config(int id);

// Cluster-resident solver geometry: R CTAs per shot (cluster), cols_per grid
// columns per CTA (a multiple of qmax; the last CTA holds the remaining grid
// columns, at least 2), G groups of nz threads per CTA (blockDim = G * nz),
// each thread owning qmax consecutive columns of one row (qmax in
// {4, 8, 10, 12, 16, 20, 24}, G * qmax = cols_per); nrec_cta = most receivers
// in one CTA's columns.
// The launch also carries the values common to all slots (grid, steps, time
// step and stencil coefficients), which the kernel reads from its parameters.
struct ClusterGeom {
    int R, cols_per, G, qmax, nrec_cta;
    int rs, dshift;  // shared-memory row stride; row shift between consecutive thread groups
    int stage;  // adjoint: stage each checkpoint in shared memory before the kernel accumulation
    int kacc;   // adjoint: accumulate the shot's kernels in shared memory, stored once after the pass
    int nx, nz, nt;
    float dt, c9x, c24x, c9z, c24z;
};

// Power-of-two scale of a 16-bit checkpoint with max |value| amax: FP16 maps
// amax to at most 2^15, BF16 to at most 1; FP32 and empty fields use 1.
#ifdef __CUDACC__
__host__ __device__
#endif
inline float ckpt_scale_of(float amax, int prec) {
    if (!(amax > 0.f) || prec == 0) return 1.f;
    const float target = prec == 2 ? 32768.f : 1.f;
    int e;
    frexpf(target / amax, &e);
    return ldexpf(1.f, e - 1);
}

// Fields of one checkpoint of a wave system. FP32 keeps the reference's
// fields (solver/fdm.h:521-560): SH uy, vy; P-SV ux, uz, vx, vz. The 16-bit
// forms keep what the kernel accumulation reads of the forward wavefield
// instead (solver/fdm.h:583-606), computed in FP32 from the displacement
// before rounding: SH d(uy)/dx, d(uy)/dz, vy; P-SV the divergence
// d(ux)/dx + d(uz)/dz, the normal-strain difference d(ux)/dx - d(uz)/dz, the
// shear sum d(ux)/dz + d(uz)/dx, vx, vz. A difference of two 16-bit
// displacements loses the digits the two values share, and so does a sum of
// two rounded normal strains where they cancel (shear waves); each rounded
// strain here keeps its own relative precision. An SH+P-SV slot stores the
// SH fields first.
#ifdef __CUDACC__
__host__ __device__
#endif
inline int ckpt_nf_sh(int prec) { return prec == 0 ? 2 : 3; }
#ifdef __CUDACC__
__host__ __device__
#endif
inline int ckpt_nf_psv(int prec) { return prec == 0 ? 4 : 5; }

// Packed tile CSR header: [0]=ntiles [1]=nentries [2]=ntraces, then
// tile_ptr[ntiles+1], local[nentries], tptr[nentries+1], traces[ntraces].
inline int csr_words(int ntiles, int nent, int ntr) { return 3 + ntiles + 1 + nent + nent + 1 + ntr; }

// ---------------------------------------------------------------- launchers
// All launchers enqueue on `st` and return cudaGetLastError().
// k is the launch's step index (see Slot::it_base).
// block_map (marching kernel only; null: none): one entry per block,
// (slot << 16) | tile, so a launch over slots of different sizes runs
// exactly their tiles instead of max_tiles blocks for every slot; nmap is
// the entry count (the grid), max_tiles is then unused.
cudaError_t launch_step(bool psv, TileCfg tc, const Slot *d_slots, int nslots, int max_tiles, int k, bool tma,
                        cudaStream_t st, const unsigned *block_map = nullptr, int nmap = 0);
// Marching kernel launch; tma = bulk tensor loads through the slots' maps.
// march_tma_error returns (and clears) the device flag a bulk-load wait that
// ran out of iterations sets.
int march_tma_error();
cudaError_t launch_march(bool psv, bool tma, int threads, int chunk, const Slot *d_slots, int nslots, int max_tiles, int k,
                         cudaStream_t st, const unsigned *block_map = nullptr, int nmap = 0);
// Checkpoint of displacement before step k (which_u = 1) or velocity after
// it (which_u = 0), for every slot with ckpt_write whose step is a
// checkpoint step ((it + 1) % sfe == 0).
cudaError_t launch_ckpt_amax(const Slot *d_slots, int nslots, int n, int k, int which_u, bool psv,
                             cudaStream_t st);
cudaError_t launch_ckpt_store(const Slot *d_slots, int nslots, int n, int k, int which_u, bool psv,
                              cudaStream_t st);
// Kernel accumulation after step k for every group slot with it % sfe == 0.
cudaError_t launch_interaction(bool psv, const Slot *d_slots, const KernelGroup *d_groups, int ngroups,
                               int max_cells, int k, cudaStream_t st);
cudaError_t launch_fill(float *p, float v, size_t n, cudaStream_t st);
// Cluster-resident passes (gb_cluster.cu): one cluster per slot runs the
// whole pass; the adjoint adds each slot's kernels to kpart[slot][3][nx*nz].
size_t cluster_smem_bytes(bool psv, const ClusterGeom &g, int nz);
void cluster_layout(ClusterGeom &g, int nz, bool shift);
int cluster_max_threads(bool psv, int qmax);
int cluster_occupancy(bool psv, ClusterGeom g, int nz);
cudaError_t launch_cluster(bool psv, bool adj, const Slot *d_slots, int nslots, ClusterGeom g, int nz, float *kpart,
                           float *snap, cudaStream_t st);
// returns (and clears) the device flag a ghost-column wait of the cluster
// kernel that ran out of iterations sets
int cluster_wait_error();
// the kernel accumulation of a cluster adjoint pass that stored its adjoint
// state (snap) instead of accumulating in the pass
cudaError_t launch_snap_interaction(bool psv, const Slot *d_slots, int nslots, const float *snap, ClusterGeom g,
                                    float *kpart, cudaStream_t st);
cudaError_t launch_cluster_reduce(const float *kpart, int nslots, size_t ncell, float *kl, float *km, float *kr,
                                  int inv_l, int inv_m, int inv_r, cudaStream_t st);
cudaError_t launch_mesh2grid(float *lambda, float *mu, float *rho, const float *px, const float *pz,
                             const float *pa, const float *pb, const float *pr, int npt, float dmax, float dx,
                             float dz, int nx, int nz, cudaStream_t st);
cudaError_t launch_scatter_points(float *lambda, float *mu, float *rho, const int *cell_of_point,
                                  const float *pa, const float *pb, const float *pr, int npt, cudaStream_t st);
cudaError_t launch_reciprocal(float *out, const float *in, size_t n, cudaStream_t st);
cudaError_t launch_vps2lm(float *lambda, float *mu, const float *rho, size_t n, cudaStream_t st);
cudaError_t launch_lm2vps(float *vp, float *vs, const float *rho, size_t n, cudaStream_t st);
cudaError_t launch_axpby(float *c, float ka, const float *a, float kb, const float *b, size_t n,
                         cudaStream_t st);

// FP64 reductions (gb_reduce.cu). `partial` holds at least reduce_partials()
// doubles; the result lands in *d_out (device).
int reduce_partials();
cudaError_t launch_dot(const float *a, const float *b, size_t n, double *partial, double *d_out,
                       cudaStream_t st);
cudaError_t launch_amax(const float *a, size_t n, double *partial, double *d_out, cudaStream_t st);

// Misfits (gb_misfit.cu).
cudaError_t launch_taper(float *tw, float dt, int nt, cudaStream_t st);
cudaError_t launch_waveform(const float *syn, const float *obs, const float *tw, float *adstf,
                            double *trace_val, int ntr, int nt, float sqrt_dt, cudaStream_t st);
cudaError_t launch_sum_traces(const double *trace_val, int ntr, double *d_out, cudaStream_t st);

// Error state.
void set_error(const std::string &msg);
const char *last_error();

}  // namespace gb

#define GB_CUDA_TRY(expr)                                                                      \
    do {                                                                                       \
        cudaError_t _e = (expr);                                                               \
        if (_e != cudaSuccess) {                                                               \
            ::gb::set_error(std::string(#expr) + ": " + cudaGetErrorString(_e) + " at " +      \
                            __FILE__ + ":" + std::to_string(__LINE__));                        \
            return GB_ERR_CUDA;                                                                \
        }                                                                                      \
    } while (0)
