// Model intake, FP64 reductions and the Gaussian gradient filter.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "gb_internal.h"
#include "gbfwi.h"

namespace gb {

// ------------------------------------------------------------ model intake
__global__ void k_fill(float *p, float v, size_t n) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) p[k] = v;
}

cudaError_t launch_fill(float *p, float v, size_t n, cudaStream_t st) {
    if (!n) return cudaSuccess;
    k_fill<<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, st>>>(p, v, n);
    return cudaGetLastError();
}

// mesh2grid (solver/fdm.h:4-24): nearest model point for each cell, strict
// "<" so the first of equally near points wins; the search starts from
// dmax = xmax^2 + zmax^2. The points are staged through shared memory in
// chunks; every thread scans them in index order, as the reference does.
__global__ void k_mesh2grid(float *lambda, float *mu, float *rho, const float *__restrict__ px,
                            const float *__restrict__ pz, const float *__restrict__ pa, const float *__restrict__ pb,
                            const float *__restrict__ pr, int npt, float dmax, float dx, float dz, int nx, int nz) {
    __shared__ float sx[256], sz[256];
    const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const bool valid = k < (size_t)nx * nz;
    const int i = valid ? (int)(k / nz) : 0, j = valid ? (int)(k % nz) : 0;
    const float x = i * dx, z = j * dz;
    float dmin = dmax;
    int best = -1;
    for (int base = 0; base < npt; base += 256) {
        const int l = base + threadIdx.x;
        if (l < npt) {
            sx[threadIdx.x] = px[l];
            sz[threadIdx.x] = pz[l];
        }
        __syncthreads();
        const int m = min(256, npt - base);
        for (int q = 0; q < m; q++) {
            const float ddx = x - sx[q], ddz = z - sz[q];
            const float d = ddx * ddx + ddz * ddz;
            if (d < dmin) {
                dmin = d;
                best = base + q;
            }
        }
        __syncthreads();
    }
    if (valid && best >= 0) {
        lambda[k] = pa[best];
        mu[k] = pb[best];
        rho[k] = pr[best];
    }
}

cudaError_t launch_mesh2grid(float *lambda, float *mu, float *rho, const float *px, const float *pz, const float *pa,
                             const float *pb, const float *pr, int npt, float dmax, float dx, float dz, int nx,
                             int nz, cudaStream_t st) {
    const size_t n = (size_t)nx * nz;
    k_mesh2grid<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(lambda, mu, rho, px, pz, pa, pb, pr, npt, dmax, dx, dz,
                                                             nx, nz);
    return cudaGetLastError();
}

// out = 1/in rounded to nearest (the factor of dt*ds/rho in the velocity
// update, solver/fdm.h:150-161); refreshed before each pass because the
// model may change between passes.
__global__ void k_reciprocal(float *out, const float *in, size_t n) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        out[k] = __frcp_rn(in[k]);
}

cudaError_t launch_reciprocal(float *out, const float *in, size_t n, cudaStream_t st) {
    if (!n) return cudaSuccess;
    k_reciprocal<<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, st>>>(out, in, n);
    return cudaGetLastError();
}

// vps2lm (solver/fdm.h:25-36), in place.
__global__ void k_vps2lm(float *lambda, float *mu, const float *rho, size_t n) {
    const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float vp = lambda[k], vs = mu[k], r = rho[k];
    lambda[k] = vp > vs ? r * (vp * vp - 2 * vs * vs) : 0.f;
    mu[k] = r * vs * vs;
}

cudaError_t launch_vps2lm(float *lambda, float *mu, const float *rho, size_t n, cudaStream_t st) {
    if (!n) return cudaSuccess;
    k_vps2lm<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(lambda, mu, rho, n);
    return cudaGetLastError();
}

// lm2vps (solver/fdm.h:37-43), in place.
__global__ void k_lm2vps(float *vp, float *vs, const float *rho, size_t n) {
    const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float l = vp[k], m = vs[k], r = rho[k];
    vp[k] = sqrtf((l + 2 * m) / r);
    vs[k] = sqrtf(m / r);
}

cudaError_t launch_lm2vps(float *vp, float *vs, const float *rho, size_t n, cudaStream_t st) {
    if (!n) return cudaSuccess;
    k_lm2vps<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(vp, vs, rho, n);
    return cudaGetLastError();
}

// c = ka*a + kb*b (device::calc, lib/device.h:157-176); b may be null.
__global__ void k_axpby(float *c, float ka, const float *a, float kb, const float *b, size_t n) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        c[k] = b ? ka * a[k] + kb * b[k] : ka * a[k];
}

cudaError_t launch_axpby(float *c, float ka, const float *a, float kb, const float *b, size_t n, cudaStream_t st) {
    if (!n) return cudaSuccess;
    k_axpby<<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, st>>>(c, ka, a, kb, b, n);
    return cudaGetLastError();
}

// ------------------------------------------------------------ reductions
// FP64 dot and max|.| over float arrays: grid-stride partial sums per
// block (warp shuffles), then one block adds the partials in index order, so
// results do not depend on scheduling.
constexpr int kRedBlocks = 608;  // 4 x 152 SMs
int reduce_partials() { return kRedBlocks; }

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
    for (int o = 16; o; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

template <bool MAX>
__global__ void k_reduce(const float *__restrict__ a, const float *__restrict__ b, size_t n, double *partial) {
    __shared__ double red[32];
    double acc = 0.0;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        if (MAX)
            acc = fmax(acc, fabs((double)a[k]));
        else
            acc += (double)a[k] * (double)b[k];
    }
    acc = MAX ? warp_max(acc) : warp_sum(acc);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        v = MAX ? warp_max(v) : warp_sum(v);
        if (threadIdx.x == 0) partial[blockIdx.x] = v;
    }
}

template <bool MAX>
__global__ void k_reduce_final(const double *partial, int np, double *out) {
    __shared__ double red[32];
    double acc = 0.0;
    for (int k = threadIdx.x; k < np; k += blockDim.x) acc = MAX ? fmax(acc, partial[k]) : acc + partial[k];
    acc = MAX ? warp_max(acc) : warp_sum(acc);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        v = MAX ? warp_max(v) : warp_sum(v);
        if (threadIdx.x == 0) *out = v;
    }
}

cudaError_t launch_dot(const float *a, const float *b, size_t n, double *partial, double *d_out, cudaStream_t st) {
    k_reduce<false><<<kRedBlocks, 256, 0, st>>>(a, b, n, partial);
    k_reduce_final<false><<<1, 1024, 0, st>>>(partial, kRedBlocks, d_out);
    return cudaGetLastError();
}

cudaError_t launch_amax(const float *a, size_t n, double *partial, double *d_out, cudaStream_t st) {
    k_reduce<true><<<kRedBlocks, 256, 0, st>>>(a, nullptr, n, partial);
    k_reduce_final<true><<<1, 1024, 0, st>>>(partial, kRedBlocks, d_out);
    return cudaGetLastError();
}

// ------------------------------------------------------------ filter
// GaussianFilter (filter/gaussian.h:4-56). The reference evaluates the
// weight through a size_t argument built as (int i) - (size_t n); for n > i it
// wraps to about 1.8e19, whose square overflows to inf in float, so those
// weights are exactly 0 and the smoothing is one-sided:
//   tmp[i,j]  = sum_{n <= i} g(i-n) data[n,j]
//   data[i,j] = sum_{n <= j} g(j-n) tmp[i,n] / (Sx(i) Sz(j)),
//   Sx(i) = sum_{n <= i} g(i-n).
// The weights are computed on the device with the reference's expression; a
// term whose weight is exactly 0 changes no sum, so each sum starts at the
// first index whose weight is nonzero and keeps the reference's order
// (ascending n, one fused multiply-add per term).
__global__ void k_gauss_weights(float *w, int m, int sigma) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= m) return;
    const float pi = 3.1415927f;
    const float xf = (float)x, sigmaf = (float)sigma;
    w[x] = (1 / (sqrtf(2 * pi) * sigmaf)) * expf(-xf * xf / (2 * sigmaf * sigmaf));
}

// The cutoff m = 1 + the index of the last nonzero weight (at least 1): the
// value gb_filter_create reads back to the host, here written to device
// memory for the allocation-free path.
__global__ void k_gauss_cutoff(const float *w, int len, int *m_out) {
    __shared__ int last;
    if (threadIdx.x == 0) last = 1;
    __syncthreads();
    for (int x = threadIdx.x; x < len; x += blockDim.x)
        if (w[x] != 0.f) atomicMax(&last, x + 1);
    __syncthreads();
    if (threadIdx.x == 0) *m_out = last;
}

// The filter kernels below take the cutoff m by value, or from device memory
// when m_dev is not null.

// Partial sums S(i) = sum_{n=0}^{i} g(i-n), added in ascending n.
__global__ void k_gauss_norm(const float *w, int m, float *s, int len, const int *m_dev) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= len) return;
    if (m_dev) m = *m_dev;
    float acc = 0.f;
    for (int n = max(0, i - m + 1); n <= i; n++) acc += w[i - n];
    s[i] = acc;
}

// X pass: tmp[i,j] = sum_n g(i-n) data[n,j]; thread per cell, consecutive
// threads along z (coalesced).
__global__ void k_gauss_x(const float *__restrict__ data, float *__restrict__ tmp, const float *__restrict__ w, int m,
                          int nx, int nz, const int *m_dev) {
    const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (k >= (size_t)nx * nz) return;
    if (m_dev) m = *m_dev;
    const int i = (int)(k / nz), j = (int)(k - (size_t)i * nz);
    float acc = 0.f;
    for (int n = max(0, i - m + 1); n <= i; n++) acc = fmaf(__ldg(w + i - n), __ldg(data + (size_t)n * nz + j), acc);
    tmp[k] = acc;
}

// Z pass with the normalisation.
__global__ void k_gauss_z(float *__restrict__ data, const float *__restrict__ tmp, const float *__restrict__ w, int m,
                          const float *__restrict__ sx, const float *__restrict__ sz, int nx, int nz,
                          const int *m_dev) {
    const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (k >= (size_t)nx * nz) return;
    if (m_dev) m = *m_dev;
    const int i = (int)(k / nz), j = (int)(k - (size_t)i * nz);
    const float *row = tmp + (size_t)i * nz;
    float acc = 0.f;
    for (int n = max(0, j - m + 1); n <= j; n++) acc = fmaf(__ldg(w + j - n), __ldg(row + n), acc);
    data[k] = acc / (sx[i] * sz[j]);
}

}  // namespace gb

// ------------------------------------------------------------ C ABI: filter
struct gb_filter {
    int nx = 0, nz = 0, sigma = 0, m = 0;
    float *w = nullptr, *sx = nullptr, *sz = nullptr, *tmp = nullptr;
    cudaStream_t st = nullptr;
};

extern "C" {

gb_filter *gb_filter_create(int nx, int nz, int sigma) {
    if (nx < 1 || nz < 1 || sigma < 1) {
        gb::set_error("gb_filter_create: nx, nz and sigma must be positive");
        return nullptr;
    }
    gb_filter *f = new gb_filter();
    f->nx = nx;
    f->nz = nz;
    f->sigma = sigma;
    const int len = std::max(nx, nz);
    cudaError_t e = cudaStreamCreateWithFlags(&f->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&f->w, (size_t)len * 4);
    if (e == cudaSuccess) e = cudaMalloc(&f->sx, (size_t)nx * 4);
    if (e == cudaSuccess) e = cudaMalloc(&f->sz, (size_t)nz * 4);
    if (e == cudaSuccess) e = cudaMalloc(&f->tmp, (size_t)nx * nz * 4);
    if (e == cudaSuccess) {
        gb::k_gauss_weights<<<(len + 255) / 256, 256, 0, f->st>>>(f->w, len, sigma);
        e = cudaGetLastError();
    }
    std::vector<float> hw(len);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hw.data(), f->w, (size_t)len * 4, cudaMemcpyDeviceToHost, f->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(f->st);
    if (e != cudaSuccess) {
        gb::set_error(std::string("gb_filter_create: ") + cudaGetErrorString(e));
        gb_filter_destroy(f);
        return nullptr;
    }
    // weights beyond the last nonzero one are exactly 0 in float
    int m = len;
    while (m > 1 && hw[m - 1] == 0.f) m--;
    f->m = m;
    gb::k_gauss_norm<<<(nx + 255) / 256, 256, 0, f->st>>>(f->w, m, f->sx, nx, nullptr);
    gb::k_gauss_norm<<<(nz + 255) / 256, 256, 0, f->st>>>(f->w, m, f->sz, nz, nullptr);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(f->st);
    if (e != cudaSuccess) {
        gb::set_error(std::string("gb_filter_create: ") + cudaGetErrorString(e));
        gb_filter_destroy(f);
        return nullptr;
    }
    return f;
}

int gb_filter_apply(gb_filter *f, float *d_data) {
    if (!f || !d_data) {
        gb::set_error("gb_filter_apply: null argument");
        return GB_ERR_ARG;
    }
    const size_t n = (size_t)f->nx * f->nz;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    gb::k_gauss_x<<<blocks, 256, 0, f->st>>>(d_data, f->tmp, f->w, f->m, f->nx, f->nz, nullptr);
    gb::k_gauss_z<<<blocks, 256, 0, f->st>>>(d_data, f->tmp, f->w, f->m, f->sx, f->sz, f->nx, f->nz, nullptr);
    GB_CUDA_TRY(cudaGetLastError());
    GB_CUDA_TRY(cudaStreamSynchronize(f->st));
    return GB_OK;
}

void gb_filter_destroy(gb_filter *f) {
    if (!f) return;
    if (f->st) cudaStreamSynchronize(f->st);
    cudaFree(f->w);
    cudaFree(f->sx);
    cudaFree(f->sz);
    cudaFree(f->tmp);
    if (f->st) cudaStreamDestroy(f->st);
    delete f;
}

// ------------------------------------------------------------ C ABI: filter
// without allocation (gb_filter_apply_noalloc)
namespace {

// Scratch of the allocation-free filter: the x-pass result, the weights,
// the partial-sum profiles and the weight cutoff. Reserved on every device
// that loads the library for the life of the process (16 MiB + 96 KiB).
// Every call writes each element it later reads (the cutoff included) before
// reading it, so nothing needs clearing between calls.
static __device__ __align__(256) float g_na_tmp[GB_NOALLOC_MAX_CELLS];
static __device__ __align__(256) float g_na_w[GB_NOALLOC_MAX_SIDE];
static __device__ __align__(256) float g_na_sx[GB_NOALLOC_MAX_SIDE];
static __device__ __align__(256) float g_na_sz[GB_NOALLOC_MAX_SIDE];
static __device__ __align__(256) int g_na_m[1];

// Device addresses of the arrays above, looked up once per device. In host
// code the array names are host-side stand-ins, never device addresses.
struct NoAllocAddr {
    float *tmp = nullptr, *w = nullptr, *sx = nullptr, *sz = nullptr;
    int *m = nullptr;
    bool ready = false;
};
constexpr int kNoAllocDevices = 64;
NoAllocAddr g_na_addr[kNoAllocDevices];
std::mutex g_na_mutex;

int noalloc_addresses(NoAllocAddr *out) {
    int dev = 0;
    GB_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocDevices) {
        gb::set_error("gb_filter_apply_noalloc: device index out of range");
        return GB_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_na_mutex);
    NoAllocAddr &a = g_na_addr[dev];
    if (!a.ready) {
        GB_CUDA_TRY(cudaGetSymbolAddress((void **)&a.tmp, g_na_tmp));
        GB_CUDA_TRY(cudaGetSymbolAddress((void **)&a.w, g_na_w));
        GB_CUDA_TRY(cudaGetSymbolAddress((void **)&a.sx, g_na_sx));
        GB_CUDA_TRY(cudaGetSymbolAddress((void **)&a.sz, g_na_sz));
        GB_CUDA_TRY(cudaGetSymbolAddress((void **)&a.m, g_na_m));
        a.ready = true;
    }
    *out = a;
    return GB_OK;
}

}  // namespace

extern "C" int gb_filter_apply_noalloc(int nx, int nz, int sigma, float *d_data) {
    if (!d_data || nx < 1 || nz < 1 || sigma < 1) {
        gb::set_error("gb_filter_apply_noalloc: need a device array and positive nx, nz, sigma");
        return GB_ERR_ARG;
    }
    if ((long long)nx * nz > GB_NOALLOC_MAX_CELLS || std::max(nx, nz) > GB_NOALLOC_MAX_SIDE) {
        gb::set_error("gb_filter_apply_noalloc: grid " + std::to_string(nx) + " x " + std::to_string(nz) +
                      " exceeds the fixed scratch (at most " + std::to_string(GB_NOALLOC_MAX_CELLS) +
                      " cells and " + std::to_string(GB_NOALLOC_MAX_SIDE) +
                      " per side); use gb_filter_create / gb_filter_apply");
        return GB_ERR_ARG;
    }
    NoAllocAddr a;
    int rc = noalloc_addresses(&a);
    if (rc) return rc;
    const int len = std::max(nx, nz);
    const size_t n = (size_t)nx * nz;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    // The weights, then the cutoff gb_filter_create uses (the last nonzero
    // weight), found on the device and read there by the filter kernels, so
    // both entry points sum exactly the same terms.
    gb::k_gauss_weights<<<(len + 255) / 256, 256>>>(a.w, len, sigma);
    gb::k_gauss_cutoff<<<1, 256>>>(a.w, len, a.m);
    gb::k_gauss_norm<<<(nx + 255) / 256, 256>>>(a.w, len, a.sx, nx, a.m);
    gb::k_gauss_norm<<<(nz + 255) / 256, 256>>>(a.w, len, a.sz, nz, a.m);
    gb::k_gauss_x<<<blocks, 256>>>(d_data, a.tmp, a.w, len, nx, nz, a.m);
    gb::k_gauss_z<<<blocks, 256>>>(d_data, a.tmp, a.w, len, a.sx, a.sz, nx, nz, a.m);
    GB_CUDA_TRY(cudaGetLastError());
    GB_CUDA_TRY(cudaStreamSynchronize(0));
    return GB_OK;
}

// ------------------------------------------------------------ C ABI: misc
int gb_dot64(const float *d_a, const float *d_b, size_t n, double *out) {
    if (!d_a || !d_b || !out) return GB_ERR_ARG;
    double *buf;
    GB_CUDA_TRY(cudaMalloc(&buf, (gb::reduce_partials() + 1) * sizeof(double)));
    cudaError_t e = gb::launch_dot(d_a, d_b, n, buf, buf + gb::reduce_partials(), 0);
    if (e == cudaSuccess) e = cudaMemcpy(out, buf + gb::reduce_partials(), sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(buf);
    GB_CUDA_TRY(e);
    return GB_OK;
}

int gb_amax64(const float *d_a, size_t n, double *out) {
    if (!d_a || !out) return GB_ERR_ARG;
    double *buf;
    GB_CUDA_TRY(cudaMalloc(&buf, (gb::reduce_partials() + 1) * sizeof(double)));
    cudaError_t e = gb::launch_amax(d_a, n, buf, buf + gb::reduce_partials(), 0);
    if (e == cudaSuccess) e = cudaMemcpy(out, buf + gb::reduce_partials(), sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(buf);
    GB_CUDA_TRY(e);
    return GB_OK;
}

void *gb_device_malloc(size_t bytes) {
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes ? bytes : 1);
    if (e != cudaSuccess) {
        gb::set_error(std::string("gb_device_malloc: ") + cudaGetErrorString(e));
        return nullptr;
    }
    return p;
}
int gb_device_free(void *d_ptr) {
    GB_CUDA_TRY(cudaFree(d_ptr));
    return GB_OK;
}
int gb_memcpy_d2h(void *dst, const void *src, size_t bytes) {
    GB_CUDA_TRY(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
    return GB_OK;
}
int gb_memcpy_h2d(void *dst, const void *src, size_t bytes) {
    GB_CUDA_TRY(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
    return GB_OK;
}
int gb_device_sync(void) {
    GB_CUDA_TRY(cudaDeviceSynchronize());
    return GB_OK;
}
void *gb_host_malloc(size_t bytes) {
    void *p = nullptr;
    cudaError_t e = cudaMallocHost(&p, bytes ? bytes : 1);
    if (e != cudaSuccess) {
        gb::set_error(std::string("gb_host_malloc: ") + cudaGetErrorString(e));
        return nullptr;
    }
    return p;
}
int gb_host_free(void *h_ptr) {
    GB_CUDA_TRY(cudaFreeHost(h_ptr));
    return GB_OK;
}
int gb_device_select(int device) {
    GB_CUDA_TRY(cudaSetDevice(device));
    return GB_OK;
}
int gb_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}

}  // extern "C"
