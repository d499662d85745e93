// md_static.cu -- an allocation-free variant of the FP64 single-centre LJ
// force evaluation, for callers that cannot allocate device memory.
//
// Some callers of this library must not call cudaMalloc (or any allocating
// routine, torch's caching allocator included): code that records its work
// into a CUDA graph owned by a larger application, host programs whose device
// memory is handed out by their own pool manager, and real-time or embedded
// drivers that forbid allocation after start-up.  For them
// md_forces_lj_noalloc computes the forces, Upot and virial of a periodic
// box of single-centre LJ molecules from device arrays the caller owns, using
// as scratch only the file-scope device array below.
//
// Scratch: one static __device__ array of MD_NOALLOC_SCRATCH_BYTES (about
// 1.9 MB) that every GPU loading this library keeps until the process exits.
// It bounds the problem: at most MD_NOALLOC_MAX_N molecules and
// MD_NOALLOC_MAX_CELLS linked cells.  Every call shares the array and it keeps
// the previous call's contents; the cell counters are cleared by each call.
// Calls whose work overlaps on the GPU (different streams, or another thread
// calling concurrently) race on the array and must be serialised by the
// caller.
//
// Set-up: the first call on a device (with that device current) looks up the
// device address of the array with cudaGetSymbolAddress and caches it for
// that device together with the device's current context; make that first
// call before any stream capture.  A call that finds another context current
// (the host program reset the device or replaced its primary context) looks
// the address up again, so that call too should come before any capture.
#include <cstdint>
#include <mutex>

#include <cuda.h>
#include <cuda_runtime.h>

#include "../../include/ls1gb300.h"

#define NA_MAX_DEVICES 64
#define NA_PARTIAL_SLOTS 2

namespace {

constexpr int64_t kMaxN = MD_NOALLOC_MAX_N;
constexpr int kMaxCells = MD_NOALLOC_MAX_CELLS;
constexpr int64_t kMaxWarps = kMaxN / 32 + 8;

// scratch layout (bytes): counts | starts | cursor | cell of molecule | perm | partials
constexpr size_t kCountsOff = 0;
constexpr size_t kStartsOff = kCountsOff + sizeof(int) * (kMaxCells + 1);
constexpr size_t kCursorOff = kStartsOff + sizeof(int) * (kMaxCells + 1);
constexpr size_t kCellOff = kCursorOff + sizeof(int) * (kMaxCells + 1);
constexpr size_t kPermOff = kCellOff + sizeof(int) * kMaxN;
constexpr size_t kPartOff = (kPermOff + sizeof(int) * kMaxN + 255) / 256 * 256;
constexpr size_t kScratchBytes = kPartOff + sizeof(double) * NA_PARTIAL_SLOTS * kMaxWarps;
static_assert(kScratchBytes <= MD_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the stated size");

}  // namespace

// The scratch array.  In host code this name is only a stand-in: kernels get
// its device address from cudaGetSymbolAddress (see na_scratch_for_device).
static __device__ __align__(256) unsigned char g_md_noalloc_scratch[MD_NOALLOC_SCRATCH_BYTES];

namespace {

std::mutex g_na_mutex;
unsigned char* g_na_ptr[NA_MAX_DEVICES] = {nullptr};
unsigned long long g_na_ctx_id[NA_MAX_DEVICES] = {0};  // context the cached address belongs to

// The driver's cuCtxGetCurrent and cuCtxGetId, fetched through the runtime
// (no link-time dependency on libcuda).  A context's id is unique for the
// life of the process, unlike its handle, which a re-created context may
// reuse.
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

cudaError_t na_driver_fn(const char* name, void** fn) {
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion(name, fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess) return e;
    return q == cudaDriverEntryPointSuccess && *fn ? cudaSuccess : cudaErrorNotSupported;
}

// id of the context current on this thread, 0 if there is none
unsigned long long na_current_ctx_id() {
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
    if (g_ctx_get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of the scratch array on the current device: looked up on
// the first call and again whenever the current context is not the one the
// cached address was taken in (a device reset invalidates the address).
// cudaGetSymbolAddress also makes the device's primary context current when
// none is.
cudaError_t na_scratch_for_device(unsigned char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= NA_MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_ctx_get_current) {
        void *f1 = nullptr, *f2 = nullptr;
        if ((e = na_driver_fn("cuCtxGetCurrent", &f1)) != cudaSuccess) return e;
        if ((e = na_driver_fn("cuCtxGetId", &f2)) != cudaSuccess) return e;
        g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f2);
        g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
    }
    const unsigned long long id = g_na_ptr[dev] ? na_current_ctx_id() : 0;
    if (!g_na_ptr[dev] || id == 0 || id != g_na_ctx_id[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_md_noalloc_scratch);
        if (e != cudaSuccess) return e;
        const unsigned long long now = na_current_ctx_id();
        if (now == 0) return cudaErrorDeviceUninitialized;
        g_na_ptr[dev] = static_cast<unsigned char*>(p);
        g_na_ctx_id[dev] = now;
    }
    *out = g_na_ptr[dev];
    return cudaSuccess;
}

struct NaGrid {
    int n[3];
    double L[3], inv[3];
};

__device__ __forceinline__ int na_cell(const NaGrid& g, const double* r) {
    int c[3];
    for (int d = 0; d < 3; ++d) {
        // periodic image into [0, L) for binning only
        double x = r[d] - floor(r[d] / g.L[d]) * g.L[d];
        int k = (int)(x * g.inv[d]);
        c[d] = k < 0 ? 0 : (k >= g.n[d] ? g.n[d] - 1 : k);
    }
    return (c[2] * g.n[1] + c[1]) * g.n[0] + c[0];
}

__global__ void na_clear(int* counts, int ncells) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i <= ncells) counts[i] = 0;
}

__global__ void na_count(const double* r, int n, NaGrid g, int* cell, int* counts) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c = na_cell(g, r + 3 * (size_t)i);
    cell[i] = c;
    atomicAdd(&counts[c], 1);
}

__global__ void na_scan(const int* counts, int* starts, int* cursor, int ncells) {
    __shared__ int sh[1024];
    int per = (ncells + blockDim.x - 1) / blockDim.x;
    int b = threadIdx.x * per, e = min(ncells, b + per);
    int s = 0;
    for (int k = b; k < e; ++k) s += counts[k];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int off = 1; off < blockDim.x; off <<= 1) {
        int v = threadIdx.x >= off ? sh[threadIdx.x - off] : 0;
        __syncthreads();
        sh[threadIdx.x] += v;
        __syncthreads();
    }
    int run = sh[threadIdx.x] - s;
    for (int k = b; k < e; ++k) {
        starts[k] = run;
        cursor[k] = run;
        run += counts[k];
    }
    if (threadIdx.x == blockDim.x - 1) starts[ncells] = sh[threadIdx.x];
}

__global__ void na_scatter(const int* cell, int n, int* cursor, int* perm) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    perm[atomicAdd(&cursor[cell[i]], 1)] = i;
}

// order inside each cell by molecule index (deterministic summation order)
__global__ void na_sort(const int* starts, int ncells, int* perm) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    int b = starts[c], e = starts[c + 1];
    for (int k = b + 1; k < e; ++k) {
        int v = perm[k];
        int q = k - 1;
        while (q >= b && perm[q] > v) { perm[q + 1] = perm[q]; --q; }
        perm[q + 1] = v;
    }
}

// Owner-computes FP64 LJ over the 27 neighbour cells with minimum-image
// shifts (the reference's halo copies r_j +- L): force on i, and Upot/virial
// counted once per pair (on the side with the smaller index).
__global__ void na_force(const double* r, int n, NaGrid g, double rc2, double eps24, double sig2, double shift6,
                         const int* cell, const int* starts, const int* perm, double* F, double* partials,
                         int pstride) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double fx = 0, fy = 0, fz = 0, u6 = 0, vir = 0;
    if (i < n) {
        const double ri[3] = {r[3 * (size_t)i], r[3 * (size_t)i + 1], r[3 * (size_t)i + 2]};
        const int ci = cell[i];
        const int cc[3] = {ci % g.n[0], (ci / g.n[0]) % g.n[1], ci / (g.n[0] * g.n[1])};
        for (int oz = -1; oz <= 1; ++oz)
            for (int oy = -1; oy <= 1; ++oy)
                for (int ox = -1; ox <= 1; ++ox) {
                    const int o[3] = {ox, oy, oz};
                    int nc[3];
                    double sh[3];
                    for (int d = 0; d < 3; ++d) {
                        nc[d] = cc[d] + o[d];
                        sh[d] = 0.0;
                        if (nc[d] < 0) { nc[d] += g.n[d]; sh[d] = -g.L[d]; }
                        else if (nc[d] >= g.n[d]) { nc[d] -= g.n[d]; sh[d] = g.L[d]; }
                    }
                    const int c = (nc[2] * g.n[1] + nc[1]) * g.n[0] + nc[0];
                    for (int k = starts[c]; k < starts[c + 1]; ++k) {
                        const int j = perm[k];
                        if (j == i) continue;
                        // positions may lie outside [0, L): take the image nearest to the cell image
                        double d[3];
                        for (int e = 0; e < 3; ++e) {
                            double xj = r[3 * (size_t)j + e];
                            double wrap = floor(xj / g.L[e]) * g.L[e];
                            double xi = ri[e] - floor(ri[e] / g.L[e]) * g.L[e];
                            d[e] = xi - ((xj - wrap) + sh[e]);
                        }
                        const double r2 = d[0] * d[0] + (d[1] * d[1] + d[2] * d[2]);
                        if (!(r2 < rc2)) continue;
                        const double r2inv = 1.0 / r2;
                        const double lj2 = sig2 * r2inv, lj6 = lj2 * lj2 * lj2, lj12 = lj6 * lj6;
                        const double lj12m6 = lj12 - lj6;
                        const double scale = eps24 * r2inv * (lj12 + lj12m6);
                        fx += d[0] * scale;
                        fy += d[1] * scale;
                        fz += d[2] * scale;
                        if (j > i) {
                            u6 += eps24 * lj12m6 + shift6;
                            vir += (d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) * scale;
                        }
                    }
                }
        F[3 * (size_t)i] = fx;
        F[3 * (size_t)i + 1] = fy;
        F[3 * (size_t)i + 2] = fz;
    }
    for (int o = 16; o > 0; o >>= 1) {
        u6 += __shfl_down_sync(0xffffffffu, u6, o);
        vir += __shfl_down_sync(0xffffffffu, vir, o);
    }
    if ((threadIdx.x & 31) == 0) {
        int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
        partials[w] = u6;
        partials[pstride + w] = vir;
    }
}

// fixed-order sum of the warp partials: out[0] = Upot = sum u6 / 6, out[1] = virial
__global__ void na_finish(const double* partials, int pstride, int nwarps, double* out) {
    __shared__ double sh[2][32];
    double a = 0, b = 0;
    for (int k = threadIdx.x; k < nwarps; k += blockDim.x) {
        a += partials[k];
        b += partials[pstride + k];
    }
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0) { sh[0][threadIdx.x >> 5] = a; sh[1][threadIdx.x >> 5] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s0 = 0, s1 = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { s0 += sh[0][w]; s1 += sh[1][w]; }
        out[0] = s0 / 6.0;
        out[1] = s1;
    }
}

}  // namespace

extern "C" int md_forces_lj_noalloc(const double* d_r, int64_t n, const double box[3], double rc, double eps,
                                    double sigma, double shift6, double* d_F, double* d_upot_virial,
                                    void* stream) {
    if (!d_r || !d_F || !d_upot_virial || !box || n < 1 || !(rc > 0) || !(sigma > 0)) return MD_ERR_ARG;
    if (n > kMaxN) return MD_ERR_CAPACITY;  // more molecules than the static scratch holds
    NaGrid g;
    int64_t ncells = 1;
    for (int d = 0; d < 3; ++d) {
        if (!(box[d] > 0)) return MD_ERR_ARG;
        const double q = box[d] / rc;  // cells of edge >= rc along this axis (before truncation)
        // more cells on one axis than the scratch holds in total (checked before the conversion to int,
        // which would overflow for a very dilute box)
        if (!(q < (double)kMaxCells + 1.0)) return MD_ERR_CAPACITY;
        g.n[d] = (int)q;
        if (g.n[d] < 3) return MD_ERR_UNSUPPORTED;  // needs at least three cells of edge >= rc per axis
        g.L[d] = box[d];
        g.inv[d] = g.n[d] / box[d];
        ncells *= g.n[d];  // <= kMaxCells^2 after any factor: no overflow
        if (ncells > kMaxCells) return MD_ERR_CAPACITY;  // more cells than the static scratch holds
    }
    unsigned char* base = nullptr;
    if (na_scratch_for_device(&base) != cudaSuccess) return MD_ERR_CUDA;
    int* counts = reinterpret_cast<int*>(base + kCountsOff);
    int* starts = reinterpret_cast<int*>(base + kStartsOff);
    int* cursor = reinterpret_cast<int*>(base + kCursorOff);
    int* cell = reinterpret_cast<int*>(base + kCellOff);
    int* perm = reinterpret_cast<int*>(base + kPermOff);
    double* partials = reinterpret_cast<double*>(base + kPartOff);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int nc = (int)ncells, nn = (int)n, T = 256;
    const int nb = (nn + T - 1) / T;
    // LJ pair parameters of one centre type (Comp2Param, same component)
    const double eps24 = 24. * eps;
    double sig2 = sigma;
    sig2 *= sig2;
    na_clear<<<(nc + 1 + T - 1) / T, T, 0, s>>>(counts, nc);
    na_count<<<nb, T, 0, s>>>(d_r, nn, g, cell, counts);
    na_scan<<<1, 1024, 0, s>>>(counts, starts, cursor, nc);
    na_scatter<<<nb, T, 0, s>>>(cell, nn, cursor, perm);
    na_sort<<<(nc + T - 1) / T, T, 0, s>>>(starts, nc, perm);
    na_force<<<nb, T, 0, s>>>(d_r, nn, g, rc * rc, eps24, sig2, shift6, cell, starts, perm, d_F, partials,
                              (int)kMaxWarps);
    na_finish<<<1, 1024, 0, s>>>(partials, (int)kMaxWarps, nb * (T / 32), d_upot_virial);
    return cudaGetLastError() == cudaSuccess ? MD_OK : MD_ERR_CUDA;
}
