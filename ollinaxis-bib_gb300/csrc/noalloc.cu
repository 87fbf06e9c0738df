// 0-D statistics of a caller-owned device grid function without any device
// allocation (ollin_gpu_norms_noalloc).
//
// Who needs it: callers that cannot call cudaMalloc -- a Fortran host that
// hands over arrays from its own CUDA allocator or from a memory pool it
// manages and must not have a second allocator carve device memory beside
// it, a region where an allocation would synchronise the device, or tools
// that may only read memory.  They own the field and the 5-number result; the
// reduction's intermediate results live in a fixed-size array that is part
// of this library's device image, reserved when the library is loaded and
// held by every GPU that loads it until the process exits.
//
// The origin value is the 4x4 bicubic interpolation of save0Dvariable with
// interporder = "bicubic" (the reference's default); with "bilinear" the
// fifth number differs from the reference's, the other four do not.
//
// The statistics are those of save0Dvariable (src/base/save0Ddata.f90:221-288,
// origin value at :370-374), computed in two fixed-order passes so that the
// result does not depend on scheduling: one block per interior z-row reduces
// that row into the scratch array, then one block reduces the rows in order.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>

#include "../../include/ollin_gpu.h"

namespace {

// Largest number of interior z-rows (Nz - ghost) one call can reduce.
constexpr int kMaxRows = 8192;
// Per row: max, min, max|f|, sum f^2, NaN flag; then the final 6 values.
constexpr int kRowSlots = 5;

// The scratch: 8192 x 5 + 8 doubles = 320 KiB per GPU.  Device code could
// name it directly; host code only ever passes the address returned by
// cudaGetSymbolAddress.
static __device__ __align__(256) double g_norms_scratch[kMaxRows * kRowSlots + 8];

constexpr int kMaxDevices = 64;
double* g_scratch_addr[kMaxDevices] = {};
std::mutex g_setup_mutex;

__device__ double rcoord(int i, double h) { return ((double)(0 + i) - 0.5) * h; }

// pass 1: one block per interior row j = 1..nz-ghost
__global__ void __launch_bounds__(256) rows_kernel(const double* __restrict__ f, int nr, int g, long ld, double* scratch) {
    __shared__ double smax[256], smin[256], snm1[256], snm2[256];
    __shared__ int snan[256];
    const int j = 1 + (int)blockIdx.x;
    const int ni = nr - g;
    double vmax = -1.0e10, vmin = 1.0e10, nm1 = 0.0, nm2 = 0.0;
    int nan = 0;
    // f points at element (1-g, 1-g)
    const double* row = f + (size_t)(j - 1 + g) * ld + (g - 1);
    for (int i = 1 + (int)threadIdx.x; i <= ni; i += blockDim.x) {
        const double v = row[i];
        if (v != v) nan = 1;
        vmax = fmax(vmax, v);
        vmin = fmin(vmin, v);
        nm1 = fmax(nm1, fabs(v));
        nm2 = nm2 + v * v;
    }
    smax[threadIdx.x] = vmax; smin[threadIdx.x] = vmin; snm1[threadIdx.x] = nm1; snm2[threadIdx.x] = nm2;
    snan[threadIdx.x] = nan;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + w]);
            smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + w]);
            snm1[threadIdx.x] = fmax(snm1[threadIdx.x], snm1[threadIdx.x + w]);
            snm2[threadIdx.x] = snm2[threadIdx.x] + snm2[threadIdx.x + w];
            snan[threadIdx.x] |= snan[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double* s = scratch + (size_t)(j - 1) * kRowSlots;
        s[0] = smax[0]; s[1] = smin[0]; s[2] = snm1[0]; s[3] = snm2[0]; s[4] = snan[0] ? 1.0 : 0.0;
    }
}

// pass 2: the rows in order, then the bicubic value at the origin
// (interp.f90:146-263 at r0 = z0 = 0, which lies one cell from the axis and
// the equator and uses the 4x4 stencil).
__global__ void __launch_bounds__(256) final_kernel(const double* __restrict__ f, int nr, int nz, int g, long ld,
                                                    double dr, double dz, double* scratch) {
    __shared__ double smax[256], smin[256], snm1[256], snm2[256];
    __shared__ int snan[256];
    const int nrows = nz - g;
    double vmax = -1.0e10, vmin = 1.0e10, nm1 = 0.0, nm2 = 0.0;
    int nan = 0;
    for (int k = threadIdx.x; k < nrows; k += blockDim.x) {
        const double* s = scratch + (size_t)k * kRowSlots;
        vmax = fmax(vmax, s[0]);
        vmin = fmin(vmin, s[1]);
        nm1 = fmax(nm1, s[2]);
        nm2 = nm2 + s[3];
        nan |= (s[4] != 0.0);
    }
    smax[threadIdx.x] = vmax; smin[threadIdx.x] = vmin; snm1[threadIdx.x] = nm1; snm2[threadIdx.x] = nm2;
    snan[threadIdx.x] = nan;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + w]);
            smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + w]);
            snm1[threadIdx.x] = fmax(snm1[threadIdx.x], snm1[threadIdx.x + w]);
            snm2[threadIdx.x] = snm2[threadIdx.x] + snm2[threadIdx.x + w];
            snan[threadIdx.x] |= snan[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double* out = scratch + (size_t)kMaxRows * kRowSlots;
        const double npts = (double)(nr - g) * (double)(nz - g);
        out[0] = smax[0];
        out[1] = smin[0];
        out[2] = snm1[0];
        out[3] = sqrt(snm2[0] / npts);
        // origin value: interp(box 0, level, 0, 0); the grid is equatorially
        // symmetric (the entry point refuses anything else)
        const double r1 = rcoord(1 - g, dr);
        const double z1 = rcoord(1 - g, dz);
        const int i0 = (int)((0.0 - r1) / dr) + 1 - g;
        const int j0 = (int)((0.0 - z1) / dz) + 1 - g;
        const double auxr = (0.0 - rcoord(i0, dr)) / dr;
        const double auxz = (0.0 - rcoord(j0, dz)) / dz;
        double v = 0.0;
        for (int ii = -1; ii <= 2; ++ii)
            for (int jj = -1; jj <= 2; ++jj) {
                double aux = 1.0;
                for (int m = -1; m <= 2; ++m) {
                    if (m == ii) continue;
                    aux = __dmul_rn(aux, __dsub_rn(auxr, (double)m)) / (double)(ii - m);
                }
                for (int n = -1; n <= 2; ++n) {
                    if (n == jj) continue;
                    aux = __dmul_rn(aux, __dsub_rn(auxz, (double)n)) / (double)(jj - n);
                }
                const double fv = f[(size_t)(i0 + ii - 1 + g) + (size_t)(j0 + jj - 1 + g) * ld];
                v = __dadd_rn(v, __dmul_rn(aux, fv));
            }
        out[4] = v;
        out[5] = snan[0] ? 1.0 : 0.0;
    }
}

thread_local char g_noalloc_err[256] = "";

int noalloc_fail(int code, const char* msg) {
    snprintf(g_noalloc_err, sizeof(g_noalloc_err), "%s", msg);
    return code;
}

// Address of the scratch array on the current device: looked up once per
// device, with that device current, and cached for the life of the process.
// The cache does not survive cudaDeviceReset (the address belongs to the
// destroyed context), so a caller that resets a device must not call this
// entry point on it afterwards.
int scratch_for_current_device(double** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return noalloc_fail(OLLIN_ECUDA, "cudaGetDevice failed");
    if (dev < 0 || dev >= kMaxDevices) return noalloc_fail(OLLIN_EINVAL, "device index out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_norms_scratch);
        if (e != cudaSuccess || p == nullptr)
            return noalloc_fail(OLLIN_ECUDA, "cudaGetSymbolAddress of the norms scratch failed");
        g_scratch_addr[dev] = (double*)p;
    }
    *out = g_scratch_addr[dev];
    return OLLIN_OK;
}

}  // namespace

extern "C" {

const char* ollin_gpu_noalloc_last_error(void) { return g_noalloc_err; }

int ollin_gpu_norms_noalloc(const double* d_field, int nr, int nz, int ghost, int ld_r, double dr, double dz,
                            int eqsym, void* stream, double out[5]) {
    if (!d_field || !out) return noalloc_fail(OLLIN_EINVAL, "null field or output pointer");
    if (ghost < 2 || ghost > 8 || nr <= ghost + 1 || nz <= ghost + 1 || ld_r < nr + ghost || !(dr > 0.0) ||
        !(dz > 0.0))
        return noalloc_fail(OLLIN_EINVAL, "bad grid description (ghost 2 to 8, ld_r >= nr+ghost)");
    if (!eqsym) return noalloc_fail(OLLIN_EINVAL, "only equatorially symmetric grids are supported");
    if (nz - ghost > kMaxRows)
        return noalloc_fail(OLLIN_EINVAL, "nz - ghost exceeds the 8192 interior rows the fixed scratch holds");
    double* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;
    // An error left pending by the caller's earlier work is reported as such,
    // not charged to these launches.
    const cudaError_t pending = cudaPeekAtLastError();
    if (pending != cudaSuccess) {
        snprintf(g_noalloc_err, sizeof(g_noalloc_err), "a CUDA error from earlier work is pending: %s",
                 cudaGetErrorString(pending));
        return OLLIN_ECUDA;
    }
    cudaStream_t s = (cudaStream_t)stream;
    // the call ends by synchronising the stream, which a capture forbids
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone)
        return noalloc_fail(OLLIN_EINVAL, "the stream is capturing (the call synchronises it)");
    rows_kernel<<<nz - ghost, 256, 0, s>>>(d_field, nr, ghost, (long)ld_r, scratch);
    if (cudaGetLastError() != cudaSuccess) return noalloc_fail(OLLIN_ECUDA, "launch of the row pass failed");
    final_kernel<<<1, 256, 0, s>>>(d_field, nr, nz, ghost, (long)ld_r, dr, dz, scratch);
    if (cudaGetLastError() != cudaSuccess) return noalloc_fail(OLLIN_ECUDA, "launch of the final pass failed");
    double res[6];
    if (cudaMemcpyAsync(res, scratch + (size_t)kMaxRows * kRowSlots, sizeof(res), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return noalloc_fail(OLLIN_ECUDA, "copying the result failed");
    if (res[5] != 0.0) return noalloc_fail(OLLIN_ENAN, "NaN found in the field (save0Ddata.f90:229-264)");
    for (int k = 0; k < 5; ++k) out[k] = res[k];
    return OLLIN_OK;
}

}  // extern "C"
