// Device-side data layout and stencil primitives of the GB300 evolution
// library for the OllinAxis-BiB time-evolution path.
//
// Layout in HBM: every grid function of a level is one FP64 array of
// (Nr+ghost) x (Nz+ghost) points, column-major with r fastest (the
// reference's (1-ghost:Nr, 1-ghost:Nz) arrays, generated allocatearrays.f90),
// with the leading dimension padded to a multiple of 32 doubles so that each
// z-row starts on a 256-byte boundary.  Kernels address element (i,j) through
// a base pointer pre-offset so that f(i,j) = base[i + j*ld].
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <vector>

namespace ollin {

// Programmatic dependent launch (sm_90+): the kernels of a level step are a
// chain of short dependent grids.  A kernel launched with launch_chained may
// be scheduled while its predecessor on the stream is still running; it
// first waits (griddepcontrol.wait) until that grid has completed and its
// writes are visible, so it reads and writes nothing early.  Then it lets
// its own successor be scheduled.  Both instructions are no-ops for a kernel
// launched the ordinary way.
__device__ __forceinline__ void chain_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Whether launch_chained adds the programmatic attribute (per host thread:
// set from the handle being stepped).  Off, the launch is an ordinary one.
extern thread_local bool g_chain_launch;

// ---- fused launches of many evolutions --------------------------------------
// While a recorder is set on the host thread, launch_chained records each
// step-path launch (the kernel, its shape and its one argument struct)
// instead of issuing it.  The fused coarse step of many evolutions records
// every evolution's step this way, then issues each kernel once for all of
// them: a multi-instance kernel (multi_kernel below) whose blocks are the
// blocks of every evolution's launch, each reading its own argument struct
// from device memory.
struct LaunchRec {
    const void* kernel;
    dim3 grid, block;
    std::vector<unsigned char> args;
};
struct LaunchRecorder {
    std::vector<LaunchRec> recs;
};
extern thread_local LaunchRecorder* g_recorder;

// Issues one multi-instance launch: ``n`` argument structs at dargs (device),
// block offsets boff[0..n] and grid widths gx[0..n-1] (device), ``total``
// blocks of shape ``block``.
using MultiLaunchFn = void (*)(const void* dargs, const int* boff, const int* gx, int n, int total, dim3 block,
                               cudaStream_t s);
// The multi-instance twin of a kernel (registered at load time by the file
// that defines both); null if the kernel has none.
void register_multi(const void* kernel, MultiLaunchFn fn);
MultiLaunchFn multi_for(const void* kernel);

// The body of a step-path kernel run for the blocks of every evolution of a
// fused launch: block b belongs to the evolution k with boff[k] <= b <
// boff[k+1], and is block (local % gx[k], local / gx[k]) of its own launch.
template <typename Args, void (*Body)(const Args&, unsigned, unsigned), int THREADS, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) multi_kernel(const Args* __restrict__ args,
                                                              const int* __restrict__ boff,
                                                              const int* __restrict__ gx, int n) {
    const int b = (int)blockIdx.x;
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(boff + mid) <= b) lo = mid;
        else hi = mid - 1;
    }
    const int local = b - __ldg(boff + lo);
    const int w = __ldg(gx + lo);
    Body(args[lo], (unsigned)(local % w), (unsigned)(local / w));
}

template <typename Args, void (*Body)(const Args&, unsigned, unsigned), int THREADS, int MINB>
void multi_launch(const void* dargs, const int* boff, const int* gx, int n, int total, dim3 block, cudaStream_t s) {
    multi_kernel<Args, Body, THREADS, MINB><<<total, block, 0, s>>>((const Args*)dargs, boff, gx, n);
}

// Registers kernel -> its multi-instance twin when the library loads.
struct MultiRegistration {
    MultiRegistration(const void* kernel, MultiLaunchFn fn) { register_multi(kernel, fn); }
};

template <typename... KArgs, typename... Args>
inline void launch_chained(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t s, Args... args) {
    if constexpr (sizeof...(Args) == 1) {
        if (g_recorder) {
            LaunchRec r;
            r.kernel = (const void*)kernel;
            r.grid = grid;
            r.block = block;
            auto put = [&](const auto& a) {
                r.args.resize(sizeof(a));
                memcpy(r.args.data(), &a, sizeof(a));
            };
            (put(args), ...);
            g_recorder->recs.push_back(std::move(r));
            return;
        }
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = g_chain_launch ? 1 : 0;
    cudaLaunchKernelEx(&cfg, kernel, args...);
}

constexpr int kMaxLevels = 12;

// Evolved fields kept on the device (a subset of the reference's EVOLVE
// arrays: the ones with non-zero sources in the supported formulation; the
// others are constant or recomputed by ``auxiliary`` and are reconstructed on
// download).
enum Field : int {
    F_ALPHA = 0, F_CHI, F_PHI, F_A, F_B, F_H, F_C,
    F_TRK, F_KTA, F_KTB, F_KTC, F_DLR, F_DLZ,
    F_BETAR, F_BETAZ, F_DTBETAR, F_DTBETAZ,
    F_SPHI, F_SXIR, F_SXIZ, F_SPI,
    F_FDRIVER,                     // the shock-avoiding drivers' fdriver
    NFIELDS
};

// Auxiliary point quantities written by the aux kernels and read by the
// right-hand side (names of the reference's auxiliary arrays).
enum AuxField : int {
    X_GA = 0, X_GB, X_GH, X_GC,    // g_A, g_B, g_H, g_C (inverse conformal metric)
    X_KTH, X_LAM, X_ALAM, X_GLAM,  // KTH, lambda, Alambda, g_lambda
    X_DELDEFR, X_DELDEFZ,          // DelDef_r, DelDef_z
    X_GDR, X_GDZ,                  // Dr_g_A + r Dz_g_C, Dz_g_B + r Dr_g_C (scalar-field source)
    // derived output arrays (analysis)
    X_HAM, X_MOMR, X_MOMZ, X_RSCAL, X_KT2, X_LAPLA,
    X_RHOS,                        // rho + trS (scalar field; source of maximal slicing)
    NAUX
};

// Geometry of one level as seen by a kernel.
struct LevelGeom {
    int nr, nz, g, ld;   // Nr, Nz, ghost, leading dimension
    int order;           // finite-difference order (param order): 2 or 4
    int jlo;             // first z-row with a source: 1 (the grid owns the equator) or 1-g
    int eqsym;           // equatorial symmetry of the run (param eqsym)
    int axis, equator;   // the grid's ghosts are the axis / equator parity images
                         // (main.f90:380-460: boxes with rbox = 0 / zbox = 0)
    int lower_r, lower_z;  // the lower r / z edge is a refinement boundary
                           // (finebound.f90:246-285, :361-397)
    double dr, dz, dt;
    double idr, idz;     // 1/dr, 1/dz
    const double* rcol;  // r(i) for i = 1-g..nr   (indexed rcol[i])
    const double* ircol; // 1/r(i)
    const double* zrow;  // z(j) for j = 1-g..nz   (indexed zrow[j])
};

__host__ __device__ inline size_t off(const LevelGeom& G, int i, int j) { return (size_t)i + (size_t)j * G.ld; }

// ---------------------------------------------------------------------------
// one-dimensional stencils of the reference (src/base/derivatives.f90,
// order four).  ``f`` is the base pointer (f(i,j) = f[i + j*ld]); ``s`` the
// stride between consecutive points along the direction; ``k`` the position
// class: 0 interior, 1 second-to-last, 2 last point (upper edge), -1 second
// point, -2 first point (lower edge, used only without equatorial symmetry).
// ``c`` is 1/(12 h) for first and 1/(12 h^2) for second derivatives.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double ld_(const double* p) { return __ldg(p); }

__device__ __forceinline__ double d1(const double* f, long s, int k, double c) {
    if (k == 0) {
        return c * (8.0 * (ld_(f + s) - ld_(f - s)) - (ld_(f + 2 * s) - ld_(f - 2 * s)));
    } else if (k == 1) {
        return c * (3.0 * ld_(f + s) + 10.0 * ld_(f) - 18.0 * ld_(f - s) + 6.0 * ld_(f - 2 * s) - ld_(f - 3 * s));
    } else if (k == 2) {
        return c * (25.0 * ld_(f) - 48.0 * ld_(f - s) + 36.0 * ld_(f - 2 * s) - 16.0 * ld_(f - 3 * s) + 3.0 * ld_(f - 4 * s));
    } else if (k == -1) {
        return -c * (3.0 * ld_(f - s) + 10.0 * ld_(f) - 18.0 * ld_(f + s) + 6.0 * ld_(f + 2 * s) - ld_(f + 3 * s));
    } else {
        return -c * (25.0 * ld_(f) - 48.0 * ld_(f + s) + 36.0 * ld_(f + 2 * s) - 16.0 * ld_(f + 3 * s) + 3.0 * ld_(f + 4 * s));
    }
}

__device__ __forceinline__ double d2(const double* f, long s, int k, double c) {
    if (k == 0) {
        return -c * fma(30.0, ld_(f), fma(-16.0, ld_(f + s) + ld_(f - s), ld_(f + 2 * s) + ld_(f - 2 * s)));
    } else if (k == 1) {
        return c * (10.0 * ld_(f + s) - 15.0 * ld_(f) - 4.0 * ld_(f - s) + 14.0 * ld_(f - 2 * s) - 6.0 * ld_(f - 3 * s) + ld_(f - 4 * s));
    } else if (k == 2) {
        return c * (45.0 * ld_(f) - 154.0 * ld_(f - s) + 214.0 * ld_(f - 2 * s) - 156.0 * ld_(f - 3 * s) + 61.0 * ld_(f - 4 * s) - 10.0 * ld_(f - 5 * s));
    } else if (k == -1) {
        return c * (10.0 * ld_(f - s) - 15.0 * ld_(f) - 4.0 * ld_(f + s) + 14.0 * ld_(f + 2 * s) - 6.0 * ld_(f + 3 * s) + ld_(f + 4 * s));
    } else {
        return c * (45.0 * ld_(f) - 154.0 * ld_(f + s) + 214.0 * ld_(f + 2 * s) - 156.0 * ld_(f + 3 * s) + 61.0 * ld_(f + 4 * s) - 10.0 * ld_(f + 5 * s));
    }
}

// Position class along one direction for first/second derivatives.
__device__ __forceinline__ int pclass(int i, int n, int g) {
    if (i <= n - 2) return (i >= 3 - g) ? 0 : (i == 2 - g ? -1 : -2);
    return (i == n - 1) ? 1 : 2;
}

// Mixed derivative d^2/(dr dz) with the reference's edge and corner rules
// (derivatives.f90:615-700): 4th order inside, 2nd order on the two outermost
// rows/columns, one-sided on the last one, and the z-edge rule overriding the
// r-edge rule where both apply.
__device__ __forceinline__ double d2rz(const double* f, long ld, int i, int j, int nr, int nz, int g, double idrz) {
    const bool ri = (i >= 3 - g && i <= nr - 2), zi = (j >= 3 - g && j <= nz - 2);
#define F_(a, b) ld_(f + (a) + (long)(b) * ld)
    if (ri && zi) {
        return fma(idrz * (1.0 / 3.0), (F_(1, 1) + F_(-1, -1)) - (F_(1, -1) + F_(-1, 1)),
                   (idrz * (-1.0 / 48.0)) * ((F_(2, 2) + F_(-2, -2)) - (F_(2, -2) + F_(-2, 2))));
    }
    const bool zedge_loop = (i >= 2 - g && i <= nr - 1);  // z-boundary loop range
    const bool redge_loop = (j >= 2 - g && j <= nz - 1);  // r-boundary loop range
    if (zedge_loop && !zi) {
        if (j == 2 - g || j == nz - 1)
            return 0.25 * idrz * (F_(1, 1) + F_(-1, -1) - F_(-1, 1) - F_(1, -1));
        if (j == nz)
            return 0.25 * idrz * ((3.0 * F_(1, 0) - 4.0 * F_(1, -1) + F_(1, -2)) - (3.0 * F_(-1, 0) - 4.0 * F_(-1, -1) + F_(-1, -2)));
        // j == 1-g
        return -0.25 * idrz * ((3.0 * F_(1, 0) - 4.0 * F_(1, 1) + F_(1, 2)) - (3.0 * F_(-1, 0) - 4.0 * F_(-1, 1) + F_(-1, 2)));
    }
    if (redge_loop && !ri) {
        if (i == 2 - g || i == nr - 1)
            return 0.25 * idrz * (F_(1, 1) + F_(-1, -1) - F_(1, -1) - F_(-1, 1));
        if (i == nr)
            return 0.25 * idrz * ((3.0 * F_(0, 1) - 4.0 * F_(-1, 1) + F_(-2, 1)) - (3.0 * F_(0, -1) - 4.0 * F_(-1, -1) + F_(-2, -1)));
        return -0.25 * idrz * ((3.0 * F_(0, 1) - 4.0 * F_(1, 1) + F_(2, 1)) - (3.0 * F_(0, -1) - 4.0 * F_(1, -1) + F_(2, -1)));
    }
    // corners
    if (i == nr && j == nz)
        return 0.25 * idrz * (9.0 * F_(0, 0) + 16.0 * F_(-1, -1) + F_(-2, -2) - 12.0 * (F_(0, -1) + F_(-1, 0))
                              + 3.0 * (F_(0, -2) + F_(-2, 0)) - 4.0 * (F_(-1, -2) + F_(-2, -1)));
    if (i == nr)  // j == 1-g
        return -0.25 * idrz * (9.0 * F_(0, 0) + 16.0 * F_(-1, 1) + F_(-2, 2) - 12.0 * (F_(0, 1) + F_(-1, 0))
                               + 3.0 * (F_(0, 2) + F_(-2, 0)) - 4.0 * (F_(-1, 2) + F_(-2, 1)));
    if (j == nz)  // i == 1-g
        return -0.25 * idrz * (9.0 * F_(0, 0) + 16.0 * F_(1, -1) + F_(2, -2) - 12.0 * (F_(1, 0) + F_(0, -1))
                               + 3.0 * (F_(2, 0) + F_(0, -2)) - 4.0 * (F_(2, -1) + F_(1, -2)));
    return 0.25 * idrz * (9.0 * F_(0, 0) + 16.0 * F_(1, 1) + F_(2, 2) - 12.0 * (F_(0, 1) + F_(1, 0))
                          + 3.0 * (F_(0, 2) + F_(2, 0)) - 4.0 * (F_(1, 2) + F_(2, 1)));
#undef F_
}

// Lopsided advective derivative (src/base/derivadvect.f90, order four).
// ``neg`` is (beta <= 0) at the point; ``k`` the upper-edge class counted as
// in diffadvr/diffadvz: 0 interior (i <= n-3), 3 second point of the
// interior range (i = 3-ghost), 10 = n-2, 11 = n-1, 12 = n.
__device__ __forceinline__ double dadv(const double* f, long s, int i, int n, int g, bool neg, double ih, bool zdir) {
    const double q = 0.25 * ih;
    auto left = [&]() { return +q * (3.0 * ld_(f + s) + 10.0 * ld_(f) - 18.0 * ld_(f - s) + 6.0 * ld_(f - 2 * s) - ld_(f - 3 * s)) * (1.0 / 3.0); };
    auto right = [&]() { return -q * (3.0 * ld_(f - s) + 10.0 * ld_(f) - 18.0 * ld_(f + s) + 6.0 * ld_(f + 2 * s) - ld_(f + 3 * s)) * (1.0 / 3.0); };
    auto cent = [&]() { return q * (8.0 * (ld_(f + s) - ld_(f - s)) - (ld_(f + 2 * s) - ld_(f - 2 * s))) * (1.0 / 3.0); };
    if (i >= 4 - g && i <= n - 3) return neg ? left() : right();
    if (i == n - 2) return neg ? left() : cent();
    if (i == n - 1) return left();
    if (i == n) return q * (25.0 * ld_(f) - 48.0 * ld_(f - s) + 36.0 * ld_(f - 2 * s) - 16.0 * ld_(f - 3 * s) + 3.0 * ld_(f - 4 * s)) * (1.0 / 3.0);
    if (i == 3 - g) {
        // the r and z lopsided routines treat this point with opposite branches
        if (!zdir) return neg ? cent() : right();
        return neg ? right() : cent();
    }
    if (i == 2 - g) return right();
    return -q * (25.0 * ld_(f) - 48.0 * ld_(f + s) + 36.0 * ld_(f + 2 * s) - 16.0 * ld_(f + 3 * s) + 3.0 * ld_(f + 4 * s)) * (1.0 / 3.0);
}

// ---------------------------------------------------------------------------
// order two (derivatives.f90 :50-58, :158-172, :285-301, :402-418, :533-599;
// derivadvect.f90 :50-100, :249-299; dissipation.f90 :121-135).  Position
// classes: 0 centred (i = 2-ghost..n-1), 2 last point, -2 first point.
// ``c`` is 1/(2h) for first and 1/h^2 for second derivatives.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int pclass2(int i, int n, int g) { return i == n ? 2 : (i >= 2 - g ? 0 : -2); }

__device__ __forceinline__ double d1_2(const double* f, long s, int k, double c) {
    if (k == 0) return c * (ld_(f + s) - ld_(f - s));
    if (k == 2) return c * (3.0 * ld_(f) - 4.0 * ld_(f - s) + ld_(f - 2 * s));
    return -c * (3.0 * ld_(f) - 4.0 * ld_(f + s) + ld_(f + 2 * s));
}

__device__ __forceinline__ double d2_2(const double* f, long s, int k, double c) {
    if (k == 0) return c * (ld_(f + s) - 2.0 * ld_(f) + ld_(f - s));
    if (k == 2) return c * (2.0 * ld_(f) - 5.0 * ld_(f - s) + 4.0 * ld_(f - 2 * s) - ld_(f - 3 * s));
    return c * (2.0 * ld_(f) - 5.0 * ld_(f + s) + 4.0 * ld_(f + 2 * s) - ld_(f + 3 * s));
}

// centred inside, one-sided on the outermost rows and columns, the corners
// from both one-sided stencils (the r- and z-edge loops do not overlap)
__device__ __forceinline__ double d2rz_2(const double* f, long ld, int i, int j, int nr, int nz, int g, double idrz) {
#define F_(a, b) ld_(f + (a) + (long)(b) * ld)
    const bool ri = (i >= 2 - g && i <= nr - 1), zi = (j >= 2 - g && j <= nz - 1);
    const double q = 0.25 * idrz;
    if (ri && zi) return q * (F_(1, 1) + F_(-1, -1) - F_(1, -1) - F_(-1, 1));
    if (zi) {  // i = 1-g or nr
        if (i == nr) return q * ((3.0 * F_(0, 1) - 4.0 * F_(-1, 1) + F_(-2, 1)) - (3.0 * F_(0, -1) - 4.0 * F_(-1, -1) + F_(-2, -1)));
        return -q * ((3.0 * F_(0, 1) - 4.0 * F_(1, 1) + F_(2, 1)) - (3.0 * F_(0, -1) - 4.0 * F_(1, -1) + F_(2, -1)));
    }
    if (ri) {  // j = 1-g or nz
        if (j == nz) return q * ((3.0 * F_(1, 0) - 4.0 * F_(1, -1) + F_(1, -2)) - (3.0 * F_(-1, 0) - 4.0 * F_(-1, -1) + F_(-1, -2)));
        return -q * ((3.0 * F_(1, 0) - 4.0 * F_(1, 1) + F_(1, 2)) - (3.0 * F_(-1, 0) - 4.0 * F_(-1, 1) + F_(-1, 2)));
    }
    if (i == nr && j == nz)
        return q * (9.0 * F_(0, 0) + 16.0 * F_(-1, -1) + F_(-2, -2) - 12.0 * (F_(0, -1) + F_(-1, 0))
                    + 3.0 * (F_(0, -2) + F_(-2, 0)) - 4.0 * (F_(-1, -2) + F_(-2, -1)));
    if (i == nr)
        return -q * (9.0 * F_(0, 0) + 16.0 * F_(-1, 1) + F_(-2, 2) - 12.0 * (F_(0, 1) + F_(-1, 0))
                     + 3.0 * (F_(0, 2) + F_(-2, 0)) - 4.0 * (F_(-1, 2) + F_(-2, 1)));
    if (j == nz)
        return -q * (9.0 * F_(0, 0) + 16.0 * F_(1, -1) + F_(2, -2) - 12.0 * (F_(1, 0) + F_(0, -1))
                     + 3.0 * (F_(2, 0) + F_(0, -2)) - 4.0 * (F_(2, -1) + F_(1, -2)));
    return q * (9.0 * F_(0, 0) + 16.0 * F_(1, 1) + F_(2, 2) - 12.0 * (F_(0, 1) + F_(1, 0))
                + 3.0 * (F_(0, 2) + F_(2, 0)) - 4.0 * (F_(1, 2) + F_(2, 1)));
#undef F_
}

// second-order lopsided advective derivative; the r and z routines treat
// every point alike
__device__ __forceinline__ double dadv_2(const double* f, long s, int i, int n, int g, bool neg, double ih) {
    const double h = 0.5 * ih;
    auto left = [&]() { return +h * (3.0 * ld_(f) - 4.0 * ld_(f - s) + ld_(f - 2 * s)); };
    auto right = [&]() { return -h * (3.0 * ld_(f) - 4.0 * ld_(f + s) + ld_(f + 2 * s)); };
    auto cent = [&]() { return h * (ld_(f + s) - ld_(f - s)); };
    if (i >= 3 - g && i <= n - 2) return neg ? left() : right();
    if (i == 2 - g) return neg ? cent() : right();
    if (i == 1 - g) return right();
    if (i == n - 1) return neg ? left() : cent();
    return left();  // i == n
}

// the fourth difference of order-two dissipation (without -eps/dt/6)
__device__ __forceinline__ double ko4(const double* f, long s) {
    return 6.0 * ld_(f) - 4.0 * (ld_(f + s) + ld_(f - s)) + (ld_(f + 2 * s) + ld_(f - 2 * s));
}

// ---- order dispatch for the kernels that take the order at run time ------
__device__ __forceinline__ int pclass_o(int ord, int i, int n, int g) { return ord == 2 ? pclass2(i, n, g) : pclass(i, n, g); }
__device__ __forceinline__ double c1_o(int ord, double ih) { return ord == 2 ? 0.5 * ih : ih * (1.0 / 12.0); }
__device__ __forceinline__ double c2_o(int ord, double ih) { return ord == 2 ? ih * ih : ih * ih * (1.0 / 12.0); }
__device__ __forceinline__ double d1_o(int ord, const double* f, long s, int k, double c) {
    return ord == 2 ? d1_2(f, s, k, c) : d1(f, s, k, c);
}
__device__ __forceinline__ double d2_o(int ord, const double* f, long s, int k, double c) {
    return ord == 2 ? d2_2(f, s, k, c) : d2(f, s, k, c);
}
__device__ __forceinline__ double d2rz_o(int ord, const double* f, long ld, int i, int j, int nr, int nz, int g, double idrz) {
    return ord == 2 ? d2rz_2(f, ld, i, j, nr, nz, g, idrz) : d2rz(f, ld, i, j, nr, nz, g, idrz);
}
// the first point whose r derivative diff1r sets: i = 1 in order four,
// i = 2-ghost in order two (lower points of a grid off the axis stay unset)
__device__ __forceinline__ int d1r_first(int ord, int g) { return ord == 2 ? 2 - g : 1; }

// Kreiss-Oliger sixth difference along one direction, the bracket of
// src/base/dissipation.f90:196-211 (without the -eps/dt/20 factor).
__device__ __forceinline__ double ko6(const double* f, long s) {
    return 20.0 * ld_(f) - 15.0 * (ld_(f + s) + ld_(f - s)) + 6.0 * (ld_(f + 2 * s) + ld_(f - 2 * s)) - (ld_(f + 3 * s) + ld_(f - 3 * s));
}

// s - k * (ko6 along stride 1 + ko6 along stride ld), for points inside both
// dissipation ranges: the two brackets share the centre and are summed
// before scaling (13 FP64 operations instead of 16).
__device__ __forceinline__ double ko6rz_apply(const double* f, long ld, double k, double s) {
    const double a1 = (ld_(f + 1) + ld_(f - 1)) + (ld_(f + ld) + ld_(f - ld));
    const double a2 = (ld_(f + 2) + ld_(f - 2)) + (ld_(f + 2 * ld) + ld_(f - 2 * ld));
    const double a3 = (ld_(f + 3) + ld_(f - 3)) + (ld_(f + 3 * ld) + ld_(f - 3 * ld));
    double t = fma(-40.0 * k, ld_(f), s);
    t = fma(15.0 * k, a1, t);
    t = fma(-6.0 * k, a2, t);
    return fma(k, a3, t);
}

}  // namespace ollin
