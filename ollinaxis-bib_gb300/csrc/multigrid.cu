// Geometric multigrid for the correction equation J d = r of the
// mixed-precision elliptic solve (the discrete system that the SOR of
// src/elliptic/sor_elliptic.f90 converges to), in FP32; the same hierarchy in
// FP64 gives the all-FP64 solve of that system that the mixed solve's error is
// measured against.
//
// Grid k of the hierarchy has n x m cells, cell centres r_I = (I-1/2) Hr,
// z_J = (J-1/2) Hz, Hr = 2^k dr.  Its equations are those of the level
// itself re-discretised with spacing H:
//   interior I <= n-1, J <= m-1:
//     a_I d(I+1,J) + b_I d(I-1,J) + cz (d(I,J+1) + d(I,J-1)) + e_IJ d = r
//     with d(0,J) = d(1,J), d(I,0) = d(I,1) (axis and equator mirrors)
//   Robin rows I = n / J = m (coarse problem), zero rows otherwise (the
//   Dirichlet problems of the finer refinement levels).
// Cell (I,J) of grid k+1 covers cells 2I-1..2I x 2J-1..2J of grid k:
// restriction averages the four residuals (the two Robin residuals on a
// boundary row), prolongation is bilinear in the cell centres (9/16, 3/16,
// 3/16, 1/16).  Smoother: red-black Gauss-Seidel, Robin rows by two-colour
// Gauss-Seidel along each edge.  Arrays are compact, (n+2) x (m+2) with one
// ghost layer: element (I,J) at [I + J (n+2)].
#include <vector>

#include "ollin_kernels.h"

namespace ollin {

namespace {

template <typename T>
struct Grid {
    int n, m, ld;
    T hr, hz;            // spacings
    T* d; T* r; T* e;
};

__device__ __forceinline__ int mirror(int k) { return k < 1 ? 1 - k : k; }

template <typename T>
__device__ __forceinline__ T Dv(const Grid<T>& G, int i, int j) { return G.d[mirror(i) + mirror(j) * G.ld]; }

// residual of one interior equation
template <typename T>
__device__ __forceinline__ T interior_res(const Grid<T>& G, int i, int j) {
    const T ri = ((T)i - T(0.5)) * G.hr;
    const T a = (T(1.0) / G.hr + T(0.5) / ri) / G.hr, b = (T(1.0) / G.hr - T(0.5) / ri) / G.hr;
    const T cz = T(1.0) / (G.hz * G.hz);
    const int o = i + j * G.ld;
    return G.r[o] - (a * Dv(G, i + 1, j) + b * Dv(G, i - 1, j) + cz * (Dv(G, i, j + 1) + Dv(G, i, j - 1)) + G.e[o] * G.d[o]);
}

// residual of a Robin row (coarse problem); cr = r_n/Hr = n - 1/2, cz = J - 1/2
template <typename T>
__device__ __forceinline__ T robin_res(const Grid<T>& G, int i, int j) {
    const int n = G.n, m = G.m;
    const T cr = (T)n - T(0.5), czn = (T)m - T(0.5);
    T lhs;
    if (i == n && j == m) {
        lhs = (T(1.0) + T(1.5) * (cr + czn)) * Dv(G, i, j) - T(0.5) * cr * (T(4.0) * Dv(G, i - 1, j) - Dv(G, i - 2, j))
              - T(0.5) * czn * (T(4.0) * Dv(G, i, j - 1) - Dv(G, i, j - 2));
    } else if (i == n) {
        const T cz = (T)j - T(0.5);
        lhs = (T(1.0) + T(1.5) * cr) * Dv(G, i, j) - T(0.5) * cr * (T(4.0) * Dv(G, i - 1, j) - Dv(G, i - 2, j))
              + T(0.5) * cz * (Dv(G, i, j + 1) - Dv(G, i, j - 1));
    } else {
        const T crr = (T)i - T(0.5);
        lhs = (T(1.0) + T(1.5) * czn) * Dv(G, i, j) - T(0.5) * czn * (T(4.0) * Dv(G, i, j - 1) - Dv(G, i, j - 2))
              + T(0.5) * crr * (Dv(G, i + 1, j) - Dv(G, i - 1, j));
    }
    return G.r[i + j * G.ld] - lhs;
}

template <typename T>
__global__ void __launch_bounds__(128) mg_smooth_kernel(Grid<T> G, int parity) {
    const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int jh = (int)(blockIdx.y * blockDim.y + threadIdx.y);
    int j = 1;
    if (((i + j) & 1) != parity) ++j;
    j += 2 * jh;
    if (i > G.n - 1 || j > G.m - 1) return;
    const T ri = ((T)i - T(0.5)) * G.hr;
    const T a = (T(1.0) / G.hr + T(0.5) / ri) / G.hr, b = (T(1.0) / G.hr - T(0.5) / ri) / G.hr;
    const T cz = T(1.0) / (G.hz * G.hz);
    const int o = i + j * G.ld;
    T diag = G.e[o];
    T off = a * G.d[o + 1] + cz * G.d[o + G.ld];
    if (i > 1) off += b * G.d[o - 1]; else diag += b;
    if (j > 1) off += cz * G.d[o - G.ld]; else diag += cz;
    G.d[o] = (G.r[o] - off) / diag;
}

// Robin rows: two-colour Gauss-Seidel along each edge, then the corner
template <typename T>
__global__ void __launch_bounds__(1024) mg_edges_kernel(Grid<T> G) {
    const int n = G.n, m = G.m;
    const T cr = (T)n - T(0.5), czn = (T)m - T(0.5);
    auto D = [&](int i, int j) -> T& { return G.d[mirror(i) + mirror(j) * G.ld]; };
    for (int colour = 0; colour < 2; ++colour) {
        for (int j = 1 + colour + 2 * (int)threadIdx.x; j <= m - 1; j += 2 * blockDim.x) {
            const T cz = (T)j - T(0.5);
            D(n, j) = (G.r[n + j * G.ld] + T(0.5) * cr * (T(4.0) * D(n - 1, j) - D(n - 2, j)) - T(0.5) * cz * (D(n, j + 1) - D(n, j - 1)))
                      / (T(1.0) + T(1.5) * cr);
        }
        for (int i = 1 + colour + 2 * (int)threadIdx.x; i <= n - 1; i += 2 * blockDim.x) {
            const T crr = (T)i - T(0.5);
            D(i, m) = (G.r[i + m * G.ld] + T(0.5) * czn * (T(4.0) * D(i, m - 1) - D(i, m - 2)) - T(0.5) * crr * (D(i + 1, m) - D(i - 1, m)))
                      / (T(1.0) + T(1.5) * czn);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        D(n, m) = (G.r[n + m * G.ld] + T(0.5) * cr * (T(4.0) * D(n - 1, m) - D(n - 2, m)) + T(0.5) * czn * (T(4.0) * D(n, m - 1) - D(n, m - 2)))
                  / (T(1.0) + T(1.5) * (cr + czn));
}

// coarsest grid: one block runs all the sweeps
template <typename T>
__global__ void __launch_bounds__(1024) mg_coarse_kernel(Grid<T> G, int robin, int sweeps) {
    const int n = G.n, m = G.m;
    const T cz2 = T(1.0) / (G.hz * G.hz);
    const T cr = (T)n - T(0.5), czn = (T)m - T(0.5);
    auto D = [&](int i, int j) -> T& { return G.d[mirror(i) + mirror(j) * G.ld]; };
    const int ncell = (n - 1) * (m - 1);
    for (int sw = 0; sw < sweeps; ++sw) {
        for (int parity = 0; parity < 2; ++parity) {
            for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
                const int i = 1 + c % (n - 1), j = 1 + c / (n - 1);
                if (((i + j) & 1) != parity) continue;
                const T ri = ((T)i - T(0.5)) * G.hr;
                const T a = (T(1.0) / G.hr + T(0.5) / ri) / G.hr, b = (T(1.0) / G.hr - T(0.5) / ri) / G.hr;
                const int o = i + j * G.ld;
                T diag = G.e[o];
                T off = a * G.d[o + 1] + cz2 * G.d[o + G.ld];
                if (i > 1) off += b * G.d[o - 1]; else diag += b;
                if (j > 1) off += cz2 * G.d[o - G.ld]; else diag += cz2;
                G.d[o] = (G.r[o] - off) / diag;
            }
            __syncthreads();
        }
        if (robin) {
            for (int colour = 0; colour < 2; ++colour) {
                for (int j = 1 + colour + 2 * (int)threadIdx.x; j <= m - 1; j += 2 * blockDim.x) {
                    const T cz = (T)j - T(0.5);
                    D(n, j) = (G.r[n + j * G.ld] + T(0.5) * cr * (T(4.0) * D(n - 1, j) - D(n - 2, j)) - T(0.5) * cz * (D(n, j + 1) - D(n, j - 1)))
                              / (T(1.0) + T(1.5) * cr);
                }
                for (int i = 1 + colour + 2 * (int)threadIdx.x; i <= n - 1; i += 2 * blockDim.x) {
                    const T crr = (T)i - T(0.5);
                    D(i, m) = (G.r[i + m * G.ld] + T(0.5) * czn * (T(4.0) * D(i, m - 1) - D(i, m - 2)) - T(0.5) * crr * (D(i + 1, m) - D(i - 1, m)))
                              / (T(1.0) + T(1.5) * czn);
                }
                __syncthreads();
            }
            if (threadIdx.x == 0)
                D(n, m) = (G.r[n + m * G.ld] + T(0.5) * cr * (T(4.0) * D(n - 1, m) - D(n - 2, m)) + T(0.5) * czn * (T(4.0) * D(n, m - 1) - D(n, m - 2)))
                          / (T(1.0) + T(1.5) * (cr + czn));
            __syncthreads();
        }
    }
}

// residual of grid F restricted to the right-hand side of grid C; d_C = 0
template <typename T>
__global__ void __launch_bounds__(128) mg_restrict_kernel(Grid<T> F, Grid<T> C, int robin) {
    const int I = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int J = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (I > C.n || J > C.m) return;
    const int o = I + J * C.ld;
    C.d[o] = T(0.0);
    const bool bI = I == C.n, bJ = J == C.m;
    T v = T(0.0);
    if (!bI && !bJ) {
        v = T(0.25) * (interior_res(F, 2 * I - 1, 2 * J - 1) + interior_res(F, 2 * I, 2 * J - 1)
                     + interior_res(F, 2 * I - 1, 2 * J) + interior_res(F, 2 * I, 2 * J));
    } else if (robin) {
        if (bI && bJ) v = robin_res(F, F.n, F.m);
        else if (bI) v = T(0.5) * (robin_res(F, F.n, 2 * J - 1) + robin_res(F, F.n, 2 * J));
        else v = T(0.5) * (robin_res(F, 2 * I - 1, F.m) + robin_res(F, 2 * I, F.m));
    }
    C.r[o] = v;
}

// d_F += bilinear interpolation of d_C (zero rows of a Dirichlet problem stay)
template <typename T>
__global__ void __launch_bounds__(128) mg_prolong_kernel(Grid<T> F, Grid<T> C, int robin) {
    const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (i > F.n || j > F.m) return;
    if (!robin && (i == F.n || j == F.m)) return;
    const int I = (i + 1) / 2, J = (j + 1) / 2;
    const int I2 = (i & 1) ? I - 1 : I + 1, J2 = (j & 1) ? J - 1 : J + 1;
    auto c = [&](int p, int q) {
        p = p < 1 ? 1 : (p > C.n ? C.n : p);
        q = q < 1 ? 1 : (q > C.m ? C.m : q);
        return C.d[p + q * C.ld];
    };
    const T v = T(0.5625) * c(I, J) + T(0.1875) * (c(I2, J) + c(I, J2)) + T(0.0625) * c(I2, J2);
    F.d[i + j * F.ld] += v;
}

// grid-k diagonal from the one below: average of S1 plus the constant part
template <typename T>
__global__ void __launch_bounds__(128) mg_diag_kernel(Grid<T> F, Grid<T> C) {
    const int I = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int J = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (I > C.n || J > C.m) return;
    const T ef = -T(2.0) * (T(1.0) / (F.hr * F.hr) + T(1.0) / (F.hz * F.hz));
    const T ec = -T(2.0) * (T(1.0) / (C.hr * C.hr) + T(1.0) / (C.hz * C.hz));
    auto s1 = [&](int p, int q) { return F.e[p + q * F.ld] - ef; };
    const T avg = T(0.25) * (s1(2 * I - 1, 2 * J - 1) + s1(2 * I, 2 * J - 1) + s1(2 * I - 1, 2 * J) + s1(2 * I, 2 * J));
    C.e[I + J * C.ld] = ec + avg;
}

// grid 0 from the level's arrays (level layout: element (i,j) at [i + j*ld])
template <typename T>
__global__ void __launch_bounds__(128) mg_load_kernel(Grid<T> G, const T* r, const T* e, long ld) {
    const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (i > G.n + 1 || j > G.m + 1) return;
    const int o = i + j * G.ld;
    G.d[o] = T(0.0);
    const bool in = i >= 1 && i <= G.n && j >= 1 && j <= G.m;
    G.r[o] = in ? r[(size_t)i + (size_t)j * ld] : T(0.0);
    G.e[o] = in ? e[(size_t)i + (size_t)j * ld] : T(0.0);
}

template <typename T>
__global__ void __launch_bounds__(128) mg_store_kernel(Grid<T> G, T* d, long ld) {
    const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (i > G.n || j > G.m) return;
    d[(size_t)i + (size_t)j * ld] = G.d[i + j * G.ld];
}

template <typename T>
dim3 cells(const Grid<T>& G, dim3 blk) { return dim3((G.n + blk.x - 1) / blk.x, (G.m + blk.y - 1) / blk.y); }

}  // namespace

// ---- host side of the hierarchy ---------------------------------------------
namespace {

template <typename T>
struct MgGrids {
    std::vector<Grid<T>> g;
    T* pool = nullptr;

    bool create(int n, int m, double dr, double dz) {
        size_t total = 0;
        int nn = n, mm = m;
        double hr = dr, hz = dz;
        for (;;) {
            Grid<T> G{};
            G.n = nn; G.m = mm; G.ld = nn + 2;
            G.hr = (T)hr; G.hz = (T)hz;
            g.push_back(G);
            total += (size_t)3 * (nn + 2) * (mm + 2);
            if ((nn & 1) || (mm & 1) || nn / 2 < 4 || mm / 2 < 4) break;
            nn /= 2; mm /= 2; hr *= 2.0; hz *= 2.0;
        }
        if (cudaMalloc(&pool, total * sizeof(T)) != cudaSuccess) { pool = nullptr; return false; }
        T* q = pool;
        for (Grid<T>& G : g) {
            const size_t sz = (size_t)(G.n + 2) * (G.m + 2);
            G.d = q; q += sz; G.r = q; q += sz; G.e = q; q += sz;
        }
        cudaMemset(pool, 0, total * sizeof(T));
        return true;
    }

    void load(const T* r, const T* e, long ld, cudaStream_t s) {
        dim3 blk(32, 4);
        const Grid<T>& G0 = g[0];
        mg_load_kernel<T><<<dim3((G0.n + 2 + 31) / 32, (G0.m + 2 + 3) / 4), blk, 0, s>>>(G0, r, e, ld);
        for (size_t k = 1; k < g.size(); ++k) mg_diag_kernel<T><<<cells(g[k], blk), blk, 0, s>>>(g[k - 1], g[k]);
    }

    void smooth(const Grid<T>& G, int robin, int sweeps, cudaStream_t s) {
        dim3 blk(32, 4);
        const int nj = (G.m + 1) / 2;
        dim3 grd((G.n + 31) / 32, (nj + 3) / 4);
        for (int k = 0; k < sweeps; ++k) {
            mg_smooth_kernel<T><<<grd, blk, 0, s>>>(G, 0);
            mg_smooth_kernel<T><<<grd, blk, 0, s>>>(G, 1);
            if (robin) mg_edges_kernel<T><<<1, 1024, 0, s>>>(G);
        }
    }

    // one V-cycle on grid k (d of grid 0 holds the current correction)
    void vcycle(size_t k, int robin, cudaStream_t s) {
        const Grid<T>& F = g[k];
        if (k + 1 == g.size()) {
            mg_coarse_kernel<T><<<1, 1024, 0, s>>>(F, robin, 60);  // coarsest grid: relax to near convergence
            return;
        }
        const Grid<T>& C = g[k + 1];
        dim3 blk(32, 4);
        smooth(F, robin, 2, s);
        mg_restrict_kernel<T><<<cells(C, blk), blk, 0, s>>>(F, C, robin);
        vcycle(k + 1, robin, s);
        mg_prolong_kernel<T><<<cells(F, blk), blk, 0, s>>>(F, C, robin);
        smooth(F, robin, 2, s);
    }

    void solve(int robin, int ncycles, T* d, long ld, cudaStream_t s) {
        for (int c = 0; c < ncycles; ++c) vcycle(0, robin, s);
        dim3 blk(32, 4);
        mg_store_kernel<T><<<cells(g[0], blk), blk, 0, s>>>(g[0], d, ld);
    }
};

}  // namespace

// One hierarchy in FP32 (the mixed-precision solve) or FP64 (the FP64 solve
// of the same system it is measured against).
struct MgHierarchy {
    int fp64 = 0;
    MgGrids<float> f;
    MgGrids<double> d;
};

MgHierarchy* mg_create(int n, int m, double dr, double dz, int fp64) {
    auto* H = new MgHierarchy();
    H->fp64 = fp64 ? 1 : 0;
    const bool ok = H->fp64 ? H->d.create(n, m, dr, dz) : H->f.create(n, m, dr, dz);
    if (!ok) { delete H; return nullptr; }
    return H;
}

void mg_destroy(MgHierarchy* H) {
    if (!H) return;
    cudaFree(H->f.pool);
    cudaFree(H->d.pool);
    delete H;
}

int mg_levels(const MgHierarchy* H) { return (int)(H->fp64 ? H->d.g.size() : H->f.g.size()); }

// load r, e of the level (the hierarchy's precision, level layout), build the
// coarse diagonals
void mg_load(MgHierarchy* H, const void* r, const void* e, long ld, cudaStream_t s) {
    if (H->fp64) H->d.load((const double*)r, (const double*)e, ld, s);
    else H->f.load((const float*)r, (const float*)e, ld, s);
}

int mg_launches_per_cycle(const MgHierarchy* H, int robin) {
    const int per_sweep = robin ? 3 : 2;
    const int L = mg_levels(H);
    return (L - 1) * (4 * per_sweep + 2) + 1;
}

// ncycles V-cycles from d = 0; the correction is stored into d (level layout)
void mg_solve(MgHierarchy* H, int robin, int ncycles, void* d, long ld, cudaStream_t s) {
    if (H->fp64) H->d.solve(robin, ncycles, (double*)d, ld, s);
    else H->f.solve(robin, ncycles, (float*)d, ld, s);
}

}  // namespace ollin
