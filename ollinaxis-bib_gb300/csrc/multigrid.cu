// FP32 geometric multigrid for the correction equation J d = r of the
// mixed-precision elliptic solve (the discrete system that the SOR of
// src/elliptic/sor_elliptic.f90 converges to).
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

struct Grid {
    int n, m, ld;
    float hr, hz;        // spacings
    float* d; float* r; float* e;
};

__device__ __forceinline__ int mirror(int k) { return k < 1 ? 1 - k : k; }

__device__ __forceinline__ float Dv(const Grid& G, int i, int j) { return G.d[mirror(i) + mirror(j) * G.ld]; }

// residual of one interior equation
__device__ __forceinline__ float interior_res(const Grid& G, int i, int j) {
    const float ri = ((float)i - 0.5f) * G.hr;
    const float a = (1.0f / G.hr + 0.5f / ri) / G.hr, b = (1.0f / G.hr - 0.5f / ri) / G.hr;
    const float cz = 1.0f / (G.hz * G.hz);
    const int o = i + j * G.ld;
    return G.r[o] - (a * Dv(G, i + 1, j) + b * Dv(G, i - 1, j) + cz * (Dv(G, i, j + 1) + Dv(G, i, j - 1)) + G.e[o] * G.d[o]);
}

// residual of a Robin row (coarse problem); cr = r_n/Hr = n - 1/2, cz = J - 1/2
__device__ __forceinline__ float robin_res(const Grid& G, int i, int j) {
    const int n = G.n, m = G.m;
    const float cr = (float)n - 0.5f, czn = (float)m - 0.5f;
    float lhs;
    if (i == n && j == m) {
        lhs = (1.0f + 1.5f * (cr + czn)) * Dv(G, i, j) - 0.5f * cr * (4.0f * Dv(G, i - 1, j) - Dv(G, i - 2, j))
              - 0.5f * czn * (4.0f * Dv(G, i, j - 1) - Dv(G, i, j - 2));
    } else if (i == n) {
        const float cz = (float)j - 0.5f;
        lhs = (1.0f + 1.5f * cr) * Dv(G, i, j) - 0.5f * cr * (4.0f * Dv(G, i - 1, j) - Dv(G, i - 2, j))
              + 0.5f * cz * (Dv(G, i, j + 1) - Dv(G, i, j - 1));
    } else {
        const float crr = (float)i - 0.5f;
        lhs = (1.0f + 1.5f * czn) * Dv(G, i, j) - 0.5f * czn * (4.0f * Dv(G, i, j - 1) - Dv(G, i, j - 2))
              + 0.5f * crr * (Dv(G, i + 1, j) - Dv(G, i - 1, j));
    }
    return G.r[i + j * G.ld] - lhs;
}

__global__ void __launch_bounds__(128) mg_smooth_kernel(Grid G, int parity) {
    const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int jh = (int)(blockIdx.y * blockDim.y + threadIdx.y);
    int j = 1;
    if (((i + j) & 1) != parity) ++j;
    j += 2 * jh;
    if (i > G.n - 1 || j > G.m - 1) return;
    const float ri = ((float)i - 0.5f) * G.hr;
    const float a = (1.0f / G.hr + 0.5f / ri) / G.hr, b = (1.0f / G.hr - 0.5f / ri) / G.hr;
    const float cz = 1.0f / (G.hz * G.hz);
    const int o = i + j * G.ld;
    float diag = G.e[o];
    float off = a * G.d[o + 1] + cz * G.d[o + G.ld];
    if (i > 1) off += b * G.d[o - 1]; else diag += b;
    if (j > 1) off += cz * G.d[o - G.ld]; else diag += cz;
    G.d[o] = (G.r[o] - off) / diag;
}

// Robin rows: two-colour Gauss-Seidel along each edge, then the corner
__global__ void __launch_bounds__(1024) mg_edges_kernel(Grid G) {
    const int n = G.n, m = G.m;
    const float cr = (float)n - 0.5f, czn = (float)m - 0.5f;
    auto D = [&](int i, int j) -> float& { return G.d[mirror(i) + mirror(j) * G.ld]; };
    for (int colour = 0; colour < 2; ++colour) {
        for (int j = 1 + colour + 2 * (int)threadIdx.x; j <= m - 1; j += 2 * blockDim.x) {
            const float cz = (float)j - 0.5f;
            D(n, j) = (G.r[n + j * G.ld] + 0.5f * cr * (4.0f * D(n - 1, j) - D(n - 2, j)) - 0.5f * cz * (D(n, j + 1) - D(n, j - 1)))
                      / (1.0f + 1.5f * cr);
        }
        for (int i = 1 + colour + 2 * (int)threadIdx.x; i <= n - 1; i += 2 * blockDim.x) {
            const float crr = (float)i - 0.5f;
            D(i, m) = (G.r[i + m * G.ld] + 0.5f * czn * (4.0f * D(i, m - 1) - D(i, m - 2)) - 0.5f * crr * (D(i + 1, m) - D(i - 1, m)))
                      / (1.0f + 1.5f * czn);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        D(n, m) = (G.r[n + m * G.ld] + 0.5f * cr * (4.0f * D(n - 1, m) - D(n - 2, m)) + 0.5f * czn * (4.0f * D(n, m - 1) - D(n, m - 2)))
                  / (1.0f + 1.5f * (cr + czn));
}

// coarsest grid: one block runs all the sweeps
__global__ void __launch_bounds__(1024) mg_coarse_kernel(Grid G, int robin, int sweeps) {
    const int n = G.n, m = G.m;
    const float cz2 = 1.0f / (G.hz * G.hz);
    const float cr = (float)n - 0.5f, czn = (float)m - 0.5f;
    auto D = [&](int i, int j) -> float& { return G.d[mirror(i) + mirror(j) * G.ld]; };
    const int ncell = (n - 1) * (m - 1);
    for (int sw = 0; sw < sweeps; ++sw) {
        for (int parity = 0; parity < 2; ++parity) {
            for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
                const int i = 1 + c % (n - 1), j = 1 + c / (n - 1);
                if (((i + j) & 1) != parity) continue;
                const float ri = ((float)i - 0.5f) * G.hr;
                const float a = (1.0f / G.hr + 0.5f / ri) / G.hr, b = (1.0f / G.hr - 0.5f / ri) / G.hr;
                const int o = i + j * G.ld;
                float diag = G.e[o];
                float off = a * G.d[o + 1] + cz2 * G.d[o + G.ld];
                if (i > 1) off += b * G.d[o - 1]; else diag += b;
                if (j > 1) off += cz2 * G.d[o - G.ld]; else diag += cz2;
                G.d[o] = (G.r[o] - off) / diag;
            }
            __syncthreads();
        }
        if (robin) {
            for (int colour = 0; colour < 2; ++colour) {
                for (int j = 1 + colour + 2 * (int)threadIdx.x; j <= m - 1; j += 2 * blockDim.x) {
                    const float cz = (float)j - 0.5f;
                    D(n, j) = (G.r[n + j * G.ld] + 0.5f * cr * (4.0f * D(n - 1, j) - D(n - 2, j)) - 0.5f * cz * (D(n, j + 1) - D(n, j - 1)))
                              / (1.0f + 1.5f * cr);
                }
                for (int i = 1 + colour + 2 * (int)threadIdx.x; i <= n - 1; i += 2 * blockDim.x) {
                    const float crr = (float)i - 0.5f;
                    D(i, m) = (G.r[i + m * G.ld] + 0.5f * czn * (4.0f * D(i, m - 1) - D(i, m - 2)) - 0.5f * crr * (D(i + 1, m) - D(i - 1, m)))
                              / (1.0f + 1.5f * czn);
                }
                __syncthreads();
            }
            if (threadIdx.x == 0)
                D(n, m) = (G.r[n + m * G.ld] + 0.5f * cr * (4.0f * D(n - 1, m) - D(n - 2, m)) + 0.5f * czn * (4.0f * D(n, m - 1) - D(n, m - 2)))
                          / (1.0f + 1.5f * (cr + czn));
            __syncthreads();
        }
    }
}

// residual of grid F restricted to the right-hand side of grid C; d_C = 0
__global__ void __launch_bounds__(128) mg_restrict_kernel(Grid F, Grid C, int robin) {
    const int I = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int J = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (I > C.n || J > C.m) return;
    const int o = I + J * C.ld;
    C.d[o] = 0.0f;
    const bool bI = I == C.n, bJ = J == C.m;
    float v = 0.0f;
    if (!bI && !bJ) {
        v = 0.25f * (interior_res(F, 2 * I - 1, 2 * J - 1) + interior_res(F, 2 * I, 2 * J - 1)
                     + interior_res(F, 2 * I - 1, 2 * J) + interior_res(F, 2 * I, 2 * J));
    } else if (robin) {
        if (bI && bJ) v = robin_res(F, F.n, F.m);
        else if (bI) v = 0.5f * (robin_res(F, F.n, 2 * J - 1) + robin_res(F, F.n, 2 * J));
        else v = 0.5f * (robin_res(F, 2 * I - 1, F.m) + robin_res(F, 2 * I, F.m));
    }
    C.r[o] = v;
}

// d_F += bilinear interpolation of d_C (zero rows of a Dirichlet problem stay)
__global__ void __launch_bounds__(128) mg_prolong_kernel(Grid F, Grid C, int robin) {
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
    const float v = 0.5625f * c(I, J) + 0.1875f * (c(I2, J) + c(I, J2)) + 0.0625f * c(I2, J2);
    F.d[i + j * F.ld] += v;
}

// grid-k diagonal from the one below: average of S1 plus the constant part
__global__ void __launch_bounds__(128) mg_diag_kernel(Grid F, Grid C) {
    const int I = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int J = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (I > C.n || J > C.m) return;
    const float ef = -2.0f * (1.0f / (F.hr * F.hr) + 1.0f / (F.hz * F.hz));
    const float ec = -2.0f * (1.0f / (C.hr * C.hr) + 1.0f / (C.hz * C.hz));
    auto s1 = [&](int p, int q) { return F.e[p + q * F.ld] - ef; };
    const float avg = 0.25f * (s1(2 * I - 1, 2 * J - 1) + s1(2 * I, 2 * J - 1) + s1(2 * I - 1, 2 * J) + s1(2 * I, 2 * J));
    C.e[I + J * C.ld] = ec + avg;
}

// grid 0 from the level's arrays (level layout: element (i,j) at [i + j*ld])
__global__ void __launch_bounds__(128) mg_load_kernel(Grid G, const float* r, const float* e, long ld) {
    const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (i > G.n + 1 || j > G.m + 1) return;
    const int o = i + j * G.ld;
    G.d[o] = 0.0f;
    const bool in = i >= 1 && i <= G.n && j >= 1 && j <= G.m;
    G.r[o] = in ? r[(size_t)i + (size_t)j * ld] : 0.0f;
    G.e[o] = in ? e[(size_t)i + (size_t)j * ld] : 0.0f;
}

__global__ void __launch_bounds__(128) mg_store_kernel(Grid G, float* d, long ld) {
    const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (i > G.n || j > G.m) return;
    d[(size_t)i + (size_t)j * ld] = G.d[i + j * G.ld];
}

dim3 cells(const Grid& G, dim3 blk) { return dim3((G.n + blk.x - 1) / blk.x, (G.m + blk.y - 1) / blk.y); }

}  // namespace

// ---- host side of the hierarchy ---------------------------------------------
struct MgHierarchy {
    std::vector<Grid> g;
    float* pool = nullptr;
};

MgHierarchy* mg_create(int n, int m, double dr, double dz) {
    auto* H = new MgHierarchy();
    size_t total = 0;
    int nn = n, mm = m;
    double hr = dr, hz = dz;
    std::vector<Grid> gs;
    for (;;) {
        Grid G{};
        G.n = nn; G.m = mm; G.ld = nn + 2;
        G.hr = (float)hr; G.hz = (float)hz;
        gs.push_back(G);
        total += (size_t)3 * (nn + 2) * (mm + 2);
        if ((nn & 1) || (mm & 1) || nn / 2 < 4 || mm / 2 < 4) break;
        nn /= 2; mm /= 2; hr *= 2.0; hz *= 2.0;
    }
    if (cudaMalloc(&H->pool, total * sizeof(float)) != cudaSuccess) { delete H; return nullptr; }
    float* q = H->pool;
    for (Grid& G : gs) {
        const size_t sz = (size_t)(G.n + 2) * (G.m + 2);
        G.d = q; q += sz; G.r = q; q += sz; G.e = q; q += sz;
    }
    cudaMemset(H->pool, 0, total * sizeof(float));
    H->g = gs;
    return H;
}

void mg_destroy(MgHierarchy* H) {
    if (!H) return;
    cudaFree(H->pool);
    delete H;
}

int mg_levels(const MgHierarchy* H) { return (int)H->g.size(); }

// load r, e of the level (FP32, level layout), build the coarse diagonals
void mg_load(MgHierarchy* H, const float* r, const float* e, long ld, cudaStream_t s) {
    dim3 blk(32, 4);
    const Grid& G0 = H->g[0];
    mg_load_kernel<<<dim3((G0.n + 2 + 31) / 32, (G0.m + 2 + 3) / 4), blk, 0, s>>>(G0, r, e, ld);
    for (size_t k = 1; k < H->g.size(); ++k) mg_diag_kernel<<<cells(H->g[k], blk), blk, 0, s>>>(H->g[k - 1], H->g[k]);
}

static void smooth(const Grid& G, int robin, int sweeps, cudaStream_t s) {
    dim3 blk(32, 4);
    const int nj = (G.m + 1) / 2;
    dim3 grd((G.n + 31) / 32, (nj + 3) / 4);
    for (int k = 0; k < sweeps; ++k) {
        mg_smooth_kernel<<<grd, blk, 0, s>>>(G, 0);
        mg_smooth_kernel<<<grd, blk, 0, s>>>(G, 1);
        if (robin) mg_edges_kernel<<<1, 1024, 0, s>>>(G);
    }
}

// one V-cycle on grid k (d of grid 0 holds the current correction)
static void vcycle(MgHierarchy* H, size_t k, int robin, cudaStream_t s) {
    const Grid& F = H->g[k];
    if (k + 1 == H->g.size()) {
        mg_coarse_kernel<<<1, 1024, 0, s>>>(F, robin, 60);  // coarsest grid: relax to near convergence
        return;
    }
    const Grid& C = H->g[k + 1];
    dim3 blk(32, 4);
    smooth(F, robin, 2, s);
    mg_restrict_kernel<<<cells(C, blk), blk, 0, s>>>(F, C, robin);
    vcycle(H, k + 1, robin, s);
    mg_prolong_kernel<<<cells(F, blk), blk, 0, s>>>(F, C, robin);
    smooth(F, robin, 2, s);
}

int mg_launches_per_cycle(const MgHierarchy* H, int robin) {
    const int per_sweep = robin ? 3 : 2;
    const int L = (int)H->g.size();
    return (L - 1) * (4 * per_sweep + 2) + 1;
}

// ncycles V-cycles from d = 0; the correction is stored into d (level layout)
void mg_solve(MgHierarchy* H, int robin, int ncycles, float* d, long ld, cudaStream_t s) {
    for (int c = 0; c < ncycles; ++c) vcycle(H, 0, robin, s);
    dim3 blk(32, 4);
    mg_store_kernel<<<cells(H->g[0], blk), blk, 0, s>>>(H->g[0], d, ld);
}

}  // namespace ollin
