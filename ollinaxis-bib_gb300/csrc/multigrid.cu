// Geometric multigrid for the correction equation J d = r of the
// mixed-precision elliptic solve (the discrete system that the SOR of
// src/elliptic/sor_elliptic.f90 converges to), in FP32; the same hierarchy in
// FP64 gives the all-FP64 solve of that system that the mixed solve's error is
// measured against.
//
// J is the five-point part of the level's stencil with variable coefficients
// (the physical Laplacian of maximal slicing has g^rr/psi^4 and g^zz/psi^4
// varying by orders of magnitude in a strong Brill wave; the flat Laplacian of
// the initial data is the case krr = kzz = 1, vr = vz = 0):
//   aE d(I+1,J) + aW d(I-1,J) + aN d(I,J+1) + aS d(I,J-1) + e d(I,J) = r
//   aE = krr (1/Hr + 1/(2 r_I))/Hr + vr/(2Hr),  aW = krr (1/Hr - 1/(2 r_I))/Hr - vr/(2Hr)
//   aN = kzz/Hz^2 + vz/(2Hz),                    aS = kzz/Hz^2 - vz/(2Hz)
//   e  = -2 (krr/Hr^2 + kzz/Hz^2) + s
// per cell of a grid of n x m cells, cell centres r_I = r0 + (I-1/2) Hr,
// z_J = (J-1/2) Hz, Hr = 2^k dr; at the lower edges d(0,J) = d(1,J),
// d(I,0) = d(I,1) (axis and equator mirrors) or, on a refinement box off the
// axis or the equator, d = 0 there (the Dirichlet row of its problem); Robin
// rows I = n / J = m on the coarse problem (and J = 0 on a coarse problem
// without equatorial symmetry, whose lowest level row is a Robin row), zero
// rows on the Dirichlet problems of the finer refinement levels and boxes.  The nine-
// point couplings of a metric with g^rz /= 0 are left to the FP64 residual of
// the outer iteration.
// Cell (I,J) of grid k+1 covers cells 2I-1..2I x 2J-1..2J of grid k: the
// coefficient fields and the residual are averaged (the two Robin residuals
// on a boundary row), prolongation is bilinear in the cell centres (9/16,
// 3/16, 3/16, 1/16).  Smoother: red-black Gauss-Seidel, Robin rows by
// two-colour Gauss-Seidel along each edge.  Arrays are compact, (n+2) x (m+2)
// with one ghost layer: element (I,J) at [I + J (n+2)].
#include <vector>

#include "ollin_kernels.h"

namespace ollin {

namespace {

template <typename T>
struct Grid {
    int n, m, ld;
    int mr, mz;                          // lower edges mirrored (1) or Dirichlet zero rows (0)
    int rz;                              // row J = 0 is a Robin row (no equatorial symmetry)
    T r0, z0;                            // r, z of the lower faces of cell (1, 1)
    T hr, hz;                            // spacings
    T* d; T* r;                          // correction, right-hand side
    T* krr; T* kzz; T* vr; T* vz; T* s;  // coefficient fields
};

__device__ __forceinline__ int mirror(int k) { return k < 1 ? 1 - k : k; }

// a Dirichlet lower edge keeps index 0 at zero and a lower Robin row holds
// its unknowns there, so both read as they are
template <typename T>
__device__ __forceinline__ T Dv(const Grid<T>& G, int i, int j) {
    return G.d[(G.mr ? mirror(i) : i) + (G.mz ? mirror(j) : j) * G.ld];
}

template <typename T>
struct Stencil { T e, w, n, s, c; };

template <typename T>
__device__ __forceinline__ Stencil<T> stencil(const Grid<T>& G, int i, int j) {
    const int o = i + j * G.ld;
    const T ri = G.r0 + ((T)i - T(0.5)) * G.hr;
    const T krr = G.krr[o], kzz = G.kzz[o];
    const T ihr = T(1.0) / G.hr, ihz = T(1.0) / G.hz;
    const T ur = T(0.5) * G.vr[o] * ihr, uz = T(0.5) * G.vz[o] * ihz;
    Stencil<T> q;
    q.e = krr * (ihr + T(0.5) / ri) * ihr + ur;
    q.w = krr * (ihr - T(0.5) / ri) * ihr - ur;
    q.n = kzz * ihz * ihz + uz;
    q.s = kzz * ihz * ihz - uz;
    q.c = T(-2.0) * (krr * ihr * ihr + kzz * ihz * ihz) + G.s[o];
    return q;
}

// residual of one interior equation
template <typename T>
__device__ __forceinline__ T interior_res(const Grid<T>& G, int i, int j) {
    const Stencil<T> q = stencil(G, i, j);
    const int o = i + j * G.ld;
    return G.r[o] - (q.e * Dv(G, i + 1, j) + q.w * Dv(G, i - 1, j) + q.n * Dv(G, i, j + 1) + q.s * Dv(G, i, j - 1)
                     + q.c * G.d[o]);
}

// residual of a Robin row (coarse problem); cr = r_n/Hr = n - 1/2, cz = J - 1/2.
// The lower Robin row J = 0 faces -z (cz < 0 there):
//   (1 - 1.5 cz) d + cz/2 (4 d(I,1) - d(I,2)) + cr_I/2 (d(I+1,0) - d(I-1,0)) = r
template <typename T>
__device__ __forceinline__ T robin_res(const Grid<T>& G, int i, int j) {
    const int n = G.n, m = G.m;
    // r/Hr and z/Hz at the cell centres of the Robin rows
    const T cr = G.r0 / G.hr + (T)n - T(0.5), czn = G.z0 / G.hz + (T)m - T(0.5);
    const T cz0 = G.z0 / G.hz - T(0.5);
    T lhs;
    if (j == 0 && i == n) {
        lhs = (T(1.0) + T(1.5) * (cr - cz0)) * Dv(G, i, 0) - T(0.5) * cr * (T(4.0) * Dv(G, i - 1, 0) - Dv(G, i - 2, 0))
              + T(0.5) * cz0 * (T(4.0) * Dv(G, i, 1) - Dv(G, i, 2));
    } else if (j == 0) {
        const T crr = G.r0 / G.hr + (T)i - T(0.5);
        lhs = (T(1.0) - T(1.5) * cz0) * Dv(G, i, 0) + T(0.5) * cz0 * (T(4.0) * Dv(G, i, 1) - Dv(G, i, 2))
              + T(0.5) * crr * (Dv(G, i + 1, 0) - Dv(G, i - 1, 0));
    } else if (i == n && j == m) {
        lhs = (T(1.0) + T(1.5) * (cr + czn)) * Dv(G, i, j) - T(0.5) * cr * (T(4.0) * Dv(G, i - 1, j) - Dv(G, i - 2, j))
              - T(0.5) * czn * (T(4.0) * Dv(G, i, j - 1) - Dv(G, i, j - 2));
    } else if (i == n) {
        const T cz = G.z0 / G.hz + (T)j - T(0.5);
        lhs = (T(1.0) + T(1.5) * cr) * Dv(G, i, j) - T(0.5) * cr * (T(4.0) * Dv(G, i - 1, j) - Dv(G, i - 2, j))
              + T(0.5) * cz * (Dv(G, i, j + 1) - Dv(G, i, j - 1));
    } else {
        const T crr = G.r0 / G.hr + (T)i - T(0.5);
        lhs = (T(1.0) + T(1.5) * czn) * Dv(G, i, j) - T(0.5) * czn * (T(4.0) * Dv(G, i, j - 1) - Dv(G, i, j - 2))
              + T(0.5) * crr * (Dv(G, i + 1, j) - Dv(G, i - 1, j));
    }
    return G.r[i + j * G.ld] - lhs;
}

// Gauss-Seidel update of one interior cell (the mirrored neighbours across
// the axis and the equator fold into the diagonal; a Dirichlet lower row
// contributes nothing)
template <typename T>
__device__ __forceinline__ void relax(const Grid<T>& G, int i, int j) {
    const Stencil<T> q = stencil(G, i, j);
    const int o = i + j * G.ld;
    T diag = q.c;
    T off = q.e * G.d[o + 1] + q.n * G.d[o + G.ld];
    if (i > 1) off += q.w * G.d[o - 1]; else if (G.mr) diag += q.w;
    if (j > 1 || G.rz) off += q.s * G.d[o - G.ld]; else if (G.mz) diag += q.s;
    G.d[o] = (G.r[o] - off) / diag;
}

template <typename T>
__global__ void __launch_bounds__(128) mg_smooth_kernel(Grid<T> G, int parity) {
    const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int jh = (int)(blockIdx.y * blockDim.y + threadIdx.y);
    int j = 1;
    if (((i + j) & 1) != parity) ++j;
    j += 2 * jh;
    if (i > G.n - 1 || j > G.m - 1) return;
    relax(G, i, j);
}

// Robin rows, two-colour Gauss-Seidel along each edge, then the corner
// (called by every thread of one block)
template <typename T>
__device__ void robin_sweep(const Grid<T>& G) {
    const int n = G.n, m = G.m;
    const T cr = G.r0 / G.hr + (T)n - T(0.5), czn = G.z0 / G.hz + (T)m - T(0.5);
    const T cz0 = G.z0 / G.hz - T(0.5);
    auto D = [&](int i, int j) -> T& { return G.d[(G.mr ? mirror(i) : i) + (G.mz ? mirror(j) : j) * G.ld]; };
    for (int colour = 0; colour < 2; ++colour) {
        for (int j = 1 + colour + 2 * (int)threadIdx.x; j <= m - 1; j += 2 * blockDim.x) {
            const T cz = G.z0 / G.hz + (T)j - T(0.5);
            D(n, j) = (G.r[n + j * G.ld] + T(0.5) * cr * (T(4.0) * D(n - 1, j) - D(n - 2, j)) - T(0.5) * cz * (D(n, j + 1) - D(n, j - 1)))
                      / (T(1.0) + T(1.5) * cr);
        }
        for (int i = 1 + colour + 2 * (int)threadIdx.x; i <= n - 1; i += 2 * blockDim.x) {
            const T crr = G.r0 / G.hr + (T)i - T(0.5);
            D(i, m) = (G.r[i + m * G.ld] + T(0.5) * czn * (T(4.0) * D(i, m - 1) - D(i, m - 2)) - T(0.5) * crr * (D(i + 1, m) - D(i - 1, m)))
                      / (T(1.0) + T(1.5) * czn);
            if (G.rz)
                D(i, 0) = (G.r[i] - T(0.5) * cz0 * (T(4.0) * D(i, 1) - D(i, 2)) - T(0.5) * crr * (D(i + 1, 0) - D(i - 1, 0)))
                          / (T(1.0) - T(1.5) * cz0);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        D(n, m) = (G.r[n + m * G.ld] + T(0.5) * cr * (T(4.0) * D(n - 1, m) - D(n - 2, m)) + T(0.5) * czn * (T(4.0) * D(n, m - 1) - D(n, m - 2)))
                  / (T(1.0) + T(1.5) * (cr + czn));
        if (G.rz)
            D(n, 0) = (G.r[n] + T(0.5) * cr * (T(4.0) * D(n - 1, 0) - D(n - 2, 0)) - T(0.5) * cz0 * (T(4.0) * D(n, 1) - D(n, 2)))
                      / (T(1.0) + T(1.5) * (cr - cz0));
    }
    __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(1024) mg_edges_kernel(Grid<T> G) { robin_sweep(G); }

// coarsest grid: one block runs all the sweeps
template <typename T>
__global__ void __launch_bounds__(1024) mg_coarse_kernel(Grid<T> G, int robin, int sweeps) {
    const int n = G.n, m = G.m;
    const int ncell = (n - 1) * (m - 1);
    for (int sw = 0; sw < sweeps; ++sw) {
        for (int parity = 0; parity < 2; ++parity) {
            for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
                const int i = 1 + c % (n - 1), j = 1 + c / (n - 1);
                if (((i + j) & 1) != parity) continue;
                relax(G, i, j);
            }
            __syncthreads();
        }
        if (robin) robin_sweep(G);
    }
}

// residual of grid F restricted to the right-hand side of grid C; d_C = 0
// (a lower Robin row J = 0 from the fine grid's row 0)
template <typename T>
__global__ void __launch_bounds__(128) mg_restrict_kernel(Grid<T> F, Grid<T> C, int robin) {
    const int I = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int J = 1 - C.rz + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (I > C.n || J > C.m) return;
    const int o = I + J * C.ld;
    C.d[o] = T(0.0);
    const bool bI = I == C.n, bJ = J == C.m;
    T v = T(0.0);
    if (J == 0) {
        v = bI ? robin_res(F, F.n, 0) : T(0.5) * (robin_res(F, 2 * I - 1, 0) + robin_res(F, 2 * I, 0));
    } else if (!bI && !bJ) {
        v = T(0.25) * (interior_res(F, 2 * I - 1, 2 * J - 1) + interior_res(F, 2 * I, 2 * J - 1)
                       + interior_res(F, 2 * I - 1, 2 * J) + interior_res(F, 2 * I, 2 * J));
    } else if (robin) {
        if (bI && bJ) v = robin_res(F, F.n, F.m);
        else if (bI) v = T(0.5) * (robin_res(F, F.n, 2 * J - 1) + robin_res(F, F.n, 2 * J));
        else v = T(0.5) * (robin_res(F, 2 * I - 1, F.m) + robin_res(F, 2 * I, F.m));
    }
    C.r[o] = v;
}

// d_F += bilinear interpolation of d_C (zero rows of a Dirichlet problem
// stay; a lower Robin row, centred half a fine cell below cell 1, takes 3/4
// of the coarse row 0 and 1/4 of the coarse row 1)
template <typename T>
__global__ void __launch_bounds__(128) mg_prolong_kernel(Grid<T> F, Grid<T> C, int robin) {
    const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = 1 - F.rz + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (i > F.n || j > F.m) return;
    if (!robin && (i == F.n || j == F.m)) return;
    const int I = (i + 1) / 2, J = (j + 1) / 2;
    const int I2 = (i & 1) ? I - 1 : I + 1, J2 = (j & 1) ? J - 1 : J + 1;
    auto c = [&](int p, int q) {
        if ((p < 1 && !C.mr) || (q < 1 && !C.mz && !C.rz)) return T(0.0);  // a Dirichlet lower row
        p = p < 1 ? 1 : (p > C.n ? C.n : p);
        q = q < 1 ? (C.rz ? 0 : 1) : (q > C.m ? C.m : q);
        return C.d[p + q * C.ld];
    };
    const T v = T(0.5625) * c(I, J) + T(0.1875) * (c(I2, J) + c(I, J2)) + T(0.0625) * c(I2, J2);
    F.d[i + j * F.ld] += v;
}

// coefficient fields of grid C: averages over the four children in grid F
template <typename T>
__global__ void __launch_bounds__(128) mg_coarsen_kernel(Grid<T> F, Grid<T> C) {
    const int I = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int J = 1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (I > C.n || J > C.m) return;
    const int a = (2 * I - 1) + (2 * J - 1) * F.ld, b = a + 1, c = a + F.ld, d = c + 1;
    const int o = I + J * C.ld;
    C.krr[o] = T(0.25) * (F.krr[a] + F.krr[b] + F.krr[c] + F.krr[d]);
    C.kzz[o] = T(0.25) * (F.kzz[a] + F.kzz[b] + F.kzz[c] + F.kzz[d]);
    C.vr[o] = T(0.25) * (F.vr[a] + F.vr[b] + F.vr[c] + F.vr[d]);
    C.vz[o] = T(0.25) * (F.vz[a] + F.vz[b] + F.vz[c] + F.vz[d]);
    C.s[o] = T(0.25) * (F.s[a] + F.s[b] + F.s[c] + F.s[d]);
}

// grid 0 from the level's FP64 five-point stencil (level layout: element
// (i,j) at [i + j*ld]; cell (I,J) is level point (I + ioff, J + joff)):
// krr = (a+b) dr^2/2, vr = (a-b) dr - krr/r, kzz = (c+d) dz^2/2,
// vz = (c-d) dz, s = e + 2 (krr/dr^2 + kzz/dz^2)
template <typename T>
__global__ void __launch_bounds__(128) mg_load_kernel(Grid<T> G, MgStencil S) {
    const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (i > G.n + 1 || j > G.m + 1) return;
    const int o = i + j * G.ld;
    const bool in = i >= 1 && i <= G.n && j >= 1 && j <= G.m;
    if (!in) {
        G.krr[o] = T(0.0); G.kzz[o] = T(0.0); G.vr[o] = T(0.0); G.vz[o] = T(0.0); G.s[o] = T(0.0);
        return;
    }
    const long li = (long)i + S.ioff, lj = (long)j + S.joff;
    const long q = li + lj * S.ld;
    const double a = S.pa ? S.pa[q] : S.ca[li], b = S.pb ? S.pb[q] : S.cb[li];
    const double c = S.pc ? S.pc[q] : S.cc, d = S.pd ? S.pd[q] : S.cc;
    const double dr = S.dr, dz = S.dz, ri = S.r0 + ((double)i - 0.5) * dr;
    const double krr = (a + b) * (dr * dr) * 0.5, kzz = (c + d) * (dz * dz) * 0.5;
    G.krr[o] = (T)krr;
    G.kzz[o] = (T)kzz;
    G.vr[o] = (T)((a - b) * dr - krr / ri);
    G.vz[o] = (T)((c - d) * dz);
    G.s[o] = (T)(S.e[q] + 2.0 * (krr / (dr * dr) + kzz / (dz * dz)));
}

// the right-hand side of grid 0 (the hierarchy's precision, level layout); d = 0
template <typename T>
__global__ void __launch_bounds__(128) mg_rhs_kernel(Grid<T> G, const T* r, long ld, int ioff, int joff) {
    const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (i > G.n + 1 || j > G.m + 1) return;
    const int o = i + j * G.ld;
    G.d[o] = T(0.0);
    const bool in = i >= 1 && i <= G.n && j >= 1 - G.rz && j <= G.m;
    G.r[o] = in ? r[(long)(i + ioff) + (long)(j + joff) * ld] : T(0.0);
}

template <typename T>
__global__ void __launch_bounds__(128) mg_store_kernel(Grid<T> G, T* d, long ld, int ioff, int joff) {
    const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = 1 - G.rz + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (i > G.n || j > G.m) return;
    d[(long)(i + ioff) + (long)(j + joff) * ld] = G.d[i + j * G.ld];
}

// the cells 1..n x 1..m, from row 0 when it is a Robin row
template <typename T>
dim3 cells(const Grid<T>& G, dim3 blk) { return dim3((G.n + blk.x - 1) / blk.x, (G.m + G.rz + blk.y - 1) / blk.y); }

// ---- host side of the hierarchy ---------------------------------------------
template <typename T>
struct MgGrids {
    std::vector<Grid<T>> g;
    T* pool = nullptr;
    int ioff = 0, joff = 0;  // level point of cell (0, 0)

    bool create(int n, int m, double dr, double dz) {
        size_t total = 0;
        int nn = n, mm = m;
        double hr = dr, hz = dz;
        for (;;) {
            Grid<T> G{};
            G.n = nn; G.m = mm; G.ld = nn + 2;
            G.hr = (T)hr; G.hz = (T)hz;
            g.push_back(G);
            total += (size_t)7 * (nn + 2) * (mm + 2);
            if ((nn & 1) || (mm & 1) || nn / 2 < 4 || mm / 2 < 4) break;
            nn /= 2; mm /= 2; hr *= 2.0; hz *= 2.0;
        }
        if (cudaMalloc(&pool, total * sizeof(T)) != cudaSuccess) { pool = nullptr; return false; }
        T* q = pool;
        for (Grid<T>& G : g) {
            const size_t sz = (size_t)(G.n + 2) * (G.m + 2);
            G.d = q; q += sz; G.r = q; q += sz;
            G.krr = q; q += sz; G.kzz = q; q += sz; G.vr = q; q += sz; G.vz = q; q += sz; G.s = q; q += sz;
        }
        cudaMemset(pool, 0, total * sizeof(T));
        return true;
    }

    void load(const MgStencil& S, cudaStream_t s) {
        dim3 blk(32, 4);
        ioff = S.ioff;
        joff = S.joff;
        for (Grid<T>& G : g) {
            G.mr = S.mr;
            G.mz = S.mz;
            G.rz = S.rz;
            G.r0 = (T)S.r0;
            G.z0 = (T)S.z0;
        }
        const Grid<T>& G0 = g[0];
        mg_load_kernel<T><<<dim3((G0.n + 2 + 31) / 32, (G0.m + 2 + 3) / 4), blk, 0, s>>>(G0, S);
        for (size_t k = 1; k < g.size(); ++k) mg_coarsen_kernel<T><<<cells(g[k], blk), blk, 0, s>>>(g[k - 1], g[k]);
    }

    void rhs(const T* r, long ld, cudaStream_t s) {
        dim3 blk(32, 4);
        const Grid<T>& G0 = g[0];
        mg_rhs_kernel<T><<<dim3((G0.n + 2 + 31) / 32, (G0.m + 2 + 3) / 4), blk, 0, s>>>(G0, r, ld, ioff, joff);
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
        mg_store_kernel<T><<<cells(g[0], blk), blk, 0, s>>>(g[0], d, ld, ioff, joff);
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

void mg_load_operator(MgHierarchy* H, const MgStencil& S, cudaStream_t s) {
    if (H->fp64) H->d.load(S, s);
    else H->f.load(S, s);
}

void mg_set_rhs(MgHierarchy* H, const void* r, long ld, cudaStream_t s) {
    if (H->fp64) H->d.rhs((const double*)r, ld, s);
    else H->f.rhs((const float*)r, ld, s);
}

int mg_launches_per_cycle(const MgHierarchy* H, int robin) {
    const int per_sweep = robin ? 3 : 2;
    const int L = mg_levels(H);
    return (L - 1) * (4 * per_sweep + 2) + 1;
}

void mg_solve(MgHierarchy* H, int robin, int ncycles, void* d, long ld, cudaStream_t s) {
    if (H->fp64) H->d.solve(robin, ncycles, (double*)d, ld, s);
    else H->f.solve(robin, ncycles, (float*)d, ld, s);
}

}  // namespace ollin
