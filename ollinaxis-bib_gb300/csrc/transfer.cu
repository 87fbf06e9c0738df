// Ghost fills, mesh-refinement transfer and reductions.
//
//  * parity ghost fill on the axis and the equator (generated
//    symmetries_r.f90 / symmetries_z.f90, tags from src/base/arrays.config);
//  * coarse -> fine boundary prolongation: bicubic Lagrange interpolation in
//    space (src/base/interp.f90:146-263) times linear/quadratic Lagrange
//    interpolation in time against the fine level's own history
//    (src/base/finebound.f90:91-316 with bound_interp.inc);
//  * fine -> coarse restriction at coarse points well inside the fine box
//    (src/base/restrict.f90:70-123 with restrict_interp.inc);
//  * the 0-D statistics of save0Ddata.f90:221-288 as a deterministic
//    fixed-order block reduction.
// The transfer arithmetic uses explicitly rounded operations (no FMA
// contraction) so that it reproduces the reference's sequence of roundings.
#include <algorithm>

#include "ollin_kernels.h"

namespace ollin {

namespace {

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }

// ---- parity ghost fill -------------------------------------------------
// thread space: the g ghost columns i <= 0 over all rows (grids that own the
// axis), then the g ghost rows j <= 0 (grids that own the equator) for the
// columns not filled already; a corner point belongs to the columns when the
// grid owns the axis
__device__ __forceinline__ void symmetry_body(const SymArgs& a, unsigned bx, unsigned) {
    if (a.skip && *a.skip) return;
    const LevelGeom& G = a.G;
    const int g = G.g;
    const int ncol = G.axis ? g * (G.nz + g) : 0;
    const int i0 = G.axis ? 1 : 1 - g, ni = G.nr - i0 + 1;
    const int nrow = G.equator ? g * ni : 0;
    const int t = (int)(bx * blockDim.x + threadIdx.x);
    if (t >= ncol + nrow) return;
    int i, j;
    if (t < ncol) {
        i = 1 - g + t % g;
        j = 1 - g + t / g;
    } else {
        const int q = t - ncol;
        i = i0 + q % ni;
        j = 1 - g + q / ni;
    }
    const bool gi = G.axis && i <= 0, gj = G.equator && j <= 0;
    const int si = gi ? 1 - i : i, sj = gj ? 1 - j : j;
    const size_t o = (size_t)i + (size_t)j * G.ld, os = (size_t)si + (size_t)sj * G.ld;
    for (int k = 0; k < a.nf; ++k) {
        double* f = a.st[k];
        double v = f[os];
        if (gi && a.symr[k] < 0) v = -v;
        if (gj && a.symz[k] < 0) v = -v;
        f[o] = v;
    }
}

__global__ void __launch_bounds__(256) symmetry_kernel(const __grid_constant__ SymArgs a) {
    chain_enter();
    symmetry_body(a, blockIdx.x, blockIdx.y);
}

// ---- interp.f90 on the device ---------------------------------------------
struct InterpPt {
    int i0, j0, mode;   // mode 0: copy node, 1: bilinear, 2: bicubic
    double w[4][4];
};

// Returns false (and mode -1) when the stencil would leave the grid, which
// a consistent box layout never asks for (interp.f90:146-157 reports it and
// reads on); the callers turn that into an error instead of a stray read.
__device__ bool interp_weights(const LevelGeom& G, double rminl, double rmaxl, double zminl, double zmaxl,
                               double r0, double z0, int bicubic, InterpPt& p) {
    const int g = G.g;
    const double dr = G.dr, dz = G.dz;
    const double r1 = G.rcol[1 - g], z1 = G.zrow[1 - g];
    p.i0 = (int)((r0 - r1) / dr) + 1 - g;
    p.j0 = (int)((z0 - z1) / dz) + 1 - g;
    p.mode = -1;
    if (p.i0 < 1 - g || p.i0 > G.nr || p.j0 < 1 - g || p.j0 > G.nz) return false;
    const double deltar = r0 - G.rcol[p.i0];
    const double deltaz = z0 - G.zrow[p.j0];
    if (deltar == 0.0 && deltaz == 0.0) { p.mode = 0; return true; }
    const bool forcelinear = ((rmaxl - r0) < dr) || ((zmaxl - z0) < dz) || ((r0 - rminl) < dr) || ((z0 - zminl) < dz);
    const double auxr = deltar / dr, auxz = deltaz / dz;
    if (!bicubic || forcelinear) {
        if (p.i0 + 1 > G.nr || p.j0 + 1 > G.nz) return false;
        // factors kept separate: the reference multiplies left to right,
        // fa(0,0)*(1-auxr)*(1-auxz) + fa(1,0)*auxr*(1-auxz) + ...
        p.mode = 1;
        p.w[0][0] = auxr;
        p.w[0][1] = auxz;
        return true;
    }
    if (p.i0 - 1 < 1 - g || p.i0 + 2 > G.nr || p.j0 - 1 < 1 - g || p.j0 + 2 > G.nz) return false;
    p.mode = 2;
    for (int ii = -1; ii <= 2; ++ii)
        for (int jj = -1; jj <= 2; ++jj) {
            double aux = 1.0;
            for (int m = -1; m <= 2; ++m) {
                if (m == ii) continue;
                aux = mul(aux, sub(auxr, (double)m)) / (double)(ii - m);
            }
            for (int n = -1; n <= 2; ++n) {
                if (n == jj) continue;
                aux = mul(aux, sub(auxz, (double)n)) / (double)(jj - n);
            }
            p.w[ii + 1][jj + 1] = aux;
        }
    return true;
}

__device__ double interp_apply(const LevelGeom& G, const double* f, const InterpPt& p) {
    const long ld = G.ld;
    if (p.mode == 0) return f[p.i0 + (long)p.j0 * ld];
    if (p.mode == 1) {
        // fa(0,0)*(1-auxr)*(1-auxz) + fa(1,0)*auxr*(1-auxz) + fa(0,1)*(1-auxr)*auxz + fa(1,1)*auxr*auxz
        const double* b = f + p.i0 + (long)p.j0 * ld;
        const double ar = p.w[0][0], az = p.w[0][1];
        double v = mul(mul(b[0], sub(1.0, ar)), sub(1.0, az));
        v = add(v, mul(mul(b[1], ar), sub(1.0, az)));
        v = add(v, mul(mul(b[ld], sub(1.0, ar)), az));
        v = add(v, mul(mul(b[1 + ld], ar), az));
        return v;
    }
    double v = 0.0;
    for (int ii = -1; ii <= 2; ++ii)
        for (int jj = -1; jj <= 2; ++jj)
            v = add(v, mul(p.w[ii + 1][jj + 1], f[(p.i0 + ii) + (long)(p.j0 + jj) * ld]));
    return v;
}

// ---- restriction -----------------------------------------------------------
__global__ void __launch_bounds__(128) restrict_kernel(const __grid_constant__ RestrictArgs a) {
    if (a.skip && *a.skip) return;
    const LevelGeom& C = a.Cg;
    const LevelGeom& F = a.F;
    const int g = C.g;
    const int m = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int n = (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (m > C.nr + g - 1 || n > C.nz + g - 1) return;
    const double r0 = add(a.rminl_c, mul((double)m, C.dr));
    const double z0 = add(a.zminl_c, mul((double)n, C.dz));
    const double deltar = add(mul((double)(2 * g), F.dr), 1.0e-10);
    const double deltaz = add(mul((double)(2 * g), F.dz), 1.0e-10);
    const double rmin = (a.rminl_f < 0.0) ? 0.0 : a.rminl_f + deltar;
    const double zmin = (a.eqsym && a.zminl_f < 0.0) ? 0.0 : a.zminl_f + deltaz;
    const double rmax = a.rmaxl_f - deltar, zmax = a.zmaxl_f - deltaz;
    if (!(r0 > rmin && r0 < rmax && z0 > zmin && z0 < zmax)) return;
    const int i = (int)round((r0 - C.rcol[1 - g]) / C.dr) + 1 - g;
    const int j = (int)round((z0 - C.zrow[1 - g]) / C.dz) + 1 - g;
    if (!(i >= 1 - g && i <= C.nr && j >= 1 - g && j <= C.nz)) return;
    InterpPt p;
    if (!interp_weights(F, a.rminl_f, a.rmaxl_f, a.zminl_f, a.zmaxl_f, r0, z0, a.bicubic, p)) return;
    const size_t o = (size_t)i + (size_t)j * C.ld;
    for (int k = 0; k < a.nf; ++k) {
        const int f = a.fid[k];
        a.cout[f][o] = interp_apply(F, a.fin[f], p);
    }
}

// ---- table-driven transfers ------------------------------------------------
__device__ void to_xfer(const InterpPt& p, XferPt& x) {
    x.i0 = p.i0;
    x.j0 = p.j0;
    x.mode = p.mode;
    for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b) x.w[a * 4 + b] = p.w[a][b];
}

__device__ __forceinline__ double xfer_apply(const LevelGeom& G, const double* f, const XferPt& p) {
    const long ld = G.ld;
    if (p.mode == 0) return f[p.i0 + (long)p.j0 * ld];
    if (p.mode == 1) {
        const double* b = f + p.i0 + (long)p.j0 * ld;
        const double ar = p.w[0], az = p.w[1];
        double v = mul(mul(b[0], sub(1.0, ar)), sub(1.0, az));
        v = add(v, mul(mul(b[1], ar), sub(1.0, az)));
        v = add(v, mul(mul(b[ld], sub(1.0, ar)), az));
        v = add(v, mul(mul(b[1 + ld], ar), az));
        return v;
    }
    double v = 0.0;
    const double* b = f + (p.i0 - 1) + (long)(p.j0 - 1) * ld;
#pragma unroll
    for (int ii = 0; ii < 4; ++ii)
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) v = add(v, mul(p.w[ii * 4 + jj], b[ii + (long)jj * ld]));
    return v;
}

// The strip points of finebound.f90 for imax = ghost+2: the upper r strip
// (:153-187), the upper z strip (:296-346) and, without equatorial symmetry,
// the lower z strip (:351-397).  The reference writes the strips in that
// order, so a point that a later strip also writes takes the later value:
// ``cover`` is the strip depth from which a later strip reaches the point.
// Strips in the order finebound.f90 writes them: upper r (rR), lower r (rL,
// boxes off the axis), upper z (zR), lower z (zL, without equatorial
// symmetry or off the equator), each (imax+1) deep for imax = ghost+2.
// ``cover`` is the smallest imax at which a later strip writes the same
// point, so that the last writer wins as in the reference.
__global__ void __launch_bounds__(128) prolong_table_kernel(const __grid_constant__ ProlongArgs a, XferPt* tab) {
    const LevelGeom& F = a.F;
    const int g = F.g;
    const int imax = g + 2;
    const int nstrip_r = (imax + 1) * (F.nz + g);
    const int nstrip_z = (imax + 1) * (F.nr + g);
    const int nr_strips = F.lower_r ? 2 : 1, nz_strips = F.lower_z ? 2 : 1;
    const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (t >= nr_strips * nstrip_r + nz_strips * nstrip_z) return;
    double r0, z0;
    int depth, strip;  // 0 rR, 1 rL, 2 zR, 3 zL
    if (t < nr_strips * nstrip_r) {
        const int q = t % nstrip_r;
        const int m = q / (F.nz + g), n = q % (F.nz + g);
        strip = t / nstrip_r;
        r0 = strip == 0 ? sub(a.rmaxl_f, mul((double)m, F.dr)) : add(a.rminl_f, mul((double)m, F.dr));
        z0 = add(a.zminl_f, mul((double)n, F.dz));
        depth = m;
    } else {
        const int q0 = t - nr_strips * nstrip_r;
        const int q = q0 % nstrip_z;
        const int n = q / (F.nr + g), m = q % (F.nr + g);
        strip = 2 + q0 / nstrip_z;
        r0 = add(a.rminl_f, mul((double)m, F.dr));
        z0 = strip == 2 ? sub(a.zmaxl_f, mul((double)n, F.dz)) : add(a.zminl_f, mul((double)n, F.dz));
        depth = n;
    }
    XferPt x{};
    x.depth = depth;
    const int i = (int)round((r0 - F.rcol[1 - g]) / F.dr) + 1 - g;
    const int j = (int)round((z0 - F.zrow[1 - g]) / F.dz) + 1 - g;
    x.o_out = kNoPoint;
    x.cover = 1 << 30;
    if (strip < 1 && F.lower_r) x.cover = min(x.cover, i - (1 - g));  // rL reaches column i
    if (strip < 2) x.cover = min(x.cover, F.nz - j);                   // zR reaches row j
    if (strip < 3 && F.lower_z) x.cover = min(x.cover, j - (1 - g));  // zL reaches row j
    if (i >= 1 - g && i <= F.nr && j >= 1 - g && j <= F.nz) {
        InterpPt p;
        if (interp_weights(a.Cg, a.rminl_c, a.rmaxl_c, a.zminl_c, a.zmaxl_c, r0, z0, a.bicubic, p)) {
            to_xfer(p, x);
            x.o_out = i + j * F.ld;
        } else {
            x.mode = -1;  // the host refuses the layout
        }
    }
    tab[t] = x;
}

// ``syncboxes`` (syncboxes.f90:48-216): the strips of grid P up to 3*ghost
// deep in the order rR, rL (P off the axis), zR, zL (P off the equator or no
// equatorial symmetry), at the points well inside grid Q, interpolated from
// Q (intersect_interp.inc).  ``depth`` holds the offset of the Q node the
// point coincides with (to rounding), or -1.
__global__ void __launch_bounds__(128) sync_table_kernel(const __grid_constant__ SyncTableArgs a, XferPt* tab) {
    const LevelGeom& F = a.P;
    const LevelGeom& Q = a.Q;
    const int g = F.g;
    const int imax = 3 * g;
    const int nstrip_r = (imax + 1) * (F.nz + g);
    const int nstrip_z = (imax + 1) * (F.nr + g);
    const int nr_strips = F.lower_r ? 2 : 1, nz_strips = F.lower_z ? 2 : 1;
    const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (t >= nr_strips * nstrip_r + nz_strips * nstrip_z) return;
    double r0, z0;
    if (t < nr_strips * nstrip_r) {
        const int q = t % nstrip_r;
        const int m = q / (F.nz + g), n = q % (F.nz + g);
        r0 = (t < nstrip_r) ? sub(a.rmaxl_p, mul((double)m, F.dr)) : add(a.rminl_p, mul((double)m, F.dr));
        z0 = add(a.zminl_p, mul((double)n, F.dz));
    } else {
        const int q0 = t - nr_strips * nstrip_r;
        const int q = q0 % nstrip_z;
        const int n = q / (F.nr + g), m = q % (F.nr + g);
        r0 = add(a.rminl_p, mul((double)m, F.dr));
        z0 = (q0 < nstrip_z) ? sub(a.zmaxl_p, mul((double)n, F.dz)) : add(a.zminl_p, mul((double)n, F.dz));
    }
    XferPt x{};
    x.o_out = kNoPoint;
    x.depth = -1;
    const double deltar = mul((double)(3 * g), F.dr), deltaz = mul((double)(3 * g), F.dz);
    if (r0 >= add(a.rminl_q, deltar) && r0 <= sub(a.rmaxl_q, deltar) && z0 >= add(a.zminl_q, deltaz) &&
        z0 <= sub(a.zmaxl_q, deltaz)) {
        const int i = (int)round((r0 - F.rcol[1 - g]) / F.dr) + 1 - g;
        const int j = (int)round((z0 - F.zrow[1 - g]) / F.dz) + 1 - g;
        if (i >= 1 - g && i <= F.nr && j >= 1 - g && j <= F.nz) {
            InterpPt p;
            if (interp_weights(Q, a.rminl_q, a.rmaxl_q, a.zminl_q, a.zmaxl_q, r0, z0, a.bicubic, p)) {
                to_xfer(p, x);
                x.o_out = i + j * F.ld;
                // the coinciding Q node
                const double er = (r0 - Q.rcol[p.i0]) / Q.dr, ez = (z0 - Q.zrow[p.j0]) / Q.dz;
                const int ni = fabs(er) < 1e-9 ? p.i0 : (fabs(er - 1.0) < 1e-9 ? p.i0 + 1 : -1 << 30);
                const int nj = fabs(ez) < 1e-9 ? p.j0 : (fabs(ez - 1.0) < 1e-9 ? p.j0 + 1 : -1 << 30);
                if (ni >= 1 - g && ni <= Q.nr && nj >= 1 - g && nj <= Q.nz) x.depth = ni + nj * Q.ld;
            } else {
                x.mode = -1;
            }
        }
    }
    tab[t] = x;
}

// thread per (stencil, field); the strips of a smaller imax are the entries
// with depth <= imax
__device__ __forceinline__ void prolong_tab_body(const ProlongArgs& a, unsigned bx, unsigned) {
    if (a.skip && *a.skip) return;
    const int t = (int)(bx * blockDim.x + threadIdx.x);
    if (t >= a.ntab * a.nf) return;
    const int e = t % a.ntab, k = t / a.ntab;
    const XferPt& P = a.tab[e];
    if (P.o_out == kNoPoint || P.depth > a.imax || P.cover <= a.imax) return;
    const int f = a.fid[k];
    const double aux2 = xfer_apply(a.Cg, a.cin[f], P);
    double v;
    if (a.tmode == 0) v = aux2;
    else if (a.tmode == 1) v = add(mul(a.wa, aux2), mul(a.wp, a.fp[f][P.o_out]));
    else v = add(add(mul(a.wa, aux2), mul(a.wp, a.fp[f][P.o_out])), mul(a.wpp, a.fpp[f][P.o_out]));
    a.fout[f][P.o_out] = v;
}

__global__ void __launch_bounds__(256) prolong_tab_kernel(const __grid_constant__ ProlongArgs a) {
    chain_enter();
    prolong_tab_body(a, blockIdx.x, blockIdx.y);
}

// the coarse points of restrict_kernel inside the overlap rectangle
// m_lo..m_lo+nm-1, n_lo..n_lo+nn-1
__global__ void __launch_bounds__(128) restrict_table_kernel(const __grid_constant__ RestrictArgs a, XferPt* tab,
                                                             int m_lo, int n_lo, int nm, int nn) {
    const LevelGeom& C = a.Cg;
    const LevelGeom& F = a.F;
    const int g = C.g;
    const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (t >= nm * nn) return;
    const int m = m_lo + t % nm, n = n_lo + t / nm;
    XferPt x{};
    x.o_out = kNoPoint;
    const double r0 = add(a.rminl_c, mul((double)m, C.dr));
    const double z0 = add(a.zminl_c, mul((double)n, C.dz));
    const double deltar = add(mul((double)(2 * g), F.dr), 1.0e-10);
    const double deltaz = add(mul((double)(2 * g), F.dz), 1.0e-10);
    const double rmin = (a.rminl_f < 0.0) ? 0.0 : a.rminl_f + deltar;
    const double zmin = (a.eqsym && a.zminl_f < 0.0) ? 0.0 : a.zminl_f + deltaz;
    const double rmax = a.rmaxl_f - deltar, zmax = a.zmaxl_f - deltaz;
    if (r0 > rmin && r0 < rmax && z0 > zmin && z0 < zmax) {
        const int i = (int)round((r0 - C.rcol[1 - g]) / C.dr) + 1 - g;
        const int j = (int)round((z0 - C.zrow[1 - g]) / C.dz) + 1 - g;
        if (i >= 1 - g && i <= C.nr && j >= 1 - g && j <= C.nz) {
            InterpPt p;
            if (interp_weights(F, a.rminl_f, a.rmaxl_f, a.zminl_f, a.zmaxl_f, r0, z0, a.bicubic, p)) {
                to_xfer(p, x);
                x.o_out = i + j * C.ld;
            } else {
                x.mode = -1;
            }
        }
    }
    tab[t] = x;
}

__device__ __forceinline__ void restrict_tab_body(const RestrictArgs& a, unsigned bx, unsigned) {
    if (a.skip && *a.skip) return;
    const int t = (int)(bx * blockDim.x + threadIdx.x);
    if (t >= a.ntab * a.nf) return;
    const int e = t % a.ntab, k = t / a.ntab;
    const XferPt& P = a.tab[e];
    if (P.o_out == kNoPoint) return;
    const int f = a.fid[k];
    a.cout[f][P.o_out] = xfer_apply(a.F, a.fin[f], P);
}

__global__ void __launch_bounds__(256) restrict_tab_kernel(const __grid_constant__ RestrictArgs a) {
    chain_enter();
    restrict_tab_body(a, blockIdx.x, blockIdx.y);
}

// ---- injection: interpolate a coarser level to every point of a finer one --
// (wave_elliptic.f90:270-328; sor_elliptic.f90:268-320)
__global__ void __launch_bounds__(128) inject_kernel(const __grid_constant__ InjectArgs a) {
    const LevelGeom& F = a.F;
    const int g = F.g;
    const int m = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int n = (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (m > F.nr + g - 1 || n > F.nz + g - 1) return;
    const double r0 = add(a.rminl_f, mul((double)m, F.dr));
    const double z0 = add(a.zminl_f, mul((double)n, F.dz));
    const int i = (int)round((r0 - F.rcol[1 - g]) / F.dr) + 1 - g;
    const int j = (int)round((z0 - F.zrow[1 - g]) / F.dz) + 1 - g;
    if (!(i >= 1 - g && i <= F.nr && j >= 1 - g && j <= F.nz)) return;
    InterpPt p;
    if (!interp_weights(a.Cg, a.rminl_c, a.rmaxl_c, a.zminl_c, a.zmaxl_c, r0, z0, a.bicubic, p)) return;
    a.fout[(size_t)i + (size_t)j * F.ld] = interp_apply(a.Cg, a.cin, p);
}

// ---- 0-D statistics (save0Ddata.f90:221-288, origin value :370-374) --------
// Two passes, both deterministic: the partial pass gives each of nb blocks a
// fixed set of points (a grid-stride walk) and combines its threads by warp
// shuffles in a fixed tree, then its 8 warps in a fixed order; the final
// pass combines the nb partials the same way in one block.  So the result
// depends on the grid size only, never on scheduling.  (The reference sums
// in loop order; the tree order changes the sum of squares by rounding
// only.)
struct NormAcc {
    double vmax, vmin, nm1, nm2;
    int nan;
};

__device__ __forceinline__ NormAcc norm_combine(NormAcc a, const NormAcc& b) {
    a.vmax = fmax(a.vmax, b.vmax);
    a.vmin = fmin(a.vmin, b.vmin);
    a.nm1 = fmax(a.nm1, b.nm1);
    a.nm2 = a.nm2 + b.nm2;
    a.nan |= b.nan;
    return a;
}

// the block's threads combined into thread 0 (blockDim.x == kNormThreads)
__device__ __forceinline__ NormAcc norm_block(NormAcc a) {
    __shared__ NormAcc warp_acc[kNormThreads / 32];
    for (int off = 16; off > 0; off >>= 1) {
        NormAcc b;
        b.vmax = __shfl_down_sync(0xffffffffu, a.vmax, off);
        b.vmin = __shfl_down_sync(0xffffffffu, a.vmin, off);
        b.nm1 = __shfl_down_sync(0xffffffffu, a.nm1, off);
        b.nm2 = __shfl_down_sync(0xffffffffu, a.nm2, off);
        b.nan = __shfl_down_sync(0xffffffffu, a.nan, off);
        a = norm_combine(a, b);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) warp_acc[warp] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        a = warp_acc[0];
        for (int w = 1; w < kNormThreads / 32; ++w) a = norm_combine(a, warp_acc[w]);
    }
    return a;
}

__global__ void __launch_bounds__(kNormThreads) norms_partial_kernel(LevelGeom G, const double* f, double* part) {
    const int ni = G.nr - G.g, nj = G.nz - G.g;
    const long npts = (long)ni * nj;
    NormAcc a{-1.0e10, 1.0e10, 0.0, 0.0, 0};
    for (long q = blockIdx.x * (long)kNormThreads + threadIdx.x; q < npts; q += (long)gridDim.x * kNormThreads) {
        const int i = 1 + (int)(q % ni), j = 1 + (int)(q / ni);
        const double v = f[(size_t)i + (size_t)j * G.ld];
        if (v != v) a.nan = 1;
        a.vmax = fmax(a.vmax, v);
        a.vmin = fmin(a.vmin, v);
        a.nm1 = fmax(a.nm1, fabs(v));
        a.nm2 = a.nm2 + v * v;
    }
    a = norm_block(a);
    if (threadIdx.x == 0) {
        double* p = part + 5 * (size_t)blockIdx.x;
        p[0] = a.vmax; p[1] = a.vmin; p[2] = a.nm1; p[3] = a.nm2; p[4] = a.nan ? 1.0 : 0.0;
    }
}

__global__ void __launch_bounds__(kNormThreads) norms_final_kernel(LevelGeom G, const double* f, int bicubic,
                                                                   double rminl, double zminl, double rmaxl,
                                                                   double zmaxl, const double* part, int nb,
                                                                   double* out) {
    NormAcc a{-1.0e10, 1.0e10, 0.0, 0.0, 0};
    for (int b = threadIdx.x; b < nb; b += kNormThreads) {
        const double* p = part + 5 * (size_t)b;
        a = norm_combine(a, NormAcc{p[0], p[1], p[2], p[3], p[4] != 0.0 ? 1 : 0});
    }
    a = norm_block(a);
    if (threadIdx.x == 0) {
        const long npts = (long)(G.nr - G.g) * (G.nz - G.g);
        out[0] = a.vmax;
        out[1] = a.vmin;
        out[2] = a.nm1;
        out[3] = sqrt(a.nm2 / (double)npts);
        if (bicubic >= 0) {
            InterpPt p;
            out[4] = interp_weights(G, rminl, rmaxl, zminl, zmaxl, 0.0, 0.0, bicubic, p) ? interp_apply(G, f, p) : 0.0;
        } else {
            out[4] = 0.0;  // save0Ddata.f90:370-374 writes origin data for box 0 only
        }
        out[5] = a.nan ? 1.0 : 0.0;
    }
}

// constraints.f90:63-93: copy the next-to-edge value onto every outer edge,
// then the axis/equator parity fill (even).  One thread per edge row/column.
__global__ void ham_edges_kernel(LevelGeom G, double* h) {
    const int g = G.g;
    const long ld = G.ld;
    auto H = [&](int i, int j) -> double& { return h[(size_t)i + (size_t)j * ld]; };
    // four sequential edge copies in the reference order
    for (int j = 1 - g + (int)threadIdx.x; j <= G.nz; j += blockDim.x) H(1 - g, j) = H(2 - g, j);
    __syncthreads();
    for (int j = 1 - g + (int)threadIdx.x; j <= G.nz; j += blockDim.x) H(G.nr, j) = H(G.nr - 1, j);
    __syncthreads();
    for (int i = 1 - g + (int)threadIdx.x; i <= G.nr; i += blockDim.x) H(i, 1 - g) = H(i, 2 - g);
    __syncthreads();
    for (int i = 1 - g + (int)threadIdx.x; i <= G.nr; i += blockDim.x) H(i, G.nz) = H(i, G.nz - 1);
    __syncthreads();
    if (G.axis)
        for (int j = 1 - g + (int)threadIdx.x; j <= G.nz; j += blockDim.x)
            for (int ii = 1; ii <= g; ++ii) H(1 - ii, j) = H(ii, j);
    __syncthreads();
    if (G.equator)
        for (int i = 1 - g + (int)threadIdx.x; i <= G.nr; i += blockDim.x)
            for (int jj = 1; jj <= g; ++jj) H(i, 1 - jj) = H(i, jj);
}

__global__ void gammadriver_init_kernel(LevelGeom G, double* dtbr, double* dtbz, const double* dlr, const double* dlz, double csi) {
    const int i = 1 - G.g + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = 1 - G.g + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (i > G.nr || j > G.nz) return;
    const size_t o = (size_t)i + (size_t)j * G.ld;
    dtbr[o] = csi * dlr[o];
    dtbz[o] = csi * dlz[o];
}

__global__ void phi_from_chi_kernel(LevelGeom G, const double* chi, double* out) {
    const int i = 1 - G.g + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = 1 - G.g + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (i > G.nr || j > G.nz) return;
    const size_t o = (size_t)i + (size_t)j * G.ld;
    out[o] = -log(chi[o]) / 2.0;
}

// FP64 issue-rate probe: eight independent DFMA chains per thread.
__global__ void fp64_probe_kernel(double* out, int iters, double seed) {
    const int gid = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    double a0 = seed + gid * 1e-9, a1 = a0 + 0.1, a2 = a0 + 0.2, a3 = a0 + 0.3;
    double a4 = a0 + 0.4, a5 = a0 + 0.5, a6 = a0 + 0.6, a7 = a0 + 0.7;
    const double m = 0.999999, c = 1e-7;
    for (int k = 0; k < iters; ++k) {
        a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
        a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
    }
    out[gid] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

// One operation of the rate table, applied to one chain value.  Every chain
// stays bounded and finite: the divide alternates between two values, sqrt,
// cbrt and exp(-x) converge to fixed points, log(x + 2) converges to 1.146.
template <int OP>
__device__ __forceinline__ double probe_op(double a, double m, double c) {
    if constexpr (OP == 0) return fma(a, m, c);
    else if constexpr (OP == 1) return a + c;
    else if constexpr (OP == 2) return a * m;
    else if constexpr (OP == 3) return m / a;
    else if constexpr (OP == 4) return sqrt(a);
    else if constexpr (OP == 5) return cbrt(a);
    else if constexpr (OP == 6) return exp(-a);
    else return log(a + 2.0);
}

template <int OP>
__global__ void op_probe_kernel(double* out, int iters, double seed) {
    const int gid = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    double a[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) a[u] = seed + 0.1 * u + gid * 1e-9;
    const double m = 0.999999, c = 1e-7;
    for (int k = 0; k < iters; ++k) {
#pragma unroll
        for (int u = 0; u < 8; ++u) a[u] = probe_op<OP>(a[u], m, c);
    }
    double t = 0.0;
#pragma unroll
    for (int u = 0; u < 8; ++u) t += a[u];
    out[gid] = t;
}

// FP32 FMA chains, for the FP32/FP64 rate ratio.
__global__ void ffma_probe_kernel(double* out, int iters, double seed) {
    const int gid = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    float a[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) a[u] = (float)seed + 0.1f * u + gid * 1e-6f;
    const float m = 0.9999f, c = 1e-4f;
    for (int k = 0; k < iters; ++k) {
#pragma unroll
        for (int u = 0; u < 8; ++u) a[u] = fmaf(a[u], m, c);
    }
    float t = 0.f;
#pragma unroll
    for (int u = 0; u < 8; ++u) t += a[u];
    out[gid] = (double)t;
}

dim3 full_grid(const LevelGeom& G, dim3 blk) {
    return dim3((G.nr + G.g + blk.x - 1) / blk.x, (G.nz + G.g + blk.y - 1) / blk.y);
}

// interp.f90 at n arbitrary points (rz[2k], rz[2k+1]) of one grid: out[k],
// or NaN where the stencil would leave the grid (counted in *bad)
__global__ void __launch_bounds__(128) interp_points_kernel(LevelGeom G, double rminl, double rmaxl, double zminl,
                                                            double zmaxl, int bicubic, const double* f,
                                                            const double* rz, int n, double* out,
                                                            unsigned int* bad) {
    const int k = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (k >= n) return;
    InterpPt p;
    if (interp_weights(G, rminl, rmaxl, zminl, zmaxl, rz[2 * k], rz[2 * k + 1], bicubic, p)) {
        out[k] = interp_apply(G, f, p);
    } else {
        out[k] = __longlong_as_double(0x7ff8000000000000LL);
        atomicAdd(bad, 1u);
    }
}

const MultiRegistration reg_symmetry((const void*)symmetry_kernel, multi_launch<SymArgs, symmetry_body, 256, 1>);
const MultiRegistration reg_prolong((const void*)prolong_tab_kernel,
                                    multi_launch<ProlongArgs, prolong_tab_body, 256, 1>);
const MultiRegistration reg_restrict((const void*)restrict_tab_kernel,
                                     multi_launch<RestrictArgs, restrict_tab_body, 256, 1>);

}  // namespace

void launch_symmetry(const SymArgs& a, cudaStream_t s) {
    const int n = (a.G.axis ? a.G.g * (a.G.nz + a.G.g) : 0) +
                  (a.G.equator ? a.G.g * (a.G.axis ? a.G.nr : a.G.nr + a.G.g) : 0);
    if (n == 0) return;
    launch_chained(symmetry_kernel, dim3((n + 255) / 256), dim3(256), s, a);
}


int prolong_table_size(const LevelGeom& F) {
    return (F.lower_r ? 2 : 1) * (F.g + 3) * (F.nz + F.g) + (F.lower_z ? 2 : 1) * (F.g + 3) * (F.nr + F.g);
}

int sync_table_size(const LevelGeom& P) {
    return (P.lower_r ? 2 : 1) * (3 * P.g + 1) * (P.nz + P.g) + (P.lower_z ? 2 : 1) * (3 * P.g + 1) * (P.nr + P.g);
}

void launch_sync_table(const SyncTableArgs& a, XferPt* tab, cudaStream_t s) {
    const int n = sync_table_size(a.P);
    sync_table_kernel<<<(n + 127) / 128, 128, 0, s>>>(a, tab);
}

void launch_prolong_table(const ProlongArgs& a, XferPt* tab, cudaStream_t s) {
    const int n = prolong_table_size(a.F);
    prolong_table_kernel<<<(n + 127) / 128, 128, 0, s>>>(a, tab);
}

void launch_prolong_tab(const ProlongArgs& a, cudaStream_t s) {
    const long n = (long)a.ntab * a.nf;
    launch_chained(prolong_tab_kernel, dim3((unsigned)((n + 255) / 256)), dim3(256), s, a);
}

void launch_restrict_table(const RestrictArgs& a, XferPt* tab, int m_lo, int n_lo, int nm, int nn, cudaStream_t s) {
    const int n = nm * nn;
    if (n > 0) restrict_table_kernel<<<(n + 127) / 128, 128, 0, s>>>(a, tab, m_lo, n_lo, nm, nn);
}

void launch_restrict_tab(const RestrictArgs& a, cudaStream_t s) {
    const long n = (long)a.ntab * a.nf;
    if (n > 0) launch_chained(restrict_tab_kernel, dim3((unsigned)((n + 255) / 256)), dim3(256), s, a);
}

void launch_inject(const InjectArgs& a, cudaStream_t s) {
    dim3 blk(32, 4);
    dim3 grd((a.F.nr + a.F.g + blk.x - 1) / blk.x, (a.F.nz + a.F.g + blk.y - 1) / blk.y);
    inject_kernel<<<grd, blk, 0, s>>>(a);
}

void launch_restrict(const RestrictArgs& a, cudaStream_t s) {
    dim3 blk(32, 4);
    dim3 grd((a.Cg.nr + a.Cg.g + blk.x - 1) / blk.x, (a.Cg.nz + a.Cg.g + blk.y - 1) / blk.y);
    restrict_kernel<<<grd, blk, 0, s>>>(a);
}

int norm_blocks(const LevelGeom& G) {
    const long npts = (long)(G.nr - G.g) * (G.nz - G.g);
    const long nb = (npts + 4L * kNormThreads - 1) / (4L * kNormThreads);  // about 4 points per thread
    return (int)std::max(1L, std::min((long)kNormMaxBlocks, nb));
}

void launch_norms(const LevelGeom& G, const double* f, int bicubic, double rminl, double zminl,
                  double rmaxl, double zmaxl, double* dev_out, double* partials, cudaStream_t s) {
    const int nb = norm_blocks(G);
    norms_partial_kernel<<<nb, kNormThreads, 0, s>>>(G, f, partials);
    norms_final_kernel<<<1, kNormThreads, 0, s>>>(G, f, bicubic, rminl, zminl, rmaxl, zmaxl, partials, nb, dev_out);
}

void launch_interp_points(const LevelGeom& G, double rminl, double rmaxl, double zminl, double zmaxl, int bicubic,
                          const double* f, const double* rz, int n, double* out, unsigned int* bad, cudaStream_t s) {
    if (n <= 0) return;
    interp_points_kernel<<<(n + 127) / 128, 128, 0, s>>>(G, rminl, rmaxl, zminl, zmaxl, bicubic, f, rz, n, out, bad);
}

void launch_ham_edges(const LevelGeom& G, double* ham, cudaStream_t s) {
    ham_edges_kernel<<<1, 256, 0, s>>>(G, ham);
}

void launch_gammadriver_init(const LevelGeom& G, double* dtbr, double* dtbz, const double* dlr,
                             const double* dlz, double csi, cudaStream_t s) {
    dim3 blk(64, 4);
    gammadriver_init_kernel<<<full_grid(G, blk), blk, 0, s>>>(G, dtbr, dtbz, dlr, dlz, csi);
}

void launch_phi_from_chi(const LevelGeom& G, const double* chi, double* out, cudaStream_t s) {
    dim3 blk(64, 4);
    phi_from_chi_kernel<<<full_grid(G, blk), blk, 0, s>>>(G, chi, out);
}

double measure_op_rate(int op, cudaStream_t s) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // the slow operations get fewer iterations, so every launch lasts ~1-10 ms
    static const int kIters[9] = {4096, 4096, 4096, 1024, 1024, 512, 512, 256, 65536};
    if (op < 0 || op > 8) return -1.0;
    const int blocks = sms * 8, threads = 256, iters = kIters[op];
    double* out = nullptr;
    if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return -1.0;
    auto launch = [&](int n) {
        switch (op) {
            case 0: fp64_probe_kernel<<<blocks, threads, 0, s>>>(out, n, 0.5); break;
            case 1: op_probe_kernel<1><<<blocks, threads, 0, s>>>(out, n, 0.5); break;
            case 2: op_probe_kernel<2><<<blocks, threads, 0, s>>>(out, n, 0.5); break;
            case 3: op_probe_kernel<3><<<blocks, threads, 0, s>>>(out, n, 0.5); break;
            case 4: op_probe_kernel<4><<<blocks, threads, 0, s>>>(out, n, 0.5); break;
            case 5: op_probe_kernel<5><<<blocks, threads, 0, s>>>(out, n, 0.5); break;
            case 6: op_probe_kernel<6><<<blocks, threads, 0, s>>>(out, n, 0.5); break;
            case 7: op_probe_kernel<7><<<blocks, threads, 0, s>>>(out, n, 0.5); break;
            default: ffma_probe_kernel<<<blocks, threads, 0, s>>>(out, n, 0.5); break;
        }
    };
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    launch(16);
    cudaEventRecord(e0, s);
    launch(iters);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (cudaGetLastError() != cudaSuccess || !(ms > 0.f)) return -1.0;
    return (double)blocks * threads * iters * 8.0 / (ms * 1e-3);
}

double measure_fp64_dfma_rate(cudaStream_t s) { return measure_op_rate(0, s); }

}  // namespace ollin
