// Auxiliary-quantity kernels: the parts of ``auxiliary`` that other points'
// stencils depend on, computed once per point after every stage
// (src/base/auxiliary.f90:26-56 -> auxiliary_geometry.f90).
#include "ollin_kernels.h"

namespace ollin {

namespace {

// Pointwise part, every point including ghosts (the reference's whole-array
// statements):
//   t = 0 : chi = exp(-2 phi)                     (auxiliary_geometry.f90:178-180)
//           hdet = 1                              (:265-271)
//   t > 0 : factordet -- rescale A,B,C,H to unit (lagrangian) determinant
//                                                 (factordet.f90:38-69)
//   g_A = B H, g_B = A H, g_H = 1/H, g_C = -C H   (:473-489, hdet = 1)
//   KTH from tracelessness                        (:747-753)
//   lambda, Alambda from their definitions        (:767-773, nolambda)
//   g_lambda = C^2 - B lambda                     (:816-821)
__device__ __forceinline__ void aux_point_body(const AuxArgs& a, unsigned bx, unsigned by) {
    const LevelGeom& G = a.G;
    const int i = 1 - G.g + (int)(bx * blockDim.x + threadIdx.x);
    const int j = 1 - G.g + (int)(by * blockDim.y + threadIdx.y);
    if (i > G.nr || j > G.nz) return;
    const size_t o = (size_t)i + (size_t)j * (size_t)G.ld;
    const double r = G.rcol[i];
    double A = a.st[F_A][o], B = a.st[F_B][o], C = a.st[F_C][o], H = a.st[F_H][o];
    if (a.t0) {
        a.st[F_CHI][o] = exp(-2.0 * a.st[F_PHI][o]);
    } else if (a.project) {
        const double rc = r * C;
        const double q = (A * B - rc * rc) * H;  // hdet = 1
        const double iq = rcbrt(q);              // 1/(det)^(1/3)
        A = A * iq; B = B * iq; C = C * iq; H = H * iq;
        a.st[F_A][o] = A; a.st[F_B][o] = B; a.st[F_C][o] = C; a.st[F_H][o] = H;
    }
    const double gA = B * H, gB = A * H, gH = 1.0 / H, gC = -C * H;
    const double kA = a.st[F_KTA][o], kB = a.st[F_KTB][o], kC = a.st[F_KTC][o];
    const double r2 = r * r, ir2 = G.ircol[i] * G.ircol[i];
    const double kH = -(gA * kA + gB * kB + 2.0 * r2 * gC * kC) * H;  // .../g_H with g_H = 1/H
    const double lam = (A - H) * ir2;
    a.aux[X_GA][o] = gA;
    a.aux[X_GB][o] = gB;
    a.aux[X_GH][o] = gH;
    a.aux[X_GC][o] = gC;
    a.aux[X_KTH][o] = kH;
    a.aux[X_LAM][o] = lam;
    a.aux[X_ALAM][o] = (kA - kH) * ir2;
    a.aux[X_GLAM][o] = C * C - B * lam;
}

__global__ void __launch_bounds__(256) aux_point_kernel(const __grid_constant__ AuxArgs a) {
    chain_enter();
    aux_point_body(a, blockIdx.x, blockIdx.y);
}

// DelDef_r/z from first derivatives of the inverse metric (:1085-1094); at
// t = 0 they overwrite Delta_r/z (:1088-1094).  Rows from jlo (the ghost rows
// of a grid that does not own the equator take the one-sided z stencils of
// derivatives.f90:179-212); on a grid off the axis the ghost columns as well,
// where the reference's diff1r leaves the r derivatives unset: they are zero
// here, as in an execution that starts them from zero.
__device__ __forceinline__ void aux_deriv_body(const AuxArgs& a, unsigned bx, unsigned by) {
    const LevelGeom& G = a.G;
    const int i = (G.axis ? 1 : 1 - G.g) + (int)(bx * blockDim.x + threadIdx.x);
    const int j = G.jlo + (int)(by * blockDim.y + threadIdx.y);
    if (i > G.nr || j > G.nz) return;
    const long ld = G.ld;
    const size_t o = (size_t)i + (size_t)j * (size_t)ld;
    const int ord = G.order;
    const int kr = pclass_o(ord, i, G.nr, G.g), kz = pclass_o(ord, j, G.nz, G.g);
    const double cr1 = c1_o(ord, G.idr), cz1 = c1_o(ord, G.idz);
    const double r = G.rcol[i];
    // a ghost column of a grid off the axis that diff1r leaves unset (all of
    // them in order four, the outermost in order two)
    const bool rg = i < d1r_first(ord, G.g);
    const double Dr_gA = rg ? 0.0 : d1_o(ord, a.aux[X_GA] + o, 1, kr, cr1);
    const double Dz_gB = d1_o(ord, a.aux[X_GB] + o, ld, kz, cz1);
    const double Dr_gC = rg ? 0.0 : d1_o(ord, a.aux[X_GC] + o, 1, kr, cr1);
    const double Dz_gC = d1_o(ord, a.aux[X_GC] + o, ld, kz, cz1);
    const double glam = a.aux[X_GLAM][o], gC = a.aux[X_GC][o];
    const double ddr = -Dr_gA - r * Dz_gC - r * glam;
    const double ddz = -Dr_gC * r - Dz_gB - 2.0 * gC;
    a.aux[X_DELDEFR][o] = ddr;
    a.aux[X_DELDEFZ][o] = ddz;
    if (a.scalar) {
        a.aux[X_GDR][o] = Dr_gA + r * Dz_gC;
        a.aux[X_GDZ][o] = Dz_gB + r * Dr_gC;
    }
    if (a.t0) {
        a.st[F_DLR][o] = ddr;
        a.st[F_DLZ][o] = ddz;
        if (a.d0r) {
            a.d0r[o] = ddr;
            a.d0z[o] = ddz;
        }
    }
}

__global__ void __launch_bounds__(256) aux_deriv_kernel(const __grid_constant__ AuxArgs a) {
    chain_enter();
    aux_deriv_body(a, blockIdx.x, blockIdx.y);
}

// KT2 and (scalar field) rho + trS on the ghost columns i = 1-g..0 of a grid
// that does not own the axis.  The reference forms both with whole-array
// statements, so they exist at every point (auxiliary_geometry.f90:1022-1031
// for KT2, the non-angmom branch; stressenergy.f90:65-205 for rho and trS);
// the fused constraint pass starts at i = 1 because its derivative stencils
// would leave the grid, and maximal slicing's SOR sweeps the ghost columns of
// such a grid (sor_elliptic.f90:648, i = 2..imax-1) with S1 = -K2 there.
// Expression order: the reference's.
__global__ void __launch_bounds__(128) ghost_kt2_kernel(const __grid_constant__ StageArgs A) {
    const LevelGeom& G = A.G;
    const int g = G.g;
    const int i = 1 - g + (int)threadIdx.x;
    const int j = 1 - g + (int)(blockIdx.x * blockDim.y + threadIdx.y);
    if (i > 0 || j > G.nz) return;
    const size_t o = (size_t)i + (size_t)j * (size_t)G.ld;
    const double r = G.rcol[i], r2 = r * r;
    const double gA = A.aux[X_GA][o], gB = A.aux[X_GB][o], gH = A.aux[X_GH][o], gC = A.aux[X_GC][o];
    const double kA = A.in[F_KTA][o], kB = A.in[F_KTB][o], kC = A.in[F_KTC][o], kH = A.aux[X_KTH][o];
    const double KT2_A = (2.0 * kA * gC * kC + kC * kC * gB) * r2 + gA * (kA * kA);
    const double KT2_B = (kC * kC * gA + 2.0 * kC * gC * kB) * r2 + gB * (kB * kB);
    const double KT2_H = (kH * kH) * gH;
    const double KT2_C = (kC * kC) * gC * r2 + kA * gA * kC + kA * gC * kB + kC * gB * kB;
    A.auxw[X_KT2][o] = gA * KT2_A + gB * KT2_B + gH * KT2_H + 2.0 * gC * KT2_C * r2;
    if (!A.P.scalar) return;
    // 1/psi^4 as the right-hand side forms it (from phi at t = 0, else chi^2)
    double ps4;
    if (A.t0) {
        const double psi = exp(A.in[F_PHI][o]);
        const double psi2 = psi * psi;
        ps4 = 1.0 / (psi2 * psi2);
    } else {
        const double chi = A.in[F_CHI][o];
        ps4 = chi * chi;
    }
    const double sphi = A.in[F_SPHI][o], sxr = A.in[F_SXIR][o], sxz = A.in[F_SXIZ][o], spi = A.in[F_SPI][o];
    const double m2 = A.P.scalar_mass * A.P.scalar_mass;
    double V = 0.0;
    if (A.P.potential == 1) V = 0.5 * m2 * (sphi * sphi);
    else if (A.P.potential == 2) V = 0.5 * m2 * (sphi * sphi) + 0.25 * A.P.scalar_lambda * ((sphi * sphi) * (sphi * sphi));
    const double grad2 = (gA * (sxr * sxr) + gB * (sxz * sxz) + 2.0 * r * gC * sxr * sxz) * ps4;
    const double rho = 0.5 * ((spi * spi) + grad2) + V;
    const double auxs = 0.5 * ((spi * spi) - grad2) - V;
    const double psi4 = 1.0 / ps4;
    const double S_A = (sxr * sxr) + A.in[F_A][o] * psi4 * auxs;
    const double S_B = (sxz * sxz) + A.in[F_B][o] * psi4 * auxs;
    const double S_C = sxr * sxz * G.ircol[i] + A.in[F_C][o] * psi4 * auxs;
    const double S_H = A.in[F_H][o] * psi4 * auxs;
    const double trS = (gA * S_A + gB * S_B + gH * S_H + 2.0 * r2 * gC * S_C) * ps4;
    A.auxw[X_RHOS][o] = rho + trS;
}

// boundtype = "flat" on level 0 (generated simpleboundary.f90): the outer
// edge points take the sources of the column Nr-1 (i = Nr, the r edge first),
// of the row Nz-1 (j = Nz) and, without equatorial symmetry, of the row
// 2-ghost (j = 1-ghost); the edge corners thereby the sources of the points
// diagonally inside.  The right-hand side stored those sources (A.flat) and
// left these arrays alone on the edges; here they take the stage's
// accumulate and update (generated accumulate.f90 / update.f90).
__device__ __forceinline__ bool not_finite(double x) {
    return ((__double_as_longlong(x) >> 52) & 0x7ff) == 0x7ff;
}

__device__ __forceinline__ void flat_edges_body(const StageArgs& A, unsigned bx, unsigned) {
    const LevelGeom& G = A.G;
    const int g = G.g, nr = G.nr, nz = G.nz;
    const int nR = nz - G.jlo + 1;                  // r edge: j = jlo..nz
    const int nZ = nr - 1, nL = G.eqsym ? 0 : nr - 1;  // z edges: i = 1..nr-1
    const int t = (int)(bx * blockDim.x + threadIdx.x);
    if (t >= nR + nZ + nL) return;
    int i, j, src;  // the point and the offset of its source in a flat strip
    if (t < nR) {
        i = nr;
        j = G.jlo + t;
        const int js = (j == nz) ? nz - 1 : ((!G.eqsym && j == 1 - g) ? 2 - g : j);
        src = js - G.jlo;
    } else if (t < nR + nZ) {
        i = 1 + (t - nR);
        j = nz;
        src = nR + i - 1;
    } else {
        i = 1 + (t - nR - nZ);
        j = 1 - g;
        src = nR + nr + i - 1;
    }
    const size_t o = (size_t)i + (size_t)j * (size_t)G.ld;
    const PhysParams& P = A.P;
    unsigned bad = 0;
    constexpr int fields[kNBound] = {F_TRK, F_KTA, F_KTB, F_KTC, F_DLR, F_DLZ, F_DTBETAR, F_DTBETAZ, F_FDRIVER, F_SPI};
#pragma unroll
    for (int b = 0; b < kNBound; ++b) {
        const int f = fields[b];
        if (b >= 6 && b <= 8 && !P.shift) continue;
        if (b == 8 && !P.shock) continue;
        if (b == 9 && !P.scalar) continue;
        const double s = A.flat[(size_t)b * (size_t)A.flat_len + (size_t)src];
        double seff = s;
        if (A.rk4) {
            double* ac = A.acc[f] + o;
            if (A.iter < A.niter) *ac = (A.iter == 1) ? A.weight * s : *ac + A.weight * s;
            else seff = *ac + A.weight * s;
        }
        const double v = A.pst[f][o] + A.dtw * seff;
        A.out[f][o] = v;
        bad |= not_finite(v);
    }
    if (bad && A.nanflag) atomicOr(A.nanflag, 1u);
}

__global__ void __launch_bounds__(128) flat_edges_kernel(const __grid_constant__ StageArgs A) {
    chain_enter();
    flat_edges_body(A, blockIdx.x, blockIdx.y);
}

const MultiRegistration reg_aux_point((const void*)aux_point_kernel, multi_launch<AuxArgs, aux_point_body, 256, 1>);
const MultiRegistration reg_aux_deriv((const void*)aux_deriv_kernel, multi_launch<AuxArgs, aux_deriv_body, 256, 1>);
const MultiRegistration reg_flat_edges((const void*)flat_edges_kernel, multi_launch<StageArgs, flat_edges_body, 128, 1>);

}  // namespace

void launch_flat_edges(const StageArgs& a, cudaStream_t s) {
    const int n = (a.G.nz - a.G.jlo + 1) + (a.G.nr - 1) + (a.G.eqsym ? 0 : a.G.nr - 1);
    launch_chained(flat_edges_kernel, dim3((n + 127) / 128), dim3(128), s, a);
}

void launch_ghost_kt2(const StageArgs& a, cudaStream_t s) {
    if (a.G.axis) return;
    dim3 blk(4, 32);  // x: the g ghost columns; y: rows
    ghost_kt2_kernel<<<(a.G.nz + a.G.g + blk.y - 1) / blk.y, blk, 0, s>>>(a);
}

void launch_aux_point(const AuxArgs& a, cudaStream_t s) {
    dim3 blk(64, 4);
    dim3 grd((a.G.nr + a.G.g + blk.x - 1) / blk.x, (a.G.nz + a.G.g + blk.y - 1) / blk.y);
    launch_chained(aux_point_kernel, grd, blk, s, a);
}

void launch_aux_deriv(const AuxArgs& a, cudaStream_t s) {
    dim3 blk(64, 4);
    const int ni = a.G.axis ? a.G.nr : a.G.nr + a.G.g;
    dim3 grd((ni + blk.x - 1) / blk.x, (a.G.nz - a.G.jlo + 1 + blk.y - 1) / blk.y);
    launch_chained(aux_deriv_kernel, grd, blk, s, a);
}

}  // namespace ollin
