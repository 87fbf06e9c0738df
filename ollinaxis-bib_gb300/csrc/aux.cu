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
__global__ void __launch_bounds__(256) aux_point_kernel(const __grid_constant__ AuxArgs a) {
    chain_enter();
    const LevelGeom& G = a.G;
    const int i = 1 - G.g + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = 1 - G.g + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (i > G.nr || j > G.nz) return;
    const size_t o = (size_t)i + (size_t)j * (size_t)G.ld;
    const double r = G.rcol[i];
    double A = a.st[F_A][o], B = a.st[F_B][o], C = a.st[F_C][o], H = a.st[F_H][o];
    if (a.t0) {
        a.st[F_CHI][o] = exp(-2.0 * a.st[F_PHI][o]);
    } else {
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

// DelDef_r/z from first derivatives of the inverse metric (:1085-1094); at
// t = 0 they overwrite Delta_r/z (:1088-1094).  Rows from jlo (the ghost rows
// of a grid that does not own the equator take the one-sided z stencils of
// derivatives.f90:179-212); on a grid off the axis the ghost columns as well,
// where the reference's diff1r leaves the r derivatives unset: they are zero
// here, as in an execution that starts them from zero.
__global__ void __launch_bounds__(256) aux_deriv_kernel(const __grid_constant__ AuxArgs a) {
    chain_enter();
    const LevelGeom& G = a.G;
    const int i = (G.axis ? 1 : 1 - G.g) + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = G.jlo + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (i > G.nr || j > G.nz) return;
    const long ld = G.ld;
    const size_t o = (size_t)i + (size_t)j * (size_t)ld;
    const int kr = pclass(i, G.nr, G.g), kz = pclass(j, G.nz, G.g);
    const double cr1 = G.idr * (1.0 / 12.0), cz1 = G.idz * (1.0 / 12.0);
    const double r = G.rcol[i];
    const bool rg = i < 1;  // a ghost column of a grid off the axis
    const double Dr_gA = rg ? 0.0 : d1(a.aux[X_GA] + o, 1, kr, cr1);
    const double Dz_gB = d1(a.aux[X_GB] + o, ld, kz, cz1);
    const double Dr_gC = rg ? 0.0 : d1(a.aux[X_GC] + o, 1, kr, cr1);
    const double Dz_gC = d1(a.aux[X_GC] + o, ld, kz, cz1);
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
    }
}

}  // namespace

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
