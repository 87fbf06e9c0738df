// The fused right-hand-side + Runge-Kutta stage kernel.
//
// One thread owns one grid point (i,j) of one level and does, in registers,
// everything the reference spreads over ~300 whole-array statements per stage:
//   * all first, second, mixed and lopsided (advective) derivatives of the
//     evolved fields (src/base/derivatives.f90, derivadvect.f90, order four);
//   * the conformal-factor, lapse and curvature algebra of
//     src/geometry/auxiliary_geometry.f90:49-1502 with calc_conformalRicci1-4
//     and calc_DIVKTA (non-angmom, BSSN branches);
//   * the sources of sources_geometry.f90, sources_lapse.f90,
//     sources_shift.f90 (Gamma-driver 2) and matter/scalar.f90 with
//     stressenergy.f90;
//   * Kreiss-Oliger dissipation (dissipation.f90), the radiative outer
//     boundary of radbound.f90/radiative_geometry.f90 on level 0;
//   * the generated ``accumulate`` and ``update`` (var = var_p + dtw*svar).
// Pointwise quantities that other points' stencils need (g_*, KTH, lambda,
// DelDef) come precomputed from the aux kernels, so no point is recomputed
// for a neighbour: on GB300 FP64 arithmetic, not HBM, bounds this kernel, and
// the redundant-halo recomputation a fully fused single pass would need costs
// more FP64 work than re-reading those arrays costs bandwidth.
#include "ollin_kernels.h"

namespace ollin {

namespace {

__device__ __forceinline__ double sq(double x) { return x * x; }

__device__ __forceinline__ bool nonfinite(double x) {
    return ((__double_as_longlong(x) >> 52) & 0x7ff) == 0x7ff;
}

struct Deriv5 { double r, z, rr, zz, rz; };

template <bool SHIFT, bool SCALAR>
__global__ void __launch_bounds__(128) rhs_kernel(const __grid_constant__ StageArgs A) {
    const LevelGeom& G = A.G;
    const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int j = G.jlo + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (i > G.nr || j > G.nz) return;
    const int g = G.g, nr = G.nr, nz = G.nz;
    const long ld = G.ld;
    const size_t o = (size_t)i + (size_t)j * (size_t)ld;
    const PhysParams& P = A.P;

    const double cr1 = G.idr * (1.0 / 12.0), cz1 = G.idz * (1.0 / 12.0);
    const double cr2 = G.idr * G.idr * (1.0 / 12.0), cz2 = G.idz * G.idz * (1.0 / 12.0);
    const double idrz = G.idr * G.idz;
    const int kr = pclass(i, nr, g), kz = pclass(j, nz, g);

    auto val = [&](int f) { return ld_(A.in[f] + o); };
    auto D5 = [&](int f) {
        const double* p = A.in[f] + o;
        Deriv5 d;
        d.r = d1(p, 1, kr, cr1);
        d.z = d1(p, ld, kz, cz1);
        d.rr = d2(p, 1, kr, cr2);
        d.zz = d2(p, ld, kz, cz2);
        d.rz = d2rz(p, ld, i, j, nr, nz, g, idrz);
        return d;
    };
    auto Dr = [&](int f) { return d1(A.in[f] + o, 1, kr, cr1); };
    auto Dz = [&](int f) { return d1(A.in[f] + o, ld, kz, cz1); };
    auto aux = [&](int x) { return ld_(A.aux[x] + o); };

    const double r = G.rcol[i], ir = G.ircol[i];
    const double zero = 0.0, half = 0.5, one = 1.0, two = 2.0, four = 4.0, six = 6.0;
    const double third = 1.0 / 3.0, sixth = 1.0 / 6.0, fourth = 0.25;
    const double smallpi = 3.141592653589793;
    const double *ft = P.ft;

    // ---- state and aux at the point
    const double alpha = val(F_ALPHA), chi = val(F_CHI);
    const double Ac = val(F_A), Bc = val(F_B), Hc = val(F_H), Cc = val(F_C);
    const double trK = val(F_TRK), kA = val(F_KTA), kB = val(F_KTB), kC = val(F_KTC);
    const double Dlr = val(F_DLR), Dlz = val(F_DLZ);
    const double gA = aux(X_GA), gB = aux(X_GB), gH = aux(X_GH), gC = aux(X_GC);
    const double kH = aux(X_KTH), lam = aux(X_LAM), Alam = aux(X_ALAM), glam = aux(X_GLAM);
    const double DDr = aux(X_DELDEFR), DDz = aux(X_DELDEFZ);

    // ---- derivatives
    const Deriv5 da = D5(F_ALPHA);
    const Deriv5 dA = D5(F_A), dB = D5(F_B), dH = D5(F_H), dC = D5(F_C);
    const double Dr_trK = Dr(F_TRK), Dz_trK = Dz(F_TRK);
    const double Dr_KTA = Dr(F_KTA), Dz_KTA = Dz(F_KTA);
    const double Dr_KTB = Dr(F_KTB), Dz_KTB = Dz(F_KTB);
    const double Dr_KTC = Dr(F_KTC), Dz_KTC = Dz(F_KTC);
    const double Dr_Dlr = Dr(F_DLR), Dz_Dlr = Dz(F_DLR);
    const double Dr_Dlz = Dr(F_DLZ), Dz_Dlz = Dz(F_DLZ);

    // conformal factor (auxiliary_geometry.f90:171-250).  The sources of a
    // stage use the derivative arrays of the previous ``auxiliary`` call, so
    // the branch follows the time of that call (A.t0), not the current one.
    double Dr_phi, Dz_phi, Drr_phi, Dzz_phi, Drz_phi, ipsi4, phi_c = 0.0;
    if (A.t0) {
        const Deriv5 dp = D5(F_PHI);
        Dr_phi = dp.r; Dz_phi = dp.z; Drr_phi = dp.rr; Dzz_phi = dp.zz; Drz_phi = dp.rz;
        phi_c = val(F_PHI);
        const double psi = exp(phi_c);
        const double psi2 = psi * psi;
        ipsi4 = one / (psi2 * psi2);
    } else {
        const Deriv5 dc = D5(F_CHI);
        const double ichi = one / chi;
        const double xr = dc.r * ichi, xz = dc.z * ichi;
        Dr_phi = -half * xr;
        Dz_phi = -half * xz;
        Drr_phi = -half * (dc.rr * ichi - xr * xr);
        Dzz_phi = -half * (dc.zz * ichi - xz * xz);
        Drz_phi = -half * (dc.rz * ichi - xr * xz);
        ipsi4 = chi * chi;  // 1/psi^4 with psi = chi^(-1/2)
    }

    const double r2 = r * r, r3 = r2 * r, r4 = r2 * r2, r5 = r4 * r, ir2 = ir * ir;
    const double gA2 = gA * gA, gB2 = gB * gB, gH2 = gH * gH, gC2 = gC * gC;
    const double gA3 = gA2 * gA, gB3 = gB2 * gB, gC3 = gC2 * gC;
    const double lamDef = (Ac - Hc) * ir2;

    // ---- lapse: covariant second derivatives and Laplacian (:1266-1324)
    double D2A = da.rr - da.r * gC * r2 * dC.r
        - (da.z * gB * dC.r + half * da.z * gC * dA.r + da.r * gC * Cc - half * da.r * gC * dA.z) * r
        - half * da.r * gA * dA.r - da.z * gB * Cc + half * da.z * gB * dA.z;
    double D2B = da.zz - da.z * gC * r2 * dC.z
        - (da.r * gA * dC.z + half * da.r * gC * dB.z - half * da.z * gC * dB.r) * r
        + half * da.r * gA * dB.r - half * da.z * gB * dB.z;
    double D2H = -(-half * da.r * gC * dH.z - half * da.z * gC * dH.r) * r
        + half * da.r * gA * dH.r + da.z * gC * Hc + half * da.z * gB * dH.z + da.r * gA * Hc * ir;
    double D2C = da.rz * ir - half * da.r * gC * dB.r - half * da.z * gC * dA.z
        - (half * da.r * gA * dA.z + half * da.z * gB * dB.r) * ir;
    {
        const double aux1 = gA * da.r * Dr_phi + gB * da.z * Dz_phi + r * gC * (da.r * Dz_phi + da.z * Dr_phi);
        D2A = D2A - two * (two * da.r * Dr_phi - Ac * aux1);
        D2B = D2B - two * (two * da.z * Dz_phi - Bc * aux1);
        D2H = D2H + two * Hc * aux1;
        D2C = D2C - two * ((da.r * ir) * Dz_phi + da.z * (Dr_phi * ir) - Cc * aux1);
    }
    const double Lapla_alpha = (gA * D2A + gB * D2B + gH * D2H + two * r2 * gC * D2C) * ipsi4;

    // ---- Ricci tensor: conformal-factor part (:1331-1469)
    double RA = -two * (Drr_phi - Dr_phi * gC * r2 * dC.r
        - (Dz_phi * gB * dC.r + half * Dz_phi * gC * dA.r + Dr_phi * gC * Cc - half * Dr_phi * gC * dA.z) * r
        - half * Dr_phi * gA * dA.r - Dz_phi * gB * Cc + half * Dz_phi * gB * dA.z);
    double RB = -two * (Dzz_phi - Dz_phi * gC * r2 * dC.z
        - (Dr_phi * gA * dC.z + half * Dr_phi * gC * dB.z - half * Dz_phi * gC * dB.r) * r
        + half * Dr_phi * gA * dB.r - half * Dz_phi * gB * dB.z);
    double RH = -two * (-(-half * Dr_phi * gC * dH.z - half * Dz_phi * gC * dH.r) * r
        + half * Dr_phi * gA * dH.r + Dz_phi * gC * Hc + half * Dz_phi * gB * dH.z + Dr_phi * gA * Hc * ir);
    double RC = -two * (Drz_phi * ir - half * Dr_phi * gC * dB.r - half * Dz_phi * gC * dA.z
        - (half * Dr_phi * gA * dA.z + half * Dz_phi * gB * dB.r) * ir);
    {
        const double tr = gA * RA + gB * RB + gH * RH + two * r2 * gC * RC;
        RA = RA + Ac * tr;
        RB = RB + Bc * tr;
        RH = RH + Hc * tr;
        RC = RC + Cc * tr;
        RA = RA + four * (Dr_phi * Dr_phi);
        RB = RB + four * (Dz_phi * Dz_phi);
        RC = RC + four * (Dr_phi * Dz_phi) * ir;
        const double q = -two * (gA * Dr_phi * Dr_phi + gB * Dz_phi * Dz_phi + two * r * gC * Dr_phi * Dz_phi);
        RA = RA + two * Ac * q;
        RB = RB + two * Bc * q;
        RH = RH + two * Hc * q;
        RC = RC + two * Cc * q;
    }
    // calc_conformalRicci1.f90:76-86
    RA = RA - gC * dA.rz * r - half * gB * dA.zz - half * gA * dA.rr - half * gH * dA.r * ir + gH * lamDef;
    RB = RB - gC * dB.rz * r - half * gA * dB.rr - half * gB * dB.zz - half * gH * dB.r * ir;
    RH = RH - gC * dH.rz * r - half * gB * dH.zz - half * gA * dH.rr - half * gH * dH.r * ir - gH * lamDef;
    RC = RC - gC * dC.rz * r - half * gA * dC.rr - gC * dC.z - half * gB * dC.zz + (-gA * dC.r - half * gH * dC.r) * ir;
    // calc_conformalRicci2.f90:73-83
    RA = RA + Cc * Dr_Dlz * r + Ac * Dr_Dlr + half * (DDr * dA.r + DDz * dA.z);
    RB = RB + Cc * Dz_Dlr * r + Bc * Dz_Dlz + half * (DDr * dB.r + DDz * dB.z);
    RH = RH + half * (DDr * dH.r + DDz * dH.z) + Dlr * Hc * ir;
    RC = RC + half * Cc * (Dr_Dlr + Dz_Dlz) + half * (DDr * dC.r + DDz * dC.z) + half * (Cc * Dlr + Ac * Dz_Dlr + Bc * Dr_Dlz) * ir;
    {
        const double dAr = dA.r, dAz = dA.z, dBr = dB.r, dBz = dB.z, dHr = dH.r, dHz = dH.z, dCr = dC.r, dCz = dC.z;
        // calc_conformalRicci3.f90:316-340
        RA = RA + (2.0 * gB * gC * dCr * dCz + gC2 * dAr * dCz + dAz * gC2 * dCr) * r3
            + (2.0 * gB * gC * Cc * dCz - gB * gC * dCr * dBr + dAr * gC * gA * dCr + dAz * gC2 * Cc) * r2
            + (dAz * gB * gC * dBr + dAz * gB * gA * dCr + dAr * gC * gA * Cc - gB * gC * Cc * dBr + dAz * gC * gA * dAr
               + gB2 * dBr * dCz) * r
            - half * gH2 * sq(dHr) - half * gB2 * sq(dBr) + gB * gA * Cc * dAz + half * sq(dAr) * gA2
            + (gH * dHr + gH2 * Ac * dHr - 2.0 * gH2 * dHr * Hc) * ir;
        RB = RB + (dBr * gC2 * dCz + gC2 * dBz * dCr + 2.0 * gA * gC * dCz * dCr) * r3
            + (2.0 * gA * gC * dCz * Cc - gA * gC * dCz * dAz + gC2 * dBz * Cc + dBz * gC * gB * dCz) * r2
            + (dBr * gA * gC * dAz + gA2 * dAz * dCr + dBr * gA * gB * dCz + dBr * gB * gC * dBz) * r
            + half * gB2 * sq(dBz) + gA2 * dAz * Cc - half * gA2 * sq(dAz) + gH2 * dHz * Cc - half * gH2 * sq(dHz);
        RH = RH - gC * dHz - r * glam * dHr;
        RC = RC + (gC2 * dBr * dCr + gC * gB * sq(dCz) + dAz * gC2 * dCz + gC * gA * sq(dCr)) * r2
            + (-half * gC * gA * dCr * dAz + 2.0 * gC * gA * dCr * Cc - half * gC2 * dBr * dAz - half * gC * gB * dCz * dBr
               + half * dBz * gB * gC * dCr + gC2 * dBr * Cc + half * dBz * gC2 * dAr + half * dAr * gA * gC * dCz) * r
            + half * dBr * gC * gA * dAr + half * dBr * gB * gA * dCr + half * gB2 * dBz * dCz + half * dAz * gA * gB * dCz
            + half * gA2 * dAr * dCr + half * sq(dBr) * gB * gC + gC * gA * sq(Cc) - half * gC * gA * Cc * dAz
            + half * dAz * gB * gC * dBz + half * sq(dAz) * gA * gC + half * dBz * gB * gC * Cc
            + (half * gH2 * Cc * dHr + half * gB * gA * dBr * Cc - half * gH2 * dHz * dHr + half * gA2 * dAr * Cc) * ir
            + half * dHz * gH2 * lam;
        // calc_conformalRicci4.f90:272-298
        RA = RA + dAz * gC2 * dCr * r3
            + (-half * sq(dAz) * gC2 + dAz * gC2 * Cc + gB * gA * sq(dCr) + half * dAr * gC2 * dBr + dAr * gC * gA * dCr
               + gB * gC * dCr * dBr) * r2
            + (-dAz * gB * gA * dCr + 2.0 * gB * gA * dCr * Cc + gB * gC * Cc * dBr + dAr * gC * gA * Cc) * r
            + fourth * gH2 * sq(dHr) - gB * gA * Cc * dAz + fourth * gB2 * sq(dBr) + gB * gA * sq(Cc)
            + fourth * sq(dAr) * gA2 + half * gB * gA * sq(dAz);
        RB = RB + dBr * gC2 * r3 * dCz
            + (gA * gB * sq(dCz) + half * dAz * gC2 * dBz - half * gC2 * sq(dBr) + dBz * gC * gB * dCz + gA * gC * dCz * dAz) * r2
            - dBr * gA * gB * dCz * r + fourth * gA2 * sq(dAz) + half * gB * gA * sq(dBr) + fourth * gH2 * sq(dHz)
            + fourth * gB2 * sq(dBz);
        RH = RH + (-half * Cc * gC * gH * dHr + gH * gC * dHz * dHr) * r + half * gH * sq(dHz) * gB
            + 3.0 * half * gC * dHz + half * gH * gA * sq(dHr) - half * Cc * gB * gH * dHz - half * gH * Ac * gC * dHz - Cc * gC
            - half * gC * dHz + half * (2.0 * gA - gH - gH * Ac * gA) * dHr * ir + gH * lam * (1.0 - gA * Hc);
        RC = RC + gC2 * dCr * dCz * r3
            + (-half * dAz * gC2 * dCz + gC2 * Cc * dCz - half * gC2 * dBr * dCr) * r2
            + (-half * gC2 * dBr * Cc + fourth * dBz * gC2 * dAr + half * dAr * gA * gC * dCz + half * gC * gB * dCz * dBr
               + 3.0 * fourth * gC2 * dBr * dAz + half * dBz * gB * gC * dCr + half * gC * gA * dCr * dAz) * r
            + half * dAz * gA * gB * dCz + half * dBz * gB * gC * Cc + half * gC * gA * Cc * dAz + half * dBr * gB * gA * dCr
            + (fourth * gH2 * dHz * dHr + half * gB * gA * dBr * Cc + fourth * gA2 * dAr * dAz + fourth * dBz * gB2 * dBr
               - half * gB * gA * dAz * dBr) * ir;
    }
    const double RSCAL = (gA * RA + gB * RB + gH * RH + two * r2 * gC * RC) * ipsi4;

    // ---- contravariant and squared traceless curvature (:944-1031)
    const double KT_up_rr = (2.0 * gA * gC * kC + gC2 * kB) * r2 + gA2 * kA;
    const double KT_up_zz = (gC2 * kA + 2.0 * gC * gB * kC) * r2 + gB2 * kB;
    const double KT_up_rz = gC2 * r3 * kC + (gC * gA * kA + gB * gA * kC + gB * gC * kB) * r;
    const double KT2_A = (2.0 * kA * gC * kC + sq(kC) * gB) * r2 + gA * sq(kA);
    const double KT2_B = (sq(kC) * gA + 2.0 * kC * gC * kB) * r2 + gB * sq(kB);
    const double KT2_H = sq(kH) * gH;
    const double KT2_C = sq(kC) * gC * r2 + kA * gA * kC + kA * gC * kB + kC * gB * kB;
    const double KT2 = gA * KT2_A + gB * KT2_B + gH * KT2_H + two * gC * KT2_C * r2;
    const double K2 = KT2 + third * sq(trK);

    // ---- divergence of the traceless curvature (calc_DIVKTA.f90:573-636)
    double DIV_KT_r, DIV_KT_z, DIVA_KT_r, DIVA_KT_z;
    {
        const double dAr = dA.r, dAz = dA.z, dBr = dB.r, dBz = dB.z, dHr = dH.r, dHz = dH.z, dCr = dC.r, dCz = dC.z;
        const double dkAr = Dr_KTA, dkAz = Dz_KTA, dkBr = Dr_KTB, dkBz = Dz_KTB, dkCr = Dr_KTC, dkCz = Dz_KTC;
        DIV_KT_r = -gC3 * dCz * kC * r5 - gA * gC2 * kC * dCr * r4
            + (gC2 * dkCz - half * gC3 * dBz * kA - gA * gC2 * kC * Cc - half * gC3 * dAz * kB - gA * dCz * gC2 * kA
               - gA * dCz * gC * gB * kC - gC2 * dCz * gB * kB - gC2 * dBz * gB * kC - gA * dAz * gC2 * kC) * r3
            + (2.0 * gA * gC * dkCr - Dlr * gC * kC - gC * dBr * gB * gA * kC - gB * gA2 * kC * dCr - dAr * gA2 * gC * kC
               - gC * gA2 * kA * dCr + gC2 * dkBr - gA * gB * gC * kB * dCr - half * gA * dAr * gC2 * kB
               - half * gC2 * dBr * gA * kA) * r2
            + (2.0 * gA * gC * kC + gA * gC * dkAz - gC * gA2 * kA * Cc + gC * gH * kC - half * gH2 * kH * gC * dHz
               - Dlz * gC * kB - gB * gA2 * kC * Cc - half * gA2 * dAz * gC * kA + gC * gB * dkBz + gA * gB * dkCz
               - Dlz * gA * kC - gA * gB * gC * kB * Cc - gC * gH2 * kH * Cc - half * gC * dBz * gB2 * kB) * r
            - half * gA * dBr * gB2 * kB - half * gH2 * kH * gA * dHr - Dlr * gA * kA + gA2 * dkAr
            - half * gA3 * dAr * kA + r * gH * (gA * Alam + gH * kH * Cc * gC);
        DIV_KT_z = -r5 * gC3 * kC * dCr + (-gC3 * kC * Cc - dCz * gC2 * gB * kC) * r4
            + (gC2 * dkCr - gB * gC2 * kB * dCr - gC * gB * gA * kC * dCr - half * gC3 * dBr * kA - gC2 * gA * kA * dCr
               - half * dAr * gC3 * kB - dAr * gA * gC2 * kC - gB * dBr * gC2 * kC) * r3
            + (-gB * dCz * gC * gA * kA + gC2 * kC - dBz * gC * gB2 * kC - Dlz * gC * kC - gC * dCz * gB2 * kB
               + gC2 * dkAz + 2.0 * gC * gB * dkCz - gC2 * gA * kA * Cc - dCz * gB2 * gA * kC - half * dAz * gB * gC2 * kB
               - gC * dAz * gB * gA * kC - gB * gC2 * kB * Cc - half * gB * dBz * gC2 * kA - gC * gB * gA * kC * Cc) * r2
            + (gB * gC * dkBr + gB * gA * dkCr + gC * gA * dkAr - half * gH2 * kH * gC * dHr - Dlr * gB * kC - Dlr * gC * kA
               - half * gB2 * dBr * gC * kB - half * gC * dAr * gA2 * kA) * r
            + gC * gH * kA + gB * gA * kC - half * dBz * gB3 * kB + gB2 * dkBz - Dlz * gB * kB - gC * gH2 * kH * Ac
            - half * gB * dAz * gA2 * kA - half * gH2 * kH * gB * dHz - gC * gH * kH + gB * gH * kC - gB * gH2 * kH * Cc;
        DIVA_KT_r = -r5 * gC3 * dCz * kC + (-gC3 * dCr * kB - gC3 * dBr * kC - 3.0 * gC2 * dCr * gA * kC) * r4
            + (-gC3 * Cc * kB - 2.0 * gA * dCz * gC2 * kA - 3.0 * gC2 * Cc * gA * kC + gC2 * dkCz - gC2 * dAz * gA * kC
               - 3.0 * gA * dCz * gC * gB * kC - 2.0 * gC2 * dBz * gB * kC - gC3 * dBz * kA - gC2 * dCz * gB * kB) * r3
            + (-gA * dBr * gC2 * kA - gA * gB * gC * kB * dCr + 2.0 * gA * gC * dkCr - 2.0 * gC * dCr * gA2 * kA - Dlr * gC * kC
               + gC2 * dkBr - gC2 * dBr * gB * kB - 2.0 * gA2 * dAr * gC * kC - gA * dAr * gC2 * kB
               - gB * gA2 * kC * dCr - gA * dBr * gC * gB * kC) * r2
            + (-gA * dCz * gB2 * kB - gB * gA2 * kC * Cc - gC * dBz * gB2 * kB + 2.0 * gA * gC * kC + gC * gB * dkBz
               + gC * gH * kC + gA * gC * dkAz + gA * gB * dkCz - gA * dAz * gB * gC * kB - gC * gH2 * kH * Cc - Dlz * gC * kB
               - gA2 * dAz * gB * kC - 2.0 * gC * Cc * gA2 * kA - Dlz * gA * kC - gA2 * dAz * gC * kA - gA * gB * gC * kB * Cc) * r
            - dAr * gA3 * kA - Dlr * gA * kA + gA2 * dkAr + r * gA * gH * (Alam - lam * gH * kH);
        DIVA_KT_z = -r5 * gC3 * kC * dCr
            + (-3.0 * dCz * gC2 * gB * kC - dAz * gC3 * kC - dCz * gC3 * kA - gC3 * kC * Cc) * r4
            + (-3.0 * gC * gB * gA * kC * dCr - 2.0 * dAr * gA * gC2 * kC + gC2 * dkCr - gB * dBr * gC2 * kC
               - dAr * gC3 * kB - 2.0 * gB * gC2 * kB * dCr - gC2 * gA * kA * dCr) * r3
            + (-gC * dAz * gB * gA * kC - gC2 * gA * kA * Cc - 2.0 * dBz * gC * gB2 * kC - dAz * gC2 * gA * kA
               - dAz * gB * gC2 * kB - 3.0 * gC * gB * gA * kC * Cc - 2.0 * gC * dCz * gB2 * kB - Dlz * gC * kC
               - dCz * gB2 * gA * kC + gC2 * kC + gC2 * dkAz + 2.0 * gC * gB * dkCz - gB * dCz * gC * gA * kA
               - gB * dBz * gC2 * kA - 2.0 * gB * gC2 * kB * Cc) * r2
            + (-Dlr * gB * kC + gB * gA * dkCr + gC * gA * dkAr + gB * gC * dkBr - gB2 * dBr * gC * kB - Dlr * gC * kA
               - gB2 * dBr * gA * kC - gC * dAr * gA2 * kA - gB * dBr * gC * gA * kA - gB * gA2 * kA * dCr) * r
            - Dlz * gB * kB - gB * gH2 * kH * Cc + gB2 * dkBz - gC * gH2 * kH * Ac - gB * gA2 * kA * Cc + gB * gH * kC
            + gC * gH * kA + gB * gA * kC - dBz * gB3 * kB;
    }

    // ---- matter: scalar field stress-energy (stressenergy.f90:65-205) and
    //      its source (scalar.f90)
    double rho = 0, J_r = 0, J_z = 0, S_A = 0, S_B = 0, S_C = 0, trS = 0;
    double s_sphi = 0, s_sxr = 0, s_sxz = 0, s_spi = 0;
    double Dr_spi = 0, Dz_spi = 0;
    if constexpr (SCALAR) {
        const double sphi_ = val(F_SPHI), sxr = val(F_SXIR), sxz = val(F_SXIZ), spi = val(F_SPI);
        const double ps4 = ipsi4;  // 1/psi4
        double V = 0, VP = 0;
        if (P.potential == 1) { V = 0.5 * sq(P.scalar_mass) * sq(sphi_); VP = sq(P.scalar_mass) * sphi_; }
        else if (P.potential == 2) {
            V = 0.5 * sq(P.scalar_mass) * sq(sphi_) + 0.25 * P.scalar_lambda * sq(sq(sphi_));
            VP = sq(P.scalar_mass) * sphi_ + P.scalar_lambda * sq(sphi_) * sphi_;
        }
        const double grad2 = (gA * sq(sxr) + gB * sq(sxz) + two * r * gC * sxr * sxz) * ps4;
        rho = half * (sq(spi) + grad2) + V;
        J_r = -(gA * sxr + r * gC * sxz) * spi * ps4;
        J_z = -(gB * sxz + r * gC * sxr) * spi * ps4;
        const double auxs = half * (sq(spi) - grad2) - V;
        const double psi4 = one / ps4;
        S_A = sq(sxr) + Ac * psi4 * auxs;
        S_B = sq(sxz) + Bc * psi4 * auxs;
        S_C = sxr * sxz * ir + Cc * psi4 * auxs;
        const double S_H = Hc * psi4 * auxs;
        trS = (gA * S_A + gB * S_B + gH * S_H + two * r2 * gC * S_C) * ps4;
        // Klein-Gordon in first-order form, second-order pi source
        const Deriv5 dsp = D5(F_SPHI);
        Dr_spi = Dr(F_SPI); Dz_spi = Dz(F_SPI);
        s_sphi = alpha * spi;
        s_sxr = alpha * Dr_spi + spi * da.r;
        s_sxz = alpha * Dz_spi + spi * da.z;
        const double GDR = aux(X_GDR), GDZ = aux(X_GDZ);
        double sp = alpha * (gA * dsp.rr + gB * dsp.zz + two * r * gC * dsp.rz);
        sp = sp + two * alpha * (Dr_phi * (gA * dsp.r + r * gC * dsp.z) + Dz_phi * (gB * dsp.z + r * gC * dsp.r));
        sp = sp + da.r * (gA * dsp.r + r * gC * dsp.z) + da.z * (gB * dsp.z + r * gC * dsp.r);
        sp = sp + alpha * (dsp.r * GDR + dsp.z * (GDZ + gC));
        sp = sp + alpha * (gA * dsp.r * ir + gC * dsp.z);
        sp = sp * ps4;
        sp = sp + alpha * spi * trK;
        if (P.potential != 0) sp = sp - alpha * VP;
        s_spi = sp;
    }

    // ---- geometric sources (sources_geometry.f90, BSSN)
    const double sigma = 1.0;  // lagrangian flavour
    double s_phi = -sixth * alpha * trK;
    double s_chi = 2.0 * sixth * alpha * chi * trK;
    double s_A = -two * alpha * kA, s_B = -two * alpha * kB, s_H = -two * alpha * kH, s_C = -two * alpha * kC;
    double s_trK = -Lapla_alpha + alpha * K2;
    double s_KTA = alpha * (trK * kA - two * KT2_A);
    double s_KTB = alpha * (trK * kB - two * KT2_B);
    double s_KTC = alpha * (trK * kC - two * KT2_C);
    {
        const double tr = -Lapla_alpha + alpha * RSCAL;
        s_KTA = s_KTA + (-D2A + alpha * RA) * ipsi4 - third * Ac * tr;
        s_KTB = s_KTB + (-D2B + alpha * RB) * ipsi4 - third * Bc * tr;
        s_KTC = s_KTC + (-D2C + alpha * RC) * ipsi4 - third * Cc * tr;
    }
    double s_Dlr = -two * (KT_up_rr * da.r + KT_up_rz * da.z) - two * alpha * DIVA_KT_r;
    s_Dlr = s_Dlr + P.eta * alpha * (DIV_KT_r + six * (KT_up_rr * Dr_phi + KT_up_rz * Dz_phi) - two * third * (gA * Dr_trK + r * gC * Dz_trK));
    double s_Dlz = -two * (KT_up_rz * da.r + KT_up_zz * da.z) - two * alpha * DIVA_KT_z;
    s_Dlz = s_Dlz + P.eta * alpha * (DIV_KT_z + six * (KT_up_rz * Dr_phi + KT_up_zz * Dz_phi) - two * third * (r * gC * Dr_trK + gB * Dz_trK));
    double s_alpha = 0.0;
    if (P.slicing == 0) s_alpha = -(alpha * P.gauge_f) * trK;                 // 1+log
    else if (P.slicing == 1) s_alpha = -(sq(alpha) * P.gauge_f) * trK;       // harmonic
    else if (P.slicing == 2) s_alpha = -(sq(alpha) + (P.gauge_f - 1.0)) * trK;  // shock avoiding

    double s_br = 0, s_bz = 0, s_dbr = 0, s_dbz = 0;
    if constexpr (SHIFT) {
        const double br = val(F_BETAR), bz = val(F_BETAZ), dbr = val(F_DTBETAR), dbz = val(F_DTBETAZ);
        const Deriv5 dbR = D5(F_BETAR), dbZ = D5(F_BETAZ);
        const bool adv = P.shiftadvect != 0;
        const bool negr = br <= 0.0, negz = bz <= 0.0;
        auto DAr = [&](int f, const double dr_) { return adv ? dadv(A.in[f] + o, 1, i, nr, g, negr, G.idr, false) : dr_; };
        auto DAz = [&](int f, const double dz_) { return adv ? dadv(A.in[f] + o, ld, j, nz, g, negz, G.idz, true) : dz_; };
        // DD_beta_rr = d/dr (beta_r / r): first derivative of beta_r/r
        double DD_beta_rr;
        {
            const double* pb = A.in[F_BETAR] + o;
            const double* ic = G.ircol + i;
            auto q = [&](int m) { return ld_(pb + m) * ic[m]; };
            if (kr == 0) DD_beta_rr = cr1 * (8.0 * (q(1) - q(-1)) - (q(2) - q(-2)));
            else if (kr == 1) DD_beta_rr = cr1 * (3.0 * q(1) + 10.0 * q(0) - 18.0 * q(-1) + 6.0 * q(-2) - q(-3));
            else DD_beta_rr = cr1 * (25.0 * q(0) - 48.0 * q(-1) + 36.0 * q(-2) - 16.0 * q(-3) + 3.0 * q(-4));
        }
        const double DIV_beta = dbR.r + dbZ.z + br * ir;
        const double Dr_DIV_beta = dbR.rr + dbZ.rz + DD_beta_rr;
        const double Dz_DIV_beta = dbR.rz + dbZ.zz + dbR.z * ir;
        const double DAr_al = DAr(F_ALPHA, da.r), DAz_al = DAz(F_ALPHA, da.z);
        const double DAr_A = DAr(F_A, dA.r), DAz_A = DAz(F_A, dA.z);
        const double DAr_B = DAr(F_B, dB.r), DAz_B = DAz(F_B, dB.z);
        const double DAr_H = DAr(F_H, dH.r), DAz_H = DAz(F_H, dH.z);
        const double DAr_C = DAr(F_C, dC.r), DAz_C = DAz(F_C, dC.z);
        const double DAr_tK = DAr(F_TRK, Dr_trK), DAz_tK = DAz(F_TRK, Dz_trK);
        const double DAr_kA = DAr(F_KTA, Dr_KTA), DAz_kA = DAz(F_KTA, Dz_KTA);
        const double DAr_kB = DAr(F_KTB, Dr_KTB), DAz_kB = DAz(F_KTB, Dz_KTB);
        const double DAr_kC = DAr(F_KTC, Dr_KTC), DAz_kC = DAz(F_KTC, Dz_KTC);
        const double DAr_Dr = DAr(F_DLR, Dr_Dlr), DAz_Dr = DAz(F_DLR, Dz_Dlr);
        const double DAr_Dz = DAr(F_DLZ, Dr_Dlz), DAz_Dz = DAz(F_DLZ, Dz_Dlz);
        if (A.t0) {
            const double DAr_ph = DAr(F_PHI, Dr_phi), DAz_ph = DAz(F_PHI, Dz_phi);
            s_phi = s_phi + br * DAr_ph + bz * DAz_ph + sixth * sigma * DIV_beta;
            // chi's lopsided derivatives are not formed while the level time is
            // zero (the t=0 branch of auxiliary_geometry.f90:178-202 only
            // differentiates phi), so the advection term of chi reads zeros
            s_chi = s_chi - sigma * 2.0 * sixth * chi * DIV_beta;
        } else {
            const double dchr = d1(A.in[F_CHI] + o, 1, kr, cr1), dchz = d1(A.in[F_CHI] + o, ld, kz, cz1);
            const double DAr_ch = DAr(F_CHI, dchr), DAz_ch = DAz(F_CHI, dchz);
            s_chi = s_chi + br * DAr_ch + bz * DAz_ch - sigma * 2.0 * sixth * chi * DIV_beta;
        }
        const double Drb = dbR.r, Dzb = dbR.z, Drbz = dbZ.r, Dzbz = dbZ.z;
        s_A = s_A + br * DAr_A + bz * DAz_A + two * (Ac * Drb + r * Cc * Drbz) - two * third * sigma * Ac * DIV_beta;
        s_B = s_B + br * DAr_B + bz * DAz_B + two * (Bc * Dzbz + r * Cc * Dzb) - two * third * sigma * Bc * DIV_beta;
        s_H = s_H + br * DAr_H + bz * DAz_H + two * Hc * br * ir - two * third * sigma * Hc * DIV_beta;
        s_C = s_C + br * DAr_C + bz * DAz_C + Cc * br * ir + Cc * (Drb + Dzbz) + (Bc * Drbz + Ac * Dzb) * ir
            - two * third * sigma * Cc * DIV_beta;
        s_trK = s_trK + br * DAr_tK + bz * DAz_tK;
        s_KTA = s_KTA + br * DAr_kA + bz * DAz_kA + two * (kA * Drb + r * kC * Drbz) - two * third * sigma * kA * DIV_beta;
        s_KTB = s_KTB + br * DAr_kB + bz * DAz_kB + two * (kB * Dzbz + r * kC * Dzb) - two * third * sigma * kB * DIV_beta;
        s_KTC = s_KTC + br * DAr_kC + bz * DAz_kC + kC * br * ir + kC * (Drb + Dzbz) + (kB * Drbz + kA * Dzb) * ir
            - two * third * sigma * kC * DIV_beta;
        s_Dlr = s_Dlr + br * DAr_Dr + bz * DAz_Dr - Dlr * Drb - Dlz * Dzb;
        s_Dlr = s_Dlr + two * r * gC * dbR.rz + gA * dbR.rr + gB * dbR.zz + gH * DD_beta_rr;
        s_Dlr = s_Dlr + third * sigma * (gA * Dr_DIV_beta + r * gC * Dz_DIV_beta + two * Dlr * DIV_beta);
        s_Dlz = s_Dlz + br * DAr_Dz + bz * DAz_Dz - Dlr * Drbz - Dlz * Dzbz;
        s_Dlz = s_Dlz + two * r * gC * dbZ.rz + gA * dbZ.rr + gB * dbZ.zz + gH * Drbz * ir;
        s_Dlz = s_Dlz + third * sigma * (r * gC * Dr_DIV_beta + gB * Dz_DIV_beta + two * Dlz * DIV_beta);
        s_alpha = s_alpha + br * DAr_al + bz * DAz_al;
        s_br = dbr;
        s_bz = dbz;
        if (P.driveradv) {
            s_br = s_br + br * DAr(F_BETAR, dbR.r) + bz * DAz(F_BETAR, dbR.z);
            s_bz = s_bz + br * DAr(F_BETAZ, dbZ.r) + bz * DAz(F_BETAZ, dbZ.z);
        }
        (void)s_dbr; (void)s_dbz;
        if constexpr (SCALAR) {
            // auxiliary_matter.f90 always forms lopsided derivatives for the
            // scalar field when a shift is present (independent of shiftadvect)
            auto LAr = [&](int f) { return dadv(A.in[f] + o, 1, i, nr, g, negr, G.idr, false); };
            auto LAz = [&](int f) { return dadv(A.in[f] + o, ld, j, nz, g, negz, G.idz, true); };
            const double sxr = val(F_SXIR), sxz = val(F_SXIZ);
            s_sphi = s_sphi + br * sxr + bz * sxz;
            s_sxr = s_sxr + br * LAr(F_SXIR) + sxr * Drb + bz * LAz(F_SXIR) + sxz * Drbz;
            s_sxz = s_sxz + br * LAr(F_SXIZ) + sxr * Dzb + bz * LAz(F_SXIZ) + sxz * Dzbz;
            s_spi = s_spi + br * LAr(F_SPI) + bz * LAz(F_SPI);
        }
    }
    if constexpr (SCALAR) {
        s_trK = s_trK + four * smallpi * alpha * (rho + trS);
        s_KTA = s_KTA - 8.0 * smallpi * alpha * (S_A * ipsi4 - third * Ac * trS);
        s_KTB = s_KTB - 8.0 * smallpi * alpha * (S_B * ipsi4 - third * Bc * trS);
        s_KTC = s_KTC - 8.0 * smallpi * alpha * (S_C * ipsi4 - third * Cc * trS);
        s_Dlr = s_Dlr - 8.0 * smallpi * P.eta * alpha * J_r / ipsi4;
        s_Dlz = s_Dlz - 8.0 * smallpi * P.eta * alpha * J_z / ipsi4;
    }

    if (A.analysis) {
        // constraints.f90:55-149
        const double spf = 3.1415927410125732;  // acos(-1.0) in single precision
        double ham = RSCAL - KT2 + two * third * sq(trK);
        if constexpr (SCALAR) ham = ham - 16.0 * spf * rho;
        double momr = DIV_KT_r + 6.0 * (KT_up_rr * Dr_phi + KT_up_rz * Dz_phi) - two * third * (gA * Dr_trK + r * gC * Dz_trK);
        double momz = DIV_KT_z + 6.0 * (KT_up_rz * Dr_phi + KT_up_zz * Dz_phi) - two * third * (r * gC * Dr_trK + gB * Dz_trK);
        if constexpr (SCALAR) {
            momr = momr - 8.0 * spf * J_r / ipsi4;
            momz = momz - 8.0 * spf * J_z / ipsi4;
        }
        A.auxw[X_HAM][o] = ham;
        A.auxw[X_MOMR][o] = momr;
        A.auxw[X_MOMZ][o] = momz;
        A.auxw[X_RSCAL][o] = RSCAL;
        A.auxw[X_KT2][o] = KT2;
        A.auxw[X_LAPLA][o] = Lapla_alpha;
        return;
    }

    // ---- Kreiss-Oliger dissipation (dissipation.f90:196-211)
    const bool diss_r = (i >= 4 - g && i <= nr - 3);
    const bool diss_z = (j >= 4 - g && j <= nz - 3);
    if (P.geodiss != 0.0) {
        const double kd = P.geodiss / G.dt * (1.0 / 20.0);
        auto diss = [&](int f, double& s) {
            const double* p = A.in[f] + o;
            if (diss_r) s = s - kd * ko6(p, 1);
            if (diss_z) s = s - kd * ko6(p, ld);
        };
        diss(F_TRK, s_trK);
        diss(F_KTA, s_KTA);
        diss(F_KTB, s_KTB);
        diss(F_KTC, s_KTC);
        diss(F_DLR, s_Dlr);
        diss(F_DLZ, s_Dlz);
    }
    if constexpr (SCALAR) {
        if (P.scalardiss != 0.0) {
            const double kd = P.scalardiss / G.dt * (1.0 / 20.0);
            auto diss = [&](int f, double& s) {
                const double* p = A.in[f] + o;
                if (diss_r) s = s - kd * ko6(p, 1);
                if (diss_z) s = s - kd * ko6(p, ld);
            };
            diss(F_SPHI, s_sphi);
            diss(F_SPI, s_spi);
            diss(F_SXIR, s_sxr);
            diss(F_SXIZ, s_sxz);
        }
    }
    if constexpr (SHIFT) {
        s_dbr = P.drivercsi * s_Dlr;
        s_dbz = P.drivercsi * s_Dlz;
        if (P.driveradv) {
            const double br = val(F_BETAR), bz = val(F_BETAZ);
            const bool negr = br <= 0.0, negz = bz <= 0.0;
            const bool adv = P.shiftadvect != 0;
            auto DAr = [&](int f) { return adv ? dadv(A.in[f] + o, 1, i, nr, g, negr, G.idr, false) : Dr(f); };
            auto DAz = [&](int f) { return adv ? dadv(A.in[f] + o, ld, j, nz, g, negz, G.idz, true) : Dz(f); };
            s_dbr = s_dbr + br * (DAr(F_DTBETAR) - DAr(F_DLR)) + bz * (DAz(F_DTBETAR) - DAz(F_DLR));
            s_dbz = s_dbz + br * (DAr(F_DTBETAZ) - DAr(F_DLZ)) + bz * (DAz(F_DTBETAZ) - DAz(F_DLZ));
        }
        s_dbr = s_dbr - P.drivereta * val(F_DTBETAR);
        s_dbz = s_dbz - P.drivereta * val(F_DTBETAZ);
    }

    // ---- outgoing-wave boundary on the outer edges (radbound.f90)
    const bool edge_r = (i == nr), edge_z = (j == nz) || (!G.eqsym && j == 1 - g);
    if (edge_r || edge_z) {
        const double z = G.zrow[j];
        const double rr = sqrt(r * r + z * z);
        auto radb = [&](int f, double v, double& s) {
            s = -v * (r * Dr(f) + z * Dz(f) + (val(f) - 0.0)) / rr;
        };
        if (A.level0 && P.boundtype == 0) {
            const double vl = 1.0, va = sqrt(P.gauge_f);
            radb(F_TRK, va, s_trK);
            radb(F_KTA, vl, s_KTA);
            radb(F_KTB, vl, s_KTB);
            if (edge_r) {
                s_KTA = s_KTA + third * (one - vl / va) * s_trK * two;
                s_KTB = s_KTB - third * (one - vl / va) * s_trK;
            }
            if (!G.eqsym && j == 1 - g) {
                s_KTA = s_KTA - third * (one - vl / va) * s_trK;
                s_KTB = s_KTB + third * (one - vl / va) * s_trK * two;
            }
            if (j == nz) {
                s_KTA = s_KTA - third * (one - vl / va) * s_trK;
                s_KTB = s_KTB + third * (one - vl / va) * s_trK * two;
            }
            radb(F_KTC, vl, s_KTC);
            if constexpr (SHIFT) {
                if (P.drivercsi != 0.0) {
                    const double vs = sqrt(4.0 * third * P.drivercsi);
                    radb(F_DTBETAR, vs, s_dbr);
                    radb(F_DTBETAZ, vs, s_dbz);
                }
            }
        }
        if constexpr (SCALAR) radb(F_SPI, 1.0, s_spi);
    }

    // ---- accumulate + update (generated accumulate.f90 / update.f90)
    unsigned bad = 0;
    auto upd = [&](int f, double s) {
        double seff = s;
        if (A.rk4) {
            double* ac = A.acc[f] + o;
            if (A.iter < A.niter) *ac = (A.iter == 1) ? A.weight * s : *ac + A.weight * s;
            else seff = *ac + A.weight * s;
        }
        const double v = ld_(A.pst[f] + o) + A.dtw * seff;
        A.out[f][o] = v;
        bad |= nonfinite(v);
    };
    upd(F_ALPHA, s_alpha);
    upd(F_CHI, s_chi);
    if (A.evolve_phi) upd(F_PHI, s_phi);
    upd(F_A, s_A); upd(F_B, s_B); upd(F_H, s_H); upd(F_C, s_C);
    upd(F_TRK, s_trK); upd(F_KTA, s_KTA); upd(F_KTB, s_KTB); upd(F_KTC, s_KTC);
    upd(F_DLR, s_Dlr); upd(F_DLZ, s_Dlz);
    if constexpr (SHIFT) { upd(F_BETAR, s_br); upd(F_BETAZ, s_bz); upd(F_DTBETAR, s_dbr); upd(F_DTBETAZ, s_dbz); }
    if constexpr (SCALAR) { upd(F_SPHI, s_sphi); upd(F_SXIR, s_sxr); upd(F_SXIZ, s_sxz); upd(F_SPI, s_spi); }
    if (bad && A.nanflag) atomicOr(A.nanflag, 1u);
    (void)zero; (void)phi_c;
}

}  // namespace

void launch_rhs(const StageArgs& a, cudaStream_t s) {
    dim3 blk(32, 4);
    const int nj = a.G.nz - a.G.jlo + 1;
    dim3 grd((a.G.nr + blk.x - 1) / blk.x, (nj + blk.y - 1) / blk.y);
    const bool sh = a.P.shift != 0, sc = a.P.scalar != 0;
    if (!sh && !sc) rhs_kernel<false, false><<<grd, blk, 0, s>>>(a);
    else if (sh && !sc) rhs_kernel<true, false><<<grd, blk, 0, s>>>(a);
    else if (!sh && sc) rhs_kernel<false, true><<<grd, blk, 0, s>>>(a);
    else rhs_kernel<true, true><<<grd, blk, 0, s>>>(a);
}

}  // namespace ollin
