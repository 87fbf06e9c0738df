// The fused right-hand-side + Runge-Kutta stage kernel.
//
// One thread owns one grid point (i,j) of one level and does, in registers,
// everything the reference spreads over ~300 whole-array statements per stage:
//   * all first, second, mixed and lopsided (advective) derivatives of the
//     evolved fields (src/base/derivatives.f90, derivadvect.f90; order four,
//     or order two with the template parameter ORD = 2);
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
#pragma once
#include "ollin_kernels.h"
#include "rhs_algebra_gen.cuh"

namespace ollin {

namespace {

__device__ __forceinline__ double sq(double x) { return x * x; }

__device__ __forceinline__ bool nonfinite(double x) {
    return ((__double_as_longlong(x) >> 52) & 0x7ff) == 0x7ff;
}

struct Deriv5 { double r, z, rr, zz, rz; };

#ifndef OLLIN_RHS_THREADS
#define OLLIN_RHS_THREADS 128
#endif
#ifndef OLLIN_RHS_MINBLOCKS
#define OLLIN_RHS_MINBLOCKS 3
#endif
// (bx, by) is the block's position in its own launch's grid: blockIdx for an
// ordinary launch, or the block of this evolution in a fused multi-instance
// launch (multi_kernel)
// the stencils of the run's finite-difference order
template <int ORD>
__device__ __forceinline__ int pcl(int i, int n, int g) {
    if constexpr (ORD == 2) return pclass2(i, n, g);
    else return pclass(i, n, g);
}
template <int ORD>
__device__ __forceinline__ double D1(const double* f, long s, int k, double c) {
    if constexpr (ORD == 2) return d1_2(f, s, k, c);
    else return d1(f, s, k, c);
}
template <int ORD>
__device__ __forceinline__ double D2(const double* f, long s, int k, double c) {
    if constexpr (ORD == 2) return d2_2(f, s, k, c);
    else return d2(f, s, k, c);
}
template <int ORD>
__device__ __forceinline__ double D2RZ(const double* f, long ld, int i, int j, int nr, int nz, int g, double idrz) {
    if constexpr (ORD == 2) return d2rz_2(f, ld, i, j, nr, nz, g, idrz);
    else return d2rz(f, ld, i, j, nr, nz, g, idrz);
}
template <int ORD>
__device__ __forceinline__ double DADV(const double* f, long s, int i, int n, int g, bool neg, double ih, bool zdir) {
    if constexpr (ORD == 2) return dadv_2(f, s, i, n, g, neg, ih);
    else return dadv(f, s, i, n, g, neg, ih, zdir);
}

template <bool SHIFT, bool SCALAR, bool ADVECT, bool STALE, bool SYNC = false, int ORD = 4>
__device__ __forceinline__ void rhs_body(const StageArgs& A, unsigned bx, unsigned by) {
    const LevelGeom& G = A.G;
    const int i = 1 + (int)(bx * blockDim.x + threadIdx.x);
    const int j = G.jlo + (int)(by * blockDim.y + threadIdx.y);
    if (i > G.nr || j > G.nz) return;
    const int g = G.g, nr = G.nr, nz = G.nz;
    const long ld = G.ld;
    const size_t o = (size_t)i + (size_t)j * (size_t)ld;
    const PhysParams& P = A.P;

    // stencil scales: 1/(12h), 1/(12h^2) in order four; 1/(2h), 1/h^2 in order two
    const double cr1 = ORD == 2 ? 0.5 * G.idr : G.idr * (1.0 / 12.0), cz1 = ORD == 2 ? 0.5 * G.idz : G.idz * (1.0 / 12.0);
    const double cr2 = ORD == 2 ? G.idr * G.idr : G.idr * G.idr * (1.0 / 12.0);
    const double cz2 = ORD == 2 ? G.idz * G.idz : G.idz * G.idz * (1.0 / 12.0);
    const double idrz = G.idr * G.idz;
    // The state the derivatives and the point values of this stage are taken
    // from: the stage input, except in the first stage after ``syncboxes``
    // (SYNC), whose auxiliary quantities the reference still holds from
    // before the copy -- the grid's own state before it at the points not
    // copied, the partner box's state (a point well inside it, so interior
    // stencils) at the copied ones.  Dissipation reads the stage input.
    const double* const* X = A.in;
    size_t ox = o;
    long ldx = ld;
    bool xin = false;  // a copied point: stencils of the partner's interior
    if constexpr (SYNC) {
        const int m = A.smap[o];
        if (m >= 0) {
            const int k = m >> kPartnerShift;
            X = A.xb[k]; ox = (size_t)(m & kPartnerOffset); ldx = A.xb_ld[k]; xin = true;
        }
        else X = A.xa;
    }
    const int pcr = xin ? 0 : pcl<ORD>(i, nr, g), pcz = xin ? 0 : pcl<ORD>(j, nz, g);
    // edge position of the mixed derivative: an interior point when copied
    const int ir_ = xin ? 4 : i, jr_ = xin ? 4 : j, nr_ = xin ? (1 << 20) : nr, nz_ = xin ? (1 << 20) : nz;

    auto val = [&](int f) { return ld_(X[f] + ox); };
    auto D5p = [&](const double* p) {
        Deriv5 d;
        d.r = D1<ORD>(p, 1, pcr, cr1);
        d.z = D1<ORD>(p, ldx, pcz, cz1);
        d.rr = D2<ORD>(p, 1, pcr, cr2);
        d.zz = D2<ORD>(p, ldx, pcz, cz2);
        d.rz = D2RZ<ORD>(p, ldx, ir_, jr_, nr_, nz_, g, idrz);
        return d;
    };
    auto D5 = [&](int f) { return D5p(X[f] + ox); };
    auto Dr = [&](int f) { return D1<ORD>(X[f] + ox, 1, pcr, cr1); };
    auto Dz = [&](int f) { return D1<ORD>(X[f] + ox, ldx, pcz, cz1); };
    auto aux = [&](int x) { return ld_(A.aux[x] + o); };

    const double r = G.rcol[i], ir = G.ircol[i];
    const double zero = 0.0, half = 0.5, one = 1.0, two = 2.0, four = 4.0, six = 6.0;
    const double third = 1.0 / 3.0, sixth = 1.0 / 6.0, fourth = 0.25;
    const double smallpi = 3.141592653589793;

    // ---- state and aux at the point
    // after a maximal-slicing solve the lapse itself is the solver's (the
    // current state), whatever the derivatives are taken from
    const double alpha = (STALE && SYNC) ? ld_(A.in[F_ALPHA] + o) : val(F_ALPHA), chi = val(F_CHI);
    const double Ac = val(F_A), Bc = val(F_B), Hc = val(F_H), Cc = val(F_C);
    const double trK = val(F_TRK), kA = val(F_KTA), kB = val(F_KTB), kC = val(F_KTC);
    const double Dlr = val(F_DLR), Dlz = val(F_DLZ);
    const double gA = aux(X_GA), gB = aux(X_GB), gH = aux(X_GH), gC = aux(X_GC);
    const double kH = aux(X_KTH), lam = aux(X_LAM), Alam = aux(X_ALAM), glam = aux(X_GLAM);
    const double DDr = aux(X_DELDEFR), DDz = aux(X_DELDEFZ);

    // ---- derivatives
    // the lapse as the last ``auxiliary`` call saw it: the same as alpha
    // except in the first stage after a maximal-slicing solve (STALE), whose
    // first derivatives ``maximalslicing`` recomputed on this grid's own
    // stencils; with SYNC as well, the old lapse's derivatives are those of
    // the state kept from before the copies
    Deriv5 da, dao;
    double alpha_o = alpha;
    if constexpr (STALE && SYNC) {
        const int kr = pcl<ORD>(i, nr, g), kz = pcl<ORD>(j, nz, g);
        const double* p = A.in[F_ALPHA] + o;
        da.r = D1<ORD>(p, 1, kr, cr1);
        da.z = D1<ORD>(p, ld, kz, cz1);
        da.rr = D2<ORD>(p, 1, kr, cr2);
        da.zz = D2<ORD>(p, ld, kz, cz2);
        da.rz = D2RZ<ORD>(p, ld, i, j, nr, nz, g, idrz);
        dao = D5(F_ALPHA);
        alpha_o = ld_(A.alpha_aux + o);
    } else if constexpr (STALE) {
        da = D5(F_ALPHA);
        dao = D5p(A.alpha_aux + o);
        alpha_o = ld_(A.alpha_aux + o);
    } else {
        da = D5(F_ALPHA);
        dao = da;
    }
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
    double Dr_chi = 0.0, Dz_chi = 0.0;
    if (A.t0) {
        const Deriv5 dp = D5(F_PHI);
        Dr_phi = dp.r; Dz_phi = dp.z; Drr_phi = dp.rr; Dzz_phi = dp.zz; Drz_phi = dp.rz;
        phi_c = val(F_PHI);
        const double psi = exp(phi_c);
        const double psi2 = psi * psi;
        ipsi4 = one / (psi2 * psi2);
    } else {
        const Deriv5 dc = D5(F_CHI);
        Dr_chi = dc.r; Dz_chi = dc.z;
        // phi = -log(chi)/2: D phi = -D chi/(2 chi),
        // DD phi = -DD chi/(2 chi) + (D chi/chi)(D chi/chi)/2
        const double ichi = one / chi;
        const double nhi = -half * ichi;
        Dr_phi = dc.r * nhi;
        Dz_phi = dc.z * nhi;
        const double xr = dc.r * ichi, xz = dc.z * ichi;
        Drr_phi = dc.rr * nhi - Dr_phi * xr;
        Dzz_phi = dc.zz * nhi - Dz_phi * xz;
        Drz_phi = dc.rz * nhi - Dr_phi * xz;
        ipsi4 = chi * chi;  // 1/psi^4 with psi = chi^(-1/2)
    }

    const double r2 = r * r;

    // ---- the pointwise algebra (Laplacian of the lapse, Ricci tensor and
    //      scalar, curvature contractions, divergence of KT, geometric
    //      sources and constraints), generated in FP64-instruction-minimised
    //      form from csrc/gen/bssn_spec.py
    AlgIn in;
    in.r = r; in.ir = ir; in.alpha = alpha; in.chi = chi;
    in.Ac = Ac; in.Bc = Bc; in.Hc = Hc; in.Cc = Cc;
    in.trK = trK; in.kA = kA; in.kB = kB; in.kC = kC; in.kH = kH;
    in.Dlr = Dlr; in.Dlz = Dlz; in.gA = gA; in.gB = gB; in.gH = gH; in.gC = gC;
    in.lam = lam; in.Alam = Alam; in.glam = glam; in.DDr = DDr; in.DDz = DDz;
    in.ipsi4 = ipsi4; in.eta = P.eta;
    in.da_r = dao.r; in.da_z = dao.z; in.da_rr = dao.rr; in.da_zz = dao.zz; in.da_rz = dao.rz;
    in.dan_r = da.r; in.dan_z = da.z;
    in.dA_r = dA.r; in.dA_z = dA.z; in.dA_rr = dA.rr; in.dA_zz = dA.zz; in.dA_rz = dA.rz;
    in.dB_r = dB.r; in.dB_z = dB.z; in.dB_rr = dB.rr; in.dB_zz = dB.zz; in.dB_rz = dB.rz;
    in.dH_r = dH.r; in.dH_z = dH.z; in.dH_rr = dH.rr; in.dH_zz = dH.zz; in.dH_rz = dH.rz;
    in.dC_r = dC.r; in.dC_z = dC.z; in.dC_rr = dC.rr; in.dC_zz = dC.zz; in.dC_rz = dC.rz;
    in.Dr_phi = Dr_phi; in.Dz_phi = Dz_phi; in.Drr_phi = Drr_phi; in.Dzz_phi = Dzz_phi; in.Drz_phi = Drz_phi;
    in.Dr_trK = Dr_trK; in.Dz_trK = Dz_trK; in.Dr_KTA = Dr_KTA; in.Dz_KTA = Dz_KTA;
    in.Dr_KTB = Dr_KTB; in.Dz_KTB = Dz_KTB; in.Dr_KTC = Dr_KTC; in.Dz_KTC = Dz_KTC;
    in.Dr_Dlr = Dr_Dlr; in.Dz_Dlr = Dz_Dlr; in.Dr_Dlz = Dr_Dlz; in.Dz_Dlz = Dz_Dlz;

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
    double s_phi = -sixth * alpha * trK;
    double s_chi = 2.0 * sixth * alpha * chi * trK;
    double s_A = -two * alpha * kA, s_B = -two * alpha * kB, s_H = -two * alpha * kH, s_C = -two * alpha * kC;
    double s_trK = 0, s_KTA = 0, s_KTB = 0, s_KTC = 0, s_Dlr = 0, s_Dlz = 0;
    if (!A.analysis) {
        SrcOut so;
        bssn_sources(in, so);
        s_trK = so.s_trK; s_KTA = so.s_KTA; s_KTB = so.s_KTB; s_KTC = so.s_KTC; s_Dlr = so.s_Dlr; s_Dlz = so.s_Dlz;
    }
    // sources_lapse.f90: -falpha trK with falpha of auxiliary_geometry.f90:
    // 116-166; zero for static and maximal slicing
    double s_alpha = 0.0;
    const bool bona_masso = P.slicing <= 2;
    if (P.slicing == 0) s_alpha = -(alpha_o * P.gauge_f) * trK;                   // 1+log
    else if (P.slicing == 1) s_alpha = -(sq(alpha_o) * P.gauge_f) * trK;         // harmonic
    else if (P.slicing == 2) s_alpha = -(sq(alpha_o) + (P.gauge_f - 1.0)) * trK;  // shock avoiding

    double s_br = 0, s_bz = 0, s_dbr = 0, s_dbz = 0;
    // the shock-avoiding drivers' fdriver source (sources_shift.f90:144,
    // :271), formed after the dissipation so that nothing of it stays live
    // through the kernel's widest region
    double s_fd = 0.0;
    if constexpr (SHIFT) {
        const double br = val(F_BETAR), bz = val(F_BETAZ), dbr = val(F_DTBETAR), dbz = val(F_DTBETAZ);
        const Deriv5 dbR = D5(F_BETAR), dbZ = D5(F_BETAZ);
        const bool negr = br <= 0.0, negz = bz <= 0.0;
        // Advection term beta^r D_r f + beta^z D_z f with lopsided derivatives
        // (derivadvect.f90).  Inside i = 4-ghost..Nr-3 (order two:
        // 3-ghost..Nr-2) the two upwind stencils are one sum taken with the
        // stride pointing against the shift, and beta times its scale is
        // -|beta|/(12 h) (order two: -|beta|/(2 h)) for either sign, so each
        // field costs one stencil and one FMA per direction.
        constexpr int lo = ORD == 2 ? 3 : 4, hi = ORD == 2 ? 2 : 3;
        const bool lint_r = xin || (i >= lo - g && i <= nr - hi), lint_z = xin || (j >= lo - g && j <= nz - hi);
        const long lsr = negr ? -1 : 1, lsz = negz ? -ldx : ldx;
        const double kr = -fabs(br) * (ORD == 2 ? 0.5 * G.idr : G.idr * (1.0 / 12.0));
        const double kz = -fabs(bz) * (ORD == 2 ? 0.5 * G.idz : G.idz * (1.0 / 12.0));
        auto lop = [&](const double* p, long st) {
            if constexpr (ORD == 2) return 3.0 * ld_(p) - 4.0 * ld_(p + st) + ld_(p + 2 * st);
            else return 3.0 * ld_(p - st) + 10.0 * ld_(p) - 18.0 * ld_(p + st) + 6.0 * ld_(p + 2 * st) - ld_(p + 3 * st);
        };
        auto ladv_r = [&](const double* p) { return lint_r ? kr * lop(p, lsr) : br * DADV<ORD>(p, 1, i, nr, g, negr, G.idr, false); };
        auto ladv_z = [&](const double* p) { return lint_z ? kz * lop(p, lsz) : bz * DADV<ORD>(p, ldx, j, nz, g, negz, G.idz, true); };
        // shiftadvect is a template parameter: with it on, the centred
        // derivatives need not stay live for this block
        auto ADVp = [&](const double* p, double dr_, double dz_) {
            if constexpr (!ADVECT) {
                (void)p;
                return br * dr_ + bz * dz_;
            } else {
                return ladv_r(p) + ladv_z(p);
            }
        };
        auto ADV = [&](int f, double dr_, double dz_) { return ADVp(X[f] + ox, dr_, dz_); };
        // DD_beta_rr = d/dr (beta_r / r): first derivative of beta_r/r
        double DD_beta_rr;
        {
            const double* pb = X[F_BETAR] + ox;
            const double* ic = G.ircol + i;
            auto q = [&](int m) { return ld_(pb + m) * ic[m]; };
            if constexpr (ORD == 2) {
                if (pcr == 0) DD_beta_rr = cr1 * (q(1) - q(-1));
                else DD_beta_rr = cr1 * (3.0 * q(0) - 4.0 * q(-1) + q(-2));
            } else {
                if (pcr == 0) DD_beta_rr = cr1 * (8.0 * (q(1) - q(-1)) - (q(2) - q(-2)));
                else if (pcr == 1) DD_beta_rr = cr1 * (3.0 * q(1) + 10.0 * q(0) - 18.0 * q(-1) + 6.0 * q(-2) - q(-3));
                else DD_beta_rr = cr1 * (25.0 * q(0) - 48.0 * q(-1) + 36.0 * q(-2) - 16.0 * q(-3) + 3.0 * q(-4));
            }
        }
        const double DIV_beta = dbR.r + dbZ.z + br * ir;
        const double Dr_DIV_beta = dbR.rr + dbZ.rz + DD_beta_rr;
        const double Dz_DIV_beta = dbR.rz + dbZ.zz + dbR.z * ir;
        // sigma = 1 (lagrangian): the -2/3 sigma f DIV_beta terms
        const double tdb = (2.0 / 3.0) * DIV_beta;
        if (A.t0) {
            s_phi = s_phi + ADV(F_PHI, Dr_phi, Dz_phi) + sixth * DIV_beta;
            // chi's lopsided derivatives are not formed while the level time is
            // zero (the t=0 branch of auxiliary_geometry.f90:178-202 only
            // differentiates phi), so the advection term of chi reads zeros
            s_chi = s_chi - chi * (0.5 * tdb);
        } else {
            s_chi = s_chi + ADV(F_CHI, Dr_chi, Dz_chi) - chi * (0.5 * tdb);
        }
        const double Drb = dbR.r, Dzb = dbR.z, Drbz = dbZ.r, Dzbz = dbZ.z;
        const double rDrbz = r * Drbz, rDzb = r * Dzb, Dsum = Drb + Dzbz, bir = br * ir;
        s_A = s_A + ADV(F_A, dA.r, dA.z) + two * (Ac * Drb + Cc * rDrbz) - Ac * tdb;
        s_B = s_B + ADV(F_B, dB.r, dB.z) + two * (Bc * Dzbz + Cc * rDzb) - Bc * tdb;
        s_H = s_H + ADV(F_H, dH.r, dH.z) + Hc * (two * bir - tdb);
        s_C = s_C + ADV(F_C, dC.r, dC.z) + Cc * (bir + Dsum - tdb) + (Bc * Drbz + Ac * Dzb) * ir;
        s_trK = s_trK + ADV(F_TRK, Dr_trK, Dz_trK);
        s_KTA = s_KTA + ADV(F_KTA, Dr_KTA, Dz_KTA) + two * (kA * Drb + kC * rDrbz) - kA * tdb;
        s_KTB = s_KTB + ADV(F_KTB, Dr_KTB, Dz_KTB) + two * (kB * Dzbz + kC * rDzb) - kB * tdb;
        s_KTC = s_KTC + ADV(F_KTC, Dr_KTC, Dz_KTC) + kC * (bir + Dsum - tdb) + (kB * Drbz + kA * Dzb) * ir;
        const double rgC = r * gC;
        s_Dlr = s_Dlr + ADV(F_DLR, Dr_Dlr, Dz_Dlr) - Dlr * Drb - Dlz * Dzb;
        s_Dlr = s_Dlr + two * rgC * dbR.rz + gA * dbR.rr + gB * dbR.zz + gH * DD_beta_rr;
        s_Dlr = s_Dlr + third * (gA * Dr_DIV_beta + rgC * Dz_DIV_beta) + Dlr * tdb;
        s_Dlz = s_Dlz + ADV(F_DLZ, Dr_Dlz, Dz_Dlz) - Dlr * Drbz - Dlz * Dzbz;
        s_Dlz = s_Dlz + two * rgC * dbZ.rz + gA * dbZ.rr + gB * dbZ.zz + gH * Drbz * ir;
        s_Dlz = s_Dlz + third * (rgC * Dr_DIV_beta + gB * Dz_DIV_beta) + Dlz * tdb;
        if (bona_masso)
            s_alpha = s_alpha + ADVp(STALE && !SYNC ? A.alpha_aux + o : X[F_ALPHA] + ox, dao.r, dao.z);
        // sources_shift.f90: Gammadriver2 d_t beta = dtbeta (:229-260),
        // Gammadriver1 d_t beta = csi Delta - eta beta (:108-186),
        // Gammadriver0 d_t beta = csi d_t Delta (below, after the Delta source
        // is complete); the shock-avoiding variants put fdriver on Delta and
        // evolve it; zero sources for the static shift and before shiftafter
        // (:43-52)
        if (A.shift_static) {
            s_br = 0.0;
            s_bz = 0.0;
        } else {
            const double cf = P.shock ? P.drivercsi * val(F_FDRIVER) : P.drivercsi;
            if (P.driver == 2) {
                s_br = dbr;
                s_bz = dbz;
            } else if (P.driver == 1) {
                s_br = cf * Dlr;
                s_bz = cf * Dlz;
            }
            if (P.driveradv && (P.driver == 1 || P.driver == 2)) {
                s_br = s_br + ADV(F_BETAR, dbR.r, dbR.z);
                s_bz = s_bz + ADV(F_BETAZ, dbZ.r, dbZ.z);
            }
            if (P.driver == 1) {
                if (P.driverD0) {
                    s_br = s_br - cf * ld_(A.d0r + o);
                    s_bz = s_bz - cf * ld_(A.d0z + o);
                }
                s_br = s_br - P.drivereta * br;
                s_bz = s_bz - P.drivereta * bz;
            }
        }
        (void)s_dbr; (void)s_dbz;
        if constexpr (SCALAR) {
            // auxiliary_matter.f90 always forms lopsided derivatives for the
            // scalar field when a shift is present (independent of shiftadvect)
            auto LADV = [&](int f) { const double* p = X[f] + ox; return ladv_r(p) + ladv_z(p); };
            const double sxr = val(F_SXIR), sxz = val(F_SXIZ);
            s_sphi = s_sphi + br * sxr + bz * sxz;
            s_sxr = s_sxr + LADV(F_SXIR) + sxr * Drb + sxz * Drbz;
            s_sxz = s_sxz + LADV(F_SXIZ) + sxr * Dzb + sxz * Dzbz;
            s_spi = s_spi + LADV(F_SPI);
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
        AnaOut ao;
        bssn_analysis(in, ao);
        double ham = ao.ham, momr = ao.mom_r, momz = ao.mom_z;
        if constexpr (SCALAR) {
            ham = ham - 16.0 * spf * rho;
            momr = momr - 8.0 * spf * J_r / ipsi4;
            momz = momz - 8.0 * spf * J_z / ipsi4;
        }
        A.auxw[X_HAM][o] = ham;
        A.auxw[X_MOMR][o] = momr;
        A.auxw[X_MOMZ][o] = momz;
        A.auxw[X_RSCAL][o] = ao.RSCAL;
        A.auxw[X_KT2][o] = ao.KT2;
        A.auxw[X_LAPLA][o] = ao.Lapla_alpha;
        if constexpr (SCALAR) A.auxw[X_RHOS][o] = rho + trS;
        return;
    }

    // ---- Kreiss-Oliger dissipation (dissipation.f90:196-211; order two: the
    //      fourth difference of :121-135 on i = 3-ghost..Nr-2)
    constexpr int dlo = ORD == 2 ? 3 : 4, dhi = ORD == 2 ? 2 : 3;
    constexpr double dscale = ORD == 2 ? 1.0 / 6.0 : 1.0 / 20.0;
    const bool diss_r = (i >= dlo - g && i <= nr - dhi);
    const bool diss_z = (j >= dlo - g && j <= nz - dhi);
    if (P.geodiss != 0.0) {
        const double kd = P.geodiss / G.dt * dscale;
        auto diss = [&](int f, double& s) {
            const double* p = A.in[f] + o;
            if constexpr (ORD == 2) {
                if (diss_r) s = s - kd * ko4(p, 1);
                if (diss_z) s = s - kd * ko4(p, ld);
                return;
            }
            if (diss_r && diss_z) { s = ko6rz_apply(p, ld, kd, s); return; }
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
            const double kd = P.scalardiss / G.dt * dscale;
            auto diss = [&](int f, double& s) {
                const double* p = A.in[f] + o;
                if constexpr (ORD == 2) {
                    if (diss_r) s = s - kd * ko4(p, 1);
                    if (diss_z) s = s - kd * ko4(p, ld);
                    return;
                }
                if (diss_r && diss_z) { s = ko6rz_apply(p, ld, kd, s); return; }
                if (diss_r) s = s - kd * ko6(p, 1);
                if (diss_z) s = s - kd * ko6(p, ld);
            };
            diss(F_SPHI, s_sphi);
            diss(F_SPI, s_spi);
            diss(F_SXIR, s_sxr);
            diss(F_SXIZ, s_sxz);
        }
    }
    if constexpr (SHIFT) if (A.shift_static || P.driver != 2) {
        // dtbeta is not evolved by the first-order and parabolic drivers, and
        // keeps a zero source while the shift is static
        s_dbr = 0.0;
        s_dbz = 0.0;
        if (P.driver == 0 && !A.shift_static) {
            s_br = P.drivercsi * s_Dlr;
            s_bz = P.drivercsi * s_Dlz;
        }
    }
    // d_t fdriver = -2/3 fdriver DIV beta (+ beta . D fdriver): lopsided
    // derivatives in the first-order driver, centred ones in the second-order
    // one (:144-151, :271-278); DIV beta again from the shift's stencils
    double s_fd0 = 0.0;
    if constexpr (SHIFT) if (P.shock && !A.shift_static) {
        const double fdv = val(F_FDRIVER), br = val(F_BETAR), bz = val(F_BETAZ);
        s_fd0 = -two * third * fdv * (Dr(F_BETAR) + Dz(F_BETAZ) + br * ir);
        s_fd = s_fd0;
        if (P.driveradv) {
            if (P.driver == 1 && ADVECT) {
                const double* pf = X[F_FDRIVER] + ox;
                s_fd = s_fd + (br * DADV<ORD>(pf, 1, xin ? 4 : i, xin ? (1 << 20) : nr, g, br <= 0.0, G.idr, false)
                               + bz * DADV<ORD>(pf, ldx, xin ? 4 : j, xin ? (1 << 20) : nz, g, bz <= 0.0, G.idz, true));
            } else {
                s_fd = s_fd + br * Dr(F_FDRIVER) + bz * Dz(F_FDRIVER);
            }
        }
    }
    if constexpr (SHIFT) if (!A.shift_static && P.driver == 2) {
        if (P.shock) {
            // d_t dtbeta = csi d_t (fdriver Delta) (:273-274)
            const double fdv = val(F_FDRIVER);
            s_dbr = P.drivercsi * (fdv * s_Dlr + s_fd0 * Dlr);
            s_dbz = P.drivercsi * (fdv * s_Dlz + s_fd0 * Dlz);
        } else {
            s_dbr = P.drivercsi * s_Dlr;
            s_dbz = P.drivercsi * s_Dlz;
        }
        if (P.driveradv) {
            const double br = val(F_BETAR), bz = val(F_BETAZ);
            const bool negr = br <= 0.0, negz = bz <= 0.0;
            auto DAr = [&](int f) {
                return ADVECT ? DADV<ORD>(X[f] + ox, 1, xin ? 4 : i, xin ? (1 << 20) : nr, g, negr, G.idr, false) : Dr(f);
            };
            auto DAz = [&](int f) {
                return ADVECT ? DADV<ORD>(X[f] + ox, ldx, xin ? 4 : j, xin ? (1 << 20) : nz, g, negz, G.idz, true) : Dz(f);
            };
            s_dbr = s_dbr + br * (DAr(F_DTBETAR) - DAr(F_DLR)) + bz * (DAz(F_DTBETAR) - DAz(F_DLR));
            s_dbz = s_dbz + br * (DAr(F_DTBETAZ) - DAr(F_DLZ)) + bz * (DAz(F_DTBETAZ) - DAz(F_DLZ));
        }
        if (P.shock && P.driverD0) {
            s_dbr = s_dbr - P.drivercsi * s_fd * ld_(A.d0r + o);
            s_dbz = s_dbz - P.drivercsi * s_fd * ld_(A.d0z + o);
        }
        s_dbr = s_dbr - P.drivereta * val(F_DTBETAR);
        s_dbz = s_dbz - P.drivereta * val(F_DTBETAZ);
    }

    // maximal slicing: strK = 0 with no dissipation, advection or matter
    // terms (sources_geometry.f90:200-204) and no radiative boundary for trK
    // (radiative_geometry.f90:70-76)
    const bool maximal = P.slicing == 4;
    if (maximal) s_trK = 0.0;

    // Gammadriver0's boundary in radiative_geometry.f90:203-211 zeroes the
    // shift sources on the column i = 0 and the row j = 0 of level 0: inside
    // the grid only where the row j = 0 is not an equator ghost row
    if constexpr (SHIFT) {
        if (P.driver == 0 && A.level0 && P.boundtype == 0 && P.drivercsi != 0.0 && (i == 0 || j == 0)) {
            s_br = 0.0;
            s_bz = 0.0;
        }
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
            if (!maximal) radb(F_TRK, va, s_trK);
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
                if (P.drivercsi != 0.0) {  // radiative_geometry.f90:195-262
                    const double vs = sqrt(4.0 * third * P.drivercsi);
                    if (P.driver == 2) {
                        radb(F_DTBETAR, vs, s_dbr);
                        radb(F_DTBETAZ, vs, s_dbz);
                    } else if (P.driver == 1) {
                        radb(F_DLR, vs, s_Dlr);
                        radb(F_DLZ, vs, s_Dlz);
                    }
                }
            }
        }
        if constexpr (SCALAR) radb(F_SPI, 1.0, s_spi);
    }

    // boundtype = "static" / "flat" on level 0 (generated simpleboundary.f90,
    // after the matter sources): the sources of the arrays without NOBOUND on
    // the outer edges are zero, or those of the column Nr-1 / row Nz-1 / row
    // 2-ghost inside.  For "flat" the points inside store theirs (A.flat), the
    // edge points leave those arrays alone, and flat_edges_kernel updates
    // them once every source of the stage is known.
    const bool simple = A.level0 && P.boundtype >= 2;
    const bool skip_bound = simple && P.boundtype == 3 && (edge_r || edge_z);
    if (simple && P.boundtype == 2 && (edge_r || edge_z)) {
        s_trK = 0.0; s_KTA = 0.0; s_KTB = 0.0; s_KTC = 0.0; s_Dlr = 0.0; s_Dlz = 0.0;
        if constexpr (SHIFT) { s_dbr = 0.0; s_dbz = 0.0; s_fd = 0.0; }
        if constexpr (SCALAR) s_spi = 0.0;
    }
    if (simple && P.boundtype == 3 && A.flat) {
        const bool in_r = i == nr - 1, in_z = j == nz - 1, in_l = !G.eqsym && j == 2 - g;
        if (in_r || in_z || in_l) {
            const int nR = nz - G.jlo + 1;
            auto put = [&](int b, double s) {
                double* base = A.flat + (size_t)b * (size_t)A.flat_len;
                if (in_r) base[j - G.jlo] = s;
                if (in_z) base[nR + i - 1] = s;
                if (in_l) base[nR + nr + i - 1] = s;
            };
            put(0, s_trK); put(1, s_KTA); put(2, s_KTB); put(3, s_KTC); put(4, s_Dlr); put(5, s_Dlz);
            if constexpr (SHIFT) { put(6, s_dbr); put(7, s_dbz); put(8, s_fd); }
            if constexpr (SCALAR) put(9, s_spi);
        }
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
    if (!skip_bound) {
        upd(F_TRK, s_trK); upd(F_KTA, s_KTA); upd(F_KTB, s_KTB); upd(F_KTC, s_KTC);
        upd(F_DLR, s_Dlr); upd(F_DLZ, s_Dlz);
    }
    if constexpr (SHIFT) {
        upd(F_BETAR, s_br); upd(F_BETAZ, s_bz);
        if (!skip_bound) {
            upd(F_DTBETAR, s_dbr); upd(F_DTBETAZ, s_dbz);
            if (P.shock) upd(F_FDRIVER, s_fd);
        }
    }
    if constexpr (SCALAR) {
        upd(F_SPHI, s_sphi); upd(F_SXIR, s_sxr); upd(F_SXIZ, s_sxz);
        if (!skip_bound) upd(F_SPI, s_spi);
    }
    if (bad && A.nanflag) atomicOr(A.nanflag, 1u);
    (void)zero; (void)phi_c;
}

template <bool SHIFT, bool SCALAR, bool ADVECT, bool STALE, bool SYNC = false, int ORD = 4>
__global__ void __launch_bounds__(OLLIN_RHS_THREADS, OLLIN_RHS_MINBLOCKS) rhs_kernel(const __grid_constant__ StageArgs A) {
    chain_enter();
    rhs_body<SHIFT, SCALAR, ADVECT, STALE, SYNC, ORD>(A, blockIdx.x, blockIdx.y);
}

// the fused multi-instance twin of one instantiation
template <bool SHIFT, bool SCALAR, bool ADVECT, bool STALE, bool SYNC = false, int ORD = 4>
void register_rhs_multi() {
    register_multi((const void*)rhs_kernel<SHIFT, SCALAR, ADVECT, STALE, SYNC, ORD>,
                   multi_launch<StageArgs, rhs_body<SHIFT, SCALAR, ADVECT, STALE, SYNC, ORD>, OLLIN_RHS_THREADS,
                                OLLIN_RHS_MINBLOCKS>);
}

// the launch of one stage: the six (shift, scalar, advection) variants of a
// (stale, sync, order) family
template <bool STALE, bool SYNC, int ORD>
void launch_rhs_family(const StageArgs& a, cudaStream_t s) {
    dim3 blk(32, OLLIN_RHS_THREADS / 32);
    const int nj = a.G.nz - a.G.jlo + 1;
    dim3 grd((a.G.nr + blk.x - 1) / blk.x, (nj + blk.y - 1) / blk.y);
    const bool sh = a.P.shift != 0, sc = a.P.scalar != 0, ad = a.P.shiftadvect != 0;
    if (!sh && !sc) launch_chained(rhs_kernel<false, false, false, STALE, SYNC, ORD>, grd, blk, s, a);
    else if (!sh && sc) launch_chained(rhs_kernel<false, true, false, STALE, SYNC, ORD>, grd, blk, s, a);
    else if (!sc && ad) launch_chained(rhs_kernel<true, false, true, STALE, SYNC, ORD>, grd, blk, s, a);
    else if (!sc) launch_chained(rhs_kernel<true, false, false, STALE, SYNC, ORD>, grd, blk, s, a);
    else if (ad) launch_chained(rhs_kernel<true, true, true, STALE, SYNC, ORD>, grd, blk, s, a);
    else launch_chained(rhs_kernel<true, true, false, STALE, SYNC, ORD>, grd, blk, s, a);
}

template <bool STALE, bool SYNC, int ORD>
void register_rhs_family() {
    register_rhs_multi<false, false, false, STALE, SYNC, ORD>();
    register_rhs_multi<false, true, false, STALE, SYNC, ORD>();
    register_rhs_multi<true, false, true, STALE, SYNC, ORD>();
    register_rhs_multi<true, false, false, STALE, SYNC, ORD>();
    register_rhs_multi<true, true, true, STALE, SYNC, ORD>();
    register_rhs_multi<true, true, false, STALE, SYNC, ORD>();
}

}  // namespace

}  // namespace ollin
