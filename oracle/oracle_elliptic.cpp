// ORACLE -- test infrastructure only.  CPU restatement of the OllinAxis-BiB
// elliptic initial data used to check the GB300 library; never linked into it.
//
// This file restates
//   src/elliptic/wave_elliptic.f90   (WaveElliptic: the elliptic equation
//       lap(u) + S1 u + S5 u^5 = S0 solved as the stationary state of the
//       damped wave equation du/dt = v, dv/dt = lap(u) + S1 u + S5 u^5 - S0
//       - eta v, with the Berger-Oliger recursion ``wavestep``),
//   src/elliptic/sor_elliptic.f90    (red-black SOR with Chebyshev
//       acceleration and Robin / Dirichlet boundaries),
//   src/matter/idata_scalarpulse.f90 and src/geometry/idata_brillwave.f90
// for the flat Laplacian that both initial-data routines use, and
//   src/geometry/maximalslicing.f90 with the physical Laplacian of the
//   conformal metric (type = 'physical' in both solvers), box 0 only.
// Arithmetic follows the Fortran expression order of those files.
#include <cmath>
#include <stdexcept>
#include <string>

#include "oracle_sim.h"

namespace oracle {

thread_local EllStats g_ell_stats;

namespace {

const double kPi = 3.141592653589793;  // acos(-1.d0)

// ---------------------------------------------------------------------------
// wave_elliptic.f90:347-770 (subroutine wavestep), type = 'flat' or
// 'physical'
// ---------------------------------------------------------------------------
static void wave_grid_step(Sim& S, Level& L, bool physical) {
    const ollin_params& P = S.P;
    const int level = L.level, gid = L.gid;
    currentgrid(S, L);
    // ell_u_p = ell_u, ell_v_p = ell_v and the boundary history
    // (wave_elliptic.f90:421-473): the generic saveold over S.evolved
    saveold(S, L);
    const bool rk4 = P.we_method == OLLIN_INTEGRATOR_RK4;
    const int niter = rk4 ? 4 : P.icniter;
    const double dt = L.dt;
    const int g = L.g, Nr = L.Nr, Nz = L.Nz;
    Arr& u = L.a("ell_u"); Arr& v = L.a("ell_v");
    Arr& su = L.a("sell_u"); Arr& sv = L.a("sell_v");
    Arr& Dr_u = L.a("Dr_ell_u"); Arr& Dz_u = L.a("Dz_ell_u");
    Arr& Drr_u = L.a("Drr_ell_u"); Arr& Dzz_u = L.a("Dzz_ell_u");
    Arr& Dr_v = L.a("Dr_ell_v"); Arr& Dz_v = L.a("Dz_ell_v");
    Arr& S0 = L.a("ell_S0"); Arr& S1 = L.a("ell_S1"); Arr& S5 = L.a("ell_S5");
    Arr& r = L.a("r");
    for (int iter = 1; iter <= niter; ++iter) {
        double dtw = 0, weight = 0;
        if (rk4) {
            switch (iter) {
                case 1: dtw = 0.5 * dt; weight = 1.0 / 6.0; break;
                case 2: dtw = 0.5 * dt; weight = 1.0 / 3.0; break;
                case 3: dtw = dt; weight = 1.0 / 3.0; break;
                default: dtw = dt; weight = 1.0 / 6.0; break;
            }
        } else {
            dtw = (iter < niter) ? 0.5 * dt : dt;
        }
        // derivatives (the mixed one is unused by the flat Laplacian)
        diff1r(L, u, Dr_u, +1);
        diff1z(L, u, Dz_u, +1);
        diff2r(L, u, Drr_u, +1);
        diff2z(L, u, Dzz_u, +1);
        if (physical) diff2rz(L, u, L.a("Drz_ell_u"), +1, +1);
        diff1r(L, v, Dr_v, +1);
        diff1z(L, v, Dz_v, +1);
        su = v;
        for (int j = 1 - g; j <= Nz; ++j)
            for (int i = 1 - g; i <= Nr; ++i) {
                double s;
                if (!physical) {
                    s = Drr_u(i, j) + Dzz_u(i, j) + Dr_u(i, j) / r(i, j);
                } else {  // wave_elliptic.f90:781-812
                    const double gA = L.a("g_A")(i, j), gB = L.a("g_B")(i, j), gC = L.a("g_C")(i, j);
                    const double rr = r(i, j), ur = Dr_u(i, j), uz = Dz_u(i, j);
                    s = gA * Drr_u(i, j) + gB * Dzz_u(i, j) + 2.0 * rr * gC * L.a("Drz_ell_u")(i, j);
                    s = s + ur * (L.a("Dr_g_A")(i, j) + rr * L.a("Dz_g_C")(i, j))
                          + uz * (L.a("Dz_g_B")(i, j) + rr * L.a("Dr_g_C")(i, j) + gC);
                    s = s + gA * ur / rr + gC * uz + 0.5 * L.a("ihdet")(i, j)
                          * (L.a("Dr_hdet")(i, j) * (gA * ur + rr * gC * uz)
                             + L.a("Dz_hdet")(i, j) * (gB * uz + rr * gC * ur));
                    s = s + 2.0 * (L.a("Dr_phi")(i, j) * (gA * ur + rr * gC * uz)
                                   + L.a("Dz_phi")(i, j) * (gB * uz + rr * gC * ur));
                    s = s / L.a("psi4")(i, j);
                }
                s = s + S1(i, j) * u(i, j) + S5(i, j) * p5(u(i, j)) - S0(i, j);
                s = s - P.we_eta * v(i, j);
                sv(i, j) = s;
            }
        dissipation(L, v, sv, +1, +1, P.we_diss);
        if (L.ownaxis)
            for (int ii = 1; ii <= g; ++ii)
                for (int j = 1 - g; j <= Nz; ++j) sv(1 - ii, j) = sv(ii, j);
        if (L.eqsym && L.ownequator)
            for (int jj = 1; jj <= g; ++jj)
                for (int i = 1 - g; i <= Nr; ++i) sv(i, 1 - jj) = sv(i, jj);
        radbound(L, v, sv, Dr_v, Dz_v, 1.0, 0.0);
        if (rk4) accumulate(S, L, iter, niter, weight);
        update(S, L, dtw);
        if (level > 0) finebound(S, gid, dtw);
    }
    S.t2[gid] = S.t1[gid];
    S.t1[gid] = S.t[gid];
    S.s[gid] = S.s[gid] + 1;
    S.t[gid] = S.t[gid] + dt;
}

// wave_elliptic.f90:578-1160 (recursive subroutine wavestep): every box that
// has the level, then the finer level twice, parity fills, ``syncboxes`` of
// ell_u and ell_v between boxes that overlap, restriction into the parents
void wavestep(Sim& S, int level, int Nlmax, bool physical) {
    for (Level& L : S.L)
        if (L.level == level) wave_grid_step(S, L, physical);
    if (level < Nlmax) {
        wavestep(S, level + 1, Nlmax, physical);
        wavestep(S, level + 1, Nlmax, physical);
    }
    if (Nlmax > 0)
        for (Level& L : S.L) {
            if (L.level != level) continue;
            if (L.ownaxis) symmetries_r(S, L);
            if (L.eqsym && L.ownequator) symmetries_z(S, L);
        }
    if (level > 0)
        for (Level& A : S.L)
            for (Level& B : S.L)
                if (A.level == level && B.level == level && A.box != B.box) {
                    syncboxes(S, A.gid, B.gid, {"ell_u"});
                    syncboxes(S, A.gid, B.gid, {"ell_v"});
                }
    if (level > 0)
        for (Level& F : S.L) {
            if (F.level != level || S.s[F.gid] % 2 != 0) continue;
            restrict_(S, F.gid);
            Level& Cl = S.L[F.parent];
            currentgrid(S, Cl);
            if (Cl.ownaxis) symmetries_r(S, Cl);
            if (Cl.eqsym && Cl.ownequator) symmetries_z(S, Cl);
        }
}

// wave_elliptic.f90:2-345 with init = 'one'.  For the physical Laplacian the
// time step follows the largest speed sqrt|g^ii/psi4| over all levels and the
// largest slicing speeds va_max[0..1] (r, z) that the caller's last analysis
// left in va_rp/va_zp (:193-263).
void wave_elliptic(Sim& S, bool physical, const double* va_max) {
    const ollin_params& P = S.P;
    const int nlev = (int)S.L.size();
    // the time counters are borrowed and given back (wave_elliptic.f90:95-103, 330-340)
    const auto s_ext = S.s; const auto t_ext = S.t, t1_ext = S.t1, t2_ext = S.t2;
    const auto evolved_ext = S.evolved;
    std::vector<double> dt_ext(nlev);
    for (int l = 0; l < nlev; ++l) dt_ext[l] = S.L[l].dt;
    std::fill(S.s.begin(), S.s.end(), 0L);
    std::fill(S.t.begin(), S.t.end(), 0.0);
    std::fill(S.t1.begin(), S.t1.end(), 0.0);
    std::fill(S.t2.begin(), S.t2.end(), 0.0);
    S.evolved = {{"ell_u", +1, +1}, {"ell_v", +1, +1}};
    for (Level& L : S.L) {
        for (double& x : L.a("ell_v").v) x = 0.0;
        for (double& x : L.a("ell_u").v) x = 1.0;
    }
    double dt0 = P.we_dtfac * std::min(P.dr0, P.dz0);
    if (physical) {
        double vrmax = 0.0, vzmax = 0.0;
        for (Level& L : S.L) {
            double vr = 0.0, vz = 0.0;
            const int g = L.g;
            Arr& gA = L.a("g_A"); Arr& gB = L.a("g_B"); Arr& psi4 = L.a("psi4");
            const double var = va_max ? std::fabs(va_max[0]) : 0.0, vaz = va_max ? std::fabs(va_max[1]) : 0.0;
            for (int j = 1 - g; j <= L.Nz; ++j)
                for (int i = 1 - g; i <= L.Nr; ++i) {
                    const double vlr = std::sqrt(std::fabs(gA(i, j) / psi4(i, j)));
                    const double vlz = std::sqrt(std::fabs(gB(i, j) / psi4(i, j)));
                    if (std::fabs(vlr) > vr) vr = std::fabs(vlr);
                    if (std::fabs(vlz) > vz) vz = std::fabs(vlz);
                    if (var > vr) vr = var;
                    if (vaz > vz) vz = vaz;
                }
            if (std::fabs(vr) > vrmax) vrmax = std::fabs(vr);
            if (std::fabs(vz) > vzmax) vzmax = std::fabs(vz);
        }
        const double cfac = P.we_dtfac;
        dt0 = cfac * std::min(std::min(P.dr0, P.dz0), std::min(P.dr0 / vrmax, P.dz0 / vzmax));
    }
    for (int l = 0; l < nlev; ++l) S.L[l].dt = dt0 / (double)(1L << S.L[l].level);
    const int Nlmax_old = S.Nlmax;
    int Nlmax = (S.Nlmax > 0) ? 0 : S.Nlmax;
    g_ell_stats = EllStats();
    for (int phase = 0;; ++phase) {
        double gres = 1.0;
        int step = 0;
        const int miniter = 100;
        Level& L0 = S.L[0];
        while (step < miniter || (gres > P.we_epsilon && step < P.we_maxiter)) {
            step = step + 1;
            wavestep(S, 0, Nlmax, physical);
            Arr& sv = L0.a("sell_v");
            double lres = 0.0;
            for (int j = 1; j <= L0.Nz - L0.g; ++j)
                for (int i = 1; i <= L0.Nr - L0.g; ++i) lres = lres + p2(sv(i, j));
            const int NNtot = L0.Nr * L0.Nz;
            lres = std::sqrt(lres / (double)NNtot);
            gres = lres;
        }
        g_ell_stats.steps[phase] = step;
        g_ell_stats.phases = phase + 1;
        g_ell_stats.gres = gres;
        if (step != P.ell_maxiter && Nlmax != Nlmax_old) {
            Nlmax = Nlmax_old;
            for (double& x : L0.a("ell_v").v) x = 0.0;
            // inject the coarse solution into every finer grid (:270-328)
            for (int gid = 1; gid < nlev; ++gid) {
                Level& F = S.L[gid];
                const int level = F.level;
                Arr& r = F.a("r"); Arr& z = F.a("z");
                Arr& u = F.a("ell_u");
                for (int m = 0; m <= F.Nr + F.g - 1; ++m)
                    for (int n = 0; n <= F.Nz + F.g - 1; ++n) {
                        const double r0 = S.rminl[gid] + (double)m * S.drl[level];
                        const double z0 = S.zminl[gid] + (double)n * S.dzl[level];
                        const int i = (int)nint_((r0 - r(1 - F.g, 0)) / S.drl[level]) + 1 - F.g;
                        const int j = (int)nint_((z0 - z(0, 1 - F.g)) / S.dzl[level]) + 1 - F.g;
                        const bool flag1 = (i >= 1 - F.g) && (i <= F.Nr) && (j >= 1 - F.g) && (j <= F.Nz);
                        const double aux2 = interp(S, 0, L0.a("ell_u"), r0, z0);
                        if (flag1) u(i, j) = aux2;
                    }
            }
            std::fill(S.s.begin(), S.s.end(), 0L);
            std::fill(S.t.begin(), S.t.end(), 0.0);
            std::fill(S.t1.begin(), S.t1.end(), 0.0);
            std::fill(S.t2.begin(), S.t2.end(), 0.0);
            continue;
        }
        break;
    }
    S.s = s_ext; S.t = t_ext; S.t1 = t1_ext; S.t2 = t2_ext;
    S.evolved = evolved_ext;
    for (int l = 0; l < nlev; ++l) S.L[l].dt = dt_ext[l];
}

// ---------------------------------------------------------------------------
// sor_elliptic.f90:2-560 (flat Laplacian): coarse solve with Robin
// boundaries, then each finer level with Dirichlet data interpolated from
// the level below, then restriction back down.  Arrays are indexed like the
// reference's sor_* arrays, 1..N+ghost.
// ---------------------------------------------------------------------------
struct SorArr {
    int nx = 0, ny = 0;
    std::vector<double> v;
    SorArr(int nx_, int ny_, double x) : nx(nx_), ny(ny_), v((size_t)nx_ * ny_, x) {}
    double& operator()(int i, int j) { return v[(size_t)(i - 1) + (size_t)(j - 1) * nx]; }
};

// subroutine sor (sor_elliptic.f90:562-802); returns the iteration count
int sor(Sim& S, Level& L, SorArr& a, SorArr& b, SorArr& c, SorArr& d, SorArr& e, SorArr& f, SorArr& cg,
        SorArr& ch, SorArr& ci, SorArr& cj, SorArr& u, int imax, int jmax, double rjac, double uinf, bool robin) {
    const ollin_params& P = S.P;
    const int g = L.g;
    Arr& r = L.a("r"); Arr& z = L.a("z"); Arr& S5 = L.a("ell_S5");
    double omega = 1.0;
    SorArr aux = e;
    for (int n = 1; n <= P.ell_maxiter; ++n) {
        double anorm = 0.0;
        int isw = 1;
        for (int i = 2; i <= imax - 1; ++i)
            for (int j = 2; j <= jmax - 1; ++j) e(i, j) = aux(i, j) + S5(i - g, j - g) * p4(u(i, j));
        for (int ipass = 1; ipass <= 2; ++ipass) {
            int jsw = isw;
            for (int i = 2; i <= imax - 1; ++i) {
                for (int j = jsw + 1; j <= jmax - 1; j += 2) {
                    // the diagonal couplings g,h,i,j are zero for the flat
                    // Laplacian; for the physical one they couple points of
                    // the same colour, so the loop order matters
                    const double resid = a(i, j) * u(i + 1, j) + b(i, j) * u(i - 1, j)
                        + c(i, j) * u(i, j + 1) + d(i, j) * u(i, j - 1)
                        + cg(i, j) * u(i + 1, j + 1) + ch(i, j) * u(i - 1, j - 1)
                        + ci(i, j) * u(i + 1, j - 1) + cj(i, j) * u(i - 1, j + 1)
                        + e(i, j) * u(i, j) - f(i, j);
                    anorm = anorm + p2(resid);
                    u(i, j) = u(i, j) - omega * resid / e(i, j);
                }
                jsw = 3 - jsw;
            }
            isw = 3 - isw;
            anorm = std::sqrt(anorm / (double)(imax * jmax));
            if (n == 1 && ipass == 1) omega = 1.0 / (1.0 - 0.5 * p2(rjac));
            else omega = 1.0 / (1.0 - 0.25 * p2(rjac) * omega);
        }
        const double ganorm = anorm;
        if (robin) {
            double cr = r(imax - g, 1) / L.dr;
            for (int j = 2; j <= jmax - 1; ++j) {
                const double cz = z(1, j - g) / L.dz;
                u(imax, j) = (uinf + 0.5 * cr * (4.0 * u(imax - 1, j) - u(imax - 2, j))
                              - 0.5 * cz * (u(imax, j + 1) - u(imax, j - 1))) / (1.0 + 1.5 * cr);
            }
            double cz = z(1, jmax - g) / L.dz;
            for (int i = 2; i <= imax - 1; ++i) {
                cr = r(i - g, 1) / L.dr;
                u(i, jmax) = (uinf + 0.5 * cz * (4.0 * u(i, jmax - 1) - u(i, jmax - 2))
                              - 0.5 * cr * (u(i + 1, jmax) - u(i - 1, jmax))) / (1.0 + 1.5 * cz);
            }
            // lower z edge without equatorial symmetry (sor_elliptic.f90:724-736)
            if (!L.eqsym) {
                cz = z(1, 1 - g) / L.dz;
                for (int i = 2; i <= imax - 1; ++i) {
                    cr = r(i - g, 1) / L.dr;
                    u(i, 1) = (uinf - 0.5 * cz * (4.0 * u(i, 2) - u(i, 3))
                               - 0.5 * cr * (u(i + 1, 1) - u(i - 1, 1))) / (1.0 - 1.5 * cz);
                }
            }
            cr = r(imax - g, jmax - g) / L.dr;
            cz = z(imax - g, jmax - g) / L.dz;
            u(imax, jmax) = (uinf + 0.5 * cr * (4.0 * u(imax - 1, jmax) - u(imax - 2, jmax))
                             + 0.5 * cz * (4.0 * u(imax, jmax - 1) - u(imax, jmax - 2))) / (1.0 + 1.5 * (cr + cz));
            // lower corner (:748-756)
            if (!L.eqsym) {
                cr = r(imax - g, 1 - g) / L.dr;
                cz = z(imax - g, 1 - g) / L.dz;
                u(imax, 1) = (uinf + 0.5 * cr * (4.0 * u(imax - 1, 1) - u(imax - 2, 1))
                              - 0.5 * cz * (4.0 * u(imax, 2) - u(imax, 3))) / (1.0 + 1.5 * (cr - cz));
            }
        }
        if (L.ownaxis)
            for (int i = 1; i <= g; ++i)
                for (int j = 1; j <= jmax; ++j) u(i, j) = u(2 * g + 1 - i, j);
        if (L.eqsym && L.ownequator)
            for (int j = 1; j <= g; ++j)
                for (int i = 1; i <= imax; ++i) u(i, j) = u(i, 2 * g + 1 - j);
        if (ganorm < P.ell_epsilon) return n;
    }
    return P.ell_maxiter;
}

// sor_elliptic.f90:154-262 (coarse grid, dr*dz) and :371-448 (finer grids,
// /dr/dz): coefficients of the physical Laplacian at one point
static void sor_physical_coeffs(Level& L, int i, int j, bool fine, double& a, double& b, double& c, double& d,
                                double& e, double& cg, double& ch, double& ci, double& cj) {
    const double one = 1.0, half = 0.5, two = 2.0;
    const double dr = L.dr, dz = L.dz;
    const double gA = L.a("g_A")(i, j), gB = L.a("g_B")(i, j), gC = L.a("g_C")(i, j), r = L.a("r")(i, j);
    const double Dr_g_A = L.a("Dr_g_A")(i, j), Dz_g_C = L.a("Dz_g_C")(i, j);
    const double Dz_g_B = L.a("Dz_g_B")(i, j), Dr_g_C = L.a("Dr_g_C")(i, j);
    const double ihdet = L.a("ihdet")(i, j), Dr_hdet = L.a("Dr_hdet")(i, j), Dz_hdet = L.a("Dz_hdet")(i, j);
    const double Dr_phi = L.a("Dr_phi")(i, j), Dz_phi = L.a("Dz_phi")(i, j), psi4 = L.a("psi4")(i, j);
    a = gA * (one / dr + half / r) / dr;
    b = gA * (one / dr - half / r) / dr;
    c = gB / p2(dz);
    d = gB / p2(dz);
    e = -two * (gA / p2(dr) + gB / p2(dz));
    if (!fine) {
        cg = +0.5 * r * gC / (dr * dz);
        ch = +0.5 * r * gC / (dr * dz);
        ci = -0.5 * r * gC / (dr * dz);
        cj = -0.5 * r * gC / (dr * dz);
    } else {
        cg = +0.5 * r * gC / dr / dz;
        ch = +0.5 * r * gC / dr / dz;
        ci = -0.5 * r * gC / dr / dz;
        cj = -0.5 * r * gC / dr / dz;
    }
    a = a + half * (Dr_g_A + r * Dz_g_C) / dr;
    b = b - half * (Dr_g_A + r * Dz_g_C) / dr;
    c = c + half * (Dz_g_B + r * Dr_g_C + gC) / dz;
    d = d - half * (Dz_g_B + r * Dr_g_C + gC) / dz;
    a = a + 0.25 * ihdet * (gA * Dr_hdet + r * gC * Dz_hdet) / dr;
    b = b - 0.25 * ihdet * (gA * Dr_hdet + r * gC * Dz_hdet) / dr;
    c = c + 0.5 * gC / dz + 0.25 * ihdet * (gB * Dz_hdet + r * gC * Dr_hdet) / dz;
    d = d - 0.5 * gC / dz - 0.25 * ihdet * (gB * Dz_hdet + r * gC * Dr_hdet) / dz;
    a = a + (gA * Dr_phi + r * gC * Dz_phi) / dr;
    b = b - (gA * Dr_phi + r * gC * Dz_phi) / dr;
    c = c + (gB * Dz_phi + r * gC * Dr_phi) / dz;
    d = d - (gB * Dz_phi + r * gC * Dr_phi) / dz;
    a = a / psi4; b = b / psi4; c = c / psi4; d = d / psi4; e = e / psi4;
    cg = cg / psi4; ch = ch / psi4; ci = ci / psi4; cj = cj / psi4;
}

void sor_elliptic(Sim& S, bool physical) {
    const ollin_params& P = S.P;
    const int nlev = (int)S.L.size();
    for (Level& L : S.L)
        for (double& x : L.a("ell_u").v) x = 1.0;
    g_ell_stats = EllStats();
    // Jacobi spectral radius (sor_elliptic.f90:126-128) from the grid that is
    // current on entry: the last box's last level (the loop of :87-110
    // leaves it current); for Nb = 0 every grid has box 0's dimensions
    const Level& Lg = S.L[nlev - 1];
    const double rjac = (Lg.dz / Lg.dr * std::cos(kPi / (double)(Lg.Nr + Lg.g))
                         + Lg.dr / Lg.dz * std::cos(kPi / (double)(Lg.Nz + Lg.g))) / (Lg.dz / Lg.dr + Lg.dr / Lg.dz);
    auto solve_level = [&](int level, bool robin) {
        Level& L = S.L[level];
        const int g = L.g;
        const int imax = L.Nr + g, jmax = L.Nz + g;
        SorArr a(imax, jmax, 0.0), b(imax, jmax, 0.0), c(imax, jmax, 0.0), d(imax, jmax, 0.0), e(imax, jmax, 1.0),
            f(imax, jmax, 0.0), u(imax, jmax, 0.0);
        SorArr cg(imax, jmax, 0.0), ch(imax, jmax, 0.0), ci(imax, jmax, 0.0), cj(imax, jmax, 0.0);
        Arr& r = L.a("r"); Arr& S1 = L.a("ell_S1"); Arr& S0 = L.a("ell_S0"); Arr& eu = L.a("ell_u");
        const double one = 1.0, half = 0.5, two = 2.0;
        const double dr = L.dr, dz = L.dz;
        for (int i = 1 - g; i <= L.Nr; ++i)
            for (int j = 1 - g; j <= L.Nz; ++j) {
                u(i + g, j + g) = eu(i, j);
                if (!physical) {
                    a(i + g, j + g) = (one / dr + half / r(i, j)) / dr;
                    b(i + g, j + g) = (one / dr - half / r(i, j)) / dr;
                    c(i + g, j + g) = one / p2(dz);
                    d(i + g, j + g) = one / p2(dz);
                    e(i + g, j + g) = -two * (one / p2(dr) + one / p2(dz)) + S1(i, j);
                } else {
                    sor_physical_coeffs(L, i, j, L.level > 0, a(i + g, j + g), b(i + g, j + g), c(i + g, j + g),
                                        d(i + g, j + g), e(i + g, j + g), cg(i + g, j + g), ch(i + g, j + g),
                                        ci(i + g, j + g), cj(i + g, j + g));
                    e(i + g, j + g) = e(i + g, j + g) + S1(i, j);
                }
                f(i + g, j + g) = S0(i, j);
            }
        const int n = sor(S, L, a, b, c, d, e, f, cg, ch, ci, cj, u, imax, jmax, rjac, 1.0, robin);
        for (int i = 1 - g; i <= L.Nr; ++i)
            for (int j = 1 - g; j <= L.Nz; ++j) eu(i, j) = u(i + g, j + g);
        return n;
    };
    g_ell_stats.steps[0] = solve_level(0, true);
    g_ell_stats.phases = 1;
    const auto evolved_ext = S.evolved;
    S.evolved = {{"ell_u", +1, +1}};
    // sor_elliptic.f90:293-491: every box, levels 1..Nl(box) in order (the
    // grid list's order), each started and bounded by interpolation from its
    // parent (box 0's level 0 for level 1, else the box's own coarser level)
    for (int gid = 1; gid < nlev; ++gid) {
        Level& F = S.L[gid];
        const int level = F.level;
        Arr& r = F.a("r"); Arr& z = F.a("z"); Arr& u = F.a("ell_u");
        for (int m = 0; m <= F.Nr + F.g - 1; ++m)
            for (int n = 0; n <= F.Nz + F.g - 1; ++n) {
                const double r0 = S.rminl[gid] + (double)m * S.drl[level];
                const double z0 = S.zminl[gid] + (double)n * S.dzl[level];
                const int i = (int)nint_((r0 - r(1 - F.g, 0)) / S.drl[level]) + 1 - F.g;
                const int j = (int)nint_((z0 - z(0, 1 - F.g)) / S.dzl[level]) + 1 - F.g;
                const bool flag1 = (i >= 1 - F.g) && (i <= F.Nr) && (j >= 1 - F.g) && (j <= F.Nz);
                const double aux1 = interp(S, F.parent, S.L[F.parent].a("ell_u"), r0, z0);
                if (flag1) u(i, j) = aux1;
            }
        const int n = solve_level(gid, false);
        if (gid == 1) g_ell_stats.steps[1] = n;
        g_ell_stats.phases = 2;
    }
    // :497-521: restriction in the same order (level 1 into level 0 first)
    for (int gid = 1; gid < nlev; ++gid) restrict_(S, gid);
    S.evolved = evolved_ext;
}

void ell_solve(Sim& S) {
    if (S.P.ell_solver == OLLIN_ELL_WAVE) wave_elliptic(S, false, nullptr);
    else if (S.P.ell_solver == OLLIN_ELL_SOR) sor_elliptic(S, false);
    else throw std::runtime_error("elliptic initial data needs ELL_solver = wave or sor");
}

// psi = ell_u and the derived conformal factors (idata_scalarpulse.f90:225-240,
// idata_brillwave.f90:200-215)
void psi_from_solution(Sim& S) {
    for (Level& L : S.L) {
        Arr& u = L.a("ell_u");
        Arr& psi = L.a("psi"); Arr& psi2 = L.a("psi2"); Arr& psi4 = L.a("psi4");
        Arr& phi = L.a("phi"); Arr& chi = L.a("chi");
        for (size_t q = 0; q < u.v.size(); ++q) {
            psi.v[q] = u.v[q];
            psi2.v[q] = p2(psi.v[q]);
            psi4.v[q] = p4(psi.v[q]);
            phi.v[q] = std::log(psi.v[q]);
            chi.v[q] = 1.0 / std::pow(psi.v[q], (double)S.P.chipower);
        }
    }
}

}  // namespace

// idata_scalarpulse.f90:46-244
void idata_scalarpulse(Sim& S) {
    const ollin_params& P = S.P;
    const double zero = 0.0, one = 1.0, two = 2.0;
    const double a0 = P.scalar_a0, r0 = P.scalar_r0, z0 = P.scalar_z0, sr0 = P.scalar_sr0, sz0 = P.scalar_sz0;
    for (Level& L : S.L) {
        currentgrid(S, L);
        const int g = L.g;
        Arr& r = L.a("r"); Arr& z = L.a("z"); Arr& rr = L.a("rr");
        Arr& sphi = L.a("scalar_phi");
        for (int j = 1 - g; j <= L.Nz; ++j)
            for (int i = 1 - g; i <= L.Nr; ++i) {
                const double R = r(i, j), Z = z(i, j), RR = rr(i, j);
                double v = 0.0;
                if (P.scalarpulse_type == OLLIN_PULSE_SHELL) {
                    if (r0 == zero && z0 == zero) {
                        v = a0 * std::exp(-(p2(R) / p2(sr0) + p2(Z) / p2(sz0)));
                    } else {
                        const double cen = (p2(R) * r0 + p2(Z) * z0) / p2(RR);
                        const double den = p2(R) * p2(sr0) + p2(Z) * p2(sz0);
                        v = a0 * (std::exp(-(p2(RR - cen) * p2(RR) / den)) + std::exp(-(p2(RR + cen) * p2(RR) / den)));
                    }
                } else if (P.scalarpulse_type == OLLIN_PULSE_TORUS) {
                    if (r0 == zero && z0 == zero) {
                        v = a0 * std::exp(-p2(R / sr0)) * std::exp(-p2(Z / sz0));
                    } else if (L.eqsym) {
                        v = a0 * (std::exp(-p2((R - r0) / sr0)) + std::exp(-p2((R + r0) / sr0)))
                            * (std::exp(-p2((Z - z0) / sz0)) + std::exp(-p2((Z + z0) / sz0)));
                    } else {
                        v = a0 * std::exp(-p2((Z - z0) / sz0)) * (std::exp(-p2((R - r0) / sr0)) + std::exp(-p2((R + r0) / sr0)));
                    }
                } else {
                    v = a0 * std::exp(-(p2(R) + (one - sz0) * p2(Z)));
                }
                sphi(i, j) = v;
            }
        diff1r(L, sphi, L.a("scalar_xi_r"), +1);
        diff1z(L, sphi, L.a("scalar_xi_z"), +1);
        for (double& x : L.a("scalar_pi").v) x = zero;
        potential(S, L);
    }
    for (Level& L : S.L) {
        Arr& xr = L.a("scalar_xi_r"); Arr& xz = L.a("scalar_xi_z"); Arr& V = L.a("scalar_V");
        Arr& S0 = L.a("ell_S0"); Arr& S1 = L.a("ell_S1"); Arr& S5 = L.a("ell_S5");
        for (size_t q = 0; q < S0.v.size(); ++q) {
            S0.v[q] = zero;
            S1.v[q] = kPi * (p2(xr.v[q]) + p2(xz.v[q]));
            S5.v[q] = (P.scalarpotential == OLLIN_POTENTIAL_NONE) ? zero : two * kPi * V.v[q];
        }
    }
    ell_solve(S);
    psi_from_solution(S);
}

// idata_brillwave.f90:60-229 (brilltype = "Holz")
void idata_brillwave(Sim& S) {
    const ollin_params& P = S.P;
    const double zero = 0.0, half = 0.5, one = 1.0, two = 2.0;
    if (P.ell_solver == OLLIN_ELL_NONE) throw std::runtime_error("For Brill wave data you need an elliptic solver");
    const double a0 = P.brill_a0, sr0 = P.brill_sr0, sz0 = P.brill_sz0;
    for (Level& L : S.L) {
        currentgrid(S, L);
        Arr& r = L.a("r"); Arr& z = L.a("z");
        Arr& q = L.a("brillq");
        Arr& S0 = L.a("ell_S0"); Arr& S1 = L.a("ell_S1"); Arr& S5 = L.a("ell_S5");
        for (size_t k = 0; k < q.v.size(); ++k) {
            const double R = r.v[k], Z = z.v[k];
            q.v[k] = a0 * p2(R) * std::exp(-p2(R / sr0) - p2(Z / sz0));
            S1.v[k] = half * q.v[k] * (one / p2(R) + two * (p2(R / p2(sr0)) + p2(Z / p2(sz0))) - 5.0 / p2(sr0) - one / p2(sz0));
            S0.v[k] = zero;
            S5.v[k] = zero;
        }
    }
    ell_solve(S);
    psi_from_solution(S);
    for (Level& L : S.L) {
        Arr& q = L.a("brillq"); Arr& r = L.a("r");
        Arr& A = L.a("A"); Arr& B = L.a("B"); Arr& C = L.a("C"); Arr& H = L.a("H");
        Arr& lam = L.a("lambda"); Arr& Dr_ = L.a("Delta_r"); Arr& Dz_ = L.a("Delta_z");
        for (size_t k = 0; k < q.v.size(); ++k) {
            A.v[k] = std::exp(two * q.v[k]);
            B.v[k] = A.v[k];
            C.v[k] = 0.0;
            H.v[k] = 1.0;
            lam.v[k] = (A.v[k] - H.v[k]) / p2(r.v[k]);
            Dr_.v[k] = (one - one / A.v[k]) / r.v[k];
            Dz_.v[k] = zero;
        }
    }
}

// maximalslicing.f90:3-175: lap(alpha) = (K_ij K^ij + 4 pi (rho + S)) alpha
// with the physical Laplacian, alpha -> 1 far away; then the lapse
// derivatives that ``auxiliary`` would give, and nothing else (the other
// auxiliary quantities of the lapse keep the values of the last
// ``auxiliary`` call)
void maximalslicing(Sim& S, const double* va_max) {
    const ollin_params& P = S.P;
    const double zero = 0.0, smallpi = std::acos(-1.0);
    for (Level& L : S.L) {
        currentgrid(S, L);
        Arr& S0 = L.a("ell_S0"); Arr& S1 = L.a("ell_S1"); Arr& S5 = L.a("ell_S5"); Arr& K2 = L.a("K2");
        for (size_t k = 0; k < S0.v.size(); ++k) {
            S0.v[k] = zero;
            S5.v[k] = zero;
            S1.v[k] = -K2.v[k];
        }
        if (P.mattertype != OLLIN_MATTER_VACUUM) {
            Arr& rho = L.a("rho"); Arr& trS = L.a("trS");
            for (size_t k = 0; k < S1.v.size(); ++k) S1.v[k] = S1.v[k] - 4.0 * smallpi * (rho.v[k] + trS.v[k]);
        }
    }
    if (P.ell_solver == OLLIN_ELL_WAVE) wave_elliptic(S, true, va_max);
    else if (P.ell_solver == OLLIN_ELL_SOR) sor_elliptic(S, true);
    else throw std::runtime_error("maximal slicing needs ELL_solver = wave or sor");
    for (Level& L : S.L) L.a("alpha").v = L.a("ell_u").v;
    for (Level& L : S.L) {
        currentgrid(S, L);
        Arr& alpha = L.a("alpha"); Arr& Dr_alpha = L.a("Dr_alpha"); Arr& r = L.a("r"); Arr& aux = L.a("auxarray");
        diff1r(L, alpha, Dr_alpha, +1);
        diff1z(L, alpha, L.a("Dz_alpha"), +1);
        diff2r(L, alpha, L.a("Drr_alpha"), +1);
        diff2z(L, alpha, L.a("Dzz_alpha"), +1);
        diff2rz(L, alpha, L.a("Drz_alpha"), +1, +1);
        for (size_t k = 0; k < aux.v.size(); ++k) aux.v[k] = Dr_alpha.v[k] / r.v[k];
        diff1r(L, aux, L.a("DD_alphar"), +1);
    }
}

}  // namespace oracle
