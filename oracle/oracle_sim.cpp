// ORACLE -- test infrastructure only.  CPU restatement of the OllinAxis-BiB
// evolution path used to check the GB300 library; never linked into it.
//
// This file restates the time stepper and the mesh-refinement transfer:
//   src/base/onestep.f90 (recursive Berger-Oliger step, RK4/ICN stages),
//   the Perl-generated saveold/accumulate/update/symmetries_r/symmetries_z
//   (prl/arrays.pl:134-218), src/base/finebound.f90 with bound_interp.inc,
//   src/base/restrict.f90 with restrict_interp.inc, src/base/interp.f90,
//   the box-0 bookkeeping of main.f90/setupboxes.f90/evolve.f90:42-219,
//   initial data of src/base/initial.f90:59-218,528-645, and the 0-D norms
//   of src/base/save0Ddata.f90:221-288,370-374.
// It exposes a C API (ollin_oracle.h) with the same parameter struct as the
// GPU library so that one harness drives both.
#include <omp.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <stdexcept>

#include "oracle_sim.h"
#include "ollin_oracle.h"

namespace oracle {

// ---------------------------------------------------------------------------
// bookkeeping
// ---------------------------------------------------------------------------
static void setup(Sim& S) {
    const ollin_params& P = S.P;
    if (P.order != 4 && P.order != 2) throw std::runtime_error("oracle: order must be two or four");
    if (P.chipower != 2 || !P.chimethod) throw std::runtime_error("oracle: chimethod with chipower 2 only");
    if (!P.lagrangian || !P.factorhdet || !P.evolveH) throw std::runtime_error("oracle: lagrangian+factorhdet+evolveH only");
    if (P.evolveKTH) throw std::runtime_error("oracle: evolveKTH unsupported");
    // main.f90:286-318: 2 ghost zones for order two, 3 for order four, or
    // the par file's number when it is not smaller
    const int gmin = P.order == 2 ? 2 : 3;
    S.g = std::max(P.ghost, gmin);
    const int g = S.g;
    // setupboxes.f90:25-80: boxes and their levels
    if (P.nb < 0 || P.nb > 3) throw std::runtime_error("The number of refinement boxes must be between 0 and 3");
    S.Nb = P.nb;
    S.Nl[0] = P.nl0;
    for (int b = 1; b <= 3; ++b) S.Nl[b] = P.nl[b - 1];
    S.Nlmax = 0;
    for (int b = 0; b <= 3; ++b) S.Nlmax = std::max(S.Nlmax, S.Nl[b]);
    if (S.Nb > 0 && S.Nlmax == 0) throw std::runtime_error("If you choose Nb>0 you must also have Nl>0 for at least one box");
    const int L = S.Nlmax;
    const double dt0 = P.dtfac * std::min(P.dr0, P.dz0);
    S.dtl.resize(L + 1); S.drl.resize(L + 1); S.dzl.resize(L + 1);
    for (int l = 0; l <= L; ++l) {  // setupboxes.f90:121-125
        S.dtl[l] = dt0 / (double)(1 << l);
        S.drl[l] = P.dr0 / (double)(1 << l);
        S.dzl[l] = P.dz0 / (double)(1 << l);
    }
    // box sizes and centres (setupboxes.f90:131-206)
    int Nrbox[4], Nzbox[4];
    Nrbox[0] = P.nrtotal;
    Nzbox[0] = P.nztotal;
    if (!P.eqsym && (Nzbox[0] + g) % 2 == 0) Nzbox[0] += 1;
    for (int b = 1; b <= 3; ++b) { Nrbox[b] = P.nrbox[b - 1]; Nzbox[b] = P.nzbox[b - 1]; }
    for (int b = 0; b <= S.Nb; ++b)
        if (Nrbox[b] < 2 + g || Nzbox[b] < 2 + g)
            throw std::runtime_error("The values of (Nrtotal,Nztotal,Nrbox,Nzbox) should be greater than 2 plus the number of ghost zones");
    S.rbox[0] = 0.0; S.zbox[0] = 0.0;
    for (int b = 1; b <= 3; ++b) { S.rbox[b] = P.rbox[b - 1]; S.zbox[b] = P.zbox[b - 1]; }
    for (int b = 1; b <= S.Nb; ++b) {
        const double d1r = S.drl[std::min(1, L)], d1z = S.dzl[std::min(1, L)];
        if (S.rbox[b] != 0.0) S.rbox[b] = ((double)(long)(S.rbox[b] / d1r) + 0.5) * d1r;
        if (S.zbox[b] != 0.0) {
            if (P.eqsym) S.zbox[b] = ((double)(long)(S.zbox[b] / d1z) + 0.5) * d1z;
            else S.zbox[b] = (double)(long)(S.zbox[b] / d1z) * d1z;
        }
    }
    for (int b = 1; b <= S.Nb; ++b) {  // setupboxes.f90:210-285
        const double d1r = S.drl[std::min(1, L)], d1z = S.dzl[std::min(1, L)];
        if (S.rbox[b] < 0.0) throw std::runtime_error("rbox must be larger than or equal to 0 for all refinement boxes");
        if (S.rbox[b] > 0.0 && S.rbox[b] - 0.5 * Nrbox[b] * d1r <= 0.0)
            throw std::runtime_error("Refinement box extends to negative values of r");
        if (S.rbox[b] + 0.5 * Nrbox[b] * d1r >= (Nrbox[0] - g) * P.dr0)
            throw std::runtime_error("Refinement box extends beyond base grid in r direction");
        if (P.eqsym) {
            if (S.zbox[b] < 0.0) throw std::runtime_error("For equatorial symmetry zbox must be larger than or equal to 0");
            if (S.zbox[b] > 0.0 && S.zbox[b] - 0.5 * Nzbox[b] * d1z <= 0.0)
                throw std::runtime_error("Refinement box extends to negative values of z");
            if (S.zbox[b] + 0.5 * Nzbox[b] * d1z >= (Nzbox[0] - g) * P.dz0)
                throw std::runtime_error("Refinement box extends beyond base grid in z direction");
        } else {
            if (S.zbox[b] - 0.5 * Nzbox[b] * d1z <= -0.5 * (Nzbox[0] - g) * P.dz0 ||
                S.zbox[b] + 0.5 * Nzbox[b] * d1z >= 0.5 * (Nzbox[0] - g) * P.dz0)
                throw std::runtime_error("Refinement box extends beyond base grid in z direction");
        }
    }
    // grids: box 0 levels 0..Nl0, then boxes 1..Nb levels 1..Nl(b)
    std::vector<std::pair<int, int>> grids;
    for (int l = 0; l <= S.Nl[0]; ++l) grids.push_back({0, l});
    for (int b = 1; b <= S.Nb; ++b)
        for (int l = 1; l <= S.Nl[b]; ++l) grids.push_back({b, l});
    const int ng = (int)grids.size();
    S.t.assign(ng, 0.0); S.t1.assign(ng, 0.0); S.t2.assign(ng, 0.0); S.s.assign(ng, 0);
    S.rminl.resize(ng); S.rmaxl.resize(ng); S.zminl.resize(ng); S.zmaxl.resize(ng);
    S.L.resize(ng);
    for (int k = 0; k < ng; ++k) {
        const int b = grids[k].first, l = grids[k].second;
        Level& lv = S.L[k];
        lv.gid = k;
        lv.level = l; lv.box = b; lv.g = g; lv.order = P.order; lv.Nr = Nrbox[b]; lv.Nz = Nzbox[b];
        // finebound/restrict partner: level 1 of any box talks to the base grid
        lv.parent = -1;
        if (l > 0) {
            const int pb = (l == 1) ? 0 : b;
            for (int q = 0; q < ng; ++q)
                if (grids[q].first == pb && grids[q].second == l - 1) lv.parent = q;
        }
        lv.dr = S.drl[l]; lv.dz = S.dzl[l]; lv.dt = S.dtl[l];
        lv.eqsym = P.eqsym != 0;
        lv.ownaxis = S.rbox[b] == 0.0;                         // main.f90:393-403
        lv.ownequator = P.eqsym != 0 && S.zbox[b] == 0.0;      // main.f90:412-424
        Arr& r = lv.a("r"); Arr& z = lv.a("z"); Arr& rr = lv.a("rr");
        for (int j = 1 - g; j <= lv.Nz; ++j)
            for (int i = 1 - g; i <= lv.Nr; ++i) {  // evolve.f90:42-70
                if (S.rbox[b] == 0.0) r(i, j) = ((double)(0 + i) - 0.5) * lv.dr;
                else r(i, j) = S.rbox[b] + ((double)(0 + i) - 0.5 * (double)(lv.Nr - g + 1)) * lv.dr;
                if (P.eqsym && S.zbox[b] == 0.0) z(i, j) = ((double)(0 + j) - 0.5) * lv.dz;
                else z(i, j) = S.zbox[b] + ((double)(0 + j) - 0.5 * (double)(lv.Nz - g + 1)) * lv.dz;
            }
        for (int j = 1 - g; j <= lv.Nz; ++j)
            for (int i = 1 - g; i <= lv.Nr; ++i) rr(i, j) = std::sqrt(p2(r(i, j)) + p2(z(i, j)));
        S.rminl[k] = r(1 - g, 0);
        S.rmaxl[k] = r(lv.Nr, 0);
        S.zminl[k] = z(0, 1 - g);
        S.zmaxl[k] = z(0, lv.Nz);
    }
    // EVOLVE arrays in generated update.f90 order, with their parity tags
    // (src/base/arrays.config:154-1045)
    auto add = [&](const char* n, int sr, int sz) { S.evolved.push_back({n, sr, sz}); };
    const bool shift = P.shift != OLLIN_SHIFT_NONE;
    add("alpha", +1, +1); add("dtalpha", +1, +1);
    if (shift) { add("beta_r", -1, +1); add("beta_z", +1, -1); add("dtbeta_r", -1, +1); add("dtbeta_z", +1, -1); add("fdriver", +1, +1); }
    add("phi", +1, +1); add("dtphi", +1, +1); add("chi", +1, +1);
    add("A", +1, +1); add("B", +1, +1); add("H", +1, +1); add("C", +1, -1);
    add("trK", +1, +1); add("KTA", +1, +1); add("KTB", +1, +1); add("KTH", +1, +1); add("KTC", +1, -1);
    add("Delta_r", -1, +1); add("Delta_z", +1, -1);
    add("lambda", +1, +1); add("Alambda", +1, +1);
    add("V_r", -1, +1); add("V_z", +1, -1); add("z4theta", +1, +1);
    if (P.mattertype == OLLIN_MATTER_SCALAR) {
        add("scalar_phi", +1, +1); add("scalar_xi_r", -1, +1); add("scalar_xi_z", +1, -1); add("scalar_pi", +1, +1);
    }
    for (Level& lv : S.L)
        for (const EvolvedVar& e : S.evolved) {
            lv.a(e.name); lv.a(e.name + "_p"); lv.a(e.name + "_a"); lv.a("s" + e.name);
            const size_t nr_hist = (size_t)g * (lv.Nz + g) * 3, nz_hist = (size_t)(lv.Nr + g) * g * 3;
            lv.hist[e.name + "_rL"].assign(nr_hist, 0.0);
            lv.hist[e.name + "_rR"].assign(nr_hist, 0.0);
            lv.hist[e.name + "_zL"].assign(nz_hist, 0.0);
            lv.hist[e.name + "_zR"].assign(nz_hist, 0.0);
        }
}

// flat offsets of the history arrays: rX(m, j, k) with m in 0:g-1,
// j in 1-g:Nz, k in 0:2; zX(i, n, k) with i in 1-g:Nr, n in 0:g-1
static inline size_t hr(const Level& L, int m, int j, int k) { return (size_t)m + (size_t)L.g * ((size_t)(j - 1 + L.g) + (size_t)(L.Nz + L.g) * k); }
static inline size_t hz(const Level& L, int i, int n, int k) { return (size_t)(i - 1 + L.g) + (size_t)(L.Nr + L.g) * ((size_t)n + (size_t)L.g * k); }

void currentgrid(Sim& S, Level& L) { L.time = S.t[L.gid]; }

// ---------------------------------------------------------------------------
// generated per-array routines
// ---------------------------------------------------------------------------
void saveold(Sim& S, Level& L) {
    const int g = L.g, Nr = L.Nr, Nz = L.Nz;
    for (const EvolvedVar& e : S.evolved) {
        Arr& v = L.a(e.name);
        L.a(e.name + "_p") = v;
        auto& rL = L.hist[e.name + "_rL"]; auto& rR = L.hist[e.name + "_rR"];
        auto& zL = L.hist[e.name + "_zL"]; auto& zR = L.hist[e.name + "_zR"];
        if (rL.empty()) {  // a variable evolved only here (the elliptic solver's ell_u, ell_v)
            const size_t nr_hist = (size_t)g * (Nz + g) * 3, nz_hist = (size_t)(Nr + g) * g * 3;
            rL.assign(nr_hist, 0.0); rR.assign(nr_hist, 0.0); zL.assign(nz_hist, 0.0); zR.assign(nz_hist, 0.0);
        }
        for (int i = 0; i <= g - 1; ++i) {
            for (int j = 1 - g; j <= Nz; ++j) {
                rL[hr(L, i, j, 2)] = rL[hr(L, i, j, 1)]; rL[hr(L, i, j, 1)] = rL[hr(L, i, j, 0)]; rL[hr(L, i, j, 0)] = v(1 - g + i, j);
                rR[hr(L, i, j, 2)] = rR[hr(L, i, j, 1)]; rR[hr(L, i, j, 1)] = rR[hr(L, i, j, 0)]; rR[hr(L, i, j, 0)] = v(Nr - i, j);
            }
            for (int ii = 1 - g; ii <= Nr; ++ii) {
                zL[hz(L, ii, i, 2)] = zL[hz(L, ii, i, 1)]; zL[hz(L, ii, i, 1)] = zL[hz(L, ii, i, 0)]; zL[hz(L, ii, i, 0)] = v(ii, 1 - g + i);
                zR[hz(L, ii, i, 2)] = zR[hz(L, ii, i, 1)]; zR[hz(L, ii, i, 1)] = zR[hz(L, ii, i, 0)]; zR[hz(L, ii, i, 0)] = v(ii, Nz - i);
            }
        }
    }
}

void accumulate(Sim& S, Level& L, int k, int niter, double w) {
    const bool first = (k == 1), last = (k == niter);
    for (const EvolvedVar& e : S.evolved) {
        Arr& a = L.a(e.name + "_a"); Arr& s = L.a("s" + e.name);
        const size_t n = a.v.size();
        double* av = a.v.data();
        double* sv = s.v.data();
        if (!last) {
            if (first) {
#pragma omp parallel for schedule(static)
                for (size_t q = 0; q < n; ++q) av[q] = w * sv[q];
            } else {
#pragma omp parallel for schedule(static)
                for (size_t q = 0; q < n; ++q) av[q] = av[q] + w * sv[q];
            }
        } else {
#pragma omp parallel for schedule(static)
            for (size_t q = 0; q < n; ++q) sv[q] = av[q] + w * sv[q];
        }
    }
}

// generated simpleboundary.f90 (prl/arrays.pl:880-905): on level 0, the
// sources of every EVOLVE array not declared NOBOUND (src/base/arrays.config)
// on the outer edges i = Nr, j = Nz and, without equatorial symmetry, the
// lower edge j = 1-ghost: zero ("static"), or the source of the row or column
// inside ("flat"), the r edge first
void simpleboundary(Sim& S, Level& L) {
    static const char* nobound[] = {"alpha", "beta_r", "beta_z", "phi", "dtphi", "chi", "A", "B", "H", "C", "lambda",
                                    "scalar_phi", "scalar_xi_r", "scalar_xi_z"};
    const bool flat = S.P.boundtype == OLLIN_BOUND_FLAT;
    const int g = L.g, Nr = L.Nr, Nz = L.Nz;
    for (const EvolvedVar& e : S.evolved) {
        bool skip = false;
        for (const char* n : nobound) skip = skip || e.name == n;
        if (skip) continue;
        Arr& s = L.a("s" + e.name);
        for (int j = 1 - g; j <= Nz; ++j) s(Nr, j) = flat ? s(Nr - 1, j) : 0.0;
        for (int i = 1 - g; i <= Nr; ++i) s(i, Nz) = flat ? s(i, Nz - 1) : 0.0;
        if (!S.P.eqsym)
            for (int i = 1 - g; i <= Nr; ++i) s(i, 1 - g) = flat ? s(i, 2 - g) : 0.0;
    }
}

void update(Sim& S, Level& L, double dtw) {
    for (const EvolvedVar& e : S.evolved) {
        Arr& v = L.a(e.name); Arr& vp = L.a(e.name + "_p"); Arr& s = L.a("s" + e.name);
        const size_t n = v.v.size();
        double* vv = v.v.data();
        const double* pv = vp.v.data();
        const double* sv = s.v.data();
#pragma omp parallel for schedule(static)
        for (size_t q = 0; q < n; ++q) vv[q] = pv[q] + dtw * sv[q];
    }
}

void symmetries_r(Sim& S, Level& L) {
    for (const EvolvedVar& e : S.evolved) {
        Arr& v = L.a(e.name);
        for (int i = 1; i <= L.g; ++i)
            for (int j = 1 - L.g; j <= L.Nz; ++j) v(1 - i, j) = e.symr * v(i, j);
    }
}

void symmetries_z(Sim& S, Level& L) {
    for (const EvolvedVar& e : S.evolved) {
        Arr& v = L.a(e.name);
        for (int j = 1; j <= L.g; ++j)
            for (int i = 1 - L.g; i <= L.Nr; ++i) v(i, 1 - j) = e.symz * v(i, j);
    }
}

// ---------------------------------------------------------------------------
// interp.f90:2-270 -- value of one grid function of grid ``gid`` (a box and
// level) at (r0,z0)
// ---------------------------------------------------------------------------
// The interpolation itself, with the grid's coordinate arrays already
// resolved (no map lookups: safe inside the parallel loops below); returns
// false when (r0, z0) lies outside the grid.
static bool interp_at(const Sim& S, int gid, const Arr& r, const Arr& z, const Arr& var, double r0, double z0,
                      double* out) {
    const Level& L = S.L[gid];
    const int g = L.g;
    const int level = L.level;
    const double small = 1.0e-10;
    const double rmin = S.rminl[gid] - small, rmax = S.rmaxl[gid];
    const double zmin = S.zminl[gid] - small, zmax = S.zmaxl[gid];
    if (r0 < rmin || r0 > rmax || z0 < zmin || z0 > zmax) return false;
    const int i0 = (int)((r0 - r(1 - g, 0)) / S.drl[level]) + 1 - g;
    const double deltar = r0 - r(i0, 0);
    const int j0 = (int)((z0 - z(0, 1 - g)) / S.dzl[level]) + 1 - g;
    const double deltaz = z0 - z(0, j0);
    if (deltar == 0.0 && deltaz == 0.0) { *out = var(i0, j0); return true; }
    const bool forcelinear = ((S.rmaxl[gid] - r0) < S.drl[level]) || ((S.zmaxl[gid] - z0) < S.dzl[level])
        || ((r0 - S.rminl[gid]) < S.drl[level]) || ((z0 - S.zminl[gid]) < S.dzl[level]);
    double fa[4][4];
    if (forcelinear) {
        for (int i = 0; i <= 1; ++i)
            for (int j = 0; j <= 1; ++j) fa[i + 1][j + 1] = var(i0 + i, j0 + j);
    } else {
        for (int i = -1; i <= 2; ++i)
            for (int j = -1; j <= 2; ++j) fa[i + 1][j + 1] = var(i0 + i, j0 + j);
    }
    const double auxr = deltar / S.drl[level];
    const double auxz = deltaz / S.dzl[level];
    if (!S.P.interp_bicubic || forcelinear) {
        *out = fa[1][1] * (1.0 - auxr) * (1.0 - auxz) + fa[2][1] * auxr * (1.0 - auxz)
            + fa[1][2] * (1.0 - auxr) * auxz + fa[2][2] * auxr * auxz;
        return true;
    }
    double res = 0.0;
    for (int i = -1; i <= 2; ++i)
        for (int j = -1; j <= 2; ++j) {
            double aux = 1.0;
            for (int m = -1; m <= 2; ++m) {
                if (m == i) continue;
                aux = aux * (auxr - (double)m) / (double)(i - m);
            }
            for (int n = -1; n <= 2; ++n) {
                if (n == j) continue;
                aux = aux * (auxz - (double)n) / (double)(j - n);
            }
            res = res + aux * fa[i + 1][j + 1];
        }
    *out = res;
    return true;
}

double interp(Sim& S, int gid, const Arr& var, double r0, double z0) {
    Level& L = S.L[gid];
    double v = 0.0;
    if (!interp_at(S, gid, L.a("r"), L.a("z"), var, r0, z0, &v))
        throw std::runtime_error("interp: interpolating point is outside the local grid");
    return v;
}

// ---------------------------------------------------------------------------
// finebound.f90:2-407 (all=.true.) with the generated bound_interp.inc, for
// grid ``gid`` from its parent (box 0's level 0 for level 1)
// ---------------------------------------------------------------------------
void finebound(Sim& S, int gid, double dtw) {
    Level& F = S.L[gid];
    const int g = F.g;
    const int level = F.level;
    const int pg = F.parent;
    const double tp = S.t[pg], t0 = S.t[gid], tm1 = S.t1[gid];
    const double tl = t0 + dtw;
    const int imax = (tp == tl) ? g + 2 : g - 1;
    const int jmax = imax;
    const int border = (tm1 == 0.0) ? 1 : 2;
    Arr& r = F.a("r"); Arr& z = F.a("z");
    Level& Cl = S.L[pg];
    const Arr& rc = Cl.a("r");
    const Arr& zc = Cl.a("z");
    // every array the strips touch, resolved once (the point loops below run
    // in parallel and must not touch the name maps)
    struct VarRefs {
        Arr* fine; const Arr* coarse; const Arr* vp;
        const std::vector<double>* h[4];  // rR, rL, zR, zL
    };
    std::vector<VarRefs> vars;
    for (const EvolvedVar& e : S.evolved) {
        VarRefs x{};
        x.fine = &F.a(e.name);
        x.coarse = &Cl.a(e.name);
        x.vp = &F.a(e.name + "_p");
        const char* sfx[4] = {"_rR", "_rL", "_zR", "_zL"};
        for (int k = 0; k < 4; ++k) {
            auto it = F.hist.find(e.name + sfx[k]);
            x.h[k] = it == F.hist.end() ? nullptr : &it->second;
        }
        vars.push_back(x);
    }
    int outside = 0;

    // one strip point: all evolving variables (bound_interp.inc); bd is the
    // strip: 'R' (rR), 'L' (rL), 'z' (zR), 'l' (zL)
    auto point = [&](double r0, double z0, int m, int n, char bd) {
        const int ii = (int)nint_((r0 - r(1 - g, 0)) / S.drl[level]) + 1 - g;
        const int jj = (int)nint_((z0 - z(0, 1 - g)) / S.dzl[level]) + 1 - g;
        const bool flag1 = (ii >= 1 - g) && (ii <= F.Nr) && (jj >= 1 - g) && (jj <= F.Nz);
        for (const VarRefs& x : vars) {
            double aux2 = 0.0;
            if (!interp_at(S, pg, rc, zc, *x.coarse, r0, z0, &aux2)) {
#pragma omp atomic write
                outside = 1;
                return;
            }
            if (!flag1) continue;
            Arr& v = *x.fine;
            if (border == 1) {
                v(ii, jj) = (tl - t0) / (tp - t0) * aux2 + (tl - tp) / (t0 - tp) * (*x.vp)(ii, jj);
            } else {
                // history terms; an index beyond the declared history depth
                // (m or n > ghost-1, reachable only when tp == tl) carries a
                // zero weight in the reference and contributes nothing here
                double h0 = 0.0, h1 = 0.0;
                if (bd == 'R' || bd == 'L') {
                    if (m <= g - 1) {
                        const auto& H = *x.h[bd == 'R' ? 0 : 1];
                        h0 = H[hr(F, m, jj, 0)]; h1 = H[hr(F, m, jj, 1)];
                    }
                } else {
                    if (n <= g - 1) {
                        const auto& H = *x.h[bd == 'z' ? 2 : 3];
                        h0 = H[hz(F, ii, n, 0)]; h1 = H[hz(F, ii, n, 1)];
                    }
                }
                v(ii, jj) = (tl - t0) * (tl - tm1) / ((tp - t0) * (tp - tm1)) * aux2
                    + (tl - tp) * (tl - tm1) / ((t0 - tp) * (t0 - tm1)) * h0
                    + (tl - tp) * (tl - t0) / ((tm1 - tp) * (tm1 - t0)) * h1;
            }
        }
    };
    // The strips are written in the reference's order (a later strip wins at
    // the corners they share); within a strip every point is its own.
    // upper r boundary (finebound.f90:153-187)
#pragma omp parallel for schedule(static)
    for (int n = 0; n <= F.Nz + g - 1; ++n)
        for (int m = 0; m <= imax; ++m) {
            const double r0 = S.rmaxl[gid] - (double)m * S.drl[level];
            const double z0 = S.zminl[gid] + (double)n * S.dzl[level];
            point(r0, z0, m, n, 'R');
        }
    // lower r boundary of a box off the axis (finebound.f90:246-285)
    if (F.box > 0 && S.rbox[F.box] != 0.0) {
#pragma omp parallel for schedule(static)
        for (int n = 0; n <= F.Nz + g - 1; ++n)
            for (int m = 0; m <= imax; ++m) {
                const double r0 = S.rminl[gid] + (double)m * S.drl[level];
                const double z0 = S.zminl[gid] + (double)n * S.dzl[level];
                point(r0, z0, m, n, 'L');
            }
    }
    // upper z boundary (finebound.f90:296-316)
#pragma omp parallel for schedule(static)
    for (int m = 0; m <= F.Nr + g - 1; ++m)
        for (int n = 0; n <= jmax; ++n) {
            const double r0 = S.rminl[gid] + (double)m * S.drl[level];
            const double z0 = S.zmaxl[gid] - (double)n * S.dzl[level];
            point(r0, z0, m, n, 'z');
        }
    // lower z boundary without equatorial symmetry or off the equator
    // (finebound.f90:351-397)
    if (!S.P.eqsym || (F.box > 0 && S.zbox[F.box] != 0.0)) {
#pragma omp parallel for schedule(static)
        for (int m = 0; m <= F.Nr + g - 1; ++m)
            for (int n = 0; n <= jmax; ++n) {
                const double r0 = S.rminl[gid] + (double)m * S.drl[level];
                const double z0 = S.zminl[gid] + (double)n * S.dzl[level];
                point(r0, z0, m, n, 'l');
            }
    }
    if (outside) throw std::runtime_error("interp: interpolating point is outside the local grid");
}

// restrict.f90:2-169 with restrict_interp.inc: grid ``gid`` into its parent
void restrict_(Sim& S, int gid) {
    Level& F = S.L[gid];
    const int pg = F.parent;
    Level& Cl = S.L[pg];
    const int g = F.g;
    const int level = F.level;
    const double deltar = (double)(2 * g) * S.drl[level] + 1.0e-10;
    const double deltaz = (double)(2 * g) * S.dzl[level] + 1.0e-10;
    Arr& rc = Cl.a("r"); Arr& zc = Cl.a("z");
    const Arr& rf = F.a("r");
    const Arr& zf = F.a("z");
    std::vector<std::pair<const Arr*, Arr*>> vars;
    for (const EvolvedVar& e : S.evolved) vars.emplace_back(&F.a(e.name), &Cl.a(e.name));
    int outside = 0;
    // every coarse point is written at most once: the rows run in parallel
#pragma omp parallel for schedule(dynamic, 4)
    for (int n = 0; n <= Cl.Nz + g - 1; ++n)
        for (int m = 0; m <= Cl.Nr + g - 1; ++m) {
            const double r0 = S.rminl[pg] + (double)m * S.drl[level - 1];
            const double z0 = S.zminl[pg] + (double)n * S.dzl[level - 1];
            const double rmin = (S.rminl[gid] < 0.0) ? 0.0 : S.rminl[gid] + deltar;
            const double zmin = (S.P.eqsym && S.zminl[gid] < 0.0) ? 0.0 : S.zminl[gid] + deltaz;
            const double rmax = S.rmaxl[gid] - deltar;
            const double zmax = S.zmaxl[gid] - deltaz;
            if (r0 > rmin && r0 < rmax && z0 > zmin && z0 < zmax) {
                const int i = (int)nint_((r0 - rc(1 - g, 0)) / S.drl[level - 1]) + 1 - g;
                const int j = (int)nint_((z0 - zc(0, 1 - g)) / S.dzl[level - 1]) + 1 - g;
                const bool flag1 = (i >= 1 - g) && (i <= Cl.Nr) && (j >= 1 - g) && (j <= Cl.Nz);
                for (const auto& fc : vars) {
                    double aux2 = 0.0;
                    if (!interp_at(S, gid, rf, zf, *fc.first, r0, z0, &aux2)) {
#pragma omp atomic write
                        outside = 1;
                        break;
                    }
                    if (flag1) (*fc.second)(i, j) = aux2;
                }
            }
        }
    if (outside) throw std::runtime_error("interp: interpolating point is outside the local grid");
}

// syncboxes.f90:2-243 with the generated intersect_interp.inc: grid ``p``
// (box b1) takes every EVOLVE and AUXILIARY array that is not NOSYNC from
// grid ``q`` (box b2, same level) on its strips up to 3*ghost deep, at the
// points well inside q.  Arrays the reference does not declare (the var_p,
// accumulator and source copies) are overwritten before they are read, so
// every array is taken but the NOSYNC coordinates and scratch and the
// arrays of INTENT = ELLIPTIC or OUTPUT (prl/arrays.pl:1431 generates the
// copies for EVOLVE and AUXILIARY only): the elliptic solution ell_u, ell_v
// and the constraint outputs.
void syncboxes(Sim& S, int p, int q, const std::vector<std::string>& only) {
    Level& A = S.L[p];
    Level& B = S.L[q];
    if (S.rmaxl[p] < S.rminl[q] || S.rmaxl[q] < S.rminl[p] || S.zmaxl[p] < S.zminl[q] || S.zmaxl[q] < S.zminl[p]) return;
    const int g = A.g, level = A.level;
    const int imax = 3 * g, jmax = 3 * g;
    const double deltar = (double)(3 * g) * S.drl[level], deltaz = (double)(3 * g) * S.dzl[level];
    Arr& r = A.a("r"); Arr& z = A.a("z");
    std::vector<std::string> names;
    if (!only.empty()) names = only;  // a single variable (all = .false.)
    else for (auto& kv : A.arrs) {
        const std::string& n = kv.first;
        if (n == "r" || n == "z" || n == "rr" || n == "auxarray" || n == "Dr_auxarray" || n == "Dz_auxarray") continue;
        if (n == "ell_u" || n == "ell_v" || n == "ham" || n == "mom_r" || n == "mom_z" || n == "mom_p" ||
            n == "CDelta_r" || n == "CDelta_z" || n == "CDelta_p" || n == "Clambda" || n == "CAlambda")
            continue;
        if (B.arrs.find(n) == B.arrs.end()) continue;
        names.push_back(n);
    }
    std::sort(names.begin(), names.end());
    auto point = [&](double r0, double z0) {
        if (!(r0 >= S.rminl[q] + deltar && r0 <= S.rmaxl[q] - deltar && z0 >= S.zminl[q] + deltaz &&
              z0 <= S.zmaxl[q] - deltaz))
            return;
        const int i = (int)nint_((r0 - r(1 - g, 0)) / S.drl[level]) + 1 - g;
        const int j = (int)nint_((z0 - z(0, 1 - g)) / S.dzl[level]) + 1 - g;
        const bool flag1 = (i >= 1 - g) && (i <= A.Nr) && (j >= 1 - g) && (j <= A.Nz);
        for (const std::string& n : names) {
            const double aux2 = interp(S, q, B.a(n), r0, z0);
            if (flag1) A.a(n)(i, j) = aux2;
        }
    };
    for (int m = 0; m <= imax; ++m)  // upper r (:60-104)
        for (int n = 0; n <= A.Nz + g - 1; ++n) point(S.rmaxl[p] - (double)m * S.drl[level], S.zminl[p] + (double)n * S.dzl[level]);
    if (A.box > 0 && S.rbox[A.box] != 0.0)  // lower r (:109-141)
        for (int m = 0; m <= imax; ++m)
            for (int n = 0; n <= A.Nz + g - 1; ++n) point(S.rminl[p] + (double)m * S.drl[level], S.zminl[p] + (double)n * S.dzl[level]);
    for (int n = 0; n <= jmax; ++n)  // upper z (:145-177)
        for (int m = 0; m <= A.Nr + g - 1; ++m) point(S.rminl[p] + (double)m * S.drl[level], S.zmaxl[p] - (double)n * S.dzl[level]);
    if (!S.P.eqsym || (A.box > 0 && S.zbox[A.box] != 0.0))  // lower z (:181-213)
        for (int n = 0; n <= jmax; ++n)
            for (int m = 0; m <= A.Nr + g - 1; ++m) point(S.rminl[p] + (double)m * S.drl[level], S.zminl[p] + (double)n * S.dzl[level]);
}

// onestep.f90:446-466 and evolve.f90:211-219: every ordered pair of boxes
// that has the level, box 0 first
void sync_level(Sim& S, int level) {
    for (Level& A : S.L)
        for (Level& B : S.L)
            if (A.level == level && B.level == level && A.box != B.box) syncboxes(S, A.gid, B.gid, {});
}

// ---------------------------------------------------------------------------
// onestep.f90:2-522: every box that has this level, one step each, then
// the finer levels twice, then the restriction of each box into its parent
// ---------------------------------------------------------------------------
static void step_grid(Sim& S, Level& L) {
    const ollin_params& P = S.P;
    const bool rk4 = P.integrator == OLLIN_INTEGRATOR_RK4;
    const bool matter = P.mattertype != OLLIN_MATTER_VACUUM;
    const int gid = L.gid;
    currentgrid(S, L);
    saveold(S, L);
    const int niter = rk4 ? 4 : P.icniter;
    const double dt = L.dt;
    for (int iter = 1; iter <= niter; ++iter) {
        double dtw = 0, weight = 0;
        if (rk4) {
            switch (iter) {
                case 1: dtw = 0.5 * dt; weight = 1.0 / 6.0; break;
                case 2: dtw = 0.5 * dt; weight = 1.0 / 3.0; break;
                case 3: dtw = dt; weight = 1.0 / 3.0; break;
                case 4: dtw = dt; weight = 1.0 / 6.0; break;
            }
        } else {
            dtw = (iter < niter) ? 0.5 * dt : dt;
        }
        sources_geometry(S, L);
        sources_lapse(S, L);
        if (P.shift != OLLIN_SHIFT_NONE) sources_shift(S, L);
        if (matter) sources_scalar(S, L);
        if (L.level == 0 && P.boundtype == OLLIN_BOUND_RADIATIVE) radiative_geometry(S, L);
        if (L.level == 0 && (P.boundtype == OLLIN_BOUND_STATIC || P.boundtype == OLLIN_BOUND_FLAT))
            simpleboundary(S, L);
        if (rk4) accumulate(S, L, iter, niter, weight);
        update(S, L, dtw);
        if (L.level > 0) finebound(S, gid, dtw);
        if (L.ownaxis) symmetries_r(S, L);
        if (L.eqsym && L.ownequator) symmetries_z(S, L);
        auxiliary(S, L);
    }
    S.t2[gid] = S.t1[gid];
    S.t1[gid] = S.t[gid];
    S.s[gid] = S.s[gid] + 1;
    S.t[gid] = S.t[gid] + dt;
    S.point_updates += (double)L.Nr * (double)(L.eqsym ? L.Nz : L.Nz + L.g);
}

static void onestep(Sim& S, int level) {
    // boxes in order 0..Nb (level 0 exists on box 0 only)
    for (Level& L : S.L)
        if (L.level == level) step_grid(S, L);
    if (level < S.Nlmax) {
        onestep(S, level + 1);
        onestep(S, level + 1);
    }
    if (level > 0) sync_level(S, level);
    if (level > 0) {
        for (Level& F : S.L) {
            if (F.level != level || S.s[F.gid] % 2 != 0) continue;
            restrict_(S, F.gid);
            Level& Cl = S.L[F.parent];
            currentgrid(S, Cl);
            if (Cl.ownaxis) symmetries_r(S, Cl);
            if (Cl.eqsym && Cl.ownequator) symmetries_z(S, Cl);
            auxiliary(S, Cl);
        }
    }
}

// ---------------------------------------------------------------------------
static void initial(Sim& S) {
    const ollin_params& P = S.P;
    const double zero = 0.0, half = 0.5, third = 1.0 / 3.0, one = 1.0, two = 2.0;
    for (Level& L : S.L) {
        currentgrid(S, L);
        const int g = L.g, Nr = L.Nr, Nz = L.Nz;
        auto setc = [&](const char* n, double v) { Arr& a = L.a(n); for (double& x : a.v) x = v; };
        setc("alpha", one); setc("dtalpha", zero);
        if (P.shift != OLLIN_SHIFT_NONE) { setc("beta_r", zero); setc("beta_z", zero); setc("dtbeta_r", zero); setc("dtbeta_z", zero); setc("fdriver", one); }
        setc("psi", one); setc("phi", zero); setc("chi", one); setc("psi2", one); setc("psi4", one);
        setc("A", one); setc("B", one); setc("H", one); setc("C", zero);
        setc("g_A", one); setc("g_B", one); setc("g_H", one); setc("g_C", zero);
        setc("trK", zero); setc("KTA", zero); setc("KTB", zero); setc("KTC", zero); setc("KTH", zero);
        setc("Delta_r", zero); setc("Delta_z", zero); setc("lambda", zero); setc("Alambda", zero); setc("z4theta", zero);
        Arr& psi = L.a("psi"); Arr& phi = L.a("phi"); Arr& chi = L.a("chi"); Arr& psi2 = L.a("psi2"); Arr& psi4 = L.a("psi4");
        Arr& rr = L.a("rr"); Arr& alpha = L.a("alpha"); Arr& r = L.a("r"); Arr& z = L.a("z");
        const double M = P.bh1mass;
        if (P.idata == OLLIN_IDATA_SCHWARZSCHILD || P.idata == OLLIN_IDATA_BRILLLINDQUIST) {
            for (int j = 1 - g; j <= Nz; ++j)
                for (int i = 1 - g; i <= Nr; ++i) {
                    if (P.idata == OLLIN_IDATA_SCHWARZSCHILD) psi(i, j) = one + half * M / std::fabs(rr(i, j));
                    else psi(i, j) = one + half * M / std::sqrt(p2(r(i, j)) + p2(z(i, j) - 0.0));
                    phi(i, j) = std::log(psi(i, j));
                    chi(i, j) = one / std::pow(psi(i, j), (double)P.chipower);
                    psi2(i, j) = p2(psi(i, j));
                    psi4(i, j) = p4(psi(i, j));
                    if (P.idata == OLLIN_IDATA_SCHWARZSCHILD && P.ilapse == OLLIN_ILAPSE_ISOTROPIC)
                        alpha(i, j) = (one - half * M / std::fabs(rr(i, j))) / (one + half * M / std::fabs(rr(i, j)));
                }
        }
        (void)psi2;
    }
    // elliptic initial data (initial.f90:336-341, 380-394)
    if (P.idata == OLLIN_IDATA_BRILLWAVE) idata_brillwave(S);
    if (P.idata == OLLIN_IDATA_SCALARPULSE) {
        if (P.mattertype != OLLIN_MATTER_SCALAR)
            throw std::runtime_error("Scalar pulse initial data needs scalar field type matter.");
        idata_scalarpulse(S);
    }
    if (P.factorhdet) {  // initial.f90:528-577
        for (Level& L : S.L) {
            const int g = L.g, Nr = L.Nr, Nz = L.Nz;
            Arr& A = L.a("A"); Arr& B = L.a("B"); Arr& C = L.a("C"); Arr& H = L.a("H"); Arr& r = L.a("r");
            Arr& hdet = L.a("hdet"); Arr& ihdet = L.a("ihdet"); Arr& phi = L.a("phi"); Arr& aux = L.a("auxarray");
            Arr& psi = L.a("psi"); Arr& psi2 = L.a("psi2"); Arr& psi4 = L.a("psi4");
            for (int j = 1 - g; j <= Nz; ++j)
                for (int i = 1 - g; i <= Nr; ++i) {
                    hdet(i, j) = (A(i, j) * B(i, j) - p2(r(i, j) * C(i, j))) * H(i, j);
                    phi(i, j) = phi(i, j) + std::log(hdet(i, j)) / 12.0;
                    aux(i, j) = std::pow(hdet(i, j), third);
                    A(i, j) = A(i, j) / aux(i, j);
                    B(i, j) = B(i, j) / aux(i, j);
                    C(i, j) = C(i, j) / aux(i, j);
                    H(i, j) = H(i, j) / aux(i, j);
                    hdet(i, j) = 1.0;
                    ihdet(i, j) = 1.0;
                    psi(i, j) = std::exp(phi(i, j));
                    psi2(i, j) = p2(psi(i, j));
                    psi4(i, j) = p4(psi(i, j));
                }
        }
    }
    for (Level& L : S.L) {  // initial.f90:583-607 traceless projection
        const int g = L.g, Nr = L.Nr, Nz = L.Nz;
        Arr& g_A = L.a("g_A"); Arr& g_B = L.a("g_B"); Arr& g_H = L.a("g_H"); Arr& g_C = L.a("g_C");
        Arr& KTA = L.a("KTA"); Arr& KTB = L.a("KTB"); Arr& KTH = L.a("KTH"); Arr& KTC = L.a("KTC");
        Arr& A = L.a("A"); Arr& B = L.a("B"); Arr& C = L.a("C"); Arr& H = L.a("H"); Arr& r = L.a("r"); Arr& aux = L.a("auxarray");
        for (int j = 1 - g; j <= Nz; ++j)
            for (int i = 1 - g; i <= Nr; ++i) aux(i, j) = g_A(i, j) * KTA(i, j) + g_B(i, j) * KTB(i, j) + g_H(i, j) * KTH(i, j) + two * p2(r(i, j)) * g_C(i, j) * KTC(i, j);
        for (int j = 1 - g; j <= Nz; ++j)
            for (int i = 1 - g; i <= Nr; ++i) {
                KTA(i, j) = KTA(i, j) - third * A(i, j) * aux(i, j);
                KTB(i, j) = KTB(i, j) - third * B(i, j) * aux(i, j);
                KTH(i, j) = KTH(i, j) - third * H(i, j) * aux(i, j);
                KTC(i, j) = KTC(i, j) - third * C(i, j) * aux(i, j);
            }
    }
    if (P.ilapse == OLLIN_ILAPSE_PSIMINUS2 || P.ilapse == OLLIN_ILAPSE_PSIMINUS4) {
        for (Level& L : S.L) {
            Arr& alpha = L.a("alpha"); Arr& psi = L.a("psi");
            for (size_t q = 0; q < alpha.v.size(); ++q)
                alpha.v[q] = (P.ilapse == OLLIN_ILAPSE_PSIMINUS2) ? one / p2(psi.v[q]) : one / p4(psi.v[q]);
        }
    }
}

// evolve.f90:128-219 (no maximal slicing); ``initial`` runs first
static void initialize(Sim& S) {
    for (Level& L : S.L) {
        currentgrid(S, L);
        if (L.ownaxis) symmetries_r(S, L);
        if (L.eqsym && L.ownequator) symmetries_z(S, L);
    }
    for (Level& L : S.L) {
        currentgrid(S, L);
        auxiliary(S, L);
    }
    // evolve.f90:174-195: dtbeta = csi Delta for the second-order drivers,
    // unless driverD0
    if ((S.P.shift == OLLIN_SHIFT_GAMMADRIVER2 || S.P.shift == OLLIN_SHIFT_GAMMADRIVERSHOCK2) && !S.P.driverD0) {
        for (Level& L : S.L) {
            Arr& b = L.a("dtbeta_r"); Arr& bz = L.a("dtbeta_z"); Arr& dr_ = L.a("Delta_r"); Arr& dz_ = L.a("Delta_z");
            for (size_t q = 0; q < b.v.size(); ++q) { b.v[q] = S.P.drivercsi * dr_.v[q]; bz.v[q] = S.P.drivercsi * dz_.v[q]; }
        }
    }
    for (int level = 1; level <= S.Nlmax; ++level) sync_level(S, level);  // :211-219
}

// save0Ddata.f90:221-288 and the origin value at :370-374
static void norms(Sim& S, int level, const Arr& v, double out[5]) {
    Level& L = S.L[level];
    double vmax = -1.0e10, vmin = +1.0e10, nm1 = 0.0, nm2 = 0.0, NN = 0.0;
    for (int j = 1; j <= L.Nz - L.g; ++j)
        for (int i = 1; i <= L.Nr - L.g; ++i) {
            const double aux = v(i, j);
            if (std::isnan(aux)) throw std::runtime_error("norms: NaN found");
            NN = NN + 1.0;
            vmin = std::min(vmin, aux);
            vmax = std::max(vmax, aux);
            nm1 = std::max(nm1, std::fabs(aux));
            nm2 = nm2 + p2(aux);
        }
    out[0] = vmax; out[1] = vmin; out[2] = nm1; out[3] = std::sqrt(nm2 / NN);
    out[4] = (L.box == 0) ? interp(S, level, v, 0.0, 0.0) : 0.0;  // origin data for box 0 only (:372-374)
}

}  // namespace oracle

// ---------------------------------------------------------------------------
// C API
// ---------------------------------------------------------------------------
using namespace oracle;

struct ollin_oracle { Sim S; };

static thread_local std::string g_oracle_err;

extern "C" {

const char* ollin_oracle_last_error(void) { return g_oracle_err.c_str(); }

int ollin_oracle_create(const ollin_params* p, ollin_oracle** out) {
    try {
        auto* o = new ollin_oracle();
        o->S.P = *p;
        setup(o->S);
        *out = o;
        return 0;
    } catch (const std::exception& e) {
        g_oracle_err = e.what();
        return 1;
    }
}

void ollin_oracle_destroy(ollin_oracle* o) { delete o; }

int ollin_oracle_initial_data(ollin_oracle* o) {
    try { initial(o->S); return 0; } catch (const std::exception& e) { g_oracle_err = e.what(); return 1; }
}

int ollin_oracle_initialize(ollin_oracle* o) {
    try { initialize(o->S); return 0; } catch (const std::exception& e) { g_oracle_err = e.what(); return 1; }
}

int ollin_oracle_step(ollin_oracle* o, double* t_out) {
    try {
        onestep(o->S, 0);
        if (t_out) *t_out = o->S.t[0];
        return 0;
    } catch (const std::exception& e) {
        g_oracle_err = e.what();
        return 1;
    }
}

int ollin_oracle_num_levels(const ollin_oracle* o) { return (int)o->S.L.size(); }

int ollin_oracle_dims(const ollin_oracle* o, int level, int* nr, int* nz, int* ghost) {
    if (level < 0 || level >= (int)o->S.L.size()) return 1;
    const Level& L = o->S.L[level];
    *nr = L.Nr; *nz = L.Nz; *ghost = L.g;
    return 0;
}

double ollin_oracle_time(const ollin_oracle* o, int level) { return o->S.t[level]; }

int ollin_oracle_grid(const ollin_oracle* o, int gid, int* box, int* level) {
    if (gid < 0 || gid >= (int)o->S.L.size()) return 1;
    *box = o->S.L[gid].box;
    *level = o->S.L[gid].level;
    return 0;
}

// Copy grid function ``name`` of ``level`` into ``a`` (column-major,
// leading dimension ld_r, element (1-ghost,1-ghost) first).
int ollin_oracle_get(ollin_oracle* o, int level, const char* name, double* a, int ld_r) {
    if (level < 0 || level >= (int)o->S.L.size()) { g_oracle_err = "bad level"; return 1; }
    Level& L = o->S.L[level];
    auto it = L.arrs.find(name);
    if (it == L.arrs.end()) { g_oracle_err = std::string("unknown array ") + name; return 1; }
    const Arr& v = it->second;
    for (int j = 0; j < L.Nz + L.g; ++j)
        for (int i = 0; i < L.Nr + L.g; ++i) a[(size_t)i + (size_t)j * ld_r] = v.v[(size_t)i + (size_t)j * v.ld];
    return 0;
}

int ollin_oracle_set(ollin_oracle* o, int level, const char* name, const double* a, int ld_r) {
    if (level < 0 || level >= (int)o->S.L.size()) { g_oracle_err = "bad level"; return 1; }
    Level& L = o->S.L[level];
    Arr& v = L.a(name);
    for (int j = 0; j < L.Nz + L.g; ++j)
        for (int i = 0; i < L.Nr + L.g; ++i) v.v[(size_t)i + (size_t)j * v.ld] = a[(size_t)i + (size_t)j * ld_r];
    return 0;
}

int ollin_oracle_aux(ollin_oracle* o, int level) {
    try {
        Level& L = o->S.L[level];
        L.time = o->S.t[level];
        auxiliary(o->S, L);
        return 0;
    } catch (const std::exception& e) {
        g_oracle_err = e.what();
        return 1;
    }
}

// maximalslicing (evolve.f90:228-230 and :388-393); va_max (r, z) may be null
int ollin_oracle_maximal_slicing(ollin_oracle* o, const double* va_max) {
    try { maximalslicing(o->S, va_max); return 0; } catch (const std::exception& e) { g_oracle_err = e.what(); return 1; }
}

int ollin_oracle_constraints(ollin_oracle* o, int level) {
    try { constraints(o->S, o->S.L[level]); return 0; } catch (const std::exception& e) { g_oracle_err = e.what(); return 1; }
}

int ollin_oracle_norms(ollin_oracle* o, int level, const char* name, double out[5]) {
    try {
        Level& L = o->S.L[level];
        auto it = L.arrs.find(name);
        if (it == L.arrs.end()) { g_oracle_err = std::string("unknown array ") + name; return 1; }
        norms(o->S, level, it->second, out);
        return 0;
    } catch (const std::exception& e) {
        g_oracle_err = e.what();
        return 1;
    }
}

// interp.f90 at n points rz = (r0, z0) pairs of grid ``level``
int ollin_oracle_interp(ollin_oracle* o, int level, const char* name, const double* rz, int n, double* out) {
    try {
        Level& L = o->S.L[level];
        auto it = L.arrs.find(name);
        if (it == L.arrs.end()) { g_oracle_err = std::string("unknown array ") + name; return 1; }
        for (int k = 0; k < n; ++k) out[k] = interp(o->S, level, it->second, rz[2 * k], rz[2 * k + 1]);
        return 0;
    } catch (const std::exception& e) {
        g_oracle_err = e.what();
        return 1;
    }
}

double ollin_oracle_point_updates(const ollin_oracle* o) { return o->S.point_updates; }

void ollin_oracle_set_threads(int n) { omp_set_num_threads(n > 0 ? n : 1); }

int ollin_oracle_max_threads(void) { return omp_get_max_threads(); }

int ollin_oracle_ell_stats(int steps[2], double* gres) {
    steps[0] = g_ell_stats.steps[0];
    steps[1] = g_ell_stats.steps[1];
    if (gres) *gres = g_ell_stats.gres;
    return g_ell_stats.phases;
}

}  // extern "C"
