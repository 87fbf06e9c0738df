// ORACLE -- test infrastructure only.  CPU restatement of the OllinAxis-BiB
// evolution path used to check the GB300 library; never linked into it.
//
// This file restates, statement for statement and in the reference's order,
// the stencil primitives and the right-hand side of the (rho,z) BSSN system:
//   src/base/derivatives.f90, src/base/derivadvect.f90,
//   src/base/dissipation.f90, src/base/radbound.f90,
//   src/geometry/auxiliary_geometry.f90 (+ calc_conformalRicci1-4,
//   calc_DIVKTA, factordet), sources_geometry/lapse/shift.f90,
//   radiative_geometry.f90, constraints.f90,
//   src/matter/auxiliary_matter.f90, potential.f90, stressenergy.f90,
//   scalar.f90 (real scalar field).
// Branches implemented: formulation bssn, angmom false, order two and four,
// chimethod, chipower 2, lagrangian flavour with factorhdet.  Each whole-array
// Fortran statement is one loop over (1-ghost:Nr, 1-ghost:Nz).
#include "oracle_sim.h"

namespace oracle {

#define GRID_DIMS const int g = L.g, Nr = L.Nr, Nz = L.Nz; (void)g; (void)Nr; (void)Nz
#define ALL _Pragma("omp parallel for schedule(static)") \
    for (int j = 1 - g; j <= Nz; ++j) for (int i = 1 - g; i <= Nr; ++i)
#define R(name) Arr& name = L.a(#name)

static inline int isign1(int s) { return s >= 0 ? 1 : -1; }

// ---------------------------------------------------------------------------
// derivatives.f90 (order two and order four branches)
// ---------------------------------------------------------------------------

// diff1r: derivatives.f90:15-117 (order two :50-58: i = 1-ghost is left unset)
void diff1r(Level& L, const Arr& f, Arr& d, int symr) {
    GRID_DIMS;
    const double idr = 1.0 / L.dr;
    const double hidr = 0.5 * idr;
    if (L.order == 2) {
#pragma omp parallel for schedule(static)
        for (int j = 1 - g; j <= Nz; ++j) {
            for (int i = 2 - g; i <= Nr - 1; ++i) d(i, j) = hidr * (f(i + 1, j) - f(i - 1, j));
            const int i = Nr;
            d(i, j) = hidr * (3.0 * f(Nr, j) - 4.0 * f(Nr - 1, j) + f(Nr - 2, j));
            if (L.ownaxis)
                for (int ii = 1; ii <= g; ++ii) d(1 - ii, j) = -isign1(symr) * d(ii, j);
        }
        return;
    }
#pragma omp parallel for schedule(static)
    for (int j = 1 - g; j <= Nz; ++j) {
        for (int i = 1; i <= Nr - 2; ++i)
            d(i, j) = idr * (8.0 * (f(i + 1, j) - f(i - 1, j)) - (f(i + 2, j) - f(i - 2, j))) / 12.0;
        int i = Nr - 1;
        d(i, j) = idr * (3.0 * f(i + 1, j) + 10.0 * f(i, j) - 18.0 * f(i - 1, j) + 6.0 * f(i - 2, j) - f(i - 3, j)) / 12.0;
        i = Nr;
        d(i, j) = idr * (25.0 * f(i, j) - 48.0 * f(i - 1, j) + 36.0 * f(i - 2, j) - 16.0 * f(i - 3, j) + 3.0 * f(i - 4, j)) / 12.0;
        if (L.ownaxis)
            for (int ii = 1; ii <= g; ++ii) d(1 - ii, j) = -isign1(symr) * d(ii, j);
    }
}

// diff1z: derivatives.f90:123-241 (order two :158-172)
void diff1z(Level& L, const Arr& f, Arr& d, int symz) {
    GRID_DIMS;
    const double idz = 1.0 / L.dz;
    const double hidz = 0.5 * idz;
    if (L.order == 2) {
#pragma omp parallel for schedule(static)
        for (int j = 2 - g; j <= Nz - 1; ++j)
            for (int i = 1 - g; i <= Nr; ++i) d(i, j) = hidz * (f(i, j + 1) - f(i, j - 1));
#pragma omp parallel for schedule(static)
        for (int i = 1 - g; i <= Nr; ++i) {
            int j = 1 - g;
            d(i, j) = -hidz * (3.0 * f(i, j) - 4.0 * f(i, j + 1) + f(i, j + 2));
            j = Nz;
            d(i, j) = +hidz * (3.0 * f(i, j) - 4.0 * f(i, j - 1) + f(i, j - 2));
            if (L.eqsym && L.ownequator)
                for (int jj = 1; jj <= g; ++jj) d(i, 1 - jj) = -isign1(symz) * d(i, jj);
        }
        return;
    }
    // the interior rows with r innermost (contiguous), then the edge rows and
    // the equator fill: every point gets the statement the reference gives it
#pragma omp parallel for schedule(static)
    for (int j = 3 - g; j <= Nz - 2; ++j)
        for (int i = 1 - g; i <= Nr; ++i)
            d(i, j) = idz * (8.0 * (f(i, j + 1) - f(i, j - 1)) - (f(i, j + 2) - f(i, j - 2))) / 12.0;
#pragma omp parallel for schedule(static)
    for (int i = 1 - g; i <= Nr; ++i) {
        int j = 2 - g;
        d(i, j) = -idz * (3.0 * f(i, j - 1) + 10.0 * f(i, j) - 18.0 * f(i, j + 1) + 6.0 * f(i, j + 2) - f(i, j + 3)) / 12.0;
        j = 1 - g;
        d(i, j) = -idz * (25.0 * f(i, j) - 48.0 * f(i, j + 1) + 36.0 * f(i, j + 2) - 16.0 * f(i, j + 3) + 3.0 * f(i, j + 4)) / 12.0;
        j = Nz - 1;
        d(i, j) = +idz * (3.0 * f(i, j + 1) + 10.0 * f(i, j) - 18.0 * f(i, j - 1) + 6.0 * f(i, j - 2) - f(i, j - 3)) / 12.0;
        j = Nz;
        d(i, j) = +idz * (25.0 * f(i, j) - 48.0 * f(i, j - 1) + 36.0 * f(i, j - 2) - 16.0 * f(i, j - 3) + 3.0 * f(i, j - 4)) / 12.0;
        if (L.eqsym && L.ownequator)
            for (int jj = 1; jj <= g; ++jj) d(i, 1 - jj) = -isign1(symz) * d(i, jj);
    }
}

// diff2r: derivatives.f90:250-359 (order two :285-301)
void diff2r(Level& L, const Arr& f, Arr& d, int symr) {
    GRID_DIMS;
    const double idr = 1.0 / L.dr;
    const double idr2 = idr * idr;
    if (L.order == 2) {
#pragma omp parallel for schedule(static)
        for (int j = 1 - g; j <= Nz; ++j) {
            for (int i = 2 - g; i <= Nr - 1; ++i) d(i, j) = idr2 * (f(i + 1, j) - 2.0 * f(i, j) + f(i - 1, j));
            int i = 1 - g;
            d(i, j) = idr2 * (2.0 * f(i, j) - 5.0 * f(i + 1, j) + 4.0 * f(i + 2, j) - f(i + 3, j));
            i = Nr;
            d(i, j) = idr2 * (2.0 * f(i, j) - 5.0 * f(i - 1, j) + 4.0 * f(i - 2, j) - f(i - 3, j));
            if (L.ownaxis)
                for (int ii = 1; ii <= g; ++ii) d(1 - ii, j) = isign1(symr) * d(ii, j);
        }
        return;
    }
#pragma omp parallel for schedule(static)
    for (int j = 1 - g; j <= Nz; ++j) {
        for (int i = 3 - g; i <= Nr - 2; ++i)
            d(i, j) = -idr2 * (30.0 * f(i, j) - 16.0 * (f(i + 1, j) + f(i - 1, j)) + f(i + 2, j) + f(i - 2, j)) / 12.0;
        int i = Nr - 1;
        d(i, j) = idr2 * (10.0 * f(i + 1, j) - 15.0 * f(i, j) - 4.0 * f(i - 1, j) + 14.0 * f(i - 2, j) - 6.0 * f(i - 3, j) + f(i - 4, j)) / 12.0;
        i = Nr;
        d(i, j) = idr2 * (45.0 * f(i, j) - 154.0 * f(i - 1, j) + 214.0 * f(i - 2, j) - 156.0 * f(i - 3, j) + 61.0 * f(i - 4, j) - 10.0 * f(i - 5, j)) / 12.0;
        if (L.ownaxis)
            for (int ii = 1; ii <= g; ++ii) d(1 - ii, j) = isign1(symr) * d(ii, j);
    }
}

// diff2z: derivatives.f90:367-488 (order two :402-418)
void diff2z(Level& L, const Arr& f, Arr& d, int symz) {
    GRID_DIMS;
    const double idz = 1.0 / L.dz;
    const double idz2 = idz * idz;
    if (L.order == 2) {
#pragma omp parallel for schedule(static)
        for (int j = 2 - g; j <= Nz - 1; ++j)
            for (int i = 1 - g; i <= Nr; ++i) d(i, j) = idz2 * (f(i, j + 1) - 2.0 * f(i, j) + f(i, j - 1));
#pragma omp parallel for schedule(static)
        for (int i = 1 - g; i <= Nr; ++i) {
            int j = 1 - g;
            d(i, j) = idz2 * (2.0 * f(i, j) - 5.0 * f(i, j + 1) + 4.0 * f(i, j + 2) - f(i, j + 3));
            j = Nz;
            d(i, j) = idz2 * (2.0 * f(i, j) - 5.0 * f(i, j - 1) + 4.0 * f(i, j - 2) - f(i, j - 3));
            if (L.eqsym && L.ownequator)
                for (int jj = 1; jj <= g; ++jj) d(i, 1 - jj) = isign1(symz) * d(i, jj);
        }
        return;
    }
#pragma omp parallel for schedule(static)
    for (int j = 3 - g; j <= Nz - 2; ++j)
        for (int i = 1 - g; i <= Nr; ++i)
            d(i, j) = -idz2 * (30.0 * f(i, j) - 16.0 * (f(i, j + 1) + f(i, j - 1)) + f(i, j + 2) + f(i, j - 2)) / 12.0;
#pragma omp parallel for schedule(static)
    for (int i = 1 - g; i <= Nr; ++i) {
        int j = 2 - g;
        d(i, j) = idz2 * (10.0 * f(i, j - 1) - 15.0 * f(i, j) - 4.0 * f(i, j + 1) + 14.0 * f(i, j + 2) - 6.0 * f(i, j + 3) + f(i, j + 4)) / 12.0;
        j = 1 - g;
        d(i, j) = idz2 * (45.0 * f(i, j) - 154.0 * f(i, j + 1) + 214.0 * f(i, j + 2) - 156.0 * f(i, j + 3) + 61.0 * f(i, j + 4) - 10.0 * f(i, j + 5)) / 12.0;
        j = Nz - 1;
        d(i, j) = idz2 * (10.0 * f(i, j + 1) - 15.0 * f(i, j) - 4.0 * f(i, j - 1) + 14.0 * f(i, j - 2) - 6.0 * f(i, j - 3) + f(i, j - 4)) / 12.0;
        j = Nz;
        d(i, j) = idz2 * (45.0 * f(i, j) - 154.0 * f(i, j - 1) + 214.0 * f(i, j - 2) - 156.0 * f(i, j - 3) + 61.0 * f(i, j - 4) - 10.0 * f(i, j - 5)) / 12.0;
        if (L.eqsym && L.ownequator)
            for (int jj = 1; jj <= g; ++jj) d(i, 1 - jj) = isign1(symz) * d(i, jj);
    }
}

// diff2rz: derivatives.f90:496-732 (fourth order branch with its
// second-order edges and corners)
void diff2rz(Level& L, const Arr& f, Arr& d, int symr, int symz) {
    GRID_DIMS;
    const double idr = 1.0 / L.dr, idz = 1.0 / L.dz;
    const double idrz = idr * idz;
    if (L.order == 2) {
        // derivatives.f90:533-599: centred inside, one-sided on the outermost
        // rows and columns, the corners from both one-sided stencils
#pragma omp parallel for schedule(static)
        for (int i = 2 - g; i <= Nr - 1; ++i)
            for (int j = 2 - g; j <= Nz - 1; ++j)
                d(i, j) = 0.25 * idrz * (f(i + 1, j + 1) + f(i - 1, j - 1) - f(i + 1, j - 1) - f(i - 1, j + 1));
        for (int j = 2 - g; j <= Nz - 1; ++j) {
            int i = 1 - g;
            d(i, j) = -0.25 * idrz * ((3.0 * f(i, j + 1) - 4.0 * f(i + 1, j + 1) + f(i + 2, j + 1))
                                      - (3.0 * f(i, j - 1) - 4.0 * f(i + 1, j - 1) + f(i + 2, j - 1)));
            i = Nr;
            d(i, j) = +0.25 * idrz * ((3.0 * f(i, j + 1) - 4.0 * f(i - 1, j + 1) + f(i - 2, j + 1))
                                      - (3.0 * f(i, j - 1) - 4.0 * f(i - 1, j - 1) + f(i - 2, j - 1)));
        }
        for (int i = 2 - g; i <= Nr - 1; ++i) {
            int j = 1 - g;
            d(i, j) = -0.25 * idrz * ((3.0 * f(i + 1, j) - 4.0 * f(i + 1, j + 1) + f(i + 1, j + 2))
                                      - (3.0 * f(i - 1, j) - 4.0 * f(i - 1, j + 1) + f(i - 1, j + 2)));
            j = Nz;
            d(i, j) = +0.25 * idrz * ((3.0 * f(i + 1, j) - 4.0 * f(i + 1, j - 1) + f(i + 1, j - 2))
                                      - (3.0 * f(i - 1, j) - 4.0 * f(i - 1, j - 1) + f(i - 1, j - 2)));
        }
    } else {
#pragma omp parallel for schedule(static)
    for (int j = 3 - g; j <= Nz - 2; ++j)
        for (int i = 3 - g; i <= Nr - 2; ++i)
            d(i, j) = idrz * ((f(i + 1, j + 1) + f(i - 1, j - 1) - f(i + 1, j - 1) - f(i - 1, j + 1)) / 3.0
                              - (f(i + 2, j + 2) + f(i - 2, j - 2) - f(i + 2, j - 2) - f(i - 2, j + 2)) / 48.0);
    // boundaries on r
    for (int j = 2 - g; j <= Nz - 1; ++j) {
        int i = 2 - g;
        d(i, j) = +0.25 * idrz * (f(i + 1, j + 1) + f(i - 1, j - 1) - f(i + 1, j - 1) - f(i - 1, j + 1));
        i = 1 - g;
        d(i, j) = -0.25 * idrz * ((3.0 * f(i, j + 1) - 4.0 * f(i + 1, j + 1) + f(i + 2, j + 1))
                                  - (3.0 * f(i, j - 1) - 4.0 * f(i + 1, j - 1) + f(i + 2, j - 1)));
        i = Nr - 1;
        d(i, j) = +0.25 * idrz * (f(i + 1, j + 1) + f(i - 1, j - 1) - f(i + 1, j - 1) - f(i - 1, j + 1));
        i = Nr;
        d(i, j) = +0.25 * idrz * ((3.0 * f(i, j + 1) - 4.0 * f(i - 1, j + 1) + f(i - 2, j + 1))
                                  - (3.0 * f(i, j - 1) - 4.0 * f(i - 1, j - 1) + f(i - 2, j - 1)));
    }
    // boundaries on z
    for (int i = 2 - g; i <= Nr - 1; ++i) {
        int j = 2 - g;
        d(i, j) = +0.25 * idrz * (f(i + 1, j + 1) + f(i - 1, j - 1) - f(i - 1, j + 1) - f(i + 1, j - 1));
        j = 1 - g;
        d(i, j) = -0.25 * idrz * ((3.0 * f(i + 1, j) - 4.0 * f(i + 1, j + 1) + f(i + 1, j + 2))
                                  - (3.0 * f(i - 1, j) - 4.0 * f(i - 1, j + 1) + f(i - 1, j + 2)));
        j = Nz - 1;
        d(i, j) = +0.25 * idrz * (f(i + 1, j + 1) + f(i - 1, j - 1) - f(i - 1, j + 1) - f(i + 1, j - 1));
        j = Nz;
        d(i, j) = +0.25 * idrz * ((3.0 * f(i + 1, j) - 4.0 * f(i + 1, j - 1) + f(i + 1, j - 2))
                                  - (3.0 * f(i - 1, j) - 4.0 * f(i - 1, j - 1) + f(i - 1, j - 2)));
    }
    // corners
    {
        int i = 1 - g, j = 1 - g;
        d(i, j) = +0.25 * idrz * (9.0 * f(i, j) + 16.0 * f(i + 1, j + 1) + f(i + 2, j + 2)
                                  - 12.0 * (f(i, j + 1) + f(i + 1, j)) + 3.0 * (f(i, j + 2) + f(i + 2, j))
                                  - 4.0 * (f(i + 1, j + 2) + f(i + 2, j + 1)));
        i = 1 - g; j = Nz;
        d(i, j) = -0.25 * idrz * (9.0 * f(i, j) + 16.0 * f(i + 1, j - 1) + f(i + 2, j - 2)
                                  - 12.0 * (f(i + 1, j) + f(i, j - 1)) + 3.0 * (f(i + 2, j) + f(i, j - 2))
                                  - 4.0 * (f(i + 2, j - 1) + f(i + 1, j - 2)));
        i = Nr; j = 1 - g;
        d(i, j) = -0.25 * idrz * (9.0 * f(i, j) + 16.0 * f(i - 1, j + 1) + f(i - 2, j + 2)
                                  - 12.0 * (f(i, j + 1) + f(i - 1, j)) + 3.0 * (f(i, j + 2) + f(i - 2, j))
                                  - 4.0 * (f(i - 1, j + 2) + f(i - 2, j + 1)));
        i = Nr; j = Nz;
        d(i, j) = +0.25 * idrz * (9.0 * f(i, j) + 16.0 * f(i - 1, j - 1) + f(i - 2, j - 2)
                                  - 12.0 * (f(i, j - 1) + f(i - 1, j)) + 3.0 * (f(i, j - 2) + f(i - 2, j))
                                  - 4.0 * (f(i - 1, j - 2) + f(i - 2, j - 1)));
    }
    }  // order four
    if (L.order == 2) {
        // the same four corner statements close the order-two branch
        // (derivatives.f90:571-597)
        int i = 1 - g, j = 1 - g;
        d(i, j) = +0.25 * idrz * (9.0 * f(i, j) + 16.0 * f(i + 1, j + 1) + f(i + 2, j + 2)
                                  - 12.0 * (f(i, j + 1) + f(i + 1, j)) + 3.0 * (f(i, j + 2) + f(i + 2, j))
                                  - 4.0 * (f(i + 1, j + 2) + f(i + 2, j + 1)));
        i = 1 - g; j = Nz;
        d(i, j) = -0.25 * idrz * (9.0 * f(i, j) + 16.0 * f(i + 1, j - 1) + f(i + 2, j - 2)
                                  - 12.0 * (f(i + 1, j) + f(i, j - 1)) + 3.0 * (f(i + 2, j) + f(i, j - 2))
                                  - 4.0 * (f(i + 2, j - 1) + f(i + 1, j - 2)));
        i = Nr; j = 1 - g;
        d(i, j) = -0.25 * idrz * (9.0 * f(i, j) + 16.0 * f(i - 1, j + 1) + f(i - 2, j + 2)
                                  - 12.0 * (f(i, j + 1) + f(i - 1, j)) + 3.0 * (f(i, j + 2) + f(i - 2, j))
                                  - 4.0 * (f(i - 1, j + 2) + f(i - 2, j + 1)));
        i = Nr; j = Nz;
        d(i, j) = +0.25 * idrz * (9.0 * f(i, j) + 16.0 * f(i - 1, j - 1) + f(i - 2, j - 2)
                                  - 12.0 * (f(i, j - 1) + f(i - 1, j)) + 3.0 * (f(i, j - 2) + f(i - 2, j))
                                  - 4.0 * (f(i - 1, j - 2) + f(i - 2, j - 1)));
    }
    // symmetries: z first, then r (derivatives.f90:702-714)
    if (L.eqsym && L.ownequator)
        for (int jj = 1; jj <= g; ++jj)
            for (int i = 1 - g; i <= Nr; ++i) d(i, 1 - jj) = -isign1(symz) * d(i, jj);
    if (L.ownaxis)
        for (int j = 1 - g; j <= Nz; ++j)
            for (int ii = 1; ii <= g; ++ii) d(1 - ii, j) = -isign1(symr) * d(ii, j);
}

// ---------------------------------------------------------------------------
// derivadvect.f90 (order two and four): lopsided derivatives, side chosen by the
// sign of the shift component at the point
// ---------------------------------------------------------------------------
void diffadvr(Level& L, const Arr& f, Arr& d, int symr) {
    GRID_DIMS;
    const Arr& beta_r = L.a("beta_r");
    const double idr = 1.0 / L.dr;
    if (L.order == 2) {
        // derivadvect.f90:50-100: second-order one-sided
        const double hidr = 0.5 * idr;
#pragma omp parallel for schedule(static)
        for (int j = 1 - g; j <= Nz; ++j) {
            for (int i = 3 - g; i <= Nr - 2; ++i) {
                if (beta_r(i, j) <= 0.0) d(i, j) = +hidr * (3.0 * f(i, j) - 4.0 * f(i - 1, j) + f(i - 2, j));
                else d(i, j) = -hidr * (3.0 * f(i, j) - 4.0 * f(i + 1, j) + f(i + 2, j));
            }
            int i = 2 - g;
            if (beta_r(i, j) <= 0.0) d(i, j) = hidr * (f(i + 1, j) - f(i - 1, j));
            else d(i, j) = -hidr * (3.0 * f(i, j) - 4.0 * f(i + 1, j) + f(i + 2, j));
            i = 1 - g;
            d(i, j) = -hidr * (3.0 * f(i, j) - 4.0 * f(i + 1, j) + f(i + 2, j));
            i = Nr - 1;
            if (beta_r(i, j) <= 0.0) d(i, j) = hidr * (3.0 * f(i, j) - 4.0 * f(i - 1, j) + f(i - 2, j));
            else d(i, j) = hidr * (f(i + 1, j) - f(i - 1, j));
            i = Nr;
            d(i, j) = hidr * (3.0 * f(i, j) - 4.0 * f(i - 1, j) + f(i - 2, j));
            if (L.ownaxis)
                for (int ii = 1; ii <= g; ++ii) d(1 - ii, j) = -symr * d(ii, j);
        }
        return;
    }
#pragma omp parallel for schedule(static)
    for (int j = 1 - g; j <= Nz; ++j) {
        for (int i = 4 - g; i <= Nr - 3; ++i) {
            if (beta_r(i, j) <= 0.0)
                d(i, j) = +0.25 * idr * (3.0 * f(i + 1, j) + 10.0 * f(i, j) - 18.0 * f(i - 1, j) + 6.0 * f(i - 2, j) - f(i - 3, j)) / 3.0;
            else
                d(i, j) = -0.25 * idr * (3.0 * f(i - 1, j) + 10.0 * f(i, j) - 18.0 * f(i + 1, j) + 6.0 * f(i + 2, j) - f(i + 3, j)) / 3.0;
        }
        int i = 3 - g;
        if (beta_r(i, j) <= 0.0)
            d(i, j) = 0.25 * idr * (8.0 * (f(i + 1, j) - f(i - 1, j)) - (f(i + 2, j) - f(i - 2, j))) / 3.0;
        else
            d(i, j) = -0.25 * idr * (3.0 * f(i - 1, j) + 10.0 * f(i, j) - 18.0 * f(i + 1, j) + 6.0 * f(i + 2, j) - f(i + 3, j)) / 3.0;
        i = 2 - g;
        d(i, j) = -0.25 * idr * (3.0 * f(i - 1, j) + 10.0 * f(i, j) - 18.0 * f(i + 1, j) + 6.0 * f(i + 2, j) - f(i + 3, j)) / 3.0;
        i = 1 - g;
        d(i, j) = -0.25 * idr * (25.0 * f(i, j) - 48.0 * f(i + 1, j) + 36.0 * f(i + 2, j) - 16.0 * f(i + 3, j) + 3.0 * f(i + 4, j)) / 3.0;
        i = Nr - 2;
        if (beta_r(i, j) <= 0.0)
            d(i, j) = 0.25 * idr * (3.0 * f(i + 1, j) + 10.0 * f(i, j) - 18.0 * f(i - 1, j) + 6.0 * f(i - 2, j) - f(i - 3, j)) / 3.0;
        else
            d(i, j) = 0.25 * idr * (8.0 * (f(i + 1, j) - f(i - 1, j)) - (f(i + 2, j) - f(i - 2, j))) / 3.0;
        i = Nr - 1;
        d(i, j) = 0.25 * idr * (3.0 * f(i + 1, j) + 10.0 * f(i, j) - 18.0 * f(i - 1, j) + 6.0 * f(i - 2, j) - f(i - 3, j)) / 3.0;
        i = Nr;
        d(i, j) = 0.25 * idr * (25.0 * f(i, j) - 48.0 * f(i - 1, j) + 36.0 * f(i - 2, j) - 16.0 * f(i - 3, j) + 3.0 * f(i - 4, j)) / 3.0;
        if (L.ownaxis)
            for (int ii = 1; ii <= g; ++ii) d(1 - ii, j) = -symr * d(ii, j);
    }
}

void diffadvz(Level& L, const Arr& f, Arr& d, int symz) {
    GRID_DIMS;
    const Arr& beta_z = L.a("beta_z");
    const double idz = 1.0 / L.dz;
    if (L.order == 2) {
        // derivadvect.f90:249-299
        const double hidz = 0.5 * idz;
#pragma omp parallel for schedule(static)
        for (int j = 3 - g; j <= Nz - 2; ++j)
            for (int i = 1 - g; i <= Nr; ++i) {
                if (beta_z(i, j) <= 0.0) d(i, j) = +hidz * (3.0 * f(i, j) - 4.0 * f(i, j - 1) + f(i, j - 2));
                else d(i, j) = -hidz * (3.0 * f(i, j) - 4.0 * f(i, j + 1) + f(i, j + 2));
            }
#pragma omp parallel for schedule(static)
        for (int i = 1 - g; i <= Nr; ++i) {
            int j = 2 - g;
            if (beta_z(i, j) <= 0.0) d(i, j) = hidz * (f(i, j + 1) - f(i, j - 1));
            else d(i, j) = -hidz * (3.0 * f(i, j) - 4.0 * f(i, j + 1) + f(i, j + 2));
            j = 1 - g;
            d(i, j) = -hidz * (3.0 * f(i, j) - 4.0 * f(i, j + 1) + f(i, j + 2));
            j = Nz - 1;
            if (beta_z(i, j) <= 0.0) d(i, j) = hidz * (3.0 * f(i, j) - 4.0 * f(i, j - 1) + f(i, j - 2));
            else d(i, j) = hidz * (f(i, j + 1) - f(i, j - 1));
            j = Nz;
            d(i, j) = hidz * (3.0 * f(i, j) - 4.0 * f(i, j - 1) + f(i, j - 2));
            if (L.eqsym && L.ownequator)
                for (int jj = 1; jj <= g; ++jj) d(i, 1 - jj) = -symz * d(i, jj);
        }
        return;
    }
#pragma omp parallel for schedule(static)
    for (int j = 4 - g; j <= Nz - 3; ++j)
        for (int i = 1 - g; i <= Nr; ++i) {
            if (beta_z(i, j) <= 0.0)
                d(i, j) = +0.25 * idz * (3.0 * f(i, j + 1) + 10.0 * f(i, j) - 18.0 * f(i, j - 1) + 6.0 * f(i, j - 2) - f(i, j - 3)) / 3.0;
            else
                d(i, j) = -0.25 * idz * (3.0 * f(i, j - 1) + 10.0 * f(i, j) - 18.0 * f(i, j + 1) + 6.0 * f(i, j + 2) - f(i, j + 3)) / 3.0;
        }
#pragma omp parallel for schedule(static)
    for (int i = 1 - g; i <= Nr; ++i) {
        int j = 3 - g;
        if (beta_z(i, j) <= 0.0)
            d(i, j) = -0.25 * idz * (3.0 * f(i, j - 1) + 10.0 * f(i, j) - 18.0 * f(i, j + 1) + 6.0 * f(i, j + 2) - f(i, j + 3)) / 3.0;
        else
            d(i, j) = 0.25 * idz * (8.0 * (f(i, j + 1) - f(i, j - 1)) - (f(i, j + 2) - f(i, j - 2))) / 3.0;
        j = 2 - g;
        d(i, j) = -0.25 * idz * (3.0 * f(i, j - 1) + 10.0 * f(i, j) - 18.0 * f(i, j + 1) + 6.0 * f(i, j + 2) - f(i, j + 3)) / 3.0;
        j = 1 - g;
        d(i, j) = -0.25 * idz * (25.0 * f(i, j) - 48.0 * f(i, j + 1) + 36.0 * f(i, j + 2) - 16.0 * f(i, j + 3) + 3.0 * f(i, j + 4)) / 3.0;
        j = Nz - 2;
        if (beta_z(i, j) <= 0.0)
            d(i, j) = 0.25 * idz * (3.0 * f(i, j + 1) + 10.0 * f(i, j) - 18.0 * f(i, j - 1) + 6.0 * f(i, j - 2) - f(i, j - 3)) / 3.0;
        else
            d(i, j) = 0.25 * idz * (8.0 * (f(i, j + 1) - f(i, j - 1)) - (f(i, j + 2) - f(i, j - 2))) / 3.0;
        j = Nz - 1;
        d(i, j) = 0.25 * idz * (3.0 * f(i, j + 1) + 10.0 * f(i, j) - 18.0 * f(i, j - 1) + 6.0 * f(i, j - 2) - f(i, j - 3)) / 3.0;
        j = Nz;
        d(i, j) = 0.25 * idz * (25.0 * f(i, j) - 48.0 * f(i, j - 1) + 36.0 * f(i, j - 2) - 16.0 * f(i, j - 3) + 3.0 * f(i, j - 4)) / 3.0;
        if (L.eqsym && L.ownequator)
            for (int jj = 1; jj <= g; ++jj) d(i, 1 - jj) = -symz * d(i, jj);
    }
}

// ---------------------------------------------------------------------------
// dissipation.f90: KO D^6 (order four) or D^4 (order two) in r then z, then
// symmetry fill
// ---------------------------------------------------------------------------
void dissipation(Level& L, const Arr& ev, Arr& src, int symr, int symz, double diss) {
    GRID_DIMS;
    const double idt = 1.0 / L.dt;
    if (L.order == 2) {
        // dissipation.f90:121-135: D^4 in r, then in z (the mixed operator is
        // commented out in the reference)
#pragma omp parallel for schedule(static)
        for (int j = 1 - g; j <= Nz; ++j)
            for (int i = 3 - g; i <= Nr - 2; ++i)
                src(i, j) = src(i, j) - diss * idt * (6.0 * ev(i, j) - 4.0 * (ev(i + 1, j) + ev(i - 1, j))
                                                      + (ev(i + 2, j) + ev(i - 2, j))) / 6.0;
#pragma omp parallel for schedule(static)
        for (int j = 3 - g; j <= Nz - 2; ++j)
            for (int i = 1 - g; i <= Nr; ++i)
                src(i, j) = src(i, j) - diss * idt * (6.0 * ev(i, j) - 4.0 * (ev(i, j + 1) + ev(i, j - 1))
                                                      + (ev(i, j + 2) + ev(i, j - 2))) / 6.0;
    } else {
#pragma omp parallel for schedule(static)
    for (int j = 1 - g; j <= Nz; ++j)
        for (int i = 4 - g; i <= Nr - 3; ++i)
            src(i, j) = src(i, j) - diss * idt * (20.0 * ev(i, j) - 15.0 * (ev(i + 1, j) + ev(i - 1, j))
                                                  + 6.0 * (ev(i + 2, j) + ev(i - 2, j)) - (ev(i + 3, j) + ev(i - 3, j))) / 20.0;
#pragma omp parallel for schedule(static)
    for (int j = 4 - g; j <= Nz - 3; ++j)
        for (int i = 1 - g; i <= Nr; ++i)
            src(i, j) = src(i, j) - diss * idt * (20.0 * ev(i, j) - 15.0 * (ev(i, j + 1) + ev(i, j - 1))
                                                  + 6.0 * (ev(i, j + 2) + ev(i, j - 2)) - (ev(i, j + 3) + ev(i, j - 3))) / 20.0;
    }
    if (L.eqsym && L.ownequator)
        for (int jj = 1; jj <= g; ++jj)
            for (int i = 1 - g; i <= Nr; ++i) src(i, 1 - jj) = symz * src(i, jj);
    if (L.ownaxis)
        for (int j = 1 - g; j <= Nz; ++j)
            for (int ii = 1; ii <= g; ++ii) src(1 - ii, j) = symr * src(ii, j);
}

// radbound.f90: outgoing-wave condition written into the source on the
// outer edges
void radbound(Level& L, const Arr& ev, Arr& src, const Arr& Dr_var, const Arr& Dz_var, double v, double var0) {
    GRID_DIMS;
    R(r); R(z); R(rr);
    {
        int i = Nr;
        for (int j = 1 - g; j <= Nz; ++j)
            src(i, j) = -v * (r(i, j) * Dr_var(i, j) + z(i, j) * Dz_var(i, j) + (ev(i, j) - var0)) / rr(i, j);
    }
    {
        int j = Nz;
        for (int i = 1 - g; i <= Nr; ++i)
            src(i, j) = -v * (r(i, j) * Dr_var(i, j) + z(i, j) * Dz_var(i, j) + (ev(i, j) - var0)) / rr(i, j);
    }
    if (!L.eqsym) {
        int j = 1 - g;
        for (int i = 1 - g; i <= Nr; ++i)
            src(i, j) = -v * (r(i, j) * Dr_var(i, j) + z(i, j) * Dz_var(i, j) + (ev(i, j) - var0)) / rr(i, j);
    }
}

// ---------------------------------------------------------------------------
// factordet.f90:2-76 (non-angmom): rescale A,B,C,H to the stored hdet
// ---------------------------------------------------------------------------
static void factordet(Level& L) {
    GRID_DIMS;
    R(A); R(B); R(C); R(H); R(r); R(hdet); R(auxarray);
    const double third = 1.0 / 3.0;
    ALL auxarray(i, j) = (A(i, j) * B(i, j) - p2(r(i, j) * C(i, j))) * H(i, j);
    ALL auxarray(i, j) = auxarray(i, j) / hdet(i, j);
    ALL auxarray(i, j) = std::pow(auxarray(i, j), third);
    ALL A(i, j) = A(i, j) / auxarray(i, j);
    ALL B(i, j) = B(i, j) / auxarray(i, j);
    ALL C(i, j) = C(i, j) / auxarray(i, j);
    ALL H(i, j) = H(i, j) / auxarray(i, j);
}

// ---------------------------------------------------------------------------
// auxiliary_geometry.f90 (non-angmom, bssn) with calc_conformalRicci1-4 and
// calc_DIVKTA
// ---------------------------------------------------------------------------
void auxiliary_geometry(Sim& S, Level& L) {
    GRID_DIMS;
    const ollin_params& P = S.P;
    const bool shift = P.shift != OLLIN_SHIFT_NONE;
    const bool adv = P.shiftadvect != 0;
    const double zero = 0.0, one = 1.0, two = 2.0, four = 4.0, half = 0.5, third = 1.0 / 3.0;
    const double fourth = half * half;
    const double time = L.time;
    const double cp = (double)P.chipower;
    const double *ft = P.ft;  // ft[0]=ft1 ...
    R(r); R(z); R(auxarray);
    R(alpha); R(dtalpha); R(phi); R(chi); R(A); R(B); R(H); R(C);
    R(trK); R(KTA); R(KTB); R(KTH); R(KTC); R(Delta_r); R(Delta_z);
    R(lambda); R(Alambda); R(z4theta);

    // ---- lapse (auxiliary_geometry.f90:49-97)
    R(Dr_alpha); R(Dz_alpha); R(Drr_alpha); R(Dzz_alpha); R(Drz_alpha); R(DD_alphar);
    diff1r(L, alpha, Dr_alpha, +1);
    diff1z(L, alpha, Dz_alpha, +1);
    diff2r(L, alpha, Drr_alpha, +1);
    diff2z(L, alpha, Dzz_alpha, +1);
    diff2rz(L, alpha, Drz_alpha, +1, +1);
    if (shift) {
        R(DAr_alpha); R(DAz_alpha);
        if (adv) { diffadvr(L, alpha, DAr_alpha, +1); diffadvz(L, alpha, DAz_alpha, +1); }
        else { DAr_alpha = Dr_alpha; DAz_alpha = Dz_alpha; }
    }
    {
        R(Dr_dtalpha); R(Dz_dtalpha);
        diff1r(L, dtalpha, Dr_dtalpha, +1);
        diff1z(L, dtalpha, Dz_dtalpha, +1);
        if (shift) {
            R(DAr_dtalpha); R(DAz_dtalpha);
            if (adv) { diffadvr(L, dtalpha, DAr_dtalpha, +1); diffadvz(L, dtalpha, DAz_dtalpha, +1); }
            else { DAr_dtalpha = Dr_dtalpha; DAz_dtalpha = Dz_dtalpha; }
        }
    }
    ALL auxarray(i, j) = Dr_alpha(i, j) / r(i, j);
    diff1r(L, auxarray, DD_alphar, +1);

    // ---- Bona-Masso function (:100-168)
    R(falpha);
    switch (P.slicing) {
        case OLLIN_SLICING_STATIC:
        case OLLIN_SLICING_MAXIMAL: ALL falpha(i, j) = 0.0; break;
        case OLLIN_SLICING_HARMONIC: ALL falpha(i, j) = p2(alpha(i, j)) * P.gauge_f; break;
        case OLLIN_SLICING_1PLUSLOG: ALL falpha(i, j) = alpha(i, j) * P.gauge_f; break;
        case OLLIN_SLICING_SHOCKAVOID: ALL falpha(i, j) = p2(alpha(i, j)) + (P.gauge_f - 1.0); break;
    }

    // ---- conformal factor (:171-250); chimethod
    R(Dr_phi); R(Dz_phi); R(Drr_phi); R(Dzz_phi); R(Drz_phi);
    R(Dr_chi); R(Dz_chi); R(Drr_chi); R(Dzz_chi); R(Drz_chi);
    if (!P.chimethod || time == zero) {
        ALL chi(i, j) = std::exp(-cp * phi(i, j));
        diff1r(L, phi, Dr_phi, +1);
        diff1z(L, phi, Dz_phi, +1);
        diff2r(L, phi, Drr_phi, +1);
        diff2z(L, phi, Dzz_phi, +1);
        diff2rz(L, phi, Drz_phi, +1, +1);
        if (shift) {
            R(DAr_phi); R(DAz_phi);
            if (adv) { diffadvr(L, phi, DAr_phi, +1); diffadvz(L, phi, DAz_phi, +1); }
            else { DAr_phi = Dr_phi; DAz_phi = Dz_phi; }
        }
    } else {
        ALL phi(i, j) = -std::log(chi(i, j)) / cp;
        diff1r(L, chi, Dr_chi, +1);
        diff1z(L, chi, Dz_chi, +1);
        diff2r(L, chi, Drr_chi, +1);
        diff2z(L, chi, Dzz_chi, +1);
        diff2rz(L, chi, Drz_chi, +1, +1);
        ALL Dr_phi(i, j) = -Dr_chi(i, j) / chi(i, j) / cp;
        ALL Dz_phi(i, j) = -Dz_chi(i, j) / chi(i, j) / cp;
        ALL Drr_phi(i, j) = -(Drr_chi(i, j) / chi(i, j) - p2(Dr_chi(i, j) / chi(i, j))) / cp;
        ALL Dzz_phi(i, j) = -(Dzz_chi(i, j) / chi(i, j) - p2(Dz_chi(i, j) / chi(i, j))) / cp;
        ALL Drz_phi(i, j) = -(Drz_chi(i, j) / chi(i, j) - Dr_chi(i, j) * Dz_chi(i, j) / p2(chi(i, j))) / cp;
        if (shift) {
            R(DAr_chi); R(DAz_chi); R(DAr_phi); R(DAz_phi);
            if (adv) { diffadvr(L, chi, DAr_chi, +1); diffadvz(L, chi, DAz_chi, +1); }
            else { DAr_chi = Dr_chi; DAz_chi = Dz_chi; }
            ALL DAr_phi(i, j) = -DAr_chi(i, j) / chi(i, j) / cp;
            ALL DAz_phi(i, j) = -DAz_chi(i, j) / chi(i, j) / cp;
        }
    }
    R(psi); R(psi2); R(psi4); R(DD_phir);
    ALL psi(i, j) = std::exp(phi(i, j));
    ALL psi2(i, j) = p2(psi(i, j));
    ALL psi4(i, j) = p4(psi(i, j));
    ALL auxarray(i, j) = Dr_phi(i, j) / r(i, j);
    diff1r(L, auxarray, DD_phir, +1);

    // ---- determinant of the conformal metric (:253-318)
    R(hdet); R(ihdet); R(Dr_hdet); R(Dz_hdet);
    if (time == zero && P.factorhdet) {
        ALL hdet(i, j) = one;
        ALL ihdet(i, j) = one;
        ALL Dr_hdet(i, j) = zero;
        ALL Dz_hdet(i, j) = zero;
    } else if (time == zero || !P.lagrangian) {
        ALL hdet(i, j) = (A(i, j) * B(i, j) - p2(r(i, j) * C(i, j))) * H(i, j);
        ALL ihdet(i, j) = one / hdet(i, j);
        diff1r(L, hdet, Dr_hdet, +1);
        diff1z(L, hdet, Dz_hdet, +1);
    } else {
        if (!P.evolveH) {
            ALL H(i, j) = hdet(i, j) / (A(i, j) * B(i, j) - p2(r(i, j) * C(i, j)));
        } else {
            factordet(L);
        }
    }

    // ---- conformal metric derivatives (:321-396)
    struct MD { const char* f; int sr, sz; };
    const MD mds[4] = {{"A", +1, +1}, {"B", +1, +1}, {"H", +1, +1}, {"C", +1, -1}};
    for (const MD& m : mds) {
        std::string n(m.f);
        Arr& F = L.a(n);
        diff1r(L, F, L.a("Dr_" + n), m.sr);
        diff1z(L, F, L.a("Dz_" + n), m.sz);
        diff2r(L, F, L.a("Drr_" + n), m.sr);
        diff2z(L, F, L.a("Dzz_" + n), m.sz);
        diff2rz(L, F, L.a("Drz_" + n), m.sr, m.sz);
        if (shift) {
            if (adv) { diffadvr(L, F, L.a("DAr_" + n), m.sr); diffadvz(L, F, L.a("DAz_" + n), m.sz); }
            else { L.a("DAr_" + n) = L.a("Dr_" + n); L.a("DAz_" + n) = L.a("Dz_" + n); }
        }
    }
    R(Dr_A); R(Dz_A); R(Drr_A); R(Dzz_A); R(Drz_A);
    R(Dr_B); R(Dz_B); R(Drr_B); R(Dzz_B); R(Drz_B);
    R(Dr_H); R(Dz_H); R(Drr_H); R(Dzz_H); R(Drz_H);
    R(Dr_C); R(Dz_C); R(Drr_C); R(Dzz_C); R(Drz_C);

    // ---- inverse conformal metric (:454-519)
    R(g_A); R(g_B); R(g_H); R(g_C);
    ALL g_A(i, j) = B(i, j) * H(i, j) * ihdet(i, j);
    ALL g_B(i, j) = A(i, j) * H(i, j) * ihdet(i, j);
    ALL g_H(i, j) = one / H(i, j);
    ALL g_C(i, j) = -C(i, j) * H(i, j) * ihdet(i, j);
    R(Dr_g_A); R(Dz_g_A); R(Dr_g_B); R(Dz_g_B); R(Dr_g_H); R(Dz_g_H); R(Dr_g_C); R(Dz_g_C);
    diff1r(L, g_A, Dr_g_A, +1); diff1z(L, g_A, Dz_g_A, +1);
    diff1r(L, g_B, Dr_g_B, +1); diff1z(L, g_B, Dz_g_B, +1);
    diff1r(L, g_H, Dr_g_H, +1); diff1z(L, g_H, Dz_g_H, +1);
    diff1r(L, g_C, Dr_g_C, +1); diff1z(L, g_C, Dz_g_C, -1);

    // ---- shift (:583-737)
    if (shift) {
        R(beta_r); R(beta_z); R(dtbeta_r); R(dtbeta_z); R(fdriver);
        R(Dr_beta_r); R(Dz_beta_r); R(Drr_beta_r); R(Dzz_beta_r); R(Drz_beta_r);
        R(Dr_beta_z); R(Dz_beta_z); R(Drr_beta_z); R(Dzz_beta_z); R(Drz_beta_z);
        R(DAr_beta_r); R(DAz_beta_r); R(DAr_beta_z); R(DAz_beta_z);
        diff1r(L, beta_r, Dr_beta_r, -1); diff1z(L, beta_r, Dz_beta_r, +1);
        diff2r(L, beta_r, Drr_beta_r, -1); diff2z(L, beta_r, Dzz_beta_r, +1);
        diff2rz(L, beta_r, Drz_beta_r, -1, +1);
        if (adv) { diffadvr(L, beta_r, DAr_beta_r, -1); diffadvz(L, beta_r, DAz_beta_r, +1); }
        else { DAr_beta_r = Dr_beta_r; DAz_beta_r = Dz_beta_r; }
        diff1r(L, beta_z, Dr_beta_z, +1); diff1z(L, beta_z, Dz_beta_z, -1);
        diff2r(L, beta_z, Drr_beta_z, +1); diff2z(L, beta_z, Dzz_beta_z, -1);
        diff2rz(L, beta_z, Drz_beta_z, +1, -1);
        if (adv) { diffadvr(L, beta_z, DAr_beta_z, +1); diffadvz(L, beta_z, DAz_beta_z, -1); }
        else { DAr_beta_z = Dr_beta_z; DAz_beta_z = Dz_beta_z; }
        R(Dr_fdriver); R(Dz_fdriver); R(DAr_fdriver); R(DAz_fdriver);
        diff1r(L, fdriver, Dr_fdriver, +1); diff1z(L, fdriver, Dz_fdriver, +1);
        if (adv) { diffadvr(L, fdriver, DAr_fdriver, +1); diffadvz(L, fdriver, DAz_fdriver, +1); }
        else { DAr_fdriver = Dr_fdriver; DAz_fdriver = Dz_fdriver; }
        R(DD_beta_rr);
        ALL auxarray(i, j) = beta_r(i, j) / r(i, j);
        diff1r(L, auxarray, DD_beta_rr, +1);
        R(Dr_dtbeta_r); R(Dz_dtbeta_r); R(DAr_dtbeta_r); R(DAz_dtbeta_r);
        diff1r(L, dtbeta_r, Dr_dtbeta_r, -1); diff1z(L, dtbeta_r, Dz_dtbeta_r, +1);
        if (adv) { diffadvr(L, dtbeta_r, DAr_dtbeta_r, -1); diffadvz(L, dtbeta_r, DAz_dtbeta_r, +1); }
        else { DAr_dtbeta_r = Dr_dtbeta_r; DAz_dtbeta_r = Dz_dtbeta_r; }
        R(Dr_dtbeta_z); R(Dz_dtbeta_z); R(DAr_dtbeta_z); R(DAz_dtbeta_z);
        diff1r(L, dtbeta_z, Dr_dtbeta_z, +1); diff1z(L, dtbeta_z, Dz_dtbeta_z, -1);
        if (adv) { diffadvr(L, dtbeta_z, DAr_dtbeta_z, +1); diffadvz(L, dtbeta_z, DAz_dtbeta_z, -1); }
        else { DAr_dtbeta_z = Dr_dtbeta_z; DAz_dtbeta_z = Dz_dtbeta_z; }
        R(DIV_beta); R(Dr_DIV_beta); R(Dz_DIV_beta);
        ALL DIV_beta(i, j) = Dr_beta_r(i, j) + Dz_beta_z(i, j) + beta_r(i, j) / r(i, j);
        ALL Dr_DIV_beta(i, j) = Drr_beta_r(i, j) + Drz_beta_z(i, j) + DD_beta_rr(i, j);
        ALL Dz_DIV_beta(i, j) = Drz_beta_r(i, j) + Dzz_beta_z(i, j) + Dz_beta_r(i, j) / r(i, j);
    }

    // ---- KTH from tracelessness (:740-756)
    ALL KTH(i, j) = -(g_A(i, j) * KTA(i, j) + g_B(i, j) * KTB(i, j) + two * p2(r(i, j)) * g_C(i, j) * KTC(i, j)) / g_H(i, j);

    // ---- lambdas (:759-821)
    R(lamDef); R(AlamDef);
    ALL lamDef(i, j) = (A(i, j) - H(i, j)) / p2(r(i, j));
    ALL AlamDef(i, j) = (KTA(i, j) - KTH(i, j)) / p2(r(i, j));
    if (P.nolambda || time == zero) {
        ALL lambda(i, j) = lamDef(i, j);
        ALL Alambda(i, j) = AlamDef(i, j);
    }
    R(Dr_lambda); R(Dz_lambda); R(Drr_lambda); R(Dzz_lambda); R(Drz_lambda);
    diff1r(L, lambda, Dr_lambda, +1); diff1z(L, lambda, Dz_lambda, +1);
    diff2r(L, lambda, Drr_lambda, +1); diff2z(L, lambda, Dzz_lambda, +1);
    diff2rz(L, lambda, Drz_lambda, +1, +1);
    if (shift) {
        R(DAr_lambda); R(DAz_lambda);
        if (adv) { diffadvr(L, lambda, DAr_lambda, +1); diffadvz(L, lambda, DAz_lambda, +1); }
        else { DAr_lambda = Dr_lambda; DAz_lambda = Dz_lambda; }
    }
    R(Dr_Alambda); R(Dz_Alambda);
    diff1r(L, Alambda, Dr_Alambda, +1); diff1z(L, Alambda, Dz_Alambda, +1);
    if (shift) {
        R(DAr_Alambda); R(DAz_Alambda);
        if (adv) { diffadvr(L, Alambda, DAr_Alambda, +1); diffadvz(L, Alambda, DAz_Alambda, +1); }
        else { DAr_Alambda = Dr_Alambda; DAz_Alambda = Dz_Alambda; }
    }
    R(g_lamDef); R(g_lambda);
    ALL g_lamDef(i, j) = (g_A(i, j) - g_H(i, j)) / p2(r(i, j));
    ALL g_lambda(i, j) = (p2(C(i, j)) - B(i, j) * lambda(i, j)) * ihdet(i, j);

    // ---- extrinsic curvature derivatives (:824-940)
    {
        const MD kds[5] = {{"trK", +1, +1}, {"KTA", +1, +1}, {"KTB", +1, +1}, {"KTH", +1, +1}, {"KTC", +1, -1}};
        for (const MD& m : kds) {
            std::string n(m.f);
            Arr& F = L.a(n);
            diff1r(L, F, L.a("Dr_" + n), m.sr);
            diff1z(L, F, L.a("Dz_" + n), m.sz);
            if (shift) {
                if (adv) { diffadvr(L, F, L.a("DAr_" + n), m.sr); diffadvz(L, F, L.a("DAz_" + n), m.sz); }
                else { L.a("DAr_" + n) = L.a("Dr_" + n); L.a("DAz_" + n) = L.a("Dz_" + n); }
            }
        }
    }
    R(KT_up_rr); R(KT_up_zz); R(KT_up_pp); R(KT_up_rz);
    ALL KT_up_rr(i, j) = (2.0 * g_A(i, j) * g_C(i, j) * KTC(i, j) + p2(g_C(i, j)) * KTB(i, j)) * p2(r(i, j)) + p2(g_A(i, j)) * KTA(i, j);
    ALL KT_up_zz(i, j) = (p2(g_C(i, j)) * KTA(i, j) + 2.0 * g_C(i, j) * g_B(i, j) * KTC(i, j)) * p2(r(i, j)) + p2(g_B(i, j)) * KTB(i, j);
    ALL KT_up_pp(i, j) = p2(g_H(i, j)) / p2(r(i, j)) * KTH(i, j);
    ALL KT_up_rz(i, j) = p2(g_C(i, j)) * p3(r(i, j)) * KTC(i, j)
        + (g_C(i, j) * g_A(i, j) * KTA(i, j) + g_B(i, j) * g_A(i, j) * KTC(i, j) + g_B(i, j) * g_C(i, j) * KTB(i, j)) * r(i, j);
    R(KT2_A); R(KT2_B); R(KT2_H); R(KT2_C); R(KT2_lambda); R(KT2); R(K2);
    ALL KT2_A(i, j) = (2.0 * KTA(i, j) * g_C(i, j) * KTC(i, j) + p2(KTC(i, j)) * g_B(i, j)) * p2(r(i, j)) + g_A(i, j) * p2(KTA(i, j));
    ALL KT2_B(i, j) = (p2(KTC(i, j)) * g_A(i, j) + 2.0 * KTC(i, j) * g_C(i, j) * KTB(i, j)) * p2(r(i, j)) + g_B(i, j) * p2(KTB(i, j));
    ALL KT2_H(i, j) = p2(KTH(i, j)) * g_H(i, j);
    ALL KT2_C(i, j) = p2(KTC(i, j)) * g_C(i, j) * p2(r(i, j)) + KTA(i, j) * g_A(i, j) * KTC(i, j)
        + KTA(i, j) * g_C(i, j) * KTB(i, j) + KTC(i, j) * g_B(i, j) * KTB(i, j);
    ALL KT2_lambda(i, j) = 2.0 * KTA(i, j) * g_C(i, j) * KTC(i, j) + p2(KTC(i, j)) * g_B(i, j)
        + ft[2] * (g_lambda(i, j) * p2(KTA(i, j)) + g_H(i, j) * Alambda(i, j) * (KTA(i, j) + KTH(i, j)))
        + (1.0 - ft[2]) * (g_lambda(i, j) * p2(KTH(i, j)) + g_A(i, j) * Alambda(i, j) * (KTA(i, j) + KTH(i, j)));
    ALL KT2(i, j) = g_A(i, j) * KT2_A(i, j) + g_B(i, j) * KT2_B(i, j) + g_H(i, j) * KT2_H(i, j) + two * g_C(i, j) * KT2_C(i, j) * p2(r(i, j));
    ALL K2(i, j) = KT2(i, j) + third * p2(trK(i, j) + two * z4theta(i, j));

    // ---- BSSN Delta (:1053-1186)
    R(DelDef_r); R(DelDef_z);
    ALL DelDef_r(i, j) = -Dr_g_A(i, j) - r(i, j) * Dz_g_C(i, j) - r(i, j) * g_lambda(i, j)
        - half * (g_A(i, j) * Dr_hdet(i, j) + r(i, j) * g_C(i, j) * Dz_hdet(i, j)) * ihdet(i, j);
    ALL DelDef_z(i, j) = -Dr_g_C(i, j) * r(i, j) - Dz_g_B(i, j) - two * g_C(i, j)
        - half * (r(i, j) * g_C(i, j) * Dr_hdet(i, j) + g_B(i, j) * Dz_hdet(i, j)) * ihdet(i, j);
    if (time == zero) {
        ALL Delta_r(i, j) = DelDef_r(i, j);
        ALL Delta_z(i, j) = DelDef_z(i, j);
        R(Delta0_r); R(Delta0_z);
        ALL Delta0_r(i, j) = Delta_r(i, j);
        ALL Delta0_z(i, j) = Delta_z(i, j);
    }
    R(Dr_Delta_r); R(Dz_Delta_r); R(Dr_Delta_z); R(Dz_Delta_z);
    diff1r(L, Delta_r, Dr_Delta_r, -1); diff1z(L, Delta_r, Dz_Delta_r, +1);
    if (shift) {
        R(DAr_Delta_r); R(DAz_Delta_r);
        if (adv) { diffadvr(L, Delta_r, DAr_Delta_r, -1); diffadvz(L, Delta_r, DAz_Delta_r, +1); }
        else { DAr_Delta_r = Dr_Delta_r; DAz_Delta_r = Dz_Delta_r; }
    }
    diff1r(L, Delta_z, Dr_Delta_z, +1); diff1z(L, Delta_z, Dz_Delta_z, -1);
    if (shift) {
        R(DAr_Delta_z); R(DAz_Delta_z);
        if (adv) { diffadvr(L, Delta_z, DAr_Delta_z, +1); diffadvz(L, Delta_z, DAz_Delta_z, -1); }
        else { DAr_Delta_z = Dr_Delta_z; DAz_Delta_z = Dz_Delta_z; }
    }
    R(DD_Delta_rr);
    ALL auxarray(i, j) = Delta_r(i, j) / r(i, j);
    diff1r(L, auxarray, DD_Delta_rr, +1);
    R(V_r); R(V_z);
    ALL V_r(i, j) = -Dr_g_A(i, j) - r(i, j) * Dz_g_C(i, j) - r(i, j) * g_lambda(i, j)
        - (g_A(i, j) * Dr_hdet(i, j) + r(i, j) * g_C(i, j) * Dz_hdet(i, j)) * ihdet(i, j);
    ALL V_z(i, j) = -Dr_g_C(i, j) * r(i, j) - Dz_g_B(i, j) - two * g_C(i, j)
        - (r(i, j) * g_C(i, j) * Dr_hdet(i, j) + g_B(i, j) * Dz_hdet(i, j)) * ihdet(i, j);

    // ---- covariant derivatives of the lapse (:1266-1324), non-angmom
    R(D2cov_alpha_A); R(D2cov_alpha_B); R(D2cov_alpha_H); R(D2cov_alpha_C); R(D2cov_alpha_lambda); R(Lapla_alpha);
    ALL {
        const double rr_ = r(i, j);
        D2cov_alpha_A(i, j) = Drr_alpha(i, j) - Dr_alpha(i, j) * g_C(i, j) * p2(rr_) * Dr_C(i, j)
            - (Dz_alpha(i, j) * g_B(i, j) * Dr_C(i, j) + half * Dz_alpha(i, j) * g_C(i, j) * Dr_A(i, j)
               + Dr_alpha(i, j) * g_C(i, j) * C(i, j) - half * Dr_alpha(i, j) * g_C(i, j) * Dz_A(i, j)) * rr_
            - half * Dr_alpha(i, j) * g_A(i, j) * Dr_A(i, j) - Dz_alpha(i, j) * g_B(i, j) * C(i, j)
            + half * Dz_alpha(i, j) * g_B(i, j) * Dz_A(i, j);
        D2cov_alpha_B(i, j) = Dzz_alpha(i, j) - Dz_alpha(i, j) * g_C(i, j) * p2(rr_) * Dz_C(i, j)
            - (Dr_alpha(i, j) * g_A(i, j) * Dz_C(i, j) + half * Dr_alpha(i, j) * g_C(i, j) * Dz_B(i, j)
               - half * Dz_alpha(i, j) * g_C(i, j) * Dr_B(i, j)) * rr_
            + half * Dr_alpha(i, j) * g_A(i, j) * Dr_B(i, j) - half * Dz_alpha(i, j) * g_B(i, j) * Dz_B(i, j);
        D2cov_alpha_H(i, j) = -(-half * Dr_alpha(i, j) * g_C(i, j) * Dz_H(i, j) - half * Dz_alpha(i, j) * g_C(i, j) * Dr_H(i, j)) * rr_
            + half * Dr_alpha(i, j) * g_A(i, j) * Dr_H(i, j) + Dz_alpha(i, j) * g_C(i, j) * H(i, j)
            + half * Dz_alpha(i, j) * g_B(i, j) * Dz_H(i, j) + Dr_alpha(i, j) * g_A(i, j) * H(i, j) / rr_;
        D2cov_alpha_C(i, j) = Drz_alpha(i, j) / rr_ - half * Dr_alpha(i, j) * g_C(i, j) * Dr_B(i, j)
            - half * Dz_alpha(i, j) * g_C(i, j) * Dz_A(i, j)
            - (half * Dr_alpha(i, j) * g_A(i, j) * Dz_A(i, j) + half * Dz_alpha(i, j) * g_B(i, j) * Dr_B(i, j)) / rr_;
        D2cov_alpha_lambda(i, j) = (DD_alphar(i, j)) / rr_
            + Dr_alpha(i, j) / rr_ * (-ft[3] * g_lambda(i, j) * H(i, j) + (1.0 - ft[3]) * (g_C(i, j) * C(i, j) + g_A(i, j) * lambda(i, j)))
            - Dr_alpha(i, j) * g_C(i, j) * Dr_C(i, j)
            - (Dz_alpha(i, j) * g_B(i, j) * Dr_C(i, j) + Dr_alpha(i, j) * g_C(i, j) * C(i, j)
               - half * Dr_alpha(i, j) * g_C(i, j) * Dz_A(i, j) + half * Dz_alpha(i, j) * g_C(i, j) * Dr_A(i, j)
               + half * Dr_alpha(i, j) * g_C(i, j) * Dz_H(i, j) + half * Dz_alpha(i, j) * g_C(i, j) * Dr_H(i, j)) / rr_
            + half * Dz_alpha(i, j) * g_B(i, j) * Dz_lambda(i, j)
            - half * Dr_alpha(i, j) * g_A(i, j) * (Dr_A(i, j) + Dr_H(i, j)) / p2(rr_)
            + Dz_alpha(i, j) * lambda(i, j) * g_C(i, j);
    }
    ALL auxarray(i, j) = g_A(i, j) * Dr_alpha(i, j) * Dr_phi(i, j) + g_B(i, j) * Dz_alpha(i, j) * Dz_phi(i, j)
        + r(i, j) * g_C(i, j) * (Dr_alpha(i, j) * Dz_phi(i, j) + Dz_alpha(i, j) * Dr_phi(i, j));
    ALL D2cov_alpha_A(i, j) = D2cov_alpha_A(i, j) - two * (two * Dr_alpha(i, j) * Dr_phi(i, j) - A(i, j) * auxarray(i, j));
    ALL D2cov_alpha_B(i, j) = D2cov_alpha_B(i, j) - two * (two * Dz_alpha(i, j) * Dz_phi(i, j) - B(i, j) * auxarray(i, j));
    ALL D2cov_alpha_H(i, j) = D2cov_alpha_H(i, j) + two * H(i, j) * auxarray(i, j);
    ALL D2cov_alpha_C(i, j) = D2cov_alpha_C(i, j) - two * ((Dr_alpha(i, j) / r(i, j)) * Dz_phi(i, j)
                                                          + Dz_alpha(i, j) * (Dr_phi(i, j) / r(i, j)) - C(i, j) * auxarray(i, j));
    ALL D2cov_alpha_lambda(i, j) = D2cov_alpha_lambda(i, j) - two * (two * (Dr_alpha(i, j) / r(i, j)) * (Dr_phi(i, j) / r(i, j))
                                                                    - lambda(i, j) * auxarray(i, j));
    ALL Lapla_alpha(i, j) = g_A(i, j) * D2cov_alpha_A(i, j) + g_B(i, j) * D2cov_alpha_B(i, j) + g_H(i, j) * D2cov_alpha_H(i, j)
        + two * p2(r(i, j)) * g_C(i, j) * D2cov_alpha_C(i, j);
    ALL Lapla_alpha(i, j) = Lapla_alpha(i, j) / psi4(i, j);

    // ---- Ricci tensor (:1331-1493)
    R(RIC_A); R(RIC_B); R(RIC_H); R(RIC_C); R(RIC_lambda); R(RSCAL);
    ALL {
        const double rr_ = r(i, j);
        RIC_A(i, j) = -two * (Drr_phi(i, j) - Dr_phi(i, j) * g_C(i, j) * p2(rr_) * Dr_C(i, j)
            - (Dz_phi(i, j) * g_B(i, j) * Dr_C(i, j) + half * Dz_phi(i, j) * g_C(i, j) * Dr_A(i, j)
               + Dr_phi(i, j) * g_C(i, j) * C(i, j) - half * Dr_phi(i, j) * g_C(i, j) * Dz_A(i, j)) * rr_
            - half * Dr_phi(i, j) * g_A(i, j) * Dr_A(i, j) - Dz_phi(i, j) * g_B(i, j) * C(i, j)
            + half * Dz_phi(i, j) * g_B(i, j) * Dz_A(i, j));
        RIC_B(i, j) = -two * (Dzz_phi(i, j) - Dz_phi(i, j) * g_C(i, j) * p2(rr_) * Dz_C(i, j)
            - (Dr_phi(i, j) * g_A(i, j) * Dz_C(i, j) + half * Dr_phi(i, j) * g_C(i, j) * Dz_B(i, j)
               - half * Dz_phi(i, j) * g_C(i, j) * Dr_B(i, j)) * rr_
            + half * Dr_phi(i, j) * g_A(i, j) * Dr_B(i, j) - half * Dz_phi(i, j) * g_B(i, j) * Dz_B(i, j));
        RIC_H(i, j) = -two * (-(-half * Dr_phi(i, j) * g_C(i, j) * Dz_H(i, j) - half * Dz_phi(i, j) * g_C(i, j) * Dr_H(i, j)) * rr_
            + half * Dr_phi(i, j) * g_A(i, j) * Dr_H(i, j) + Dz_phi(i, j) * g_C(i, j) * H(i, j)
            + half * Dz_phi(i, j) * g_B(i, j) * Dz_H(i, j) + Dr_phi(i, j) * g_A(i, j) * H(i, j) / rr_);
        RIC_C(i, j) = -two * (Drz_phi(i, j) / rr_ - half * Dr_phi(i, j) * g_C(i, j) * Dr_B(i, j)
            - half * Dz_phi(i, j) * g_C(i, j) * Dz_A(i, j)
            - (half * Dr_phi(i, j) * g_A(i, j) * Dz_A(i, j) + half * Dz_phi(i, j) * g_B(i, j) * Dr_B(i, j)) / rr_);
        RIC_lambda(i, j) = -two * ((DD_phir(i, j)) / rr_
            + Dr_phi(i, j) / rr_ * (-ft[4] * g_lambda(i, j) * H(i, j) + (1.0 - ft[4]) * (g_C(i, j) * C(i, j) + g_A(i, j) * lambda(i, j)))
            - Dr_phi(i, j) * g_C(i, j) * Dr_C(i, j)
            - (Dz_phi(i, j) * g_B(i, j) * Dr_C(i, j) + Dr_phi(i, j) * g_C(i, j) * C(i, j)
               - half * Dr_phi(i, j) * g_C(i, j) * Dz_A(i, j) + half * Dz_phi(i, j) * g_C(i, j) * Dr_A(i, j)
               + half * Dr_phi(i, j) * g_C(i, j) * Dz_H(i, j) + half * Dz_phi(i, j) * g_C(i, j) * Dr_H(i, j)) / rr_
            + half * Dz_phi(i, j) * g_B(i, j) * Dz_lambda(i, j)
            - half * Dr_phi(i, j) * g_A(i, j) * (Dr_A(i, j) / rr_ + Dr_H(i, j) / rr_) / rr_
            + Dz_phi(i, j) * lambda(i, j) * g_C(i, j));
    }
    ALL auxarray(i, j) = g_A(i, j) * RIC_A(i, j) + g_B(i, j) * RIC_B(i, j) + g_H(i, j) * RIC_H(i, j) + two * p2(r(i, j)) * g_C(i, j) * RIC_C(i, j);
    ALL RIC_A(i, j) = RIC_A(i, j) + A(i, j) * auxarray(i, j);
    ALL RIC_B(i, j) = RIC_B(i, j) + B(i, j) * auxarray(i, j);
    ALL RIC_H(i, j) = RIC_H(i, j) + H(i, j) * auxarray(i, j);
    ALL RIC_C(i, j) = RIC_C(i, j) + C(i, j) * auxarray(i, j);
    ALL RIC_lambda(i, j) = RIC_lambda(i, j) + lambda(i, j) * auxarray(i, j);
    ALL RIC_A(i, j) = RIC_A(i, j) + four * (p2(Dr_phi(i, j)));
    ALL RIC_B(i, j) = RIC_B(i, j) + four * (p2(Dz_phi(i, j)));
    ALL RIC_C(i, j) = RIC_C(i, j) + four * (Dr_phi(i, j) * Dz_phi(i, j)) / r(i, j);
    ALL RIC_lambda(i, j) = RIC_lambda(i, j) + four * p2(Dr_phi(i, j) / r(i, j));
    ALL auxarray(i, j) = -two * (g_A(i, j) * Dr_phi(i, j) * Dr_phi(i, j) + g_B(i, j) * Dz_phi(i, j) * Dz_phi(i, j)
                                 + two * r(i, j) * g_C(i, j) * Dr_phi(i, j) * Dz_phi(i, j));
    ALL RIC_A(i, j) = RIC_A(i, j) + two * A(i, j) * auxarray(i, j);
    ALL RIC_B(i, j) = RIC_B(i, j) + two * B(i, j) * auxarray(i, j);
    ALL RIC_H(i, j) = RIC_H(i, j) + two * H(i, j) * auxarray(i, j);
    ALL RIC_C(i, j) = RIC_C(i, j) + two * C(i, j) * auxarray(i, j);
    ALL RIC_lambda(i, j) = RIC_lambda(i, j) + two * lambda(i, j) * auxarray(i, j);

    // calc_conformalRicci1.f90:74-92 (non-angmom)
    ALL {
        const double rr_ = r(i, j);
        RIC_A(i, j) = RIC_A(i, j) - g_C(i, j) * Drz_A(i, j) * rr_ - half * g_B(i, j) * Dzz_A(i, j) - half * g_A(i, j) * Drr_A(i, j)
            - half * g_H(i, j) * Dr_A(i, j) / rr_ + g_H(i, j) * lamDef(i, j);
        RIC_B(i, j) = RIC_B(i, j) - g_C(i, j) * Drz_B(i, j) * rr_ - half * g_A(i, j) * Drr_B(i, j) - half * g_B(i, j) * Dzz_B(i, j)
            - half * g_H(i, j) * Dr_B(i, j) / rr_;
        RIC_H(i, j) = RIC_H(i, j) - g_C(i, j) * Drz_H(i, j) * rr_ - half * g_B(i, j) * Dzz_H(i, j) - half * g_A(i, j) * Drr_H(i, j)
            - half * g_H(i, j) * Dr_H(i, j) / rr_ - g_H(i, j) * lamDef(i, j);
        RIC_C(i, j) = RIC_C(i, j) - g_C(i, j) * Drz_C(i, j) * rr_ - half * g_A(i, j) * Drr_C(i, j) - g_C(i, j) * Dz_C(i, j)
            - half * g_B(i, j) * Dzz_C(i, j) + (-g_A(i, j) * Dr_C(i, j) - half * g_H(i, j) * Dr_C(i, j)) / rr_;
        RIC_lambda(i, j) = RIC_lambda(i, j) - g_C(i, j) * (rr_ * Drz_lambda(i, j) + 2.0 * Dz_lambda(i, j))
            - half * g_B(i, j) * Dzz_lambda(i, j) - half * g_A(i, j) * Drr_lambda(i, j)
            - (2.0 * g_A(i, j) + half * g_H(i, j)) * Dr_lambda(i, j) / rr_;
    }
    // calc_conformalRicci2.f90:73-88 (non-angmom)
    ALL {
        const double rr_ = r(i, j);
        RIC_A(i, j) = RIC_A(i, j) + C(i, j) * Dr_Delta_z(i, j) * rr_ + A(i, j) * Dr_Delta_r(i, j)
            + half * (DelDef_r(i, j) * Dr_A(i, j) + DelDef_z(i, j) * Dz_A(i, j));
        RIC_B(i, j) = RIC_B(i, j) + C(i, j) * Dz_Delta_r(i, j) * rr_ + B(i, j) * Dz_Delta_z(i, j)
            + half * (DelDef_r(i, j) * Dr_B(i, j) + DelDef_z(i, j) * Dz_B(i, j));
        RIC_H(i, j) = RIC_H(i, j) + half * (DelDef_r(i, j) * Dr_H(i, j) + DelDef_z(i, j) * Dz_H(i, j)) + Delta_r(i, j) * H(i, j) / rr_;
        RIC_C(i, j) = RIC_C(i, j) + half * C(i, j) * (Dr_Delta_r(i, j) + Dz_Delta_z(i, j))
            + half * (DelDef_r(i, j) * Dr_C(i, j) + DelDef_z(i, j) * Dz_C(i, j))
            + half * (C(i, j) * Delta_r(i, j) + A(i, j) * Dz_Delta_r(i, j) + B(i, j) * Dr_Delta_z(i, j)) / rr_;
        RIC_lambda(i, j) = RIC_lambda(i, j) + (Dr_Delta_z(i, j) * C(i, j) + Delta_r(i, j) * lamDef(i, j)) / rr_
            + half * (DelDef_r(i, j) * Dr_lambda(i, j) + DelDef_z(i, j) * Dz_lambda(i, j))
            + ft[5] * (A(i, j) * DD_Delta_rr(i, j) + lamDef(i, j) * Delta_r(i, j)) / rr_
            + (1.0 - ft[5]) * (H(i, j) * DD_Delta_rr(i, j) / rr_ + lamDef(i, j) * Dr_Delta_r(i, j));
    }
    // calc_conformalRicci3.f90:314-357 (non-angmom)
    ALL {
        const double rr_ = r(i, j);
        const double gA = g_A(i, j), gB = g_B(i, j), gH = g_H(i, j), gC = g_C(i, j);
        const double dAr = Dr_A(i, j), dAz = Dz_A(i, j), dBr = Dr_B(i, j), dBz = Dz_B(i, j);
        const double dHr = Dr_H(i, j), dHz = Dz_H(i, j), dCr = Dr_C(i, j), dCz = Dz_C(i, j);
        const double Cc = C(i, j), Ac = A(i, j), Hc = H(i, j);
        RIC_A(i, j) = RIC_A(i, j) + (2.0 * gB * gC * dCr * dCz + p2(gC) * dAr * dCz + dAz * p2(gC) * dCr) * p3(rr_)
            + (2.0 * gB * gC * Cc * dCz - gB * gC * dCr * dBr + dAr * gC * gA * dCr + dAz * p2(gC) * Cc) * p2(rr_)
            + (dAz * gB * gC * dBr + dAz * gB * gA * dCr + dAr * gC * gA * Cc - gB * gC * Cc * dBr + dAz * gC * gA * dAr
               + p2(gB) * dBr * dCz) * rr_
            - half * p2(gH) * p2(dHr) - half * p2(gB) * p2(dBr) + gB * gA * Cc * dAz + half * p2(dAr) * p2(gA)
            + (gH * dHr + p2(gH) * Ac * dHr - 2.0 * p2(gH) * dHr * Hc) / rr_;
        RIC_B(i, j) = RIC_B(i, j) + (dBr * p2(gC) * dCz + p2(gC) * dBz * dCr + 2.0 * gA * gC * dCz * dCr) * p3(rr_)
            + (2.0 * gA * gC * dCz * Cc - gA * gC * dCz * dAz + p2(gC) * dBz * Cc + dBz * gC * gB * dCz) * p2(rr_)
            + (dBr * gA * gC * dAz + p2(gA) * dAz * dCr + dBr * gA * gB * dCz + dBr * gB * gC * dBz) * rr_
            + half * p2(gB) * p2(dBz) + p2(gA) * dAz * Cc - half * p2(gA) * p2(dAz) + p2(gH) * dHz * Cc - half * p2(gH) * p2(dHz);
        RIC_H(i, j) = RIC_H(i, j) - gC * dHz - rr_ * g_lambda(i, j) * dHr;
        RIC_C(i, j) = RIC_C(i, j) + (p2(gC) * dBr * dCr + gC * gB * p2(dCz) + dAz * p2(gC) * dCz + gC * gA * p2(dCr)) * p2(rr_)
            + (-half * gC * gA * dCr * dAz + 2.0 * gC * gA * dCr * Cc - half * p2(gC) * dBr * dAz - half * gC * gB * dCz * dBr
               + half * dBz * gB * gC * dCr + p2(gC) * dBr * Cc + half * dBz * p2(gC) * dAr + half * dAr * gA * gC * dCz) * rr_
            + half * dBr * gC * gA * dAr + half * dBr * gB * gA * dCr + half * p2(gB) * dBz * dCz + half * dAz * gA * gB * dCz
            + half * p2(gA) * dAr * dCr + half * p2(dBr) * gB * gC + gC * gA * p2(Cc) - half * gC * gA * Cc * dAz
            + half * dAz * gB * gC * dBz + half * p2(dAz) * gA * gC + half * dBz * gB * gC * Cc
            + (half * p2(gH) * Cc * dHr + half * gB * gA * dBr * Cc - half * p2(gH) * dHz * dHr + half * p2(gA) * dAr * Cc) / rr_
            + half * dHz * p2(gH) * lambda(i, j);
        const double gl = g_lambda(i, j), dlz = Dz_lambda(i, j);
        RIC_lambda(i, j) = RIC_lambda(i, j) + (two * gB * gC * dCr * dCz + p2(gC) * dAr * dCz + two * dAz * p2(gC) * dCr) * rr_
            + two * dAr * gC * gA * dCr + gB * gA * p2(dCr) + half * dAr * p2(gC) * dBr + two * dAz * p2(gC) * Cc
            + two * gB * gC * Cc * dCz - half * p2(dAz) * p2(gC)
            + (p2(gB) * dBr * dCz + dAz * gC * gA * dAr + half * Cc * gC * gH * dHr + dAz * gB * gC * dBr
               + two * gB * gA * dCr * Cc + two * dAr * gC * gA * Cc - gH * gC * dHz * dHr) / rr_
            + (-fourth * p2(gH) * p2(dHr) - fourth * p2(gB) * p2(dBr) + 3.0 * fourth * p2(dAr) * p2(gA)
               - half * gH * gA * p2(dHr)) / p2(rr_)
            + half * gB * (ft[6] * (gl * p2(dAz) + gH * dlz * (dAz + dHz)) + (1.0 - ft[6]) * (gA * dlz * (dAz + dHz) + gl * p2(dHz)))
            + p2(Cc) * p2(gC) - gH * (half * Cc * gC - gH * lambda(i, j)) * dHr / rr_;
    }
    // calc_conformalRicci4.f90:270-302 (non-angmom)
    ALL {
        const double rr_ = r(i, j);
        const double gA = g_A(i, j), gB = g_B(i, j), gH = g_H(i, j), gC = g_C(i, j);
        const double dAr = Dr_A(i, j), dAz = Dz_A(i, j), dBr = Dr_B(i, j), dBz = Dz_B(i, j);
        const double dHr = Dr_H(i, j), dHz = Dz_H(i, j), dCr = Dr_C(i, j), dCz = Dz_C(i, j);
        const double Cc = C(i, j), Ac = A(i, j), Hc = H(i, j);
        RIC_A(i, j) = RIC_A(i, j) + dAz * p2(gC) * dCr * p3(rr_)
            + (-half * p2(dAz) * p2(gC) + dAz * p2(gC) * Cc + gB * gA * p2(dCr) + half * dAr * p2(gC) * dBr + dAr * gC * gA * dCr
               + gB * gC * dCr * dBr) * p2(rr_)
            + (-dAz * gB * gA * dCr + 2.0 * gB * gA * dCr * Cc + gB * gC * Cc * dBr + dAr * gC * gA * Cc) * rr_
            + 1.0 * fourth * p2(gH) * p2(dHr) - gB * gA * Cc * dAz + fourth * p2(gB) * p2(dBr) + gB * gA * p2(Cc)
            + fourth * p2(dAr) * p2(gA) + half * gB * gA * p2(dAz);
        RIC_B(i, j) = RIC_B(i, j) + dBr * p2(gC) * p3(rr_) * dCz
            + (gA * gB * p2(dCz) + half * dAz * p2(gC) * dBz - half * p2(gC) * p2(dBr) + dBz * gC * gB * dCz + gA * gC * dCz * dAz) * p2(rr_)
            - dBr * gA * gB * dCz * rr_ + fourth * p2(gA) * p2(dAz) + half * gB * gA * p2(dBr) + fourth * p2(gH) * p2(dHz)
            + fourth * p2(gB) * p2(dBz);
        RIC_H(i, j) = RIC_H(i, j) + (-half * Cc * gC * gH * dHr + gH * gC * dHz * dHr) * rr_ + half * gH * p2(dHz) * gB
            + 3.0 * half * gC * dHz + half * gH * gA * p2(dHr) - half * Cc * gB * gH * dHz - half * gH * Ac * gC * dHz - Cc * gC
            - half * gC * dHz + half * (2.0 * gA - gH - gH * Ac * gA) * dHr / rr_ + gH * lambda(i, j) * (1.0 - gA * Hc);
        RIC_C(i, j) = RIC_C(i, j) + p2(gC) * dCr * dCz * p3(rr_)
            + (-half * dAz * p2(gC) * dCz + p2(gC) * Cc * dCz - half * p2(gC) * dBr * dCr) * p2(rr_)
            + (-half * p2(gC) * dBr * Cc + fourth * dBz * p2(gC) * dAr + half * dAr * gA * gC * dCz + half * gC * gB * dCz * dBr
               + 3.0 * fourth * p2(gC) * dBr * dAz + half * dBz * gB * gC * dCr + half * gC * gA * dCr * dAz) * rr_
            + half * dAz * gA * gB * dCz + half * dBz * gB * gC * Cc + half * gC * gA * Cc * dAz + half * dBr * gB * gA * dCr
            + (fourth * p2(gH) * dHz * dHr + half * gB * gA * dBr * Cc + fourth * p2(gA) * dAr * dAz + fourth * dBz * p2(gB) * dBr
               - half * gB * gA * dAz * dBr) / rr_;
    }
    ALL RSCAL(i, j) = g_A(i, j) * RIC_A(i, j) + g_B(i, j) * RIC_B(i, j) + g_H(i, j) * RIC_H(i, j) + two * p2(r(i, j)) * g_C(i, j) * RIC_C(i, j);
    ALL RSCAL(i, j) = RSCAL(i, j) / psi4(i, j);

    // ---- divergence of KT: calc_DIVKTA.f90:571-638 (non-angmom)
    R(DIV_KT_r); R(DIV_KT_z); R(DIVA_KT_r); R(DIVA_KT_z);
    R(Dr_KTA); R(Dz_KTA); R(Dr_KTB); R(Dz_KTB); R(Dr_KTC); R(Dz_KTC);
    ALL {
        const double rr_ = r(i, j);
        const double gA = g_A(i, j), gB = g_B(i, j), gH = g_H(i, j), gC = g_C(i, j);
        const double dAr = Dr_A(i, j), dAz = Dz_A(i, j), dBr = Dr_B(i, j), dBz = Dz_B(i, j);
        const double dHr = Dr_H(i, j), dHz = Dz_H(i, j), dCr = Dr_C(i, j), dCz = Dz_C(i, j);
        const double Cc = C(i, j), Ac = A(i, j);
        const double kA = KTA(i, j), kB = KTB(i, j), kH = KTH(i, j), kC = KTC(i, j);
        const double dkAr = Dr_KTA(i, j), dkAz = Dz_KTA(i, j), dkBr = Dr_KTB(i, j), dkBz = Dz_KTB(i, j);
        const double dkCr = Dr_KTC(i, j), dkCz = Dz_KTC(i, j);
        const double Dlr = Delta_r(i, j), Dlz = Delta_z(i, j);
        DIV_KT_r(i, j) = -p3(gC) * dCz * kC * p5(rr_) - gA * p2(gC) * kC * dCr * p4(rr_)
            + (p2(gC) * dkCz - half * p3(gC) * dBz * kA - gA * p2(gC) * kC * Cc - half * p3(gC) * dAz * kB - gA * dCz * p2(gC) * kA
               - gA * dCz * gC * gB * kC - p2(gC) * dCz * gB * kB - p2(gC) * dBz * gB * kC - gA * dAz * p2(gC) * kC) * p3(rr_)
            + (2.0 * gA * gC * dkCr - Dlr * gC * kC - gC * dBr * gB * gA * kC - gB * p2(gA) * kC * dCr - dAr * p2(gA) * gC * kC
               - gC * p2(gA) * kA * dCr + p2(gC) * dkBr - gA * gB * gC * kB * dCr - half * gA * dAr * p2(gC) * kB
               - half * p2(gC) * dBr * gA * kA) * p2(rr_)
            + (2.0 * gA * gC * kC + gA * gC * dkAz - gC * p2(gA) * kA * Cc + gC * gH * kC - half * p2(gH) * kH * gC * dHz
               - Dlz * gC * kB - gB * p2(gA) * kC * Cc - half * p2(gA) * dAz * gC * kA + gC * gB * dkBz + gA * gB * dkCz
               - Dlz * gA * kC - gA * gB * gC * kB * Cc - gC * p2(gH) * kH * Cc - half * gC * dBz * p2(gB) * kB) * rr_
            - half * gA * dBr * p2(gB) * kB - half * p2(gH) * kH * gA * dHr - Dlr * gA * kA + p2(gA) * dkAr
            - half * p3(gA) * dAr * kA + rr_ * gH * (gA * Alambda(i, j) + gH * kH * Cc * gC);
        DIV_KT_z(i, j) = -p5(rr_) * p3(gC) * kC * dCr + (-p3(gC) * kC * Cc - dCz * p2(gC) * gB * kC) * p4(rr_)
            + (p2(gC) * dkCr - gB * p2(gC) * kB * dCr - gC * gB * gA * kC * dCr - half * p3(gC) * dBr * kA - p2(gC) * gA * kA * dCr
               - half * dAr * p3(gC) * kB - dAr * gA * p2(gC) * kC - gB * dBr * p2(gC) * kC) * p3(rr_)
            + (-gB * dCz * gC * gA * kA + p2(gC) * kC - dBz * gC * p2(gB) * kC - Dlz * gC * kC - gC * dCz * p2(gB) * kB
               + p2(gC) * dkAz + 2.0 * gC * gB * dkCz - p2(gC) * gA * kA * Cc - dCz * p2(gB) * gA * kC - half * dAz * gB * p2(gC) * kB
               - gC * dAz * gB * gA * kC - gB * p2(gC) * kB * Cc - half * gB * dBz * p2(gC) * kA - gC * gB * gA * kC * Cc) * p2(rr_)
            + (gB * gC * dkBr + gB * gA * dkCr + gC * gA * dkAr - half * p2(gH) * kH * gC * dHr - Dlr * gB * kC - Dlr * gC * kA
               - half * p2(gB) * dBr * gC * kB - half * gC * dAr * p2(gA) * kA) * rr_
            + gC * gH * kA + gB * gA * kC - half * dBz * p3(gB) * kB + p2(gB) * dkBz - Dlz * gB * kB - gC * p2(gH) * kH * Ac
            - half * gB * dAz * p2(gA) * kA - half * p2(gH) * kH * gB * dHz - gC * gH * kH + gB * gH * kC - gB * p2(gH) * kH * Cc;
        DIVA_KT_r(i, j) = -p5(rr_) * p3(gC) * dCz * kC + (-p3(gC) * dCr * kB - p3(gC) * dBr * kC - 3.0 * p2(gC) * dCr * gA * kC) * p4(rr_)
            + (-p3(gC) * Cc * kB - 2.0 * gA * dCz * p2(gC) * kA - 3.0 * p2(gC) * Cc * gA * kC + p2(gC) * dkCz - p2(gC) * dAz * gA * kC
               - 3.0 * gA * dCz * gC * gB * kC - 2.0 * p2(gC) * dBz * gB * kC - p3(gC) * dBz * kA - p2(gC) * dCz * gB * kB) * p3(rr_)
            + (-gA * dBr * p2(gC) * kA - gA * gB * gC * kB * dCr + 2.0 * gA * gC * dkCr - 2.0 * gC * dCr * p2(gA) * kA - Dlr * gC * kC
               + p2(gC) * dkBr - p2(gC) * dBr * gB * kB - 2.0 * p2(gA) * dAr * gC * kC - gA * dAr * p2(gC) * kB
               - gB * p2(gA) * kC * dCr - gA * dBr * gC * gB * kC) * p2(rr_)
            + (-gA * dCz * p2(gB) * kB - gB * p2(gA) * kC * Cc - gC * dBz * p2(gB) * kB + 2.0 * gA * gC * kC + gC * gB * dkBz
               + gC * gH * kC + gA * gC * dkAz + gA * gB * dkCz - gA * dAz * gB * gC * kB - gC * p2(gH) * kH * Cc - Dlz * gC * kB
               - p2(gA) * dAz * gB * kC - 2.0 * gC * Cc * p2(gA) * kA - Dlz * gA * kC - p2(gA) * dAz * gC * kA - gA * gB * gC * kB * Cc) * rr_
            - dAr * p3(gA) * kA - Dlr * gA * kA + p2(gA) * dkAr + rr_ * gA * gH * (Alambda(i, j) - lambda(i, j) * gH * kH);
        DIVA_KT_z(i, j) = -p5(rr_) * p3(gC) * kC * dCr
            + (-3.0 * dCz * p2(gC) * gB * kC - dAz * p3(gC) * kC - dCz * p3(gC) * kA - p3(gC) * kC * Cc) * p4(rr_)
            + (-3.0 * gC * gB * gA * kC * dCr - 2.0 * dAr * gA * p2(gC) * kC + p2(gC) * dkCr - gB * dBr * p2(gC) * kC
               - dAr * p3(gC) * kB - 2.0 * gB * p2(gC) * kB * dCr - p2(gC) * gA * kA * dCr) * p3(rr_)
            + (-gC * dAz * gB * gA * kC - p2(gC) * gA * kA * Cc - 2.0 * dBz * gC * p2(gB) * kC - dAz * p2(gC) * gA * kA
               - dAz * gB * p2(gC) * kB - 3.0 * gC * gB * gA * kC * Cc - 2.0 * gC * dCz * p2(gB) * kB - Dlz * gC * kC
               - dCz * p2(gB) * gA * kC + p2(gC) * kC + p2(gC) * dkAz + 2.0 * gC * gB * dkCz - gB * dCz * gC * gA * kA
               - gB * dBz * p2(gC) * kA - 2.0 * gB * p2(gC) * kB * Cc) * p2(rr_)
            + (-Dlr * gB * kC + gB * gA * dkCr + gC * gA * dkAr + gB * gC * dkBr - p2(gB) * dBr * gC * kB - Dlr * gC * kA
               - p2(gB) * dBr * gA * kC - gC * dAr * p2(gA) * kA - gB * dBr * gC * gA * kA - gB * p2(gA) * kA * dCr) * rr_
            - Dlz * gB * kB - gB * p2(gH) * kH * Cc + p2(gB) * dkBz - gC * p2(gH) * kH * Ac - gB * p2(gA) * kA * Cc + gB * gH * kC
            + gC * gH * kA + gB * gA * kC - dBz * p3(gB) * kB;
    }
}

// ---------------------------------------------------------------------------
// scalar field: auxiliary_matter.f90:28-77, potential.f90:27-73,
// stressenergy.f90:65-205
// ---------------------------------------------------------------------------
void auxiliary_matter(Sim& S, Level& L) {
    GRID_DIMS;
    const bool shift = S.P.shift != OLLIN_SHIFT_NONE;
    R(scalar_phi); R(scalar_pi); R(scalar_xi_r); R(scalar_xi_z);
    diff1r(L, scalar_phi, L.a("Dr_scalar_phi"), +1);
    diff1z(L, scalar_phi, L.a("Dz_scalar_phi"), +1);
    diff2r(L, scalar_phi, L.a("Drr_scalar_phi"), +1);
    diff2z(L, scalar_phi, L.a("Dzz_scalar_phi"), +1);
    diff2rz(L, scalar_phi, L.a("Drz_scalar_phi"), +1, +1);
    diff1r(L, scalar_pi, L.a("Dr_scalar_pi"), +1);
    diff1z(L, scalar_pi, L.a("Dz_scalar_pi"), +1);
    diff1r(L, scalar_xi_r, L.a("Dr_scalar_xi_r"), -1);
    diff1z(L, scalar_xi_r, L.a("Dz_scalar_xi_r"), +1);
    diff1r(L, scalar_xi_z, L.a("Dr_scalar_xi_z"), +1);
    diff1z(L, scalar_xi_z, L.a("Dz_scalar_xi_z"), -1);
    if (shift) {
        diffadvr(L, scalar_pi, L.a("DAr_scalar_pi"), +1);
        diffadvz(L, scalar_pi, L.a("DAz_scalar_pi"), +1);
        diffadvr(L, scalar_xi_r, L.a("DAr_scalar_xi_r"), -1);
        diffadvz(L, scalar_xi_r, L.a("DAz_scalar_xi_r"), +1);
        diffadvr(L, scalar_xi_z, L.a("DAr_scalar_xi_z"), +1);
        diffadvz(L, scalar_xi_z, L.a("DAz_scalar_xi_z"), -1);
    }
}

void potential(Sim& S, Level& L) {
    GRID_DIMS;
    R(scalar_phi); R(scalar_V); R(scalar_VP);
    const double m = S.P.scalar_mass, lam = S.P.scalar_lambda;
    ALL scalar_V(i, j) = 0.0;
    ALL scalar_VP(i, j) = 0.0;
    if (S.P.scalarpotential == OLLIN_POTENTIAL_PHI2) {
        ALL scalar_V(i, j) = 0.5 * p2(m) * p2(scalar_phi(i, j));
        ALL scalar_VP(i, j) = p2(m) * scalar_phi(i, j);
    } else if (S.P.scalarpotential == OLLIN_POTENTIAL_PHI4) {
        ALL scalar_V(i, j) = 0.5 * p2(m) * p2(scalar_phi(i, j)) + 0.25 * lam * p4(scalar_phi(i, j));
        ALL scalar_VP(i, j) = p2(m) * scalar_phi(i, j) + lam * p3(scalar_phi(i, j));
    }
}

void stressenergy(Sim& S, Level& L) {
    GRID_DIMS;
    const double zero = 0.0, half = 0.5, two = 2.0;
    R(phi); R(chi); R(psi); R(psi4); R(r);
    R(rho); R(J_r); R(J_z); R(S_A); R(S_B); R(S_H); R(S_C); R(S_lambda); R(trS); R(auxarray);
    R(g_A); R(g_B); R(g_H); R(g_C); R(A); R(B); R(H); R(C); R(lambda);
    R(scalar_pi); R(scalar_xi_r); R(scalar_xi_z); R(scalar_V);
    if (S.P.chimethod) ALL phi(i, j) = -half * std::log(chi(i, j));
    ALL psi(i, j) = std::exp(phi(i, j));
    ALL psi4(i, j) = p4(psi(i, j));
    ALL rho(i, j) = zero;
    ALL J_r(i, j) = zero;
    ALL J_z(i, j) = zero;
    ALL S_A(i, j) = zero;
    ALL S_B(i, j) = zero;
    ALL S_H(i, j) = zero;
    ALL S_C(i, j) = zero;
    ALL S_lambda(i, j) = zero;
    ALL rho(i, j) = rho(i, j) + half * (p2(scalar_pi(i, j)) + (g_A(i, j) * p2(scalar_xi_r(i, j)) + g_B(i, j) * p2(scalar_xi_z(i, j))
                                                                + two * r(i, j) * g_C(i, j) * scalar_xi_r(i, j) * scalar_xi_z(i, j)) / psi4(i, j))
        + scalar_V(i, j);
    ALL J_r(i, j) = J_r(i, j) - (g_A(i, j) * scalar_xi_r(i, j) + r(i, j) * g_C(i, j) * scalar_xi_z(i, j)) * scalar_pi(i, j) / psi4(i, j);
    ALL J_z(i, j) = J_z(i, j) - (g_B(i, j) * scalar_xi_z(i, j) + r(i, j) * g_C(i, j) * scalar_xi_r(i, j)) * scalar_pi(i, j) / psi4(i, j);
    ALL auxarray(i, j) = half * (p2(scalar_pi(i, j)) - (g_A(i, j) * p2(scalar_xi_r(i, j)) + g_B(i, j) * p2(scalar_xi_z(i, j))
                                                        + two * r(i, j) * g_C(i, j) * scalar_xi_r(i, j) * scalar_xi_z(i, j)) / psi4(i, j))
        - scalar_V(i, j);
    ALL S_A(i, j) = S_A(i, j) + p2(scalar_xi_r(i, j)) + A(i, j) * psi4(i, j) * auxarray(i, j);
    ALL S_B(i, j) = S_B(i, j) + p2(scalar_xi_z(i, j)) + B(i, j) * psi4(i, j) * auxarray(i, j);
    ALL S_C(i, j) = S_C(i, j) + scalar_xi_r(i, j) * scalar_xi_z(i, j) / r(i, j) + C(i, j) * psi4(i, j) * auxarray(i, j);
    ALL S_H(i, j) = S_H(i, j) + H(i, j) * psi4(i, j) * auxarray(i, j);
    if (!S.P.nolambda)
        ALL S_lambda(i, j) = S_lambda(i, j) + p2(scalar_xi_r(i, j) / r(i, j)) + lambda(i, j) * psi4(i, j) * auxarray(i, j);
    ALL trS(i, j) = g_A(i, j) * S_A(i, j) + g_B(i, j) * S_B(i, j) + g_H(i, j) * S_H(i, j) + two * p2(r(i, j)) * g_C(i, j) * S_C(i, j);
    ALL trS(i, j) = trS(i, j) / psi4(i, j);
}

// auxiliary.f90:26-56
void auxiliary(Sim& S, Level& L) {
    auxiliary_geometry(S, L);
    if (S.P.mattertype == OLLIN_MATTER_SCALAR) {
        auxiliary_matter(S, L);
        potential(S, L);
        stressenergy(S, L);
    }
}

// ---------------------------------------------------------------------------
// sources_geometry.f90 (bssn), sources_lapse.f90, sources_shift.f90
// ---------------------------------------------------------------------------
void sources_geometry(Sim& S, Level& L) {
    GRID_DIMS;
    const ollin_params& P = S.P;
    const bool shift = P.shift != OLLIN_SHIFT_NONE;
    const bool matter = P.mattertype != OLLIN_MATTER_VACUUM;
    const double zero = 0.0, half = 0.5, third = 1.0 / 3.0, sixth = 1.0 / 6.0, one = 1.0, two = 2.0, four = 4.0, six = 6.0;
    const double smallpi = std::acos(-one);
    const double sigma = P.lagrangian ? 1.0 : 0.0;
    const double cp = (double)P.chipower;
    const double eta = P.eta;
    (void)zero; (void)half;
    R(r); R(alpha); R(trK); R(chi); R(A); R(B); R(H); R(C); R(KTA); R(KTB); R(KTH); R(KTC); R(z4theta);
    R(lambda); R(Alambda); R(Delta_r); R(Delta_z);
    R(sphi); R(schi); R(sA); R(sB); R(sH); R(sC); R(slambda); R(strK); R(sKTA); R(sKTB); R(sKTC); R(sKTH);
    R(sAlambda); R(sDelta_r); R(sDelta_z); R(sz4theta);
    R(psi4); R(Lapla_alpha); R(K2); R(RSCAL); R(KT2_A); R(KT2_B); R(KT2_C); R(KT2_lambda);
    R(RIC_A); R(RIC_B); R(RIC_C); R(RIC_lambda);
    R(D2cov_alpha_A); R(D2cov_alpha_B); R(D2cov_alpha_C); R(D2cov_alpha_lambda);
    R(KT_up_rr); R(KT_up_rz); R(KT_up_zz); R(Dr_alpha); R(Dz_alpha); R(Dr_phi); R(Dz_phi);
    R(Dr_trK); R(Dz_trK); R(g_A); R(g_B); R(g_C); R(g_H); R(DIVA_KT_r); R(DIVA_KT_z); R(DIV_KT_r); R(DIV_KT_z);

    // conformal factor (:63-101)
    ALL sphi(i, j) = -sixth * alpha(i, j) * trK(i, j);
    if (shift) {
        R(beta_r); R(beta_z); R(DAr_phi); R(DAz_phi); R(DIV_beta);
        ALL sphi(i, j) = sphi(i, j) + beta_r(i, j) * DAr_phi(i, j) + beta_z(i, j) * DAz_phi(i, j) + sixth * sigma * DIV_beta(i, j);
    }
    if (P.chimethod) {
        ALL schi(i, j) = cp * sixth * alpha(i, j) * chi(i, j) * trK(i, j);
        if (shift) {
            R(beta_r); R(beta_z); R(DAr_chi); R(DAz_chi); R(DIV_beta);
            ALL schi(i, j) = schi(i, j) + beta_r(i, j) * DAr_chi(i, j) + beta_z(i, j) * DAz_chi(i, j)
                - sigma * cp * sixth * chi(i, j) * DIV_beta(i, j);
        }
    }
    // conformal metric (:104-156)
    ALL sA(i, j) = -two * alpha(i, j) * KTA(i, j);
    ALL sB(i, j) = -two * alpha(i, j) * KTB(i, j);
    ALL sH(i, j) = -two * alpha(i, j) * KTH(i, j);
    ALL sC(i, j) = -two * alpha(i, j) * KTC(i, j);
    if (shift) {
        R(beta_r); R(beta_z); R(DIV_beta); R(Dr_beta_r); R(Dz_beta_r); R(Dr_beta_z); R(Dz_beta_z);
        R(DAr_A); R(DAz_A); R(DAr_B); R(DAz_B); R(DAr_H); R(DAz_H); R(DAr_C); R(DAz_C);
        ALL sA(i, j) = sA(i, j) + beta_r(i, j) * DAr_A(i, j) + beta_z(i, j) * DAz_A(i, j)
            + two * (A(i, j) * Dr_beta_r(i, j) + r(i, j) * C(i, j) * Dr_beta_z(i, j)) - two * third * sigma * A(i, j) * DIV_beta(i, j);
        ALL sB(i, j) = sB(i, j) + beta_r(i, j) * DAr_B(i, j) + beta_z(i, j) * DAz_B(i, j)
            + two * (B(i, j) * Dz_beta_z(i, j) + r(i, j) * C(i, j) * Dz_beta_r(i, j)) - two * third * sigma * B(i, j) * DIV_beta(i, j);
        ALL sH(i, j) = sH(i, j) + beta_r(i, j) * DAr_H(i, j) + beta_z(i, j) * DAz_H(i, j)
            + two * H(i, j) * beta_r(i, j) / r(i, j) - two * third * sigma * H(i, j) * DIV_beta(i, j);
        ALL sC(i, j) = sC(i, j) + beta_r(i, j) * DAr_C(i, j) + beta_z(i, j) * DAz_C(i, j)
            + C(i, j) * beta_r(i, j) / r(i, j) + C(i, j) * (Dr_beta_r(i, j) + Dz_beta_z(i, j))
            + (B(i, j) * Dr_beta_z(i, j) + A(i, j) * Dz_beta_r(i, j)) / r(i, j) - two * third * sigma * C(i, j) * DIV_beta(i, j);
    }
    // lambda (:159-193)
    if (!P.nolambda) {
        ALL slambda(i, j) = -two * alpha(i, j) * Alambda(i, j);
        if (shift) {
            R(beta_r); R(beta_z); R(DAr_lambda); R(DAz_lambda); R(Dr_beta_r); R(Dr_beta_z); R(DD_beta_rr); R(DIV_beta);
            ALL slambda(i, j) = slambda(i, j) + beta_r(i, j) * DAr_lambda(i, j) + beta_z(i, j) * DAz_lambda(i, j)
                + two * (lambda(i, j) * beta_r(i, j) + C(i, j) * Dr_beta_z(i, j)) / r(i, j)
                + two * (P.ft[0] * (lambda(i, j) * Dr_beta_r(i, j) + H(i, j) * DD_beta_rr(i, j) / r(i, j))
                         + (one - P.ft[0]) * (lambda(i, j) * beta_r(i, j) + A(i, j) * DD_beta_rr(i, j)) / r(i, j))
                - two * third * sigma * lambda(i, j) * DIV_beta(i, j);
        }
    }
    // trK (:196-252)
    if (P.slicing == OLLIN_SLICING_MAXIMAL) {  // :200-204
        ALL strK(i, j) = zero;
    } else {
        ALL strK(i, j) = -Lapla_alpha(i, j);
        ALL strK(i, j) = strK(i, j) + alpha(i, j) * K2(i, j);
        if (shift) {
            R(beta_r); R(beta_z); R(DAr_trK); R(DAz_trK);
            ALL strK(i, j) = strK(i, j) + beta_r(i, j) * DAr_trK(i, j) + beta_z(i, j) * DAz_trK(i, j);
        }
        if (matter) {
            R(rho); R(trS);
            ALL strK(i, j) = strK(i, j) + four * smallpi * alpha(i, j) * (rho(i, j) + trS(i, j));
        }
        if (P.geodiss != 0.0) dissipation(L, trK, strK, +1, +1, P.geodiss);
    }
    // traceless extrinsic curvature (:255-392)
    ALL sKTA(i, j) = alpha(i, j) * ((trK(i, j) + two * z4theta(i, j)) * KTA(i, j) - two * KT2_A(i, j));
    ALL sKTB(i, j) = alpha(i, j) * ((trK(i, j) + two * z4theta(i, j)) * KTB(i, j) - two * KT2_B(i, j));
    ALL sKTC(i, j) = alpha(i, j) * ((trK(i, j) + two * z4theta(i, j)) * KTC(i, j) - two * KT2_C(i, j));
    ALL sKTA(i, j) = sKTA(i, j) + (-D2cov_alpha_A(i, j) + alpha(i, j) * RIC_A(i, j)) / psi4(i, j)
        - third * A(i, j) * (-Lapla_alpha(i, j) + alpha(i, j) * RSCAL(i, j));
    ALL sKTB(i, j) = sKTB(i, j) + (-D2cov_alpha_B(i, j) + alpha(i, j) * RIC_B(i, j)) / psi4(i, j)
        - third * B(i, j) * (-Lapla_alpha(i, j) + alpha(i, j) * RSCAL(i, j));
    ALL sKTC(i, j) = sKTC(i, j) + (-D2cov_alpha_C(i, j) + alpha(i, j) * RIC_C(i, j)) / psi4(i, j)
        - third * C(i, j) * (-Lapla_alpha(i, j) + alpha(i, j) * RSCAL(i, j));
    if (shift) {
        R(beta_r); R(beta_z); R(DIV_beta); R(Dr_beta_r); R(Dz_beta_r); R(Dr_beta_z); R(Dz_beta_z);
        R(DAr_KTA); R(DAz_KTA); R(DAr_KTB); R(DAz_KTB); R(DAr_KTC); R(DAz_KTC);
        ALL sKTA(i, j) = sKTA(i, j) + beta_r(i, j) * DAr_KTA(i, j) + beta_z(i, j) * DAz_KTA(i, j)
            + two * (KTA(i, j) * Dr_beta_r(i, j) + r(i, j) * KTC(i, j) * Dr_beta_z(i, j)) - two * third * sigma * KTA(i, j) * DIV_beta(i, j);
        ALL sKTB(i, j) = sKTB(i, j) + beta_r(i, j) * DAr_KTB(i, j) + beta_z(i, j) * DAz_KTB(i, j)
            + two * (KTB(i, j) * Dz_beta_z(i, j) + r(i, j) * KTC(i, j) * Dz_beta_r(i, j)) - two * third * sigma * KTB(i, j) * DIV_beta(i, j);
        ALL sKTC(i, j) = sKTC(i, j) + beta_r(i, j) * DAr_KTC(i, j) + beta_z(i, j) * DAz_KTC(i, j) + KTC(i, j) * beta_r(i, j) / r(i, j)
            + KTC(i, j) * (Dr_beta_r(i, j) + Dz_beta_z(i, j)) + (KTB(i, j) * Dr_beta_z(i, j) + KTA(i, j) * Dz_beta_r(i, j)) / r(i, j)
            - two * third * sigma * KTC(i, j) * DIV_beta(i, j);
    }
    if (matter) {
        R(S_A); R(S_B); R(S_C); R(trS);
        ALL sKTA(i, j) = sKTA(i, j) - 8.0 * smallpi * alpha(i, j) * (S_A(i, j) / psi4(i, j) - third * A(i, j) * trS(i, j));
        ALL sKTB(i, j) = sKTB(i, j) - 8.0 * smallpi * alpha(i, j) * (S_B(i, j) / psi4(i, j) - third * B(i, j) * trS(i, j));
        ALL sKTC(i, j) = sKTC(i, j) - 8.0 * smallpi * alpha(i, j) * (S_C(i, j) / psi4(i, j) - third * C(i, j) * trS(i, j));
    }
    if (P.geodiss != 0.0) {
        dissipation(L, KTA, sKTA, +1, +1, P.geodiss);
        dissipation(L, KTB, sKTB, +1, +1, P.geodiss);
        dissipation(L, KTC, sKTC, +1, -1, P.geodiss);
    }
    // Alambda (:395-442)
    if (!P.nolambda) {
        ALL sAlambda(i, j) = alpha(i, j) * (trK(i, j) * Alambda(i, j) - two * KT2_lambda(i, j));
        ALL sAlambda(i, j) = sAlambda(i, j) + (-D2cov_alpha_lambda(i, j) + alpha(i, j) * RIC_lambda(i, j)) / psi4(i, j)
            - third * lambda(i, j) * (-Lapla_alpha(i, j) + alpha(i, j) * RSCAL(i, j));
        if (shift) {
            R(beta_r); R(beta_z); R(DAr_Alambda); R(DAz_Alambda); R(Dr_beta_r); R(Dr_beta_z); R(DD_beta_rr); R(DIV_beta);
            ALL sAlambda(i, j) = sAlambda(i, j) + beta_r(i, j) * DAr_Alambda(i, j) + beta_z(i, j) * DAz_Alambda(i, j)
                + two * (Alambda(i, j) * beta_r(i, j) + KTC(i, j) * Dr_beta_z(i, j)) / r(i, j)
                + two * (P.ft[1] * (Alambda(i, j) * Dr_beta_r(i, j) + KTH(i, j) * DD_beta_rr(i, j) / r(i, j))
                         + (one - P.ft[1]) * (Alambda(i, j) * beta_r(i, j) + KTA(i, j) * DD_beta_rr(i, j)) / r(i, j))
                - two * third * sigma * Alambda(i, j) * DIV_beta(i, j);
        }
        if (matter) {
            R(S_lambda); R(trS);
            ALL sAlambda(i, j) = sAlambda(i, j) - 8.0 * smallpi * alpha(i, j) * (S_lambda(i, j) / psi4(i, j) - third * lambda(i, j) * trS(i, j));
        }
        if (P.geodiss != 0.0) dissipation(L, Alambda, sAlambda, +1, +1, P.geodiss);
    }
    // Delta_r (:445-520)
    ALL sDelta_r(i, j) = -two * (KT_up_rr(i, j) * Dr_alpha(i, j) + KT_up_rz(i, j) * Dz_alpha(i, j)) - two * alpha(i, j) * DIVA_KT_r(i, j);
    ALL sDelta_r(i, j) = sDelta_r(i, j) + eta * alpha(i, j) * (DIV_KT_r(i, j)
        + six * (KT_up_rr(i, j) * Dr_phi(i, j) + KT_up_rz(i, j) * Dz_phi(i, j))
        - two * third * (g_A(i, j) * Dr_trK(i, j) + r(i, j) * g_C(i, j) * Dz_trK(i, j)));
    if (shift) {
        R(beta_r); R(beta_z); R(DAr_Delta_r); R(DAz_Delta_r); R(Dr_beta_r); R(Dz_beta_r);
        R(Drz_beta_r); R(Drr_beta_r); R(Dzz_beta_r); R(DD_beta_rr); R(Dr_DIV_beta); R(Dz_DIV_beta); R(DIV_beta);
        ALL sDelta_r(i, j) = sDelta_r(i, j) + beta_r(i, j) * DAr_Delta_r(i, j) + beta_z(i, j) * DAz_Delta_r(i, j)
            - Delta_r(i, j) * Dr_beta_r(i, j) - Delta_z(i, j) * Dz_beta_r(i, j);
        ALL sDelta_r(i, j) = sDelta_r(i, j) + two * r(i, j) * g_C(i, j) * Drz_beta_r(i, j)
            + g_A(i, j) * Drr_beta_r(i, j) + g_B(i, j) * Dzz_beta_r(i, j) + g_H(i, j) * DD_beta_rr(i, j);
        ALL sDelta_r(i, j) = sDelta_r(i, j) + third * sigma * (g_A(i, j) * Dr_DIV_beta(i, j)
            + r(i, j) * g_C(i, j) * Dz_DIV_beta(i, j) + two * Delta_r(i, j) * DIV_beta(i, j));
    }
    if (matter) {
        R(J_r);
        ALL sDelta_r(i, j) = sDelta_r(i, j) - 8.0 * smallpi * eta * alpha(i, j) * J_r(i, j) * psi4(i, j);
    }
    if (P.geodiss != 0.0) dissipation(L, Delta_r, sDelta_r, -1, +1, P.geodiss);
    // Delta_z (:523-580)
    ALL sDelta_z(i, j) = -two * (KT_up_rz(i, j) * Dr_alpha(i, j) + KT_up_zz(i, j) * Dz_alpha(i, j)) - two * alpha(i, j) * DIVA_KT_z(i, j);
    ALL sDelta_z(i, j) = sDelta_z(i, j) + eta * alpha(i, j) * (DIV_KT_z(i, j)
        + six * (KT_up_rz(i, j) * Dr_phi(i, j) + KT_up_zz(i, j) * Dz_phi(i, j))
        - two * third * (r(i, j) * g_C(i, j) * Dr_trK(i, j) + g_B(i, j) * Dz_trK(i, j)));
    if (shift) {
        R(beta_r); R(beta_z); R(DAr_Delta_z); R(DAz_Delta_z); R(Dr_beta_z); R(Dz_beta_z);
        R(Drz_beta_z); R(Drr_beta_z); R(Dzz_beta_z); R(Dr_DIV_beta); R(Dz_DIV_beta); R(DIV_beta);
        ALL sDelta_z(i, j) = sDelta_z(i, j) + beta_r(i, j) * DAr_Delta_z(i, j) + beta_z(i, j) * DAz_Delta_z(i, j)
            - Delta_r(i, j) * Dr_beta_z(i, j) - Delta_z(i, j) * Dz_beta_z(i, j);
        ALL sDelta_z(i, j) = sDelta_z(i, j) + two * r(i, j) * g_C(i, j) * Drz_beta_z(i, j)
            + g_A(i, j) * Drr_beta_z(i, j) + g_B(i, j) * Dzz_beta_z(i, j) + g_H(i, j) * Dr_beta_z(i, j) / r(i, j);
        ALL sDelta_z(i, j) = sDelta_z(i, j) + third * sigma * (r(i, j) * g_C(i, j) * Dr_DIV_beta(i, j)
            + g_B(i, j) * Dz_DIV_beta(i, j) + two * Delta_z(i, j) * DIV_beta(i, j));
    }
    if (matter) {
        R(J_z);
        ALL sDelta_z(i, j) = sDelta_z(i, j) - 8.0 * smallpi * eta * alpha(i, j) * J_z(i, j) * psi4(i, j);
    }
    if (P.geodiss != 0.0) dissipation(L, Delta_z, sDelta_z, +1, -1, P.geodiss);
    // Z4 theta (:640-683): BSSN
    ALL sz4theta(i, j) = 0.0;
    (void)sKTH;
}

void sources_lapse(Sim& S, Level& L) {
    GRID_DIMS;
    R(salpha); R(falpha); R(trK); R(alpha);
    if (S.P.slicing == OLLIN_SLICING_STATIC || S.P.slicing == OLLIN_SLICING_MAXIMAL) {
        ALL salpha(i, j) = 0.0;
    } else {
        ALL salpha(i, j) = -falpha(i, j) * trK(i, j);
        if (S.P.shift != OLLIN_SHIFT_NONE) {
            R(beta_r); R(beta_z); R(DAr_alpha); R(DAz_alpha);
            ALL salpha(i, j) = salpha(i, j) + beta_r(i, j) * DAr_alpha(i, j) + beta_z(i, j) * DAz_alpha(i, j);
        }
        // gauge_eta = 0 (param.f90:313): no damping term
    }
}

void sources_shift(Sim& S, Level& L) {
    GRID_DIMS;
    const ollin_params& P = S.P;
    const double two = 2.0, third = 1.0 / 3.0;
    R(sbeta_r); R(sbeta_z); R(sdtbeta_r); R(sdtbeta_z); R(beta_r); R(beta_z); R(dtbeta_r); R(dtbeta_z);
    // static shift (:40-52), also before shiftafter (the time of box 0's
    // level 0); sdtbeta keeps what it holds
    if (P.shift == OLLIN_SHIFT_ZERO || P.shift == OLLIN_SHIFT_STATIC || S.t[0] < P.shiftafter) {
        ALL sbeta_r(i, j) = 0.0;
        ALL sbeta_z(i, j) = 0.0;
        return;
    }
    if (P.shift == OLLIN_SHIFT_GAMMADRIVER0) {  // parabolic driver (:62-85)
        R(sDelta_r); R(sDelta_z);
        ALL sbeta_r(i, j) = P.drivercsi * sDelta_r(i, j);
        ALL sbeta_z(i, j) = P.drivercsi * sDelta_z(i, j);
        ALL sdtbeta_r(i, j) = 0.0;
        ALL sdtbeta_z(i, j) = 0.0;
        return;
    }
    auto shift_advection = [&]() {
        R(DAr_beta_r); R(DAz_beta_r); R(DAr_beta_z); R(DAz_beta_z);
        ALL sbeta_r(i, j) = sbeta_r(i, j) + beta_r(i, j) * DAr_beta_r(i, j) + beta_z(i, j) * DAz_beta_r(i, j);
        ALL sbeta_z(i, j) = sbeta_z(i, j) + beta_r(i, j) * DAr_beta_z(i, j) + beta_z(i, j) * DAz_beta_z(i, j);
    };
    const bool shock = P.shift == OLLIN_SHIFT_GAMMADRIVERSHOCK1 || P.shift == OLLIN_SHIFT_GAMMADRIVERSHOCK2;
    if (P.shift == OLLIN_SHIFT_GAMMADRIVER1 || P.shift == OLLIN_SHIFT_GAMMADRIVERSHOCK1) {  // (:113-186)
        R(Delta_r); R(Delta_z);
        if (!shock) {
            ALL sbeta_r(i, j) = P.drivercsi * Delta_r(i, j);
            ALL sbeta_z(i, j) = P.drivercsi * Delta_z(i, j);
            if (P.driveradv) shift_advection();
            if (P.driverD0) {
                R(Delta0_r); R(Delta0_z);
                ALL sbeta_r(i, j) = sbeta_r(i, j) - P.drivercsi * Delta0_r(i, j);
                ALL sbeta_z(i, j) = sbeta_z(i, j) - P.drivercsi * Delta0_z(i, j);
            }
        } else {
            R(sfdriver); R(fdriver); R(DIV_beta);
            ALL sfdriver(i, j) = -two * third * fdriver(i, j) * DIV_beta(i, j);
            ALL sbeta_r(i, j) = P.drivercsi * fdriver(i, j) * Delta_r(i, j);
            ALL sbeta_z(i, j) = P.drivercsi * fdriver(i, j) * Delta_z(i, j);
            if (P.driveradv) {
                R(DAr_fdriver); R(DAz_fdriver);
                ALL sfdriver(i, j) = sfdriver(i, j) + beta_r(i, j) * DAr_fdriver(i, j) + beta_z(i, j) * DAz_fdriver(i, j);
                shift_advection();
            }
            if (P.driverD0) {
                R(Delta0_r); R(Delta0_z);
                ALL sbeta_r(i, j) = sbeta_r(i, j) - P.drivercsi * fdriver(i, j) * Delta0_r(i, j);
                ALL sbeta_z(i, j) = sbeta_z(i, j) - P.drivercsi * fdriver(i, j) * Delta0_z(i, j);
            }
        }
        ALL sbeta_r(i, j) = sbeta_r(i, j) - P.drivereta * beta_r(i, j);
        ALL sbeta_z(i, j) = sbeta_z(i, j) - P.drivereta * beta_z(i, j);
        ALL sdtbeta_r(i, j) = 0.0;
        ALL sdtbeta_z(i, j) = 0.0;
        return;
    }
    // Gammadriver2 and Gammadrivershock2 (:229-306)
    ALL sbeta_r(i, j) = dtbeta_r(i, j);
    ALL sbeta_z(i, j) = dtbeta_z(i, j);
    if (P.driveradv) shift_advection();
    R(sDelta_r); R(sDelta_z);
    auto dtbeta_advection = [&]() {
        R(DAr_dtbeta_r); R(DAz_dtbeta_r); R(DAr_Delta_r); R(DAz_Delta_r);
        R(DAr_dtbeta_z); R(DAz_dtbeta_z); R(DAr_Delta_z); R(DAz_Delta_z);
        ALL sdtbeta_r(i, j) = sdtbeta_r(i, j) + beta_r(i, j) * (DAr_dtbeta_r(i, j) - DAr_Delta_r(i, j))
            + beta_z(i, j) * (DAz_dtbeta_r(i, j) - DAz_Delta_r(i, j));
        ALL sdtbeta_z(i, j) = sdtbeta_z(i, j) + beta_r(i, j) * (DAr_dtbeta_z(i, j) - DAr_Delta_z(i, j))
            + beta_z(i, j) * (DAz_dtbeta_z(i, j) - DAz_Delta_z(i, j));
    };
    if (!shock) {
        ALL sdtbeta_r(i, j) = P.drivercsi * sDelta_r(i, j);
        ALL sdtbeta_z(i, j) = P.drivercsi * sDelta_z(i, j);
        if (P.driveradv) dtbeta_advection();
    } else {
        R(sfdriver); R(fdriver); R(DIV_beta); R(Delta_r); R(Delta_z);
        ALL sfdriver(i, j) = -two * third * fdriver(i, j) * DIV_beta(i, j);
        ALL sdtbeta_r(i, j) = P.drivercsi * (fdriver(i, j) * sDelta_r(i, j) + sfdriver(i, j) * Delta_r(i, j));
        ALL sdtbeta_z(i, j) = P.drivercsi * (fdriver(i, j) * sDelta_z(i, j) + sfdriver(i, j) * Delta_z(i, j));
        if (P.driveradv) {
            R(Dr_fdriver); R(Dz_fdriver);
            ALL sfdriver(i, j) = sfdriver(i, j) + beta_r(i, j) * Dr_fdriver(i, j) + beta_z(i, j) * Dz_fdriver(i, j);
            dtbeta_advection();
        }
        if (P.driverD0) {
            R(Delta0_r); R(Delta0_z);
            ALL sdtbeta_r(i, j) = sdtbeta_r(i, j) - P.drivercsi * sfdriver(i, j) * Delta0_r(i, j);
            ALL sdtbeta_z(i, j) = sdtbeta_z(i, j) - P.drivercsi * sfdriver(i, j) * Delta0_z(i, j);
        }
    }
    ALL sdtbeta_r(i, j) = sdtbeta_r(i, j) - P.drivereta * dtbeta_r(i, j);
    ALL sdtbeta_z(i, j) = sdtbeta_z(i, j) - P.drivereta * dtbeta_z(i, j);
}

// scalar.f90:2-258 (second-order form of the Klein-Gordon source for pi)
void sources_scalar(Sim& S, Level& L) {
    GRID_DIMS;
    const ollin_params& P = S.P;
    const bool shift = P.shift != OLLIN_SHIFT_NONE;
    const double zero = 0.0, half = 0.5, one = 1.0, two = 2.0;
    R(alpha); R(r); R(scalar_pi); R(scalar_xi_r); R(scalar_xi_z); R(scalar_phi);
    R(sscalar_phi); R(sscalar_xi_r); R(sscalar_xi_z); R(sscalar_pi);
    R(Dr_scalar_pi); R(Dz_scalar_pi); R(Dr_alpha); R(Dz_alpha);
    R(g_A); R(g_B); R(g_C); R(Dr_phi); R(Dz_phi); R(Dr_g_A); R(Dz_g_C); R(Dz_g_B); R(Dr_g_C);
    R(ihdet); R(Dr_hdet); R(Dz_hdet); R(psi4); R(trK);
    R(Drr_scalar_phi); R(Dzz_scalar_phi); R(Drz_scalar_phi); R(Dr_scalar_phi); R(Dz_scalar_phi);
    ALL sscalar_phi(i, j) = alpha(i, j) * scalar_pi(i, j);
    if (shift) {
        R(beta_r); R(beta_z);
        ALL sscalar_phi(i, j) = sscalar_phi(i, j) + beta_r(i, j) * scalar_xi_r(i, j) + beta_z(i, j) * scalar_xi_z(i, j);
    }
    ALL sscalar_xi_r(i, j) = alpha(i, j) * Dr_scalar_pi(i, j) + scalar_pi(i, j) * Dr_alpha(i, j);
    if (shift) {
        R(beta_r); R(beta_z); R(DAr_scalar_xi_r); R(DAz_scalar_xi_r); R(Dr_beta_r); R(Dr_beta_z);
        ALL sscalar_xi_r(i, j) = sscalar_xi_r(i, j) + beta_r(i, j) * DAr_scalar_xi_r(i, j) + scalar_xi_r(i, j) * Dr_beta_r(i, j)
            + beta_z(i, j) * DAz_scalar_xi_r(i, j) + scalar_xi_z(i, j) * Dr_beta_z(i, j);
    }
    ALL sscalar_xi_z(i, j) = alpha(i, j) * Dz_scalar_pi(i, j) + scalar_pi(i, j) * Dz_alpha(i, j);
    if (shift) {
        R(beta_r); R(beta_z); R(DAr_scalar_xi_z); R(DAz_scalar_xi_z); R(Dz_beta_r); R(Dz_beta_z);
        ALL sscalar_xi_z(i, j) = sscalar_xi_z(i, j) + beta_r(i, j) * DAr_scalar_xi_z(i, j) + scalar_xi_r(i, j) * Dz_beta_r(i, j)
            + beta_z(i, j) * DAz_scalar_xi_z(i, j) + scalar_xi_z(i, j) * Dz_beta_z(i, j);
    }
    // scalarmethod = "second" (param.f90:634)
    ALL sscalar_pi(i, j) = alpha(i, j) * (g_A(i, j) * Drr_scalar_phi(i, j) + g_B(i, j) * Dzz_scalar_phi(i, j)
                                          + two * r(i, j) * g_C(i, j) * Drz_scalar_phi(i, j));
    ALL sscalar_pi(i, j) = sscalar_pi(i, j) + two * alpha(i, j)
        * (Dr_phi(i, j) * (g_A(i, j) * Dr_scalar_phi(i, j) + r(i, j) * g_C(i, j) * Dz_scalar_phi(i, j))
           + Dz_phi(i, j) * (g_B(i, j) * Dz_scalar_phi(i, j) + r(i, j) * g_C(i, j) * Dr_scalar_phi(i, j)));
    ALL sscalar_pi(i, j) = sscalar_pi(i, j)
        + Dr_alpha(i, j) * (g_A(i, j) * Dr_scalar_phi(i, j) + r(i, j) * g_C(i, j) * Dz_scalar_phi(i, j))
        + Dz_alpha(i, j) * (g_B(i, j) * Dz_scalar_phi(i, j) + r(i, j) * g_C(i, j) * Dr_scalar_phi(i, j));
    ALL sscalar_pi(i, j) = sscalar_pi(i, j) + alpha(i, j)
        * (Dr_scalar_phi(i, j) * (Dr_g_A(i, j) + r(i, j) * Dz_g_C(i, j))
           + Dz_scalar_phi(i, j) * (Dz_g_B(i, j) + r(i, j) * Dr_g_C(i, j) + g_C(i, j)));
    ALL sscalar_pi(i, j) = sscalar_pi(i, j) + alpha(i, j) * (g_A(i, j) * Dr_scalar_phi(i, j) / r(i, j) + g_C(i, j) * Dz_scalar_phi(i, j));
    ALL sscalar_pi(i, j) = sscalar_pi(i, j) + half * alpha(i, j) * ihdet(i, j)
        * (Dr_hdet(i, j) * (g_A(i, j) * Dr_scalar_phi(i, j) + r(i, j) * g_C(i, j) * Dz_scalar_phi(i, j))
           + Dz_hdet(i, j) * (g_B(i, j) * Dz_scalar_phi(i, j) + r(i, j) * g_C(i, j) * Dr_scalar_phi(i, j)));
    ALL sscalar_pi(i, j) = sscalar_pi(i, j) / psi4(i, j);
    ALL sscalar_pi(i, j) = sscalar_pi(i, j) + alpha(i, j) * scalar_pi(i, j) * trK(i, j);
    if (P.scalarpotential != OLLIN_POTENTIAL_NONE) {
        R(scalar_VP);
        ALL sscalar_pi(i, j) = sscalar_pi(i, j) - alpha(i, j) * scalar_VP(i, j);
    }
    if (shift) {
        R(beta_r); R(beta_z); R(DAr_scalar_pi); R(DAz_scalar_pi);
        ALL sscalar_pi(i, j) = sscalar_pi(i, j) + beta_r(i, j) * DAr_scalar_pi(i, j) + beta_z(i, j) * DAz_scalar_pi(i, j);
    }
    if (P.scalardiss != zero) {
        dissipation(L, scalar_phi, sscalar_phi, +1, +1, P.scalardiss);
        dissipation(L, scalar_pi, sscalar_pi, +1, +1, P.scalardiss);
        dissipation(L, scalar_xi_r, sscalar_xi_r, -1, +1, P.scalardiss);
        dissipation(L, scalar_xi_z, sscalar_xi_z, +1, -1, P.scalardiss);
    }
    radbound(L, scalar_pi, sscalar_pi, Dr_scalar_pi, Dz_scalar_pi, one, zero);
}

// radiative_geometry.f90:2-291
void radiative_geometry(Sim& S, Level& L) {
    GRID_DIMS;
    const ollin_params& P = S.P;
    const double zero = 0.0, one = 1.0, two = 2.0, third = 1.0 / 3.0;
    const double var0 = zero;
    const double vl = 1.0;
    const double va = std::sqrt(P.gauge_f);
    const double vs = std::sqrt(4.0 * third * P.drivercsi);
    R(trK); R(strK); R(Dr_trK); R(Dz_trK);
    R(KTA); R(sKTA); R(Dr_KTA); R(Dz_KTA);
    R(KTB); R(sKTB); R(Dr_KTB); R(Dz_KTB);
    R(KTC); R(sKTC); R(Dr_KTC); R(Dz_KTC);
    if (P.slicing != OLLIN_SLICING_MAXIMAL) radbound(L, trK, strK, Dr_trK, Dz_trK, va, var0);  // :70-76
    radbound(L, KTA, sKTA, Dr_KTA, Dz_KTA, vl, var0);
    radbound(L, KTB, sKTB, Dr_KTB, Dz_KTB, vl, var0);
    for (int j = 1 - g; j <= Nz; ++j) {
        sKTA(Nr, j) = sKTA(Nr, j) + third * (one - vl / va) * strK(Nr, j) * two;
        sKTB(Nr, j) = sKTB(Nr, j) - third * (one - vl / va) * strK(Nr, j);
    }
    if (!L.eqsym) {
        for (int i = 1 - g; i <= Nr; ++i) {
            sKTA(i, 1 - g) = sKTA(i, 1 - g) - third * (one - vl / va) * strK(i, 1 - g);
            sKTB(i, 1 - g) = sKTB(i, 1 - g) + third * (one - vl / va) * strK(i, 1 - g) * two;
        }
    }
    for (int i = 1 - g; i <= Nr; ++i) {
        sKTA(i, Nz) = sKTA(i, Nz) - third * (one - vl / va) * strK(i, Nz);
        sKTB(i, Nz) = sKTB(i, Nz) + third * (one - vl / va) * strK(i, Nz) * two;
    }
    radbound(L, KTC, sKTC, Dr_KTC, Dz_KTC, vl, var0);
    if (!P.nolambda) {
        R(Alambda); R(sAlambda); R(Dr_Alambda); R(Dz_Alambda);
        radbound(L, Alambda, sAlambda, Dr_Alambda, Dz_Alambda, vl, var0);
    }
    // radiative_geometry.f90:195-262: the Gamma drivers' boundary
    if (P.shift == OLLIN_SHIFT_GAMMADRIVER0 && P.drivercsi != 0.0) {
        // zeroes the shift sources on the column i = 0 and the row j = 0
        R(sbeta_r); R(sbeta_z);
        for (int j = 1 - g; j <= Nz; ++j) { sbeta_r(0, j) = 0.0; sbeta_z(0, j) = 0.0; }
        for (int i = 1 - g; i <= Nr; ++i) { sbeta_r(i, 0) = 0.0; sbeta_z(i, 0) = 0.0; }
    }
    if ((P.shift == OLLIN_SHIFT_GAMMADRIVER1 || P.shift == OLLIN_SHIFT_GAMMADRIVERSHOCK1) && P.drivercsi != 0.0) {
        R(Delta_r); R(sDelta_r); R(Dr_Delta_r); R(Dz_Delta_r);
        R(Delta_z); R(sDelta_z); R(Dr_Delta_z); R(Dz_Delta_z);
        radbound(L, Delta_r, sDelta_r, Dr_Delta_r, Dz_Delta_r, vs, var0);
        radbound(L, Delta_z, sDelta_z, Dr_Delta_z, Dz_Delta_z, vs, var0);
    }
    if ((P.shift == OLLIN_SHIFT_GAMMADRIVER2 || P.shift == OLLIN_SHIFT_GAMMADRIVERSHOCK2) && P.drivercsi != 0.0) {
        R(dtbeta_r); R(sdtbeta_r); R(Dr_dtbeta_r); R(Dz_dtbeta_r);
        R(dtbeta_z); R(sdtbeta_z); R(Dr_dtbeta_z); R(Dz_dtbeta_z);
        radbound(L, dtbeta_r, sdtbeta_r, Dr_dtbeta_r, Dz_dtbeta_r, vs, var0);
        radbound(L, dtbeta_z, sdtbeta_z, Dr_dtbeta_z, Dz_dtbeta_z, vs, var0);
    }
}

// constraints.f90:55-149 (ham, mom_r, mom_z)
void constraints(Sim& S, Level& L) {
    GRID_DIMS;
    const double two = 2.0, third = 1.0 / 3.0;
    const double smallpi = (double)std::acos(-1.0f);  // single-precision pi (constraints.f90:41)
    R(ham); R(mom_r); R(mom_z); R(RSCAL); R(KT2); R(trK); R(r);
    ALL ham(i, j) = RSCAL(i, j) - KT2(i, j) + two * third * p2(trK(i, j));
    if (S.P.mattertype != OLLIN_MATTER_VACUUM) {
        R(rho);
        ALL ham(i, j) = ham(i, j) - 16.0 * smallpi * rho(i, j);
    }
    for (int j = 1 - g; j <= Nz; ++j) ham(1 - g, j) = ham(2 - g, j);
    for (int j = 1 - g; j <= Nz; ++j) ham(Nr, j) = ham(Nr - 1, j);
    for (int i = 1 - g; i <= Nr; ++i) ham(i, 1 - g) = ham(i, 2 - g);
    for (int i = 1 - g; i <= Nr; ++i) ham(i, Nz) = ham(i, Nz - 1);
    if (L.ownaxis)
        for (int j = 1 - g; j <= Nz; ++j)
            for (int ii = 1; ii <= g; ++ii) ham(1 - ii, j) = ham(ii, j);
    if (L.eqsym && L.ownequator)
        for (int jj = 1; jj <= g; ++jj)
            for (int i = 1 - g; i <= Nr; ++i) ham(i, 1 - jj) = ham(i, jj);
    R(DIV_KT_r); R(DIV_KT_z); R(KT_up_rr); R(KT_up_rz); R(KT_up_zz); R(Dr_phi); R(Dz_phi);
    R(g_A); R(g_B); R(g_C); R(Dr_trK); R(Dz_trK);
    ALL mom_r(i, j) = DIV_KT_r(i, j) + 6.0 * (KT_up_rr(i, j) * Dr_phi(i, j) + KT_up_rz(i, j) * Dz_phi(i, j))
        - two * third * (g_A(i, j) * Dr_trK(i, j) + r(i, j) * g_C(i, j) * Dz_trK(i, j));
    ALL mom_z(i, j) = DIV_KT_z(i, j) + 6.0 * (KT_up_rz(i, j) * Dr_phi(i, j) + KT_up_zz(i, j) * Dz_phi(i, j))
        - two * third * (r(i, j) * g_C(i, j) * Dr_trK(i, j) + g_B(i, j) * Dz_trK(i, j));
    if (S.P.mattertype != OLLIN_MATTER_VACUUM) {
        R(J_r); R(J_z); R(psi4);
        ALL mom_r(i, j) = mom_r(i, j) - 8.0 * smallpi * J_r(i, j) * psi4(i, j);
        ALL mom_z(i, j) = mom_z(i, j) - 8.0 * smallpi * J_z(i, j) * psi4(i, j);
    }
}

}  // namespace oracle
