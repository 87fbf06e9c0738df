// ORACLE -- test infrastructure only.  CPU restatement of the OllinAxis-BiB
// evolution path used to check the GB300 library; never linked into it.
#pragma once
#include <string>
#include <unordered_map>
#include <vector>

#include "../include/ollin_gpu.h"
#include "oracle_grid.h"

namespace oracle {

struct Level {
    int level = 0, g = 3, Nr = 0, Nz = 0;
    int order = 4;             // finite-difference order (param order: 2 or 4)
    int box = 0, parent = -1;  // refinement box; grid of the next coarser level (finebound/restrict)
    int gid = 0;               // index in Sim::L
    double dr = 0, dz = 0, dt = 0, time = 0;
    bool ownaxis = true, ownequator = true, eqsym = true;
    std::unordered_map<std::string, Arr> arrs;
    Arr& a(const std::string& n) {
        auto it = arrs.find(n);
        if (it != arrs.end()) return it->second;
        return arrs.emplace(n, Arr(g, Nr, Nz)).first->second;
    }
    // boundary history var_bound_{rL,rR,zL,zR}(.,.,0:2), flattened
    std::unordered_map<std::string, std::vector<double>> hist;
};

struct EvolvedVar {
    std::string name;
    int symr, symz;
};

// The grids are box 0's levels 0..Nl0 (grid index = level), then levels
// 1..Nl(b) of boxes b = 1..Nb; t, t1, t2, s and the extents rminl.. are per
// grid, dtl, drl, dzl per level.
struct Sim {
    ollin_params P;
    int g = 3, Nlmax = 0, Nb = 0;
    int Nl[4] = {0, 0, 0, 0};
    double rbox[4] = {0, 0, 0, 0}, zbox[4] = {0, 0, 0, 0};
    std::vector<Level> L;
    std::vector<double> t, t1, t2, dtl, drl, dzl, rminl, rmaxl, zminl, zmaxl;
    std::vector<long> s;
    std::vector<EvolvedVar> evolved;  // update/saveold order (generated update.f90)
    double point_updates = 0;
};

// physics (oracle_physics.cpp)
void auxiliary(Sim& S, Level& L);
void sources_geometry(Sim& S, Level& L);
void sources_lapse(Sim& S, Level& L);
void sources_shift(Sim& S, Level& L);
void sources_scalar(Sim& S, Level& L);
void radiative_geometry(Sim& S, Level& L);
void constraints(Sim& S, Level& L);
void diff1r(Level& L, const Arr& f, Arr& d, int symr);
void diff1z(Level& L, const Arr& f, Arr& d, int symz);
void diff2r(Level& L, const Arr& f, Arr& d, int symr);
void diff2z(Level& L, const Arr& f, Arr& d, int symz);
void diff2rz(Level& L, const Arr& f, Arr& d, int symr, int symz);
void dissipation(Level& L, const Arr& ev, Arr& src, int symr, int symz, double diss);
void radbound(Level& L, const Arr& ev, Arr& src, const Arr& Dr_var, const Arr& Dz_var, double v, double var0);
void potential(Sim& S, Level& L);

// Berger-Oliger machinery over the variables listed in Sim::evolved
// (oracle_sim.cpp)
void currentgrid(Sim& S, Level& L);
void saveold(Sim& S, Level& L);
void accumulate(Sim& S, Level& L, int k, int niter, double w);
void update(Sim& S, Level& L, double dtw);
void symmetries_r(Sim& S, Level& L);
void symmetries_z(Sim& S, Level& L);
double interp(Sim& S, int level, const Arr& var, double r0, double z0);
void finebound(Sim& S, int level, double dtw);
void restrict_(Sim& S, int level);
// syncboxes.f90 onto grid p from grid q: every synchronised array, or only
// the named ones (the single-variable mode of the elliptic solver)
void syncboxes(Sim& S, int p, int q, const std::vector<std::string>& only);

// elliptic initial data (oracle_elliptic.cpp)
void idata_scalarpulse(Sim& S);
void idata_brillwave(Sim& S);
void maximalslicing(Sim& S, const double* va_max);

// solver statistics of the last elliptic solve: iterations of each phase
struct EllStats { int steps[2] = {0, 0}; int phases = 0; double gres = 0.0; };
extern thread_local EllStats g_ell_stats;

}  // namespace oracle
