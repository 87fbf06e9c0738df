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

struct Sim {
    ollin_params P;
    int g = 3, Nlmax = 0;
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

}  // namespace oracle
