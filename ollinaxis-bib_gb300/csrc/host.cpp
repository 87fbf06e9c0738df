// Host side of the GB300 evolution library: level hierarchy, buffer
// rotation, the Berger-Oliger schedule of src/base/onestep.f90 and the C ABI
// declared in include/ollin_gpu.h.
//
// Schedule per level step (onestep.f90:90-357):
//   saveold          -> rotate state slots: pp <- p, p <- cur (no copy)
//   per RK4 stage    -> rhs (sources + dissipation + radiative boundary +
//                       accumulate + update), prolongation of the fine-level
//                       boundary strips, parity ghost fill, aux_point,
//                       aux_deriv (the ``auxiliary`` of the next stage)
//   then two steps of the next finer level, and restriction to the coarser
//   level when both coincide in time (onestep.f90:375-469).
// The boundary history var_bound_* of the reference is the strip of the
// state at the start of the current (p) and previous (pp) step, so it is read
// straight from those slots.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/ollin_gpu.h"
#include "ollin_kernels.h"

using namespace ollin;

namespace ollin {
thread_local bool g_chain_launch = false;
thread_local LaunchRecorder* g_recorder = nullptr;

static std::unordered_map<const void*, MultiLaunchFn>& multi_registry() {
    static std::unordered_map<const void*, MultiLaunchFn> m;
    return m;
}
void register_multi(const void* kernel, MultiLaunchFn fn) { multi_registry()[kernel] = fn; }
MultiLaunchFn multi_for(const void* kernel) {
    auto it = multi_registry().find(kernel);
    return it == multi_registry().end() ? nullptr : it->second;
}
}

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

#define CUDA_OR_FAIL(x)                                                               \
    do {                                                                              \
        cudaError_t e_ = (x);                                                         \
        if (e_ != cudaSuccess) return fail(OLLIN_ECUDA, std::string(#x ": ") + cudaGetErrorString(e_)); \
    } while (0)

constexpr int kSlots = 4;

struct DLevel {
    int level = 0, nr = 0, nz = 0, g = 3, ld = 0, rows = 0;
    int box = 0, parent = -1;  // refinement box; grid of the next coarser level
    size_t n = 0;  // elements per grid function
    double dr = 0, dz = 0, dt = 0;
    double* pool = nullptr;
    double* slot[kSlots][NFIELDS] = {};
    double* acc[NFIELDS] = {};
    double* aux[NAUX] = {};
    double* coords = nullptr;  // rcol | ircol | zrow
    int cur = 0, p = 1, pp = 2;
    LevelGeom G{};
    bool last_aux_t0 = true;
    std::vector<double> rh, zh;  // host copies of the coordinates
    // transfer stencils with the next coarser level (levels >= 1): the
    // boundary strips this level receives, the overlap it restricts to
    XferPt* ptab = nullptr;
    int nptab = 0;
    XferPt* rtab = nullptr;
    int nrtab = 0;
    // the lapse of the last ``auxiliary`` call, kept while a maximal-slicing
    // solve has replaced the lapse and no ``auxiliary`` has run since
    double* alpha_aux = nullptr;
    bool alpha_stale = false;
    // driverD0: Delta_r | Delta_z of the last t = 0 ``auxiliary`` call
    // (auxiliary_geometry.f90:1107-1113)
    double* delta0 = nullptr;
    double* flat = nullptr;  // boundtype = "flat", level 0: the edge sources (StageArgs::flat)
    // syncboxes: this grid's state before the copies of its level (kept for
    // the partner's next first stage and its own), the map of the points
    // another box copies onto it (offset in the partner's state, or -1), the
    // partner grid, and whether the copy has happened since the last
    // ``auxiliary``
    double* snap = nullptr;
    int* smap = nullptr;
    std::vector<int> spartners;  // the grids copied from (index k of a copied point's smap entry)
    std::vector<int> hsmap;      // host copy of smap
    bool sync_pending = false;
};

// One ``syncboxes`` copy onto grid p from grid q (same level), in the order
// of onestep.f90:452-464.
struct SyncPair {
    int p = -1, q = -1;
    XferPt* tab = nullptr;
    int ntab = 0;
    // (offset in p from its element (0, 0), offset of the coinciding node in q) of each copied point
    std::vector<std::pair<int, int>> copies;
};

}  // namespace

struct ollin_handle {
    ollin_params P{};
    // grids: box 0's levels 0..Nl0 (index = level), then levels 1..Nl(b) of
    // boxes b = 1..Nb; nlev counts the grids, t..zmaxl are per grid
    int g = 3, nlev = 0, nb = 0, nlmax = 0;
    int nl[4] = {0, 0, 0, 0}, nrbox[4] = {0, 0, 0, 0}, nzbox[4] = {0, 0, 0, 0};
    double rbox[4] = {0, 0, 0, 0}, zbox[4] = {0, 0, 0, 0};
    std::vector<DLevel> L;
    std::vector<SyncPair> sync;  // nonempty copies, in the reference's order
    std::vector<double> t, t1, t2, rminl, rmaxl, zminl, zmaxl;
    std::vector<long> s;
    std::vector<int> fields;  // active field slots
    int symr[NFIELDS] = {}, symz[NFIELDS] = {};
    cudaStream_t stream = nullptr;
    unsigned int* d_flag = nullptr;
    double* d_norm = nullptr;
    double point_updates = 0;
    long long launches = 0;
    bool initialized = false;
    bool step_queued = false;  // ollin_gpu_step_begin ran, ollin_gpu_step_end not yet
    // ollin_gpu_step_graphs: a coarse step is captured and replayed as one
    // graph launch (the executable graph is updated in place each step)
    bool graphs = false;
    // ollin_gpu_step_chaining: the kernels of a step launched as a
    // programmatic dependent chain (on by default)
    bool chain = true;
    cudaGraphExec_t gexec = nullptr;
    long long graph_updates = 0, graph_instantiations = 0;
    bool shift = false, scalar = false;
    PhysParams phys{};
    // optional per-launch timing of the right-hand-side kernel
    bool ktime = false;
    std::vector<cudaEvent_t> ev;  // start/stop pairs
    size_t ev_used = 0;
    double rhs_point_stages = 0;
    long long rhs_launches = 0;
    // iterations of the last elliptic solve (coarse phase, all-level phase)
    int ell_steps[2] = {0, 0};
    double ell_gres = 0.0;
    // RMS residual after each FP64 refinement of the last mixed / fp64mg
    // solve, per level (entry 0: before the first correction)
    std::vector<std::vector<double>> ell_hist;
};

namespace {

// parity tags of the evolved fields (src/base/arrays.config)
void parity_table(ollin_handle* h) {
    auto set = [&](int f, int sr, int sz) { h->symr[f] = sr; h->symz[f] = sz; };
    for (int f = 0; f < NFIELDS; ++f) set(f, +1, +1);
    set(F_C, +1, -1); set(F_KTC, +1, -1);
    set(F_DLR, -1, +1); set(F_DLZ, +1, -1);
    set(F_BETAR, -1, +1); set(F_BETAZ, +1, -1);
    set(F_DTBETAR, -1, +1); set(F_DTBETAZ, +1, -1);
    set(F_SXIR, -1, +1); set(F_SXIZ, +1, -1);
}

// ghost zones of every grid (main.f90:286-318)
int ghost_zones(const ollin_params& P) { return std::max(P.ghost, P.order == 2 ? 2 : 3); }

double* base_ptr(const DLevel& L, double* p) { return p ? p + (L.g - 1) + (size_t)(L.g - 1) * L.ld : nullptr; }

int check_params(const ollin_params& P) {
    if (P.order != 4 && P.order != 2) return fail(OLLIN_EINVAL, "order must be \"two\" (2) or \"four\" (4)");
    if (P.nrtotal < 8 || P.nztotal < 8) return fail(OLLIN_EINVAL, "Nrtotal and Nztotal must be at least 8");
    if (P.nl0 < 0 || P.nl0 >= kMaxLevels) return fail(OLLIN_EINVAL, "Nl0 out of range");
    // main.f90:286-318: 0 or fewer than the order needs gives the order's own
    // number (ghost_zones), a larger one is kept
    if (P.ghost < 0 || P.ghost > kMaxGhost)
        return fail(OLLIN_EINVAL, "ghost must be between 0 and " + std::to_string(kMaxGhost));
    if (!P.chimethod || P.chipower != 2) return fail(OLLIN_EINVAL, "chimethod with chipower = 2 is required");
    if (!P.lagrangian || !P.factorhdet || !P.evolveH) return fail(OLLIN_EINVAL, "lagrangian flavour with factorhdet and evolveH is required");
    if (P.evolveKTH || !P.nolambda) return fail(OLLIN_EINVAL, "evolveKTH must be off and nolambda on");
    if (P.shift < OLLIN_SHIFT_NONE || P.shift > OLLIN_SHIFT_GAMMADRIVERSHOCK2)
        return fail(OLLIN_EINVAL, "shift must be none, zero, static, Gammadriver0, Gammadriver1, Gammadriver2, Gammadrivershock1 or Gammadrivershock2");
    if (P.slicing < 0 || P.slicing > OLLIN_SLICING_MAXIMAL) return fail(OLLIN_EINVAL, "unknown slicing");
    if (P.ilapse < OLLIN_ILAPSE_ONE || P.ilapse > OLLIN_ILAPSE_MAXIMAL) return fail(OLLIN_EINVAL, "unknown ilapse");
    if (P.integrator != OLLIN_INTEGRATOR_RK4 && P.integrator != OLLIN_INTEGRATOR_ICN) return fail(OLLIN_EINVAL, "unknown integrator");
    if (P.integrator == OLLIN_INTEGRATOR_ICN && P.icniter < 1) return fail(OLLIN_EINVAL, "icniter must be positive");
    if (P.mattertype != OLLIN_MATTER_VACUUM && P.mattertype != OLLIN_MATTER_SCALAR) return fail(OLLIN_EINVAL, "unknown mattertype");
    if (P.boundtype < OLLIN_BOUND_RADIATIVE || P.boundtype > OLLIN_BOUND_FLAT) return fail(OLLIN_EINVAL, "unknown boundtype");
    if (!(P.dr0 > 0 && P.dz0 > 0 && P.dtfac > 0)) return fail(OLLIN_EINVAL, "dr0, dz0 and dtfac must be positive");
    if (P.idata < OLLIN_IDATA_MINKOWSKI || P.idata > OLLIN_IDATA_SCALARPULSE) return fail(OLLIN_EINVAL, "unknown idata");
    if (P.idata == OLLIN_IDATA_SCALARPULSE && P.mattertype != OLLIN_MATTER_SCALAR)
        return fail(OLLIN_EINVAL, "Scalar pulse initial data needs scalar field type matter.");
    if ((P.idata == OLLIN_IDATA_SCALARPULSE || P.idata == OLLIN_IDATA_BRILLWAVE) && P.ell_solver != OLLIN_ELL_WAVE &&
        P.ell_solver != OLLIN_ELL_SOR && P.ell_solver != OLLIN_ELL_MIXED && P.ell_solver != OLLIN_ELL_FP64MG)
        return fail(OLLIN_EINVAL,
                    "elliptic initial data needs an elliptic solver (ELL_solver = wave, sor, mixed or fp64mg)");
    if (P.idata == OLLIN_IDATA_BRILLWAVE && P.brilltype != 0) return fail(OLLIN_EINVAL, "brilltype must be Holz");
    if (P.nb < 0 || P.nb > 3) return fail(OLLIN_EINVAL, "The number of refinement boxes must be between 0 and 3");
    for (int b = 0; b < P.nb; ++b)
        if (P.nl[b] < 0 || P.nl[b] >= kMaxLevels) return fail(OLLIN_EINVAL, "Nl of a refinement box out of range");
    return OLLIN_OK;
}

// setupboxes.f90:25-285: box sizes, centres aligned with the fine grids,
// sanity checks; then the grid list of the handle
int setup_boxes(ollin_handle* h) {
    const ollin_params& P = h->P;
    const int g = h->g;
    h->nb = P.nb;
    h->nl[0] = P.nl0;
    for (int b = 1; b <= 3; ++b) h->nl[b] = P.nl[b - 1];
    h->nlmax = 0;
    for (int b = 0; b <= h->nb; ++b) h->nlmax = std::max(h->nlmax, h->nl[b]);
    if (h->nb > 0 && h->nlmax == 0) return fail(OLLIN_EINVAL, "If you choose Nb>0 you must also have Nl>0 for at least one box");
    h->nrbox[0] = P.nrtotal;
    h->nzbox[0] = P.nztotal;
    if (!P.eqsym && (h->nzbox[0] + g) % 2 == 0) h->nzbox[0] += 1;  // setupboxes.f90:131-135
    for (int b = 1; b <= 3; ++b) { h->nrbox[b] = P.nrbox[b - 1]; h->nzbox[b] = P.nzbox[b - 1]; }
    for (int b = 0; b <= h->nb; ++b)
        if (h->nrbox[b] < 2 + g || h->nzbox[b] < 2 + g)
            return fail(OLLIN_EINVAL, "The values of (Nrtotal,Nztotal,Nrbox,Nzbox) should be greater than 2 plus the number of ghost zones");
    const double d1r = P.dr0 / 2.0, d1z = P.dz0 / 2.0;  // drl(1), dzl(1)
    h->rbox[0] = 0.0; h->zbox[0] = 0.0;
    for (int b = 1; b <= 3; ++b) { h->rbox[b] = P.rbox[b - 1]; h->zbox[b] = P.zbox[b - 1]; }
    for (int b = 1; b <= h->nb; ++b) {
        if (h->rbox[b] != 0.0) h->rbox[b] = ((double)(long)(h->rbox[b] / d1r) + 0.5) * d1r;
        if (h->zbox[b] != 0.0)
            h->zbox[b] = P.eqsym ? ((double)(long)(h->zbox[b] / d1z) + 0.5) * d1z : (double)(long)(h->zbox[b] / d1z) * d1z;
        const double rb = h->rbox[b], zb = h->zbox[b];
        if (rb < 0.0) return fail(OLLIN_EINVAL, "rbox must be larger than or equal to 0 for all refinement boxes");
        if (rb > 0.0 && rb - 0.5 * h->nrbox[b] * d1r <= 0.0) return fail(OLLIN_EINVAL, "Refinement box extends to negative values of r");
        if (rb + 0.5 * h->nrbox[b] * d1r >= (h->nrbox[0] - g) * P.dr0)
            return fail(OLLIN_EINVAL, "Refinement box extends beyond base grid in r direction");
        if (P.eqsym) {
            if (zb < 0.0) return fail(OLLIN_EINVAL, "For equatorial symmetry zbox must be larger than or equal to 0");
            if (zb > 0.0 && zb - 0.5 * h->nzbox[b] * d1z <= 0.0) return fail(OLLIN_EINVAL, "Refinement box extends to negative values of z");
            if (zb + 0.5 * h->nzbox[b] * d1z >= (h->nzbox[0] - g) * P.dz0)
                return fail(OLLIN_EINVAL, "Refinement box extends beyond base grid in z direction");
        } else if (zb - 0.5 * h->nzbox[b] * d1z <= -0.5 * (h->nzbox[0] - g) * P.dz0 ||
                   zb + 0.5 * h->nzbox[b] * d1z >= 0.5 * (h->nzbox[0] - g) * P.dz0) {
            return fail(OLLIN_EINVAL, "Refinement box extends beyond base grid in z direction");
        }
    }
    std::vector<std::pair<int, int>> grids;
    for (int l = 0; l <= h->nl[0]; ++l) grids.push_back({0, l});
    for (int b = 1; b <= h->nb; ++b)
        for (int l = 1; l <= h->nl[b]; ++l) grids.push_back({b, l});
    h->nlev = (int)grids.size();
    h->L.resize(h->nlev);
    for (int k = 0; k < h->nlev; ++k) {
        DLevel& L = h->L[k];
        L.box = grids[k].first;
        L.level = grids[k].second;
        L.parent = -1;
        if (L.level > 0) {
            const int pb = L.level == 1 ? 0 : L.box;  // finebound.f90:66-70
            for (int q = 0; q < h->nlev; ++q)
                if (grids[q].first == pb && grids[q].second == L.level - 1) L.parent = q;
        }
    }
    return OLLIN_OK;
}

int alloc_level(ollin_handle* h, DLevel& L, int gid) {
    const ollin_params& P = h->P;
    const int g = h->g;
    const int level = L.level, box = L.box;
    L.g = g;
    L.nr = h->nrbox[box];
    L.nz = h->nzbox[box];
    L.ld = ((L.nr + g + 31) / 32) * 32;
    L.rows = L.nz + g;
    L.n = (size_t)L.ld * L.rows;
    const double dt0 = P.dtfac * std::min(P.dr0, P.dz0);
    L.dt = dt0 / (double)(1 << level);  // setupboxes.f90:121-125
    L.dr = P.dr0 / (double)(1 << level);
    L.dz = P.dz0 / (double)(1 << level);
    const size_t ncoord = (size_t)(L.nr + g) * 2 + (size_t)(L.nz + g);
    const size_t narrays = (size_t)kSlots * NFIELDS + NFIELDS + NAUX;
    const size_t bytes = (narrays * L.n + ncoord + 64) * sizeof(double);
    if (cudaMalloc(&L.pool, bytes) != cudaSuccess) return fail(OLLIN_ENOMEM, "device allocation failed for level " + std::to_string(level));
    CUDA_OR_FAIL(cudaMemsetAsync(L.pool, 0, bytes, h->stream));
    double* q = L.pool;
    for (int k = 0; k < kSlots; ++k)
        for (int f = 0; f < NFIELDS; ++f) { L.slot[k][f] = q; q += L.n; }
    for (int f = 0; f < NFIELDS; ++f) { L.acc[f] = q; q += L.n; }
    for (int x = 0; x < NAUX; ++x) { L.aux[x] = q; q += L.n; }
    L.coords = q;
    // coordinates (evolve.f90:42-70, one process): the axis on a cell face
    // for boxes on it, else centred on the box
    L.rh.resize(L.nr + g);
    L.zh.resize(L.nz + g);
    std::vector<double> host(ncoord);
    const double rb = h->rbox[box], zb = h->zbox[box];
    for (int i = 1 - g; i <= L.nr; ++i) {
        const double r = (rb == 0.0) ? ((double)(0 + i) - 0.5) * L.dr
                                     : rb + ((double)(0 + i) - 0.5 * (double)(L.nr - g + 1)) * L.dr;
        L.rh[i - 1 + g] = r;
        host[i - 1 + g] = r;
        host[(size_t)(L.nr + g) + (i - 1 + g)] = 1.0 / r;
    }
    for (int j = 1 - g; j <= L.nz; ++j) {
        // evolve.f90:57-70: the equator on a cell face (eqsym, boxes on it) or
        // z centred on the box
        const double z = (P.eqsym && zb == 0.0) ? ((double)(0 + j) - 0.5) * L.dz
                                                : zb + ((double)(0 + j) - 0.5 * (double)(L.nz - g + 1)) * L.dz;
        L.zh[j - 1 + g] = z;
        host[(size_t)(L.nr + g) * 2 + (j - 1 + g)] = z;
    }
    CUDA_OR_FAIL(cudaMemcpyAsync(L.coords, host.data(), ncoord * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
    LevelGeom& G = L.G;
    G.nr = L.nr; G.nz = L.nz; G.g = g; G.ld = L.ld;
    G.order = P.order;
    G.eqsym = P.eqsym ? 1 : 0;
    G.axis = rb == 0.0 ? 1 : 0;                        // main.f90:393-403
    G.equator = (P.eqsym && zb == 0.0) ? 1 : 0;        // main.f90:412-424
    G.lower_r = (box > 0 && rb != 0.0) ? 1 : 0;        // finebound.f90:246
    G.lower_z = (!P.eqsym || (box > 0 && zb != 0.0)) ? 1 : 0;  // finebound.f90:361
    G.jlo = G.equator ? 1 : 1 - g;
    G.dr = L.dr; G.dz = L.dz; G.dt = L.dt;
    G.idr = 1.0 / L.dr; G.idz = 1.0 / L.dz;
    G.rcol = L.coords + (g - 1);                 // rcol[i] for i >= 1-g
    G.ircol = L.coords + (L.nr + g) + (g - 1);
    G.zrow = L.coords + 2 * (L.nr + g) + (g - 1);
    h->rminl[gid] = L.rh[0];
    h->rmaxl[gid] = L.rh[L.nr - 1 + g];
    h->zminl[gid] = L.zh[0];
    h->zmaxl[gid] = L.zh[L.nz - 1 + g];
    L.cur = 0; L.p = 1; L.pp = 2;
    return OLLIN_OK;
}

PhysParams make_phys(const ollin_params& P) {
    PhysParams q{};
    q.slicing = P.slicing;
    q.gauge_f = P.gauge_f;
    q.shift = P.shift != OLLIN_SHIFT_NONE ? 1 : 0;
    // sources_shift.f90: 2 the second-order drivers, 1 the first-order ones,
    // 0 the parabolic one, 3 zero or static (no sources, no boundary)
    q.driver = (P.shift == OLLIN_SHIFT_GAMMADRIVER1 || P.shift == OLLIN_SHIFT_GAMMADRIVERSHOCK1) ? 1
               : P.shift == OLLIN_SHIFT_GAMMADRIVER0                                             ? 0
               : (P.shift == OLLIN_SHIFT_ZERO || P.shift == OLLIN_SHIFT_STATIC)                  ? 3
                                                                                                  : 2;
    q.shock = (P.shift == OLLIN_SHIFT_GAMMADRIVERSHOCK1 || P.shift == OLLIN_SHIFT_GAMMADRIVERSHOCK2) ? 1 : 0;
    q.driverD0 = P.driverD0 ? 1 : 0;
    q.shiftadvect = P.shiftadvect;
    q.driveradv = P.driveradv;
    q.drivercsi = P.drivercsi;
    q.drivereta = P.drivereta;
    q.eta = P.eta;
    q.geodiss = P.geodiss;
    q.scalardiss = P.scalardiss;
    for (int k = 0; k < 8; ++k) q.ft[k] = P.ft[k];
    q.scalar = P.mattertype == OLLIN_MATTER_SCALAR;
    q.potential = P.scalarpotential;
    q.scalar_mass = P.scalar_mass;
    q.scalar_lambda = P.scalar_lambda;
    q.boundtype = P.boundtype;
    return q;
}

// ---- kernel launch helpers ---------------------------------------------------
// d_norm: 8 result slots per grid, then the first pass's block partials
size_t norm_scratch(const ollin_handle* h) { return 8 * (size_t)h->nlev + 5 * (size_t)kNormMaxBlocks; }
double* norm_partials(const ollin_handle* h) { return h->d_norm + 8 * (size_t)h->nlev; }

int after_launch(ollin_handle* h) {
    h->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(OLLIN_ECUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    return OLLIN_OK;
}

int do_symmetry(ollin_handle* h, DLevel& L, int slot, const std::vector<int>& fl) {
    SymArgs a{};
    a.G = L.G;
    a.nf = 0;
    for (int f : fl) {
        a.st[a.nf] = base_ptr(L, L.slot[slot][f]);
        a.symr[a.nf] = h->symr[f];
        a.symz[a.nf] = h->symz[f];
        a.fid[a.nf] = f;
        a.nf++;
    }
    launch_symmetry(a, h->stream);
    return after_launch(h);
}

std::vector<int> active_fields(const ollin_handle* h, bool with_phi) {
    std::vector<int> v;
    for (int f : h->fields)
        if (f != F_PHI || with_phi) v.push_back(f);
    return v;
}

// ``auxiliary`` on one level's current slot (auxiliary_geometry.f90 parts
// that feed the right-hand side).
int do_aux(ollin_handle* h, DLevel& L, int slot, bool t0, bool project = true) {
    AuxArgs a{};
    a.G = L.G;
    for (int f = 0; f < NFIELDS; ++f) a.st[f] = base_ptr(L, L.slot[slot][f]);
    for (int x = 0; x < NAUX; ++x) a.aux[x] = base_ptr(L, L.aux[x]);
    a.t0 = t0 ? 1 : 0;
    a.scalar = h->scalar ? 1 : 0;
    a.project = project ? 1 : 0;
    if (t0 && h->shift && h->P.driverD0) {
        if (!L.delta0) {
            if (cudaMalloc(&L.delta0, 2 * L.n * sizeof(double)) != cudaSuccess)
                return fail(OLLIN_ENOMEM, "device allocation failed for the t = 0 Delta");
            CUDA_OR_FAIL(cudaMemsetAsync(L.delta0, 0, 2 * L.n * sizeof(double), h->stream));
        }
        a.d0r = base_ptr(L, L.delta0);
        a.d0z = base_ptr(L, L.delta0 + L.n);
    }
    launch_aux_point(a, h->stream);
    int rc = after_launch(h);
    if (rc) return rc;
    launch_aux_deriv(a, h->stream);
    rc = after_launch(h);
    if (rc) return rc;
    if (t0) {
        rc = do_symmetry(h, L, slot, {F_DLR, F_DLZ});
        if (rc) return rc;
    }
    L.last_aux_t0 = t0;
    L.alpha_stale = false;
    L.sync_pending = false;
    return OLLIN_OK;
}

StageArgs stage_args(ollin_handle* h, DLevel& L, int in_slot, int out_slot, bool t0) {
    StageArgs a{};
    a.G = L.G;
    a.P = h->phys;
    for (int f = 0; f < NFIELDS; ++f) {
        a.in[f] = base_ptr(L, L.slot[in_slot][f]);
        a.pst[f] = base_ptr(L, L.slot[L.p][f]);
        a.out[f] = base_ptr(L, L.slot[out_slot][f]);
        a.acc[f] = base_ptr(L, L.acc[f]);
    }
    for (int x = 0; x < NAUX; ++x) {
        a.aux[x] = base_ptr(L, L.aux[x]);
        a.auxw[x] = base_ptr(L, L.aux[x]);
    }
    a.t0 = L.last_aux_t0 ? 1 : 0;
    a.evolve_phi = t0 ? 1 : 0;
    a.level0 = L.level == 0;
    // sources_shift.f90:43 reads the time of box 0's level 0 when the stage runs
    a.shift_static = (h->phys.driver == 3 || h->t[0] < h->P.shiftafter) ? 1 : 0;
    a.d0r = L.delta0 ? base_ptr(L, L.delta0) : nullptr;
    a.d0z = L.delta0 ? base_ptr(L, L.delta0 + L.n) : nullptr;
    a.rk4 = h->P.integrator == OLLIN_INTEGRATOR_RK4;
    a.nanflag = h->d_flag;
    a.alpha_aux = L.alpha_stale ? base_ptr(L, L.alpha_aux) : nullptr;
    if (L.sync_pending) {
        a.smap = L.smap + (L.g - 1) + (size_t)(L.g - 1) * L.ld;
        for (int f = 0; f < NFIELDS; ++f) a.xa[f] = base_ptr(L, L.snap + (size_t)f * L.n);
        for (size_t k = 0; k < L.spartners.size(); ++k) {
            const DLevel& Q = h->L[L.spartners[k]];
            for (int f = 0; f < NFIELDS; ++f) a.xb[k][f] = base_ptr(Q, Q.snap + (size_t)f * Q.n);
            a.xb_ld[k] = Q.ld;
        }
    }
    return a;
}

// the right-hand side of a stage: the ordinary kernels, or the ones that read
// the lapse quantities of the last ``auxiliary`` call from alpha_aux, the
// derivatives from the state kept from before ``syncboxes``, or both
void launch_stage_rhs(const StageArgs& a, cudaStream_t s) {
    const bool o2 = a.G.order == 2;
    if (a.alpha_aux && a.smap) (o2 ? launch_rhs_o2_stale_sync : launch_rhs_stale_sync)(a, s);
    else if (a.alpha_aux) (o2 ? launch_rhs_o2_stale : launch_rhs_stale)(a, s);
    else if (a.smap) (o2 ? launch_rhs_o2_sync : launch_rhs_sync)(a, s);
    else (o2 ? launch_rhs_o2 : launch_rhs)(a, s);
}

// Geometry part of the transfer arguments of grid ``gid`` and its parent
// (the next coarser level of its box, or box 0's level 0 for level 1).
ProlongArgs prolong_geometry(ollin_handle* h, int gid) {
    const int pg = h->L[gid].parent;
    ProlongArgs a{};
    a.F = h->L[gid].G;
    a.Cg = h->L[pg].G;
    a.rminl_f = h->rminl[gid]; a.rmaxl_f = h->rmaxl[gid];
    a.zminl_f = h->zminl[gid]; a.zmaxl_f = h->zmaxl[gid];
    a.rminl_c = h->rminl[pg]; a.rmaxl_c = h->rmaxl[pg];
    a.zminl_c = h->zminl[pg]; a.zmaxl_c = h->zmaxl[pg];
    a.bicubic = h->P.interp_bicubic;
    a.tab = h->L[gid].ptab;
    a.ntab = h->L[gid].nptab;
    return a;
}

RestrictArgs restrict_geometry(ollin_handle* h, int gid) {
    const int pg = h->L[gid].parent;
    RestrictArgs a{};
    a.F = h->L[gid].G;
    a.Cg = h->L[pg].G;
    a.rminl_f = h->rminl[gid]; a.rmaxl_f = h->rmaxl[gid];
    a.zminl_f = h->zminl[gid]; a.zmaxl_f = h->zmaxl[gid];
    a.rminl_c = h->rminl[pg]; a.zminl_c = h->zminl[pg];
    a.eqsym = h->P.eqsym;
    a.bicubic = h->P.interp_bicubic;
    a.tab = h->L[gid].rtab;
    a.ntab = h->L[gid].nrtab;
    return a;
}

// Time weights of finebound.f90:118-145 (the same expressions the oracle
// evaluates), fixed per launch.
void prolong_time(ProlongArgs& a, int g) {
    const double tp = a.tp, t0 = a.t0, tm1 = a.tm1, tl = a.tl;
    a.imax = (tp == tl) ? g + 2 : g - 1;  // finebound.f90:106-112
    a.border = (tm1 == 0.0) ? 1 : 2;
    if (tp == tl) {
        a.tmode = 0;  // the history weights vanish exactly
    } else if (a.border == 1) {
        a.tmode = 1;
        a.wa = (tl - t0) / (tp - t0);
        a.wp = (tl - tp) / (t0 - tp);
    } else {
        a.tmode = 2;
        a.wa = ((tl - t0) * (tl - tm1)) / ((tp - t0) * (tp - tm1));
        a.wp = ((tl - tp) * (tl - tm1)) / ((t0 - tp) * (t0 - tm1));
        a.wpp = ((tl - tp) * (tl - t0)) / ((tm1 - tp) * (tm1 - t0));
    }
}

// Build the transfer stencils of every grid and its parent once.
int build_transfer_tables(ollin_handle* h) {
    const int g = h->g;
    for (int l = 0; l < h->nlev; ++l) {
        DLevel& F = h->L[l];
        if (F.parent < 0) continue;
        DLevel& C = h->L[F.parent];
        F.nptab = prolong_table_size(F.G);
        if (cudaMalloc(&F.ptab, (size_t)F.nptab * sizeof(XferPt)) != cudaSuccess)
            return fail(OLLIN_ENOMEM, "device allocation failed for the transfer tables");
        launch_prolong_table(prolong_geometry(h, l), F.ptab, h->stream);
        int rc = after_launch(h);
        if (rc) return rc;
        // the coarse points restrict_kernel writes form a rectangle in (m, n);
        // find it with the kernel's own expressions, one point wider on each side
        RestrictArgs ra = restrict_geometry(h, l);
        const double deltar = (double)(2 * g) * F.dr + 1.0e-10, deltaz = (double)(2 * g) * F.dz + 1.0e-10;
        const double rmin = (ra.rminl_f < 0.0) ? 0.0 : ra.rminl_f + deltar;
        const double zmin = (ra.eqsym && ra.zminl_f < 0.0) ? 0.0 : ra.zminl_f + deltaz;
        const double rmax = ra.rmaxl_f - deltar, zmax = ra.zmaxl_f - deltaz;
        int m_lo = 1 << 30, m_hi = -1, n_lo = 1 << 30, n_hi = -1;
        for (int m = 0; m <= C.nr + g - 1; ++m) {
            const double r0 = ra.rminl_c + (double)m * C.dr;
            if (r0 > rmin && r0 < rmax) { m_lo = std::min(m_lo, m); m_hi = std::max(m_hi, m); }
        }
        for (int n = 0; n <= C.nz + g - 1; ++n) {
            const double z0 = ra.zminl_c + (double)n * C.dz;
            if (z0 > zmin && z0 < zmax) { n_lo = std::min(n_lo, n); n_hi = std::max(n_hi, n); }
        }
        if (m_hi < 0 || n_hi < 0) { F.nrtab = 0; continue; }
        m_lo = std::max(0, m_lo - 1); n_lo = std::max(0, n_lo - 1);
        m_hi = std::min(C.nr + g - 1, m_hi + 1); n_hi = std::min(C.nz + g - 1, n_hi + 1);
        const int nm = m_hi - m_lo + 1, nn = n_hi - n_lo + 1;
        F.nrtab = nm * nn;
        if (cudaMalloc(&F.rtab, (size_t)F.nrtab * sizeof(XferPt)) != cudaSuccess)
            return fail(OLLIN_ENOMEM, "device allocation failed for the transfer tables");
        launch_restrict_table(ra, F.rtab, m_lo, n_lo, nm, nn, h->stream);
        rc = after_launch(h);
        if (rc) return rc;
    }
    CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
    // a stencil that would leave its source grid marks the layout as unusable
    for (int l = 0; l < h->nlev; ++l) {
        DLevel& F = h->L[l];
        for (int k = 0; k < 2; ++k) {
            const XferPt* t = k == 0 ? F.ptab : F.rtab;
            const int n = k == 0 ? F.nptab : F.nrtab;
            if (!t || n == 0) continue;
            std::vector<XferPt> host(n);
            CUDA_OR_FAIL(cudaMemcpy(host.data(), t, (size_t)n * sizeof(XferPt), cudaMemcpyDeviceToHost));
            for (const XferPt& x : host)
                if (x.mode == -1)
                    return fail(OLLIN_EINVAL, "grid " + std::to_string(l) + ": a boundary or restriction point lies too close to "
                                              "the edge of the grid it interpolates from (interp.f90:146-157)");
        }
    }
    return OLLIN_OK;
}

int prolong(ollin_handle* h, int level, int out_slot, double dtw) {
    DLevel& F = h->L[level];
    const int pg = F.parent;
    DLevel& C = h->L[pg];
    ProlongArgs a{};
    a.F = F.G;
    a.Cg = C.G;
    const bool t0 = h->t[level] == 0.0;
    a.nf = 0;
    for (int f : active_fields(h, t0)) {
        a.fid[a.nf++] = f;
    }
    for (int f = 0; f < NFIELDS; ++f) {
        a.fout[f] = base_ptr(F, F.slot[out_slot][f]);
        a.fp[f] = base_ptr(F, F.slot[F.p][f]);
        a.fpp[f] = base_ptr(F, F.slot[F.pp][f]);
        a.cin[f] = base_ptr(C, C.slot[C.cur][f]);
    }
    a.rminl_f = h->rminl[level]; a.rmaxl_f = h->rmaxl[level];
    a.zminl_f = h->zminl[level]; a.zmaxl_f = h->zmaxl[level];
    a.rminl_c = h->rminl[pg]; a.rmaxl_c = h->rmaxl[pg];
    a.zminl_c = h->zminl[pg]; a.zmaxl_c = h->zmaxl[pg];
    a.tp = h->t[pg];
    a.t0 = h->t[level];
    a.tm1 = h->t1[level];
    a.tl = a.t0 + dtw;
    a.bicubic = h->P.interp_bicubic;
    a.tab = F.ptab;
    a.ntab = F.nptab;
    prolong_time(a, h->g);
    launch_prolong_tab(a, h->stream);
    return after_launch(h);
}

int restrict_level(ollin_handle* h, int level) {
    DLevel& F = h->L[level];
    const int pg = F.parent;
    DLevel& C = h->L[pg];
    RestrictArgs a{};
    a.F = F.G;
    a.Cg = C.G;
    a.nf = 0;
    for (int f : active_fields(h, false)) a.fid[a.nf++] = f;
    for (int f = 0; f < NFIELDS; ++f) {
        a.fin[f] = base_ptr(F, F.slot[F.cur][f]);
        a.cout[f] = base_ptr(C, C.slot[C.cur][f]);
    }
    a.rminl_f = h->rminl[level]; a.rmaxl_f = h->rmaxl[level];
    a.zminl_f = h->zminl[level]; a.zmaxl_f = h->zmaxl[level];
    a.rminl_c = h->rminl[pg]; a.zminl_c = h->zminl[pg];
    a.eqsym = h->P.eqsym;
    a.bicubic = h->P.interp_bicubic;
    a.tab = F.rtab;
    a.ntab = F.nrtab;
    launch_restrict_tab(a, h->stream);
    return after_launch(h);
}

// One time step of one grid (the body of the box loop of onestep.f90:73-388).
int step_grid(ollin_handle* h, int level) {
    DLevel& L = h->L[level];
    const bool rk4 = h->P.integrator == OLLIN_INTEGRATOR_RK4;
    const bool t0 = h->t[level] == 0.0;  // currentgrid: time = t(box,level)
    // saveold: pp <- p, p <- cur
    L.pp = L.p;
    L.p = L.cur;
    int freeslots[2], nfree = 0;
    for (int k = 0; k < kSlots && nfree < 2; ++k)
        if (k != L.p && k != L.pp) freeslots[nfree++] = k;
    const int niter = rk4 ? 4 : h->P.icniter;
    const double dt = L.dt;
    int in_slot = L.p;
    const bool flat = L.level == 0 && h->P.boundtype == OLLIN_BOUND_FLAT;
    const int flat_len = (L.nz - L.G.jlo + 1) + 2 * L.nr;
    if (flat && !L.flat && cudaMalloc(&L.flat, (size_t)kNBound * flat_len * sizeof(double)) != cudaSuccess)
        return fail(OLLIN_ENOMEM, "device allocation failed for the flat boundary");
    for (int iter = 1; iter <= niter; ++iter) {
        double dtw, weight = 0;
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
        const int out_slot = freeslots[(iter - 1) & 1];
        StageArgs a = stage_args(h, L, in_slot, out_slot, t0);
        a.iter = iter;
        a.niter = niter;
        if (flat) {
            a.flat = L.flat;
            a.flat_len = flat_len;
        }
        a.dtw = dtw;
        a.weight = weight;
        if (h->ktime) {
            if (h->ev_used + 2 > h->ev.size()) {
                for (int k = 0; k < 256; ++k) {
                    cudaEvent_t e;
                    CUDA_OR_FAIL(cudaEventCreate(&e));
                    h->ev.push_back(e);
                }
            }
            CUDA_OR_FAIL(cudaEventRecord(h->ev[h->ev_used], h->stream));
        }
        launch_stage_rhs(a, h->stream);
        int rc = after_launch(h);
        if (rc) return rc;
        if (h->ktime) {
            CUDA_OR_FAIL(cudaEventRecord(h->ev[h->ev_used + 1], h->stream));
            h->ev_used += 2;
            h->rhs_point_stages += (double)L.nr * (double)(L.nz - L.G.jlo + 1);
            h->rhs_launches++;
        }
        if (flat) {
            launch_flat_edges(a, h->stream);
            rc = after_launch(h);
            if (rc) return rc;
        }
        if (L.level > 0) {
            rc = prolong(h, level, out_slot, dtw);
            if (rc) return rc;
        }
        rc = do_symmetry(h, L, out_slot, active_fields(h, t0));
        if (rc) return rc;
        rc = do_aux(h, L, out_slot, t0);
        if (rc) return rc;
        in_slot = out_slot;
    }
    L.cur = in_slot;
    h->t2[level] = h->t1[level];
    h->t1[level] = h->t[level];
    h->s[level] = h->s[level] + 1;
    h->t[level] = h->t[level] + dt;
    h->point_updates += (double)L.nr * (double)(L.nz - (L.G.eqsym ? 1 : 1 - L.g) + 1);
    return OLLIN_OK;
}

int sync_level(ollin_handle* h, int level);

// onestep.f90:2-522: a step of every box that has this level (boxes 0..Nb),
// two steps of the next level, the ``syncboxes`` copies between boxes that
// overlap on this level (:446-466), then each box restricts into its parent
// with the parent's symmetries and ``auxiliary`` (:472-514).
int onestep(ollin_handle* h, int level) {
    for (int k = 0; k < h->nlev; ++k) {
        if (h->L[k].level != level) continue;
        int rc = step_grid(h, k);
        if (rc) return rc;
    }
    if (level < h->nlmax) {
        int rc = onestep(h, level + 1);
        if (rc) return rc;
        rc = onestep(h, level + 1);
        if (rc) return rc;
    }
    if (level > 0) {
        int rc = sync_level(h, level);  // onestep.f90:446-466
        if (rc) return rc;
        for (int k = 0; k < h->nlev; ++k) {
            if (h->L[k].level != level || h->s[k] % 2 != 0) continue;
            int rc = restrict_level(h, k);
            if (rc) return rc;
            const int pg = h->L[k].parent;
            DLevel& C = h->L[pg];
            rc = do_symmetry(h, C, C.cur, active_fields(h, false));
            if (rc) return rc;
            rc = do_aux(h, C, C.cur, h->t[pg] == 0.0);
            if (rc) return rc;
        }
    }
    return OLLIN_OK;
}

// ``syncboxes`` tables of every ordered pair of boxes on a level that
// overlap (onestep.f90:446-466).  The device reproduces the copy and, for
// the next first stage, the auxiliary quantities it carries; that needs each
// copied point to coincide with a node of the partner.
//
// The copies of a level run in this order, so a copy that reads a node an
// earlier copy wrote (a chain) takes the value that copy brought, and with
// it, in the reference, that copy's auxiliary arrays.  The copy map of each
// grid therefore records the origin of every copied point: the grid and node
// whose state before the level's copies the value and its auxiliary
// quantities come from (possibly the grid itself).
int build_sync_tables(ollin_handle* h) {
    for (int level = 1; level <= h->nlmax; ++level)
        for (int p = 0; p < h->nlev; ++p) {
            if (h->L[p].level != level) continue;
            for (int q = 0; q < h->nlev; ++q) {
                if (q == p || h->L[q].level != level) continue;
                if (h->rmaxl[p] < h->rminl[q] || h->rmaxl[q] < h->rminl[p] || h->zmaxl[p] < h->zminl[q] ||
                    h->zmaxl[q] < h->zminl[p])
                    continue;  // syncboxes.f90:48-52
                DLevel& P = h->L[p];
                SyncTableArgs a{};
                a.P = P.G; a.Q = h->L[q].G;
                a.rminl_p = h->rminl[p]; a.rmaxl_p = h->rmaxl[p]; a.zminl_p = h->zminl[p]; a.zmaxl_p = h->zmaxl[p];
                a.rminl_q = h->rminl[q]; a.rmaxl_q = h->rmaxl[q]; a.zminl_q = h->zminl[q]; a.zmaxl_q = h->zmaxl[q];
                a.bicubic = h->P.interp_bicubic;
                const int n = sync_table_size(P.G);
                std::vector<XferPt> host(n);
                XferPt* tab = nullptr;
                if (cudaMalloc(&tab, (size_t)n * sizeof(XferPt)) != cudaSuccess)
                    return fail(OLLIN_ENOMEM, "device allocation failed for the syncboxes tables");
                launch_sync_table(a, tab, h->stream);
                int rc = after_launch(h);
                if (rc) { cudaFree(tab); return rc; }
                CUDA_OR_FAIL(cudaMemcpyAsync(host.data(), tab, (size_t)n * sizeof(XferPt), cudaMemcpyDeviceToHost, h->stream));
                CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
                int used = 0;
                for (const XferPt& x : host) {
                    if (x.mode == -1) { cudaFree(tab); return fail(OLLIN_EINVAL, "syncboxes: a stencil leaves the partner box"); }
                    if (x.o_out == kNoPoint) continue;
                    ++used;
                    if (x.depth < 0) {
                        cudaFree(tab);
                        return fail(OLLIN_EINVAL, "overlapping boxes whose grid points do not coincide are not supported");
                    }
                }
                if (used == 0) { cudaFree(tab); continue; }
                SyncPair sp;
                sp.p = p; sp.q = q; sp.tab = tab; sp.ntab = n;
                for (const XferPt& x : host)
                    if (x.o_out != kNoPoint) sp.copies.emplace_back(x.o_out, x.depth);
                h->sync.push_back(std::move(sp));
            }
        }
    // origin of every copied point, in the order the copies run: origin[g][o]
    // = (source grid, offset from its element (0, 0)) of array element o of
    // grid g, or (-1, -1)
    std::vector<std::vector<std::pair<int, long>>> origin(h->nlev);
    for (const SyncPair& sp : h->sync) {
        const DLevel& P = h->L[sp.p];
        const DLevel& Q = h->L[sp.q];
        const size_t shp = (size_t)(P.g - 1) + (size_t)(P.g - 1) * P.ld;
        const size_t shq = (size_t)(Q.g - 1) + (size_t)(Q.g - 1) * Q.ld;
        if (origin[sp.p].empty()) origin[sp.p].assign(P.n, {-1, -1L});
        // the reads of this copy see the writes of the copies before it only
        std::vector<std::pair<size_t, std::pair<int, long>>> upd;
        for (const auto& c : sp.copies) {
            std::pair<int, long> src{sp.q, c.second};
            const size_t oq = (size_t)c.second + shq;
            if (!origin[sp.q].empty() && oq < Q.n && origin[sp.q][oq].first >= 0) src = origin[sp.q][oq];
            upd.emplace_back((size_t)c.first + shp, src);
        }
        for (const auto& u : upd) origin[sp.p][u.first] = u.second;
    }
    for (int p = 0; p < h->nlev; ++p) {
        if (origin[p].empty()) continue;
        DLevel& P = h->L[p];
        P.spartners.clear();
        P.hsmap.assign(P.n, -1);
        for (size_t o = 0; o < P.n; ++o) {
            const std::pair<int, long>& src = origin[p][o];
            if (src.first < 0) continue;
            int k = (int)(std::find(P.spartners.begin(), P.spartners.end(), src.first) - P.spartners.begin());
            if (k == (int)P.spartners.size()) {
                if (k == kMaxPartners)
                    return fail(OLLIN_EINVAL, "syncboxes: the copies onto a grid come from more than four grids");
                P.spartners.push_back(src.first);
            }
            if (src.second > kPartnerOffset)
                return fail(OLLIN_EINVAL, "syncboxes: a partner grid too large for the copy map");
            P.hsmap[o] = (int)src.second | (k << kPartnerShift);
        }
        if (!P.smap && cudaMalloc(&P.smap, P.n * sizeof(int)) != cudaSuccess)
            return fail(OLLIN_ENOMEM, "device allocation failed for the syncboxes map");
        CUDA_OR_FAIL(cudaMemcpy(P.smap, P.hsmap.data(), P.n * sizeof(int), cudaMemcpyHostToDevice));
    }
    for (const SyncPair& sp : h->sync)
        for (int g2 : {sp.p, sp.q}) {
            DLevel& G = h->L[g2];
            if (!G.snap && cudaMalloc(&G.snap, (size_t)(NFIELDS + 3) * G.n * sizeof(double)) != cudaSuccess)
                return fail(OLLIN_ENOMEM, "device allocation failed for the syncboxes state");
        }
    return OLLIN_OK;
}

// The copies of one level (syncboxes.f90): the state of every grid involved
// is kept first, then each copy takes the evolved fields and the stored
// auxiliary quantities, and the targets' next first stage reads the kept
// states (StageArgs::smap).
int sync_level(ollin_handle* h, int level) {
    bool any = false;
    for (const SyncPair& sp : h->sync)
        if (h->L[sp.p].level == level) any = true;
    if (!any) return OLLIN_OK;
    std::vector<int> kept;
    for (const SyncPair& sp : h->sync) {
        if (h->L[sp.p].level != level) continue;
        for (int g2 : {sp.p, sp.q}) {
            if (std::find(kept.begin(), kept.end(), g2) != kept.end()) continue;
            kept.push_back(g2);
            DLevel& G = h->L[g2];
            for (int f : h->fields)
                CUDA_OR_FAIL(cudaMemcpyAsync(G.snap + (size_t)f * G.n, G.slot[G.cur][f], G.n * sizeof(double),
                                             cudaMemcpyDeviceToDevice, h->stream));
            // and the inverse metric the maximal-slicing coefficients differentiate
            static const int kGSlots[3] = {X_GA, X_GB, X_GC};
            for (int k = 0; k < 3; ++k)
                CUDA_OR_FAIL(cudaMemcpyAsync(G.snap + (size_t)(NFIELDS + k) * G.n, G.aux[kGSlots[k]], G.n * sizeof(double),
                                             cudaMemcpyDeviceToDevice, h->stream));
        }
    }
    static const int kSyncAux[] = {X_GA, X_GB, X_GH, X_GC, X_KTH, X_LAM, X_ALAM, X_GLAM, X_DELDEFR, X_DELDEFZ, X_GDR, X_GDZ};
    for (const SyncPair& sp : h->sync) {
        if (h->L[sp.p].level != level) continue;
        DLevel& P = h->L[sp.p];
        DLevel& Q = h->L[sp.q];
        for (int part = 0; part < 2; ++part) {
            RestrictArgs a{};
            a.F = Q.G;
            a.Cg = P.G;
            a.nf = 0;
            if (part == 0) {
                for (int f : active_fields(h, h->t[sp.p] == 0.0)) {
                    a.fid[a.nf] = a.nf;
                    a.fin[a.nf] = base_ptr(Q, Q.slot[Q.cur][f]);
                    a.cout[a.nf] = base_ptr(P, P.slot[P.cur][f]);
                    ++a.nf;
                }
            } else {
                for (int x : kSyncAux) {
                    a.fid[a.nf] = a.nf;
                    a.fin[a.nf] = base_ptr(Q, Q.aux[x]);
                    a.cout[a.nf] = base_ptr(P, P.aux[x]);
                    ++a.nf;
                }
            }
            a.tab = sp.tab;
            a.ntab = sp.ntab;
            launch_restrict_tab(a, h->stream);
            int rc = after_launch(h);
            if (rc) return rc;
        }
        P.sync_pending = true;
    }
    return OLLIN_OK;
}
int internal_field(int field, bool* is_aux) {
    *is_aux = false;
    switch (field) {
        case OLLIN_F_ALPHA: return F_ALPHA;
        case OLLIN_F_PHI: return F_PHI;
        case OLLIN_F_CHI: return F_CHI;
        case OLLIN_F_A: return F_A;
        case OLLIN_F_B: return F_B;
        case OLLIN_F_H: return F_H;
        case OLLIN_F_C: return F_C;
        case OLLIN_F_TRK: return F_TRK;
        case OLLIN_F_KTA: return F_KTA;
        case OLLIN_F_KTB: return F_KTB;
        case OLLIN_F_KTC: return F_KTC;
        case OLLIN_F_DELTA_R: return F_DLR;
        case OLLIN_F_DELTA_Z: return F_DLZ;
        case OLLIN_F_BETA_R: return F_BETAR;
        case OLLIN_F_BETA_Z: return F_BETAZ;
        case OLLIN_F_DTBETA_R: return F_DTBETAR;
        case OLLIN_F_DTBETA_Z: return F_DTBETAZ;
        case OLLIN_F_SCALAR_PHI: return F_SPHI;
        case OLLIN_F_SCALAR_XI_R: return F_SXIR;
        case OLLIN_F_SCALAR_XI_Z: return F_SXIZ;
        case OLLIN_F_SCALAR_PI: return F_SPI;
        case OLLIN_F_FDRIVER: return F_FDRIVER;
        case OLLIN_F_KTH: *is_aux = true; return X_KTH;
        case OLLIN_F_LAMBDA: *is_aux = true; return X_LAM;
        case OLLIN_F_ALAMBDA: *is_aux = true; return X_ALAM;
        case OLLIN_F_HAM: *is_aux = true; return X_HAM;
        case OLLIN_F_MOM_R: *is_aux = true; return X_MOMR;
        case OLLIN_F_MOM_Z: *is_aux = true; return X_MOMZ;
        case OLLIN_F_RSCAL: *is_aux = true; return X_RSCAL;
        case OLLIN_F_KT2: *is_aux = true; return X_KT2;
        case OLLIN_F_LAPLA_ALPHA: *is_aux = true; return X_LAPLA;
        default: return -1;
    }
}

bool field_active(const ollin_handle* h, int f) {
    for (int x : h->fields)
        if (x == f) return true;
    return false;
}

// constraints.f90 on the current state: ham, mom_r, mom_z (+ RSCAL, KT2,
// Lapla_alpha) of one level.
int analysis(ollin_handle* h, int level) {
    DLevel& L = h->L[level];
    StageArgs a = stage_args(h, L, L.cur, L.cur, L.last_aux_t0);
    a.analysis = 1;
    launch_stage_rhs(a, h->stream);
    int rc = after_launch(h);
    if (rc) return rc;
    launch_ghost_kt2(a, h->stream);
    rc = after_launch(h);
    if (rc) return rc;
    launch_ham_edges(L.G, base_ptr(L, L.aux[X_HAM]), h->stream);
    rc = after_launch(h);
    if (rc) return rc;
    SymArgs s{};
    s.G = L.G;
    s.nf = 2;
    s.st[0] = base_ptr(L, L.aux[X_MOMR]); s.symr[0] = -1; s.symz[0] = +1;
    s.st[1] = base_ptr(L, L.aux[X_MOMZ]); s.symr[1] = +1; s.symz[1] = -1;
    launch_symmetry(s, h->stream);
    return after_launch(h);
}

// ---------------------------------------------------------------------------
// Elliptic initial data: WaveElliptic (wave_elliptic.f90) on the device.
// The solver keeps its own (u, v) arrays per level, rotated like the
// evolution's state slots, and its own time counters (the reference borrows
// and restores the global ones, wave_elliptic.f90:95-103, 330-340).
// ---------------------------------------------------------------------------
struct WLevel {
    double* pool = nullptr;
    double* u[kSlots] = {};
    double* v[kSlots] = {};
    double* ua = nullptr; double* va = nullptr;
    double* S0 = nullptr; double* S1 = nullptr; double* S5 = nullptr;
    int cur = 0, p = 1, pp = 2;
    double dt = 0;
    // physical Laplacian (maximal slicing): P1, P2, Drphi, Dzphi, psi4
    double* cpool = nullptr;
    WavePhys ph{};
};

struct WaveSolve {
    ollin_handle* h = nullptr;
    std::vector<WLevel> W;
    std::vector<double> t, t1, t2;
    std::vector<long> s;
    EllCtl* ctl = nullptr;
    double* partial = nullptr;
    double* partial2 = nullptr;
    int nparts = 0;
    int Nlmax = 0;
    int steps[2] = {0, 0};
    double gres = 0.0;
    struct Snap {
        std::vector<int> cur, p, pp;
        std::vector<double> t, t1, t2;
        std::vector<long> s;
    };
    bool physical = false;  // type = 'physical' (maximal slicing)
    ~WaveSolve() {
        for (WLevel& w : W) { cudaFree(w.pool); cudaFree(w.cpool); }
        cudaFree(ctl);
        cudaFree(partial);
        cudaFree(partial2);
    }
    Snap snap() const {
        Snap q;
        for (const WLevel& w : W) { q.cur.push_back(w.cur); q.p.push_back(w.p); q.pp.push_back(w.pp); }
        q.t = t; q.t1 = t1; q.t2 = t2; q.s = s;
        return q;
    }
    void restore(const Snap& q) {
        for (size_t l = 0; l < W.size(); ++l) { W[l].cur = q.cur[l]; W[l].p = q.p[l]; W[l].pp = q.pp[l]; }
        t = q.t; t1 = q.t1; t2 = q.t2; s = q.s;
    }
};

int wave_alloc(ollin_handle* h, WaveSolve& S) {
    const ollin_params& P = h->P;
    S.h = h;
    S.W.resize(h->nlev);
    S.t.assign(h->nlev, 0.0); S.t1.assign(h->nlev, 0.0); S.t2.assign(h->nlev, 0.0); S.s.assign(h->nlev, 0);
    const double dt0 = P.we_dtfac * std::min(P.dr0, P.dz0);  // wave_elliptic.f90:148-151
    for (int l = 0; l < h->nlev; ++l) {
        DLevel& L = h->L[l];
        WLevel& w = S.W[l];
        const size_t narr = 2 * kSlots + 5;
        if (cudaMalloc(&w.pool, narr * L.n * sizeof(double)) != cudaSuccess)
            return fail(OLLIN_ENOMEM, "device allocation failed for the elliptic solver");
        CUDA_OR_FAIL(cudaMemsetAsync(w.pool, 0, narr * L.n * sizeof(double), h->stream));
        double* q = w.pool;
        for (int k = 0; k < kSlots; ++k) { w.u[k] = q; q += L.n; }
        for (int k = 0; k < kSlots; ++k) { w.v[k] = q; q += L.n; }
        w.ua = q; q += L.n; w.va = q; q += L.n;
        w.S0 = q; q += L.n; w.S1 = q; q += L.n; w.S5 = q; q += L.n;
        w.dt = dt0 / (double)(1L << L.level);
    }
    S.nparts = wave_stage_blocks(h->L[0].G);
    if (cudaMalloc(&S.ctl, sizeof(EllCtl)) != cudaSuccess || cudaMalloc(&S.partial, S.nparts * sizeof(double)) != cudaSuccess)
        return fail(OLLIN_ENOMEM, "device allocation failed for the elliptic solver");
    return OLLIN_OK;
}

int wave_symmetry(ollin_handle* h, WaveSolve& S, int level) {
    DLevel& L = h->L[level];
    WLevel& w = S.W[level];
    SymArgs a{};
    a.G = L.G;
    a.nf = 2;
    a.st[0] = base_ptr(L, w.u[w.cur]); a.symr[0] = +1; a.symz[0] = +1;
    a.st[1] = base_ptr(L, w.v[w.cur]); a.symr[1] = +1; a.symz[1] = +1;
    a.skip = &S.ctl->done;
    launch_symmetry(a, h->stream);
    return after_launch(h);
}

int wave_prolong(ollin_handle* h, WaveSolve& S, int level, int out, double dtw) {
    DLevel& F = h->L[level];
    const int pg = F.parent;
    DLevel& C = h->L[pg];
    WLevel& wf = S.W[level];
    WLevel& wc = S.W[pg];
    ProlongArgs a{};
    a.F = F.G;
    a.Cg = C.G;
    a.nf = 2;
    a.fid[0] = 0; a.fid[1] = 1;
    a.fout[0] = base_ptr(F, wf.u[out]); a.fout[1] = base_ptr(F, wf.v[out]);
    a.fp[0] = base_ptr(F, wf.u[wf.p]); a.fp[1] = base_ptr(F, wf.v[wf.p]);
    a.fpp[0] = base_ptr(F, wf.u[wf.pp]); a.fpp[1] = base_ptr(F, wf.v[wf.pp]);
    a.cin[0] = base_ptr(C, wc.u[wc.cur]); a.cin[1] = base_ptr(C, wc.v[wc.cur]);
    a.rminl_f = h->rminl[level]; a.rmaxl_f = h->rmaxl[level];
    a.zminl_f = h->zminl[level]; a.zmaxl_f = h->zmaxl[level];
    a.rminl_c = h->rminl[pg]; a.rmaxl_c = h->rmaxl[pg];
    a.zminl_c = h->zminl[pg]; a.zmaxl_c = h->zmaxl[pg];
    a.tp = S.t[pg];
    a.t0 = S.t[level];
    a.tm1 = S.t1[level];
    a.tl = a.t0 + dtw;
    a.bicubic = h->P.interp_bicubic;
    a.skip = &S.ctl->done;
    a.tab = F.ptab;
    a.ntab = F.nptab;
    prolong_time(a, h->g);
    launch_prolong_tab(a, h->stream);
    return after_launch(h);
}

int wave_restrict(ollin_handle* h, WaveSolve& S, int level) {
    DLevel& F = h->L[level];
    const int pg = F.parent;
    DLevel& C = h->L[pg];
    WLevel& wf = S.W[level];
    WLevel& wc = S.W[pg];
    RestrictArgs a{};
    a.F = F.G;
    a.Cg = C.G;
    a.nf = 2;
    a.fid[0] = 0; a.fid[1] = 1;
    a.fin[0] = base_ptr(F, wf.u[wf.cur]); a.fin[1] = base_ptr(F, wf.v[wf.cur]);
    a.cout[0] = base_ptr(C, wc.u[wc.cur]); a.cout[1] = base_ptr(C, wc.v[wc.cur]);
    a.rminl_f = h->rminl[level]; a.rmaxl_f = h->rmaxl[level];
    a.zminl_f = h->zminl[level]; a.zmaxl_f = h->zmaxl[level];
    a.rminl_c = h->rminl[pg]; a.zminl_c = h->zminl[pg];
    a.eqsym = h->P.eqsym;
    a.bicubic = h->P.interp_bicubic;
    a.skip = &S.ctl->done;
    a.tab = F.rtab;
    a.ntab = F.nrtab;
    launch_restrict_tab(a, h->stream);
    return after_launch(h);
}

// One step of one grid in wave_elliptic.f90:578-1005 (the body of the box
// loop of subroutine wavestep), type = 'flat' or 'physical'
int wave_grid_step(ollin_handle* h, WaveSolve& S, int level) {
    const ollin_params& P = h->P;
    DLevel& L = h->L[level];
    WLevel& w = S.W[level];
    w.pp = w.p;
    w.p = w.cur;
    int freeslots[2], nfree = 0;
    for (int k = 0; k < kSlots && nfree < 2; ++k)
        if (k != w.p && k != w.pp) freeslots[nfree++] = k;
    const bool rk4 = P.we_method == OLLIN_INTEGRATOR_RK4;
    const int niter = rk4 ? 4 : P.icniter;
    const double dt = w.dt;
    int in = w.p;
    for (int iter = 1; iter <= niter; ++iter) {
        double dtw, weight = 0;
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
        const int out = freeslots[(iter - 1) & 1];
        WaveArgs a{};
        a.G = L.G;
        a.u_in = base_ptr(L, w.u[in]); a.v_in = base_ptr(L, w.v[in]);
        a.u_p = base_ptr(L, w.u[w.p]); a.v_p = base_ptr(L, w.v[w.p]);
        a.u_out = base_ptr(L, w.u[out]); a.v_out = base_ptr(L, w.v[out]);
        a.u_acc = base_ptr(L, w.ua); a.v_acc = base_ptr(L, w.va);
        a.S0 = base_ptr(L, w.S0); a.S1 = base_ptr(L, w.S1); a.S5 = base_ptr(L, w.S5);
        a.eta = P.we_eta;
        a.kdiss = P.we_diss / dt;
        a.dtw = dtw;
        a.weight = weight;
        a.rk4 = rk4 ? 1 : 0;
        a.iter = iter;
        a.niter = niter;
        a.res_partial = (level == 0 && iter == niter) ? S.partial : nullptr;
        a.skip = &S.ctl->done;
        a.physical = S.physical ? 1 : 0;
        a.ph = w.ph;
        launch_wave_stage(a, h->stream);
        int rc = after_launch(h);
        if (rc) return rc;
        if (L.level > 0) {
            rc = wave_prolong(h, S, level, out, dtw);
            if (rc) return rc;
        }
        in = out;
    }
    w.cur = in;
    S.t2[level] = S.t1[level];
    S.t1[level] = S.t[level];
    S.s[level] = S.s[level] + 1;
    S.t[level] = S.t[level] + dt;
    return OLLIN_OK;
}

// wave_elliptic.f90:578-1160 (recursive subroutine wavestep): a step of every
// box that has the level, the next level twice, the parity fills,
// ``syncboxes`` of ell_u and ell_v between boxes that overlap (plain copies:
// the solver differentiates ell_u afresh in every stage), and the
// restriction of each box into its parent.
int wavestep(ollin_handle* h, WaveSolve& S, int level) {
    for (int k = 0; k < h->nlev; ++k) {
        if (h->L[k].level != level) continue;
        int rc = wave_grid_step(h, S, k);
        if (rc) return rc;
    }
    if (level < S.Nlmax) {
        int rc = wavestep(h, S, level + 1);
        if (rc) return rc;
        rc = wavestep(h, S, level + 1);
        if (rc) return rc;
    }
    if (S.Nlmax > 0)
        for (int k = 0; k < h->nlev; ++k) {
            if (h->L[k].level != level) continue;
            int rc = wave_symmetry(h, S, k);
            if (rc) return rc;
        }
    if (level > 0)
        for (const SyncPair& sp : h->sync) {
            if (h->L[sp.p].level != level) continue;
            DLevel& P = h->L[sp.p];
            DLevel& Q = h->L[sp.q];
            WLevel& wp = S.W[sp.p];
            WLevel& wq = S.W[sp.q];
            RestrictArgs a{};
            a.F = Q.G;
            a.Cg = P.G;
            a.nf = 2;
            a.fid[0] = 0; a.fid[1] = 1;
            a.fin[0] = base_ptr(Q, wq.u[wq.cur]); a.fin[1] = base_ptr(Q, wq.v[wq.cur]);
            a.cout[0] = base_ptr(P, wp.u[wp.cur]); a.cout[1] = base_ptr(P, wp.v[wp.cur]);
            a.tab = sp.tab;
            a.ntab = sp.ntab;
            a.skip = &S.ctl->done;
            launch_restrict_tab(a, h->stream);
            int rc = after_launch(h);
            if (rc) return rc;
        }
    if (level > 0)
        for (int k = 0; k < h->nlev; ++k) {
            if (h->L[k].level != level || S.s[k] % 2 != 0) continue;
            int rc = wave_restrict(h, S, k);
            if (rc) return rc;
            rc = wave_symmetry(h, S, h->L[k].parent);
            if (rc) return rc;
        }
    return OLLIN_OK;
}

// One solver phase: iterate until the stop condition of wave_elliptic.f90:206
// holds.  Iterations are queued in batches; the device turns the ones after
// convergence into no-ops, and the host takes back the slot rotation and the
// time counters of the last iteration that ran.
int wave_phase(ollin_handle* h, WaveSolve& S, int* steps) {
    const ollin_params& P = h->P;
    std::fill(S.t.begin(), S.t.end(), 0.0);
    std::fill(S.t1.begin(), S.t1.end(), 0.0);
    std::fill(S.t2.begin(), S.t2.end(), 0.0);
    std::fill(S.s.begin(), S.s.end(), 0L);
    EllCtl c{};
    c.step = 0; c.done = 0; c.miniter = 100; c.maxiter = P.we_maxiter; c.eps = P.we_epsilon; c.gres = 1.0;
    CUDA_OR_FAIL(cudaMemcpyAsync(S.ctl, &c, sizeof(c), cudaMemcpyHostToDevice, h->stream));
    int queued = 0;
    int batch = 100;
    for (;;) {
        std::vector<WaveSolve::Snap> snaps;
        snaps.reserve(batch);
        for (int k = 0; k < batch; ++k) {
            int rc = wavestep(h, S, 0);
            if (rc) return rc;
            launch_wave_residual(S.partial, S.nparts, h->L[0].nr, h->L[0].nz, S.ctl, h->stream);
            rc = after_launch(h);
            if (rc) return rc;
            snaps.push_back(S.snap());
        }
        EllCtl hc{};
        CUDA_OR_FAIL(cudaMemcpyAsync(&hc, S.ctl, sizeof(hc), cudaMemcpyDeviceToHost, h->stream));
        CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
        if (hc.done) {
            const int idx = hc.step - queued - 1;
            if (idx < 0 || idx >= batch) return fail(OLLIN_ESTATE, "elliptic solver: inconsistent iteration count");
            S.restore(snaps[idx]);
            *steps = hc.step;
            S.gres = hc.gres;
            return OLLIN_OK;
        }
        queued += batch;
        batch = std::min(256, std::max(16, queued / 4));
    }
}

// wave_elliptic.f90:2-345 with type = 'flat' and init = 'one'; the
// coefficient arrays S0, S1, S5 are set by the caller.
int wave_elliptic(ollin_handle* h, WaveSolve& S) {
    const ollin_params& P = h->P;
    for (int l = 0; l < h->nlev; ++l) {
        DLevel& L = h->L[l];
        WLevel& w = S.W[l];
        std::vector<double> ones(L.n, 1.0);
        CUDA_OR_FAIL(cudaMemcpyAsync(w.u[w.cur], ones.data(), L.n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        CUDA_OR_FAIL(cudaMemsetAsync(w.v[w.cur], 0, L.n * sizeof(double), h->stream));
        CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
    }
    const int Nlmax_old = h->nlmax;
    S.Nlmax = Nlmax_old > 0 ? 0 : Nlmax_old;
    for (int phase = 0;; ++phase) {
        int steps = 0;
        int rc = wave_phase(h, S, &steps);
        if (rc) return rc;
        S.steps[phase] = steps;
        if (steps != P.ell_maxiter && S.Nlmax != Nlmax_old) {
            S.Nlmax = Nlmax_old;
            WLevel& w0 = S.W[0];
            DLevel& L0 = h->L[0];
            CUDA_OR_FAIL(cudaMemsetAsync(w0.v[w0.cur], 0, L0.n * sizeof(double), h->stream));
            for (int l = 1; l < h->nlev; ++l) {
                DLevel& F = h->L[l];
                WLevel& w = S.W[l];
                InjectArgs a{};
                a.F = F.G;
                a.Cg = L0.G;
                a.cin = base_ptr(L0, w0.u[w0.cur]);
                a.fout = base_ptr(F, w.u[w.cur]);
                a.rminl_f = h->rminl[l]; a.zminl_f = h->zminl[l];
                a.rminl_c = h->rminl[0]; a.rmaxl_c = h->rmaxl[0];
                a.zminl_c = h->zminl[0]; a.zmaxl_c = h->zmaxl[0];
                a.bicubic = P.interp_bicubic;
                launch_inject(a, h->stream);
                rc = after_launch(h);
                if (rc) return rc;
            }
            continue;
        }
        break;
    }
    return OLLIN_OK;
}

// ---------------------------------------------------------------------------
// SOR (sor_elliptic.f90) on the device: coarse solve with Robin boundaries,
// then every finer level with Dirichlet data interpolated from the level
// below, then restriction back down.  The iteration is in place; batches of
// iterations are queued and turned into no-ops by the device stop flag.
// ---------------------------------------------------------------------------
int sor_level_physical(ollin_handle* h, WaveSolve& S, int level, bool robin, double rjac, int* iters);

int sor_level(ollin_handle* h, WaveSolve& S, int level, bool robin, double rjac, int* iters) {
    if (S.physical) return sor_level_physical(h, S, level, robin, rjac, iters);
    const ollin_params& P = h->P;
    DLevel& L = h->L[level];
    WLevel& w = S.W[level];
    const int g = h->g;
    // coefficient columns a(i), b(i) and the constant part of e
    // (sor_elliptic.f90:141-151), evaluated as written
    std::vector<double> cab(2 * (size_t)(L.nr + g));
    for (int i = 1 - g; i <= L.nr; ++i) {
        const double r = L.rh[i - 1 + g];
        cab[i - 1 + g] = (1.0 / L.dr + 0.5 / r) / L.dr;
        cab[(L.nr + g) + (i - 1 + g)] = (1.0 / L.dr - 0.5 / r) / L.dr;
    }
    double* dcab = nullptr;
    if (cudaMalloc(&dcab, cab.size() * sizeof(double)) != cudaSuccess) return fail(OLLIN_ENOMEM, "device allocation failed");
    struct FreeOnExit { double* p; ~FreeOnExit() { cudaFree(p); } } free_cab{dcab};
    CUDA_OR_FAIL(cudaMemcpyAsync(dcab, cab.data(), cab.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    const double ec = -2.0 * (1.0 / (L.dr * L.dr) + 1.0 / (L.dz * L.dz));
    double* eaux = w.ua;  // the WaveElliptic accumulators are free during SOR
    double* e = w.va;
    launch_add(L.G, base_ptr(L, eaux), ec, base_ptr(L, w.S1), h->stream);
    int rc = after_launch(h);
    if (rc) return rc;
    // with S5 = 0, e = aux + 0*u^4 = aux exactly, so the update is skipped
    const bool s5 = P.idata == OLLIN_IDATA_SCALARPULSE && P.scalarpotential != OLLIN_POTENTIAL_NONE;
    EllCtl c{};
    c.maxiter = P.ell_maxiter; c.eps = P.ell_epsilon; c.gres = 1.0;
    CUDA_OR_FAIL(cudaMemcpyAsync(S.ctl, &c, sizeof(c), cudaMemcpyHostToDevice, h->stream));
    double omega = 1.0;
    int n = 0, batch = 64;
    for (;;) {
        for (int k = 0; k < batch; ++k) {
            ++n;
            if (s5) {
                launch_sor_e(L.G, base_ptr(L, e), base_ptr(L, eaux), base_ptr(L, w.S5), base_ptr(L, w.u[w.cur]),
                             &S.ctl->done, h->stream);
                rc = after_launch(h);
                if (rc) return rc;
            }
            for (int ipass = 1; ipass <= 2; ++ipass) {
                SorPassArgs a{};
                a.G = L.G;
                a.u = base_ptr(L, w.u[w.cur]);
                a.ca = dcab + (g - 1);
                a.cb = dcab + (L.nr + g) + (g - 1);
                a.cc = 1.0 / (L.dz * L.dz);
                a.e = base_ptr(L, s5 ? e : eaux);
                a.f = base_ptr(L, w.S0);
                a.omega = omega;
                a.parity = ipass == 1 ? 0 : 1;
                a.partial = ipass == 1 ? S.partial : S.partial2;
                a.skip = &S.ctl->done;
                launch_sor_pass(a, h->stream);
                rc = after_launch(h);
                if (rc) return rc;
                // Chebyshev acceleration (sor_elliptic.f90:690-694)
                if (n == 1 && ipass == 1) omega = 1.0 / (1.0 - 0.5 * (rjac * rjac));
                else omega = 1.0 / (1.0 - 0.25 * (rjac * rjac) * omega);
            }
            SorFinishArgs f{};
            f.G = L.G;
            f.u = base_ptr(L, w.u[w.cur]);
            f.partial1 = S.partial;
            f.partial2 = S.partial2;
            f.nparts = sor_pass_blocks(L.G);
            f.robin = robin ? 1 : 0;
            f.uinf = 1.0;
            f.ctl = S.ctl;
            if (launch_sor_finish(f, h->stream))
                return fail(OLLIN_ECUDA, "SOR boundary kernel: shared memory for the Robin edges not available");
            rc = after_launch(h);
            if (rc) return rc;
        }
        EllCtl hc{};
        CUDA_OR_FAIL(cudaMemcpyAsync(&hc, S.ctl, sizeof(hc), cudaMemcpyDeviceToHost, h->stream));
        CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
        if (hc.done) {
            *iters = hc.step;
            S.gres = hc.gres;
            return OLLIN_OK;
        }
        batch = std::min(1024, std::max(64, n / 4));
    }
}

// sor on one level with the nine-point stencil of the physical Laplacian
// (maximal slicing, S5 = 0 so the diagonal stays fixed).  While every
// diagonal coefficient is zero the colours decouple and the pass runs over
// all points at once; otherwise one block sweeps the columns in the
// reference's order.
int sor_level_physical(ollin_handle* h, WaveSolve& S, int level, bool robin, double rjac, int* iters) {
    const ollin_params& P = h->P;
    DLevel& L = h->L[level];
    WLevel& w = S.W[level];
    double* pool = nullptr;
    unsigned long long* dflag = nullptr;
    if (cudaMalloc(&pool, 9 * L.n * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&dflag, sizeof(unsigned long long)) != cudaSuccess) {
        cudaFree(pool);
        return fail(OLLIN_ENOMEM, "device allocation failed for the SOR coefficients");
    }
    struct FreeOnExit { void* a; void* b; ~FreeOnExit() { cudaFree(a); cudaFree(b); } } fr{pool, dflag};
    CUDA_OR_FAIL(cudaMemsetAsync(pool, 0, 9 * L.n * sizeof(double), h->stream));
    CUDA_OR_FAIL(cudaMemsetAsync(dflag, 0, sizeof(unsigned long long), h->stream));
    double* arr[9];
    for (int k = 0; k < 9; ++k) arr[k] = pool + (size_t)k * L.n;
    SorCoeffArgs c{};
    c.G = L.G;
    c.ph = w.ph;
    c.S1 = base_ptr(L, w.S1);
    c.fine = level > 0 ? 1 : 0;
    c.a = base_ptr(L, arr[0]); c.b = base_ptr(L, arr[1]); c.c = base_ptr(L, arr[2]); c.d = base_ptr(L, arr[3]);
    c.e = base_ptr(L, arr[4]);
    c.cg = base_ptr(L, arr[5]); c.ch = base_ptr(L, arr[6]); c.ci = base_ptr(L, arr[7]); c.cj = base_ptr(L, arr[8]);
    c.diag_nonzero = dflag;
    launch_sor_coeffs(c, h->stream);
    int rc = after_launch(h);
    if (rc) return rc;
    unsigned long long hdiag = 0;
    CUDA_OR_FAIL(cudaMemcpyAsync(&hdiag, dflag, sizeof(hdiag), cudaMemcpyDeviceToHost, h->stream));
    CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
    const bool seq = hdiag != 0;
    EllCtl ctl{};
    ctl.maxiter = P.ell_maxiter; ctl.eps = P.ell_epsilon; ctl.gres = 1.0;
    CUDA_OR_FAIL(cudaMemcpyAsync(S.ctl, &ctl, sizeof(ctl), cudaMemcpyHostToDevice, h->stream));
    double omega = 1.0;
    int n = 0, batch = 64;
    for (;;) {
        for (int k = 0; k < batch; ++k) {
            ++n;
            for (int ipass = 1; ipass <= 2; ++ipass) {
                SorPhysPassArgs a{};
                a.G = L.G;
                a.u = base_ptr(L, w.u[w.cur]);
                a.a = c.a; a.b = c.b; a.c = c.c; a.d = c.d; a.e = c.e;
                a.cg = c.cg; a.ch = c.ch; a.ci = c.ci; a.cj = c.cj;
                a.f = base_ptr(L, w.S0);
                a.omega = omega;
                a.parity = ipass == 1 ? 0 : 1;
                a.partial = ipass == 1 ? S.partial : S.partial2;
                a.skip = &S.ctl->done;
                if (seq) launch_sor_phys_pass_seq(a, h->stream);
                else launch_sor_phys_pass(a, h->stream);
                rc = after_launch(h);
                if (rc) return rc;
                if (n == 1 && ipass == 1) omega = 1.0 / (1.0 - 0.5 * (rjac * rjac));
                else omega = 1.0 / (1.0 - 0.25 * (rjac * rjac) * omega);
            }
            SorFinishArgs f{};
            f.G = L.G;
            f.u = base_ptr(L, w.u[w.cur]);
            f.partial1 = S.partial;
            f.partial2 = S.partial2;
            f.nparts = seq ? 1 : sor_pass_blocks(L.G);
            f.robin = robin ? 1 : 0;
            f.uinf = 1.0;
            f.ctl = S.ctl;
            if (launch_sor_finish(f, h->stream))
                return fail(OLLIN_ECUDA, "SOR boundary kernel: shared memory for the Robin edges not available");
            rc = after_launch(h);
            if (rc) return rc;
        }
        EllCtl hc{};
        CUDA_OR_FAIL(cudaMemcpyAsync(&hc, S.ctl, sizeof(hc), cudaMemcpyDeviceToHost, h->stream));
        CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
        if (hc.done) {
            *iters = hc.step;
            S.gres = hc.gres;
            return OLLIN_OK;
        }
        batch = std::min(1024, std::max(64, n / 4));
    }
}

int sor_elliptic(ollin_handle* h, WaveSolve& S) {
    const ollin_params& P = h->P;
    // the Robin edges are staged in shared memory (six doubles per edge point)
    if (sor_finish_smem(h->L[0].G) > (size_t)200 * 1024)
        return fail(OLLIN_EINVAL, "ELL_solver = sor on the device supports Nrtotal + Nztotal up to 4260");
    // partial sums of the two passes (the largest grid's count)
    int nparts = 1;
    for (const DLevel& L : h->L) nparts = std::max(nparts, sor_pass_blocks(L.G));
    if (S.nparts < nparts) {
        cudaFree(S.partial);
        S.partial = nullptr;
        if (cudaMalloc(&S.partial, nparts * sizeof(double)) != cudaSuccess)
            return fail(OLLIN_ENOMEM, "device allocation failed for the elliptic solver");
        S.nparts = nparts;
    }
    if (cudaMalloc(&S.partial2, nparts * sizeof(double)) != cudaSuccess)
        return fail(OLLIN_ENOMEM, "device allocation failed for the elliptic solver");
    for (int l = 0; l < h->nlev; ++l) {
        DLevel& L = h->L[l];
        WLevel& w = S.W[l];
        std::vector<double> ones(L.n, 1.0);
        CUDA_OR_FAIL(cudaMemcpyAsync(w.u[w.cur], ones.data(), L.n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
    }
    // Jacobi spectral radius (sor_elliptic.f90:126-128) from the grid that is
    // current on entry: the last box's last level
    const DLevel& L0 = h->L[h->nlev - 1];
    const double pi = 3.141592653589793;
    const double rjac = (L0.dz / L0.dr * std::cos(pi / (double)(L0.nr + L0.g))
                         + L0.dr / L0.dz * std::cos(pi / (double)(L0.nz + L0.g))) / (L0.dz / L0.dr + L0.dr / L0.dz);
    int rc = sor_level(h, S, 0, true, rjac, &S.steps[0]);
    if (rc) return rc;
    // sor_elliptic.f90:293-491: every box, levels 1..Nl(box), in the grid
    // list's order; each grid starts from and is bounded by interpolation
    // from its parent (box 0's level 0 for level 1, else its box's coarser level)
    for (int l = 1; l < h->nlev; ++l) {
        DLevel& F = h->L[l];
        const int pl = F.parent;
        DLevel& C = h->L[pl];
        InjectArgs a{};
        a.F = F.G;
        a.Cg = C.G;
        a.cin = base_ptr(C, S.W[pl].u[S.W[pl].cur]);
        a.fout = base_ptr(F, S.W[l].u[S.W[l].cur]);
        a.rminl_f = h->rminl[l]; a.zminl_f = h->zminl[l];
        a.rminl_c = h->rminl[pl]; a.rmaxl_c = h->rmaxl[pl];
        a.zminl_c = h->zminl[pl]; a.zmaxl_c = h->zmaxl[pl];
        a.bicubic = P.interp_bicubic;
        launch_inject(a, h->stream);
        rc = after_launch(h);
        if (rc) return rc;
        int it = 0;
        rc = sor_level(h, S, l, false, rjac, &it);
        if (rc) return rc;
        if (l == 1) S.steps[1] = it;
    }
    for (int l = 1; l < h->nlev; ++l) {  // sor_elliptic.f90:497-521, the same order
        DLevel& F = h->L[l];
        const int pl = F.parent;
        DLevel& C = h->L[pl];
        RestrictArgs a{};
        a.F = F.G;
        a.Cg = C.G;
        a.nf = 1;
        a.fid[0] = 0;
        a.fin[0] = base_ptr(F, S.W[l].u[S.W[l].cur]);
        a.cout[0] = base_ptr(C, S.W[pl].u[S.W[pl].cur]);
        a.rminl_f = h->rminl[l]; a.rmaxl_f = h->rmaxl[l];
        a.zminl_f = h->zminl[l]; a.zmaxl_f = h->zmaxl[l];
        a.rminl_c = h->rminl[pl]; a.zminl_c = h->zminl[pl];
        a.eqsym = P.eqsym;
        a.bicubic = P.interp_bicubic;
        launch_restrict(a, h->stream);
        rc = after_launch(h);
        if (rc) return rc;
    }
    return OLLIN_OK;
}

// ---------------------------------------------------------------------------
// Mixed precision (ELL_solver = "mixed", no counterpart in the reference):
// the discrete system of sor_elliptic.f90 solved by iterative refinement --
// FP64 residual and update, the correction from FP32 multigrid V-cycles --
// until the RMS residual of the interior equations is below ELL_epsilon or
// stops falling (the FP64 rounding floor, about 1e-16 of the diagonal terms
// e*u, which on fine grids lies above 1e-12).  FP32 rounding limits one correction to
// about 1e-3 of its residual, so each refinement runs a few V-cycles.  Same
// level sequence as SOR (coarse Robin problem, Dirichlet problems of the
// finer levels).
// ---------------------------------------------------------------------------
int mix_level(ollin_handle* h, WaveSolve& S, int level, bool robin, int* outer_out, int* cycles_out, double* rms_out) {
    const ollin_params& P = h->P;
    DLevel& L = h->L[level];
    WLevel& w = S.W[level];
    const int g = h->g;
    const size_t ncol = (size_t)(L.nr + g);
    std::vector<double> cab(2 * ncol);
    for (int i = 1 - g; i <= L.nr; ++i) {
        const double r = L.rh[i - 1 + g];
        cab[i - 1 + g] = (1.0 / L.dr + 0.5 / r) / L.dr;
        cab[ncol + (i - 1 + g)] = (1.0 / L.dr - 0.5 / r) / L.dr;
    }
    // the correction's precision: FP32 ("mixed") or FP64 ("fp64mg", the
    // all-FP64 solve of the same system)
    const bool fp64 = P.ell_solver == OLLIN_ELL_FP64MG;
    const size_t csize = fp64 ? sizeof(double) : sizeof(float);
    double* dcol = nullptr;
    void* cbuf = nullptr;
    if (cudaMalloc(&dcol, 2 * ncol * sizeof(double)) != cudaSuccess || cudaMalloc(&cbuf, 3 * L.n * csize) != cudaSuccess) {
        cudaFree(dcol);
        return fail(OLLIN_ENOMEM, "device allocation failed for the mixed-precision solver");
    }
    // the unknowns: from 1 on a grid owning the axis / equator, from 2-ghost on
    // a refinement box off them (its outermost ghost row is Dirichlet data)
    const int ilo = L.G.axis ? 1 : 2 - g, jlo = L.G.equator ? 1 : 2 - g;
    MgHierarchy* mg = mg_create(L.nr - ilo + 1, L.nz - jlo + 1, L.dr, L.dz, fp64 ? 1 : 0);
    struct FreeOnExit {
        double* a; void* b; MgHierarchy* m;
        ~FreeOnExit() { cudaFree(a); cudaFree(b); mg_destroy(m); }
    } free_all{dcol, cbuf, mg};
    if (!mg) return fail(OLLIN_ENOMEM, "device allocation failed for the multigrid hierarchy");
    CUDA_OR_FAIL(cudaMemcpyAsync(dcol, cab.data(), 2 * ncol * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CUDA_OR_FAIL(cudaMemsetAsync(cbuf, 0, 3 * L.n * csize, h->stream));
    const size_t off = (size_t)(g - 1) + (size_t)(g - 1) * L.ld;  // correction arrays share the level layout
    float* f32 = fp64 ? nullptr : (float*)cbuf;
    double* f64 = fp64 ? (double*)cbuf : nullptr;
    float* d = fp64 ? nullptr : f32 + off;
    float* r32 = fp64 ? nullptr : f32 + L.n + off;
    double* d64 = fp64 ? f64 + off : nullptr;
    double* r64 = fp64 ? f64 + L.n + off : nullptr;
    const double ec = -2.0 * (1.0 / (L.dr * L.dr) + 1.0 / (L.dz * L.dz));
    double* eaux = w.ua;
    double* e = w.va;
    launch_add(L.G, base_ptr(L, eaux), ec, base_ptr(L, w.S1), h->stream);
    int rc = after_launch(h);
    if (rc) return rc;
    const bool s5 = !S.physical && P.idata == OLLIN_IDATA_SCALARPULSE && P.scalarpotential != OLLIN_POTENTIAL_NONE;
    const int nparts = mix_blocks(L.G, robin ? 1 : 0);
    if (S.nparts < 3 * nparts) {
        cudaFree(S.partial);
        S.partial = nullptr;
        if (cudaMalloc(&S.partial, 3 * nparts * sizeof(double)) != cudaSuccess)
            return fail(OLLIN_ENOMEM, "device allocation failed for the mixed-precision solver");
        S.nparts = 3 * nparts;
    }
    // maximal slicing: the nine-point stencil of the physical Laplacian
    double* phys = nullptr;
    struct FreePhys { double* p; ~FreePhys() { cudaFree(p); } } free_phys{nullptr};
    if (S.physical) {
        if (cudaMalloc(&phys, (9 * L.n + 1) * sizeof(double)) != cudaSuccess)
            return fail(OLLIN_ENOMEM, "device allocation failed for the mixed-precision solver");
        free_phys.p = phys;
        CUDA_OR_FAIL(cudaMemsetAsync(phys, 0, (9 * L.n + 1) * sizeof(double), h->stream));
    }
    MixArgs a{};
    a.G = L.G;
    a.u = base_ptr(L, w.u[w.cur]);
    a.e64 = base_ptr(L, s5 ? e : eaux);
    if (S.physical) {
        double* q[9];
        for (int k = 0; k < 9; ++k) q[k] = base_ptr(L, phys + (size_t)k * L.n);
        SorCoeffArgs c{};
        c.G = L.G;
        c.ph = w.ph;
        c.S1 = base_ptr(L, w.S1);
        c.fine = level > 0 ? 1 : 0;
        c.a = q[0]; c.b = q[1]; c.c = q[2]; c.d = q[3]; c.e = q[4];
        c.cg = q[5]; c.ch = q[6]; c.ci = q[7]; c.cj = q[8];
        c.diag_nonzero = reinterpret_cast<unsigned long long*>(phys + 9 * L.n);  // not needed here
        launch_sor_coeffs(c, h->stream);
        rc = after_launch(h);
        if (rc) return rc;
        a.pa = q[0]; a.pb = q[1]; a.pc = q[2]; a.pd = q[3]; a.e64 = q[4];
        a.pg = q[5]; a.ph = q[6]; a.pi = q[7]; a.pj = q[8];
    }
    a.f64 = base_ptr(L, w.S0);
    a.ca = dcol + (g - 1);
    a.cb = dcol + ncol + (g - 1);
    a.cc = 1.0 / (L.dz * L.dz);
    a.d = d;
    a.r32 = r32;
    a.d64 = d64;
    a.r64 = r64;
    a.robin = robin ? 1 : 0;
    a.uinf = 1.0;
    a.partial = S.partial;
    // the five-point part of the level's stencil, which the multigrid
    // coarsens (the variable coefficients of the physical Laplacian included)
    MgStencil ms{};
    ms.pa = a.pa; ms.pb = a.pb; ms.pc = a.pc; ms.pd = a.pd;
    ms.ca = a.ca; ms.cb = a.cb; ms.cc = a.cc;
    ms.e = a.e64;
    ms.ld = L.ld;
    ms.dr = L.dr; ms.dz = L.dz;
    ms.ioff = ilo - 1; ms.joff = jlo - 1;
    ms.r0 = L.G.axis ? 0.0 : L.rh[ilo - 1 + g] - 0.5 * L.dr;
    ms.z0 = L.G.equator ? 0.0 : L.zh[jlo - 1 + g] - 0.5 * L.dz;
    ms.mr = L.G.axis; ms.mz = L.G.equator;
    // without equatorial symmetry the coarse problem's lowest row j = 1-ghost
    // is a Robin row: the multigrid holds it as its row 0
    ms.rz = robin && !L.G.equator ? 1 : 0;
    // Orthomin storage: a ring of kOrthoSlots directions z and their images
    // q = A z, the FP64 residual for the FP32 solve, per-block dot products
    constexpr int kOrthoSlots = 7;  // the new direction + up to 6 kept
    static_assert(kOrthoSlots - 1 <= kOrthoMax, "Orthomin ring larger than the kernels take");
    const size_t nvec = 2 * (size_t)kOrthoSlots + (fp64 ? 0 : 1);
    double* ortho = nullptr;
    double* dpart = nullptr;
    struct FreeOrtho { double* a; double* b; ~FreeOrtho() { cudaFree(a); cudaFree(b); } } free_ortho{nullptr, nullptr};
    if (cudaMalloc(&ortho, nvec * L.n * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&dpart, (size_t)(kOrthoMax + 2) * nparts * sizeof(double)) != cudaSuccess) {
        cudaFree(ortho);
        return fail(OLLIN_ENOMEM, "device allocation failed for the mixed-precision solver");
    }
    free_ortho.a = ortho;
    free_ortho.b = dpart;
    CUDA_OR_FAIL(cudaMemsetAsync(ortho, 0, nvec * L.n * sizeof(double), h->stream));
    double* Zs[kOrthoSlots];
    double* Qs[kOrthoSlots];
    for (int k = 0; k < kOrthoSlots; ++k) {
        Zs[k] = base_ptr(L, ortho + (size_t)k * L.n);
        Qs[k] = base_ptr(L, ortho + (size_t)(kOrthoSlots + k) * L.n);
    }
    if (!fp64) a.r64 = base_ptr(L, ortho + (size_t)(2 * kOrthoSlots) * L.n);
    double qq[kOrthoSlots] = {0};
    int head = 0, stored = 0;
    std::vector<double> hd((size_t)(kOrthoMax + 2) * nparts);
    // sums over the blocks of the first n dot products, in block order
    auto dots = [&](const double* x, const OrthoVecs& y, int n, double* out) -> int {
        launch_mix_dots(L.G, a.robin, x, y, n, dpart, h->stream);
        int rc2 = after_launch(h);
        if (rc2) return rc2;
        CUDA_OR_FAIL(cudaMemcpyAsync(hd.data(), dpart, (size_t)n * nparts * sizeof(double), cudaMemcpyDeviceToHost,
                                     h->stream));
        CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
        for (int k = 0; k < n; ++k) {
            double acc = 0.0;
            for (int b = 0; b < nparts; ++b) acc += hd[(size_t)k * nparts + b];
            out[k] = acc;
        }
        return OLLIN_OK;
    };
    std::vector<double> hp(3 * nparts);
    int outer = 0, cycles = 0, ncyc = 2, flat = 0, post = 0;
    double rms = 0.0, last = 0.0;
    if ((int)h->ell_hist.size() != h->nlev) h->ell_hist.assign(h->nlev, {});
    std::vector<double>& hist = h->ell_hist[level];
    hist.clear();
    for (;;) {
        if (s5) {
            launch_sor_e(L.G, base_ptr(L, e), base_ptr(L, eaux), base_ptr(L, w.S5), base_ptr(L, w.u[w.cur]), nullptr,
                         h->stream);
            rc = after_launch(h);
            if (rc) return rc;
        }
        launch_mix_resid(a, h->stream);
        rc = after_launch(h);
        if (rc) return rc;
        CUDA_OR_FAIL(cudaMemcpyAsync(hp.data(), S.partial, 3 * nparts * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
        double sum = 0.0, scale = 0.0, sumb = 0.0;
        for (int k = 0; k < nparts; ++k) { sum += hp[k]; scale += hp[nparts + k]; sumb += hp[2 * nparts + k]; }
        const double nint = (double)(L.nr - ilo) * (double)(L.nz - jlo);
        const double rms_in = std::sqrt(sum / nint);
        // the Robin rows (level 0): a smooth offset of the whole solution moves
        // them by its size while the interior rows hardly see it, so they are
        // held to the tolerance on their own
        const double nrob = !robin ? 0.0 : L.G.equator ? (double)(L.nr + L.nz - 1)
                                                        : (double)(L.nz + g + 2 * (L.nr - 1));
        const double rms_b = robin ? std::sqrt(sumb / nrob) : 0.0;
        rms = std::max(rms_in, rms_b);
        // the FP64 floor of a row: the residual of the solution rounded to
        // FP64, about a unit roundoff of the diagonal term (e*u inside, the
        // Robin row's 1 + 1.5 (r/dr + z/dz) on the edges)
        const double floor64 = 1.1e-16 * std::sqrt(scale / nint);
        const double floor_b = 1.1e-16 * (1.0 + 1.5 * (L.rh[L.nr - 1 + g] / L.dr + L.zh[L.nz - 1 + g] / L.dz));
        const bool near_floor = rms_in < 100.0 * floor64 && rms_b < 100.0 * floor_b;
        hist.push_back(rms);
        if (!std::isfinite(rms))
            return fail(OLLIN_ENAN, "non-finite residual in the multigrid solve of level " + std::to_string(level)
                                        + " (refinement " + std::to_string(outer) + ")");
        // converged: two more refinements past the tolerance take out the
        // smooth error its residual hides (the lowest modes of the operator
        // have eigenvalues near 1e-3, so a residual of 1e-12 still allows an
        // offset near 1e-9)
        if (rms < P.ell_epsilon) {
            if (++post > 2) break;
        } else if (outer >= 60) {
            if (near_floor) break;
            return fail(OLLIN_ECONV, "the multigrid solve of level " + std::to_string(level) + " did not converge: RMS "
                                         + "residual " + std::to_string(rms) + " after 60 refinements");
        }
        if (outer > 0 && post == 0) {
            // at the FP64 floor the residual stops falling; a few more
            // refinements still take out the smooth error that the floor's
            // rounding residual hides (the residual sums are exact)
            flat = (rms > 0.5 * last && near_floor) ? flat + 1 : 0;
            if (flat >= 3) break;
            // a refinement that gained less than a decade gets more cycles next time
            if (rms > 0.1 * last) ncyc = std::min(ncyc * 2, 16);
        }
        last = rms;
        ++outer;
        // the operator once, or every refinement when S5 u^4 enters the diagonal
        if (outer == 1 || s5) {
            mg_load_operator(mg, ms, h->stream);
            h->launches += mg_levels(mg);
        }
        mg_set_rhs(mg, fp64 ? (const void*)r64 : (const void*)r32, L.ld, h->stream);
        mg_solve(mg, a.robin, ncyc, fp64 ? (void*)d64 : (void*)d, L.ld, h->stream);
        h->launches += 2 + (long long)ncyc * mg_launches_per_cycle(mg, a.robin);
        CUDA_OR_FAIL(cudaGetLastError());
        cycles += ncyc;
        // the correction as a search direction: q = A z, orthogonal to the
        // kept images (none when S5 u^4 changed the operator), then the step
        // that minimises the residual along q
        if (s5) stored = 0;
        launch_mix_apply(a, Zs[head], Qs[head], h->stream);
        rc = after_launch(h);
        if (rc) return rc;
        const int nprev = std::min(stored, kOrthoSlots - 1);
        if (nprev > 0) {
            OrthoVecs zy{}, qy{};
            OrthoCoef beta{};
            for (int k = 0; k < nprev; ++k) {
                const int sl = (head - 1 - k + kOrthoSlots) % kOrthoSlots;
                zy.v[k] = Zs[sl];
                qy.v[k] = Qs[sl];
            }
            double dq[kOrthoMax];
            rc = dots(Qs[head], qy, nprev, dq);
            if (rc) return rc;
            for (int k = 0; k < nprev; ++k) {
                const int sl = (head - 1 - k + kOrthoSlots) % kOrthoSlots;
                beta.c[k] = qq[sl] > 0.0 ? dq[k] / qq[sl] : 0.0;
            }
            launch_mix_orth(L.G, a.robin, Zs[head], Qs[head], zy, qy, beta, nprev, h->stream);
            rc = after_launch(h);
            if (rc) return rc;
        }
        OrthoVecs rq{};
        rq.v[0] = a.r64;
        rq.v[1] = Qs[head];
        double d2[2];
        rc = dots(Qs[head], rq, 2, d2);
        if (rc) return rc;
        if (!(d2[1] > 0.0) || !std::isfinite(d2[0])) break;  // no direction left (the residual is zero)
        launch_mix_step(L.G, a.robin, a.u, Zs[head], d2[0] / d2[1], h->stream);
        rc = after_launch(h);
        if (rc) return rc;
        qq[head] = d2[1];
        head = (head + 1) % kOrthoSlots;
        ++stored;
    }
    // parity fill of the solution (the ghosts mirror the first points)
    SymArgs sy{};
    sy.G = L.G;
    sy.nf = 1;
    sy.st[0] = base_ptr(L, w.u[w.cur]);
    sy.symr[0] = +1;
    sy.symz[0] = +1;
    launch_symmetry(sy, h->stream);
    rc = after_launch(h);
    if (rc) return rc;
    *outer_out = outer;
    *cycles_out = cycles;
    *rms_out = rms;
    return OLLIN_OK;
}

int mixed_elliptic(ollin_handle* h, WaveSolve& S) {
    const ollin_params& P = h->P;
    for (int l = 0; l < h->nlev; ++l) {
        DLevel& L = h->L[l];
        WLevel& w = S.W[l];
        std::vector<double> ones(L.n, 1.0);
        CUDA_OR_FAIL(cudaMemcpyAsync(w.u[w.cur], ones.data(), L.n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
    }
    int outer = 0, inner = 0;
    double rms = 0.0;
    int rc = mix_level(h, S, 0, true, &outer, &inner, &rms);
    if (rc) return rc;
    S.steps[0] = outer;
    S.steps[1] = inner;
    S.gres = rms;
    for (int l = 1; l < h->nlev; ++l) {
        DLevel& F = h->L[l];
        const int pl = F.parent;
        DLevel& C = h->L[pl];
        InjectArgs a{};
        a.F = F.G;
        a.Cg = C.G;
        a.cin = base_ptr(C, S.W[pl].u[S.W[pl].cur]);
        a.fout = base_ptr(F, S.W[l].u[S.W[l].cur]);
        a.rminl_f = h->rminl[l]; a.zminl_f = h->zminl[l];
        a.rminl_c = h->rminl[pl]; a.rmaxl_c = h->rmaxl[pl];
        a.zminl_c = h->zminl[pl]; a.zmaxl_c = h->zmaxl[pl];
        a.bicubic = P.interp_bicubic;
        launch_inject(a, h->stream);
        rc = after_launch(h);
        if (rc) return rc;
        int o2 = 0, i2 = 0;
        double r2 = 0.0;
        rc = mix_level(h, S, l, false, &o2, &i2, &r2);
        if (rc) return rc;
        S.gres = std::max(S.gres, r2);
    }
    for (int l = 1; l < h->nlev; ++l) {
        DLevel& F = h->L[l];
        const int pl = F.parent;
        DLevel& C = h->L[pl];
        RestrictArgs a{};
        a.F = F.G;
        a.Cg = C.G;
        a.nf = 1;
        a.fid[0] = 0;
        a.fin[0] = base_ptr(F, S.W[l].u[S.W[l].cur]);
        a.cout[0] = base_ptr(C, S.W[pl].u[S.W[pl].cur]);
        a.rminl_f = h->rminl[l]; a.rmaxl_f = h->rmaxl[l];
        a.zminl_f = h->zminl[l]; a.zmaxl_f = h->zmaxl[l];
        a.rminl_c = h->rminl[pl]; a.zminl_c = h->zminl[pl];
        a.eqsym = P.eqsym;
        a.bicubic = P.interp_bicubic;
        launch_restrict(a, h->stream);
        rc = after_launch(h);
        if (rc) return rc;
    }
    return OLLIN_OK;
}

// The pre-solve part of the elliptic initial data, the solve, and the
// solution of every level copied to the host (``ell_u``, all points).
// Scalar pulse (idata_scalarpulse.f90:46-170): the pulse is evaluated here,
// its gradient and the coefficients on the device, and the four scalar
// fields are returned in ``scal``.  Brill wave (idata_brillwave.f90:60-118):
// brillq and S1 are evaluated here, brillq is returned.
int elliptic_data(ollin_handle* h, std::vector<std::vector<double>>& ell_u, std::vector<std::vector<double>>& brillq,
                  std::vector<std::vector<std::vector<double>>>& scal) {
    const ollin_params& P = h->P;
    const int g = h->g;
    WaveSolve S;
    int rc = wave_alloc(h, S);
    if (rc) return rc;
    const bool pulse = P.idata == OLLIN_IDATA_SCALARPULSE;
    const double pi = 3.141592653589793;
    ell_u.assign(h->nlev, {});
    brillq.assign(h->nlev, {});
    scal.assign(h->nlev, {});
    for (int l = 0; l < h->nlev; ++l) {
        DLevel& L = h->L[l];
        WLevel& w = S.W[l];
        auto at = [&](int i, int j) { return (size_t)(i - 1 + g) + (size_t)(j - 1 + g) * L.ld; };
        if (pulse) {
            const double a0 = P.scalar_a0, r0 = P.scalar_r0, z0 = P.scalar_z0, sr0 = P.scalar_sr0, sz0 = P.scalar_sz0;
            std::vector<double> ph(L.n, 0.0);
            for (int j = 1 - g; j <= L.nz; ++j)
                for (int i = 1 - g; i <= L.nr; ++i) {
                    const double R = L.rh[i - 1 + g], Z = L.zh[j - 1 + g];
                    const double RR = std::sqrt(R * R + Z * Z);
                    double v;
                    if (P.scalarpulse_type == OLLIN_PULSE_SHELL) {
                        if (r0 == 0.0 && z0 == 0.0) {
                            v = a0 * std::exp(-((R * R) / (sr0 * sr0) + (Z * Z) / (sz0 * sz0)));
                        } else {
                            const double cen = ((R * R) * r0 + (Z * Z) * z0) / (RR * RR);
                            const double den = (R * R) * (sr0 * sr0) + (Z * Z) * (sz0 * sz0);
                            v = a0 * (std::exp(-(((RR - cen) * (RR - cen)) * (RR * RR) / den))
                                      + std::exp(-(((RR + cen) * (RR + cen)) * (RR * RR) / den)));
                        }
                    } else if (P.scalarpulse_type == OLLIN_PULSE_TORUS) {
                        auto sq = [](double x) { return x * x; };
                        if (r0 == 0.0 && z0 == 0.0) v = a0 * std::exp(-sq(R / sr0)) * std::exp(-sq(Z / sz0));
                        else v = a0 * (std::exp(-sq((R - r0) / sr0)) + std::exp(-sq((R + r0) / sr0)))
                                 * (std::exp(-sq((Z - z0) / sz0)) + std::exp(-sq((Z + z0) / sz0)));
                    } else {
                        v = a0 * std::exp(-((R * R) + (1.0 - sz0) * (Z * Z)));
                    }
                    ph[at(i, j)] = v;
                }
            CUDA_OR_FAIL(cudaMemcpyAsync(L.slot[L.cur][F_SPHI], ph.data(), L.n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
            PulseCoeffArgs a{};
            a.G = L.G;
            a.sphi = base_ptr(L, L.slot[L.cur][F_SPHI]);
            a.xir = base_ptr(L, L.slot[L.cur][F_SXIR]);
            a.xiz = base_ptr(L, L.slot[L.cur][F_SXIZ]);
            a.spi = base_ptr(L, L.slot[L.cur][F_SPI]);
            a.S0 = base_ptr(L, w.S0); a.S1 = base_ptr(L, w.S1); a.S5 = base_ptr(L, w.S5);
            a.potential = P.scalarpotential;
            a.mass = P.scalar_mass;
            a.lambda = P.scalar_lambda;
            launch_pulse_xi(a, h->stream);
            rc = after_launch(h);
            if (rc) return rc;
            SymArgs sy{};
            sy.G = L.G;
            sy.nf = 2;
            sy.st[0] = a.xir; sy.symr[0] = -1; sy.symz[0] = +1;
            sy.st[1] = a.xiz; sy.symr[1] = +1; sy.symz[1] = -1;
            launch_symmetry(sy, h->stream);
            rc = after_launch(h);
            if (rc) return rc;
            launch_pulse_coeffs(a, h->stream);
            rc = after_launch(h);
            if (rc) return rc;
        } else {
            const double a0 = P.brill_a0, sr0 = P.brill_sr0, sz0 = P.brill_sz0;
            std::vector<double>& q = brillq[l];
            q.assign(L.n, 0.0);
            std::vector<double> s1(L.n, 0.0);
            auto sq = [](double x) { return x * x; };
            for (int j = 1 - g; j <= L.nz; ++j)
                for (int i = 1 - g; i <= L.nr; ++i) {
                    const double R = L.rh[i - 1 + g], Z = L.zh[j - 1 + g];
                    const size_t o = at(i, j);
                    q[o] = a0 * (R * R) * std::exp(-sq(R / sr0) - sq(Z / sz0));
                    s1[o] = 0.5 * q[o] * (1.0 / (R * R) + 2.0 * (sq(R / (sr0 * sr0)) + sq(Z / (sz0 * sz0)))
                                          - 5.0 / (sr0 * sr0) - 1.0 / (sz0 * sz0));
                }
            CUDA_OR_FAIL(cudaMemcpyAsync(w.S1, s1.data(), L.n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
            CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
        }
    }
    rc = (P.ell_solver == OLLIN_ELL_SOR) ? sor_elliptic(h, S)
         : (P.ell_solver == OLLIN_ELL_MIXED || P.ell_solver == OLLIN_ELL_FP64MG) ? mixed_elliptic(h, S)
                                                                                  : wave_elliptic(h, S);
    if (rc) return rc;
    h->ell_steps[0] = S.steps[0];
    h->ell_steps[1] = S.steps[1];
    h->ell_gres = S.gres;
    for (int l = 0; l < h->nlev; ++l) {
        DLevel& L = h->L[l];
        WLevel& w = S.W[l];
        ell_u[l].resize(L.n);
        CUDA_OR_FAIL(cudaMemcpyAsync(ell_u[l].data(), w.u[w.cur], L.n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        if (pulse) {
            scal[l].assign(4, std::vector<double>(L.n));
            const int ids[4] = {F_SPHI, F_SXIR, F_SXIZ, F_SPI};
            for (int k = 0; k < 4; ++k)
                CUDA_OR_FAIL(cudaMemcpyAsync(scal[l][k].data(), L.slot[L.cur][ids[k]], L.n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        }
    }
    CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
    (void)pi;
    return OLLIN_OK;
}

// Host restatement of initial.f90:59-218,528-645 for the supported data,
// written straight into host arrays of every level (field slots of the
// device layout), then uploaded.
int initial_data(ollin_handle* h) {
    const ollin_params& P = h->P;
    const int g = h->g;
    const bool ell = P.idata == OLLIN_IDATA_BRILLWAVE || P.idata == OLLIN_IDATA_SCALARPULSE;
    std::vector<std::vector<double>> ell_u, brillq;
    std::vector<std::vector<std::vector<double>>> scal;
    if (ell) {
        int rc = elliptic_data(h, ell_u, brillq, scal);
        if (rc) return rc;
    }
    for (int l = 0; l < h->nlev; ++l) {
        DLevel& L = h->L[l];
        const size_t n = L.n;
        std::vector<std::vector<double>> F(NFIELDS, std::vector<double>(n, 0.0));
        auto at = [&](int i, int j) { return (size_t)(i - 1 + g) + (size_t)(j - 1 + g) * L.ld; };
        for (int j = 1 - g; j <= L.nz; ++j)
            for (int i = 1 - g; i <= L.nr; ++i) {
                const size_t o = at(i, j);
                const double r = L.rh[i - 1 + g], z = L.zh[j - 1 + g];
                const double rr = std::sqrt(r * r + z * z);
                double alpha = 1.0, psi = 1.0, phi = 0.0, chi = 1.0;
                double A = 1.0, B = 1.0, H = 1.0, C = 0.0;
                if (P.idata == OLLIN_IDATA_SCHWARZSCHILD || P.idata == OLLIN_IDATA_BRILLLINDQUIST) {
                    const double M = P.bh1mass;
                    psi = (P.idata == OLLIN_IDATA_SCHWARZSCHILD) ? 1.0 + 0.5 * M / std::fabs(rr)
                                                                 : 1.0 + 0.5 * M / std::sqrt(r * r + (z - 0.0) * (z - 0.0));
                    phi = std::log(psi);
                    chi = 1.0 / std::pow(psi, (double)P.chipower);
                    if (P.idata == OLLIN_IDATA_SCHWARZSCHILD && P.ilapse == OLLIN_ILAPSE_ISOTROPIC)
                        alpha = (1.0 - 0.5 * M / std::fabs(rr)) / (1.0 + 0.5 * M / std::fabs(rr));
                }
                if (ell) {
                    // psi = ell_u (idata_scalarpulse.f90:225-240, idata_brillwave.f90:200-215)
                    psi = ell_u[l][o];
                    phi = std::log(psi);
                    chi = 1.0 / std::pow(psi, (double)P.chipower);
                    if (P.idata == OLLIN_IDATA_BRILLWAVE) {
                        A = std::exp(2.0 * brillq[l][o]);
                        B = A;
                        C = 0.0;
                        H = 1.0;
                    }
                }
                // factorhdet (initial.f90:528-577): unit-determinant conformal
                // metric, the determinant moved into phi
                if (P.factorhdet) {
                    const double hdet = (A * B - (r * C) * (r * C)) * H;
                    phi = phi + std::log(hdet) / 12.0;
                    const double aux = std::pow(hdet, 1.0 / 3.0);
                    A = A / aux;
                    B = B / aux;
                    C = C / aux;
                    H = H / aux;
                    psi = std::exp(phi);
                }
                if (P.ilapse == OLLIN_ILAPSE_PSIMINUS2) alpha = 1.0 / (psi * psi);
                else if (P.ilapse == OLLIN_ILAPSE_PSIMINUS4) alpha = 1.0 / ((psi * psi) * (psi * psi));
                F[F_ALPHA][o] = alpha;
                F[F_PHI][o] = phi;
                F[F_CHI][o] = chi;
                F[F_A][o] = A; F[F_B][o] = B; F[F_H][o] = H; F[F_C][o] = C;
            }
        if (P.idata == OLLIN_IDATA_SCALARPULSE) {
            F[F_SPHI] = scal[l][0]; F[F_SXIR] = scal[l][1]; F[F_SXIZ] = scal[l][2]; F[F_SPI] = scal[l][3];
        }
        // initial.f90:71-82: zero shift, fdriver = 1
        F[F_FDRIVER].assign(n, 1.0);
        for (int f : h->fields) {
            CUDA_OR_FAIL(cudaMemcpyAsync(L.slot[L.cur][f], F[f].data(), n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        }
        CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
    }
    return OLLIN_OK;
}

// maximalslicing.f90:3-175 on every level: lap(alpha) = (K_ij K^ij +
// 4 pi (rho + S)) alpha with the physical Laplacian of the conformal metric,
// solved by the elliptic solver of ELL_solver ('physical', init 'one'), then
// alpha = ell_u.  The reference recomputes the lapse's first and second
// derivatives and nothing else, so until a level's next ``auxiliary`` the
// right-hand side reads the other lapse quantities from the lapse before the
// solve (DLevel::alpha_aux).  va_max: the largest slicing speeds (r, z) that
// the caller's last analysis left in va_rp/va_zp, or null for none.
int maximal_slicing(ollin_handle* h, const double* va_max) {
    const ollin_params& P = h->P;
    if (!h->initialized) return fail(OLLIN_ESTATE, "ollin_gpu_initialize must run before a maximal-slicing solve");
    if (P.ell_solver != OLLIN_ELL_WAVE && P.ell_solver != OLLIN_ELL_SOR && P.ell_solver != OLLIN_ELL_MIXED &&
        P.ell_solver != OLLIN_ELL_FP64MG)
        return fail(OLLIN_EINVAL, "maximal slicing needs ELL_solver = wave, sor, mixed or fp64mg");
    // K_ij K^ij and rho + S of the current state (the last ``auxiliary``)
    for (int l = 0; l < h->nlev; ++l) {
        int rc = analysis(h, l);
        if (rc) return rc;
    }
    WaveSolve S;
    int rc = wave_alloc(h, S);
    if (rc) return rc;
    S.physical = true;
    double vrmax = 0.0, vzmax = 0.0;
    for (int l = 0; l < h->nlev; ++l) {
        DLevel& L = h->L[l];
        WLevel& w = S.W[l];
        const int nb = max_coeff_blocks(L.G);
        if (cudaMalloc(&w.cpool, (5 * L.n + 2 * (size_t)nb) * sizeof(double)) != cudaSuccess)
            return fail(OLLIN_ENOMEM, "device allocation failed for the maximal-slicing coefficients");
        CUDA_OR_FAIL(cudaMemsetAsync(w.cpool, 0, (5 * L.n + 2 * (size_t)nb) * sizeof(double), h->stream));
        double* q[5];
        for (int k = 0; k < 5; ++k) q[k] = w.cpool + (size_t)k * L.n;
        double* vmax = w.cpool + 5 * L.n;
        MaxCoeffArgs a{};
        a.G = L.G;
        a.gA = base_ptr(L, L.aux[X_GA]); a.gB = base_ptr(L, L.aux[X_GB]); a.gC = base_ptr(L, L.aux[X_GC]);
        a.chi = base_ptr(L, L.slot[L.cur][F_CHI]);
        a.phi = base_ptr(L, L.slot[L.cur][F_PHI]);
        a.trK = base_ptr(L, L.slot[L.cur][F_TRK]);
        a.KT2 = base_ptr(L, L.aux[X_KT2]);
        a.rhos = h->scalar ? base_ptr(L, L.aux[X_RHOS]) : nullptr;
        a.t0 = L.last_aux_t0 ? 1 : 0;
        if (L.sync_pending) {
            a.smap = L.smap + (L.g - 1) + (size_t)(L.g - 1) * L.ld;
            const int slots[5] = {NFIELDS, NFIELDS + 1, NFIELDS + 2, F_CHI, F_PHI};
            for (int k = 0; k < 5; ++k) a.xa[k] = base_ptr(L, L.snap + (size_t)slots[k] * L.n);
            for (size_t p = 0; p < L.spartners.size(); ++p) {
                const DLevel& Q = h->L[L.spartners[p]];
                for (int k = 0; k < 5; ++k) a.xb[p][k] = base_ptr(Q, Q.snap + (size_t)slots[k] * Q.n);
                a.xb_ld[p] = Q.ld;
            }
        }
        a.S1 = base_ptr(L, w.S1);
        a.P1 = base_ptr(L, q[0]); a.P2 = base_ptr(L, q[1]);
        a.Drphi = base_ptr(L, q[2]); a.Dzphi = base_ptr(L, q[3]); a.psi4 = base_ptr(L, q[4]);
        a.vmax = vmax;
        launch_max_coeffs(a, h->stream);
        rc = after_launch(h);
        if (rc) return rc;
        w.ph.gA = a.gA; w.ph.gB = a.gB; w.ph.gC = a.gC;
        w.ph.P1 = a.P1; w.ph.P2 = a.P2; w.ph.Drphi = a.Drphi; w.ph.Dzphi = a.Dzphi; w.ph.psi4 = a.psi4;
        std::vector<double> hv(2 * (size_t)nb);
        CUDA_OR_FAIL(cudaMemcpyAsync(hv.data(), vmax, hv.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
        // wave_elliptic.f90:211-258: maxima over the level, then over levels
        double vr = 0.0, vz = 0.0;
        for (int b = 0; b < nb; ++b) { vr = std::max(vr, hv[2 * b]); vz = std::max(vz, hv[2 * b + 1]); }
        if (va_max) { vr = std::max(vr, std::fabs(va_max[0])); vz = std::max(vz, std::fabs(va_max[1])); }
        vrmax = std::max(vrmax, vr);
        vzmax = std::max(vzmax, vz);
    }
    if (P.ell_solver == OLLIN_ELL_WAVE) {
        // wave_elliptic.f90:263-271
        const double dt0 = P.we_dtfac * std::min(std::min(P.dr0, P.dz0), std::min(P.dr0 / vrmax, P.dz0 / vzmax));
        for (int l = 0; l < h->nlev; ++l) S.W[l].dt = dt0 / (double)(1L << h->L[l].level);
        rc = wave_elliptic(h, S);
    } else if (P.ell_solver == OLLIN_ELL_SOR) {
        rc = sor_elliptic(h, S);
    } else {
        rc = mixed_elliptic(h, S);
    }
    if (rc) return rc;
    // alpha = ell_u (maximalslicing.f90:148-154)
    for (int l = 0; l < h->nlev; ++l) {
        DLevel& L = h->L[l];
        WLevel& w = S.W[l];
        if (!L.alpha_aux && cudaMalloc(&L.alpha_aux, L.n * sizeof(double)) != cudaSuccess)
            return fail(OLLIN_ENOMEM, "device allocation failed for the lapse of the last auxiliary call");
        // a second solve before any ``auxiliary`` keeps the older lapse
        if (!L.alpha_stale)
            CUDA_OR_FAIL(cudaMemcpyAsync(L.alpha_aux, L.slot[L.cur][F_ALPHA], L.n * sizeof(double),
                                         cudaMemcpyDeviceToDevice, h->stream));
        CUDA_OR_FAIL(cudaMemcpyAsync(L.slot[L.cur][F_ALPHA], w.u[w.cur], L.n * sizeof(double), cudaMemcpyDeviceToDevice,
                                     h->stream));
        L.alpha_stale = true;
    }
    CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
    h->ell_steps[0] = S.steps[0];
    h->ell_steps[1] = S.steps[1];
    h->ell_gres = S.gres;
    return OLLIN_OK;
}

}  // namespace

// =============================================================================
// C ABI
// =============================================================================
extern "C" {

void ollin_params_default(ollin_params* p) {
    std::memset(p, 0, sizeof(*p));
    p->nrtotal = 10; p->nztotal = 10; p->nl0 = 0; p->ghost = 0; p->eqsym = 0;
    p->dr0 = 1.0; p->dz0 = 1.0; p->dtfac = 0.5;
    p->integrator = OLLIN_INTEGRATOR_ICN; p->icniter = 3; p->order = 2;
    p->slicing = OLLIN_SLICING_HARMONIC; p->gauge_f = 1.0;
    p->shift = OLLIN_SHIFT_NONE; p->drivercsi = 0.75; p->drivereta = 0.0;
    p->driveradv = 0; p->shiftadvect = 1;
    p->chimethod = 1; p->chipower = 2;
    p->evolveH = 1; p->evolveKTH = 0; p->nolambda = 1;
    p->lagrangian = 1; p->factorhdet = 1;
    p->eta = 2.0;
    p->geodiss = (double)0.01f;     // real(8) :: geodiss = 0.01 (a default-real literal)
    p->scalardiss = (double)0.01f;
    p->boundtype = OLLIN_BOUND_RADIATIVE; p->interp_bicubic = 1;
    p->mattertype = OLLIN_MATTER_VACUUM; p->scalarpotential = OLLIN_POTENTIAL_NONE;
    p->idata = OLLIN_IDATA_MINKOWSKI; p->ilapse = OLLIN_ILAPSE_ONE; p->bh1mass = 1.0;
    p->ell_solver = OLLIN_ELL_WAVE; p->ell_maxiter = 100000; p->ell_epsilon = 1.0e-8;
    p->we_method = OLLIN_INTEGRATOR_ICN; p->we_maxiter = 100000;
    p->we_eta = 0.0; p->we_diss = 0.1; p->we_dtfac = 0.6; p->we_epsilon = 1.0e-8;
    p->scalarpulse_type = OLLIN_PULSE_SHELL; p->brilltype = 0;
    p->scalar_a0 = 0.0; p->scalar_r0 = 0.0; p->scalar_z0 = 0.0; p->scalar_sr0 = 1.0; p->scalar_sz0 = 1.0;
    p->brill_a0 = 0.0; p->brill_sr0 = 1.0; p->brill_sz0 = 1.0;
    p->nb = 0;  // param.f90:114-139
    for (int b = 0; b < 3; ++b) {
        p->nl[b] = 0; p->nrbox[b] = 1; p->nzbox[b] = 1; p->rbox[b] = 0.0; p->zbox[b] = 0.0;
    }
    p->driverD0 = 0; p->shiftafter = 0.0;  // param.f90:347-350
}

const char* ollin_gpu_last_error(void) { return g_err.c_str(); }

int ollin_gpu_create(const ollin_params* p, ollin_handle** out) {
    if (!p || !out) return fail(OLLIN_EINVAL, "null argument");
    *out = nullptr;
    int rc = check_params(*p);
    if (rc) return rc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(OLLIN_ECUDA, "no CUDA device is available");
    auto* h = new ollin_handle();
    h->P = *p;
    h->g = ghost_zones(*p);
    h->shift = p->shift != OLLIN_SHIFT_NONE;
    h->scalar = p->mattertype == OLLIN_MATTER_SCALAR;
    h->phys = make_phys(*p);
    parity_table(h);
    for (int f : {F_ALPHA, F_CHI, F_PHI, F_A, F_B, F_H, F_C, F_TRK, F_KTA, F_KTB, F_KTC, F_DLR, F_DLZ}) h->fields.push_back(f);
    if (h->shift)
        for (int f : {F_BETAR, F_BETAZ, F_DTBETAR, F_DTBETAZ}) h->fields.push_back(f);
    // fdriver has a source only with the shock-avoiding drivers (it stays 1
    // under the others)
    if (h->phys.shock) h->fields.push_back(F_FDRIVER);
    if (h->scalar)
        for (int f : {F_SPHI, F_SXIR, F_SXIZ, F_SPI}) h->fields.push_back(f);
    rc = setup_boxes(h);
    if (rc) {
        delete h;
        return rc;
    }
    const int L = h->nlev;
    h->t.assign(L, 0.0); h->t1.assign(L, 0.0); h->t2.assign(L, 0.0); h->s.assign(L, 0);
    h->rminl.resize(L); h->rmaxl.resize(L); h->zminl.resize(L); h->zmaxl.resize(L);
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete h;
        return fail(OLLIN_ECUDA, "cudaStreamCreate failed");
    }
    if (cudaMalloc(&h->d_flag, 64) != cudaSuccess || cudaMalloc(&h->d_norm, norm_scratch(h) * sizeof(double)) != cudaSuccess) {
        ollin_gpu_destroy(h);
        return fail(OLLIN_ENOMEM, "device allocation failed");
    }
    cudaMemsetAsync(h->d_flag, 0, 64, h->stream);
    for (int l = 0; l < L; ++l) {
        rc = alloc_level(h, h->L[l], l);
        if (rc) {
            ollin_gpu_destroy(h);
            return rc;
        }
    }
    rc = build_sync_tables(h);
    if (rc) {
        ollin_gpu_destroy(h);
        return rc;
    }
    rc = build_transfer_tables(h);
    if (rc) {
        ollin_gpu_destroy(h);
        return rc;
    }
    *out = h;
    return OLLIN_OK;
}

void ollin_gpu_destroy(ollin_handle* h) {
    if (!h) return;
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (DLevel& L : h->L) {
        if (L.pool) cudaFree(L.pool);
        if (L.ptab) cudaFree(L.ptab);
        if (L.rtab) cudaFree(L.rtab);
        if (L.alpha_aux) cudaFree(L.alpha_aux);
        if (L.delta0) cudaFree(L.delta0);
        if (L.flat) cudaFree(L.flat);
        if (L.snap) cudaFree(L.snap);
        if (L.smap) cudaFree(L.smap);
    }
    for (SyncPair& sp : h->sync) cudaFree(sp.tab);
    if (h->d_flag) cudaFree(h->d_flag);
    if (h->d_norm) cudaFree(h->d_norm);
    for (cudaEvent_t e : h->ev) cudaEventDestroy(e);
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

static int captured_step(ollin_handle* h);

int ollin_gpu_num_levels(const ollin_handle* h) { return h ? h->nlev : 0; }

int ollin_gpu_level_desc(const ollin_handle* h, int level, ollin_level_desc* out) {
    if (!h || !out || level < 0 || level >= h->nlev) return fail(OLLIN_EINVAL, "bad level");
    const DLevel& L = h->L[level];
    out->level = L.level; out->nr = L.nr; out->nz = L.nz; out->ghost = L.g;
    out->box = L.box;
    out->dr = L.dr; out->dz = L.dz; out->dt = L.dt;
    out->rmin = h->rminl[level]; out->rmax = h->rmaxl[level];
    out->zmin = h->zminl[level]; out->zmax = h->zmaxl[level];
    out->time = h->t[level];
    out->steps = (int)h->s[level];
    out->rbox = h->rbox[L.box];
    out->zbox = h->zbox[L.box];
    return OLLIN_OK;
}

int ollin_gpu_coords(const ollin_handle* h, int level, double* r, double* z) {
    if (!h || !r || !z || level < 0 || level >= h->nlev) return fail(OLLIN_EINVAL, "bad level or pointer");
    const DLevel& L = h->L[level];
    for (int k = 0; k < L.nr + L.g; ++k) r[k] = L.rh[k];
    for (int k = 0; k < L.nz + L.g; ++k) z[k] = L.zh[k];
    return OLLIN_OK;
}

int ollin_gpu_upload(ollin_handle* h, int level, int field, const double* a, int ld_r) {
    if (!h || !a || level < 0 || level >= h->nlev) return fail(OLLIN_EINVAL, "bad handle, level or pointer");
    DLevel& L = h->L[level];
    bool is_aux;
    const int f = internal_field(field, &is_aux);
    if (f < 0 || is_aux) return fail(OLLIN_EINVAL, "field cannot be uploaded (unknown or recomputed by auxiliary)");
    if (!field_active(h, f)) return fail(OLLIN_EINVAL, "field is not evolved with these parameters");
    if (ld_r < L.nr + L.g) return fail(OLLIN_EINVAL, "ld_r smaller than Nr+ghost");
    CUDA_OR_FAIL(cudaMemcpy2DAsync(L.slot[L.cur][f], (size_t)L.ld * sizeof(double), a, (size_t)ld_r * sizeof(double),
                                   (size_t)(L.nr + L.g) * sizeof(double), (size_t)(L.nz + L.g), cudaMemcpyHostToDevice, h->stream));
    CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
    return OLLIN_OK;
}

int ollin_gpu_upload_many(ollin_handle* h, int n, const int* levels, const int* fields, const double* const* a,
                          const int* ld_r) {
    if (!h || n < 0 || (n > 0 && (!levels || !fields || !a || !ld_r))) return fail(OLLIN_EINVAL, "null argument");
    // every copy checked before any is queued
    for (int k = 0; k < n; ++k) {
        if (levels[k] < 0 || levels[k] >= h->nlev || !a[k]) return fail(OLLIN_EINVAL, "bad level or pointer");
        const DLevel& L = h->L[levels[k]];
        bool is_aux;
        const int f = internal_field(fields[k], &is_aux);
        if (f < 0 || is_aux || !field_active(h, f)) return fail(OLLIN_EINVAL, "not an evolved field of these parameters");
        if (ld_r[k] < L.nr + L.g) return fail(OLLIN_EINVAL, "ld_r smaller than Nr+ghost");
    }
    for (int k = 0; k < n; ++k) {
        DLevel& L = h->L[levels[k]];
        bool is_aux;
        const int f = internal_field(fields[k], &is_aux);
        CUDA_OR_FAIL(cudaMemcpy2DAsync(L.slot[L.cur][f], (size_t)L.ld * sizeof(double), a[k],
                                       (size_t)ld_r[k] * sizeof(double), (size_t)(L.nr + L.g) * sizeof(double),
                                       (size_t)(L.nz + L.g), cudaMemcpyHostToDevice, h->stream));
    }
    CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
    return OLLIN_OK;
}

static int field_source(ollin_handle* h, int level, int field, const double** out);

int ollin_gpu_download_many(ollin_handle* h, int n, const int* levels, const int* fields, double* const* a,
                            const int* ld_r) {
    if (!h || n < 0 || (n > 0 && (!levels || !fields || !a || !ld_r))) return fail(OLLIN_EINVAL, "null argument");
    for (int k = 0; k < n; ++k) {
        if (levels[k] < 0 || levels[k] >= h->nlev || !a[k]) return fail(OLLIN_EINVAL, "bad level or pointer");
        if (ld_r[k] < h->L[levels[k]].nr + h->L[levels[k]].g) return fail(OLLIN_EINVAL, "ld_r smaller than Nr+ghost");
        bool is_aux;
        const int f = internal_field(fields[k], &is_aux);
        if (f < 0 || is_aux || !field_active(h, f))
            return fail(OLLIN_EINVAL, "ollin_gpu_download_many copies evolved fields (derived ones one at a time)");
    }
    for (int k = 0; k < n; ++k) {
        DLevel& L = h->L[levels[k]];
        const double* src = nullptr;
        int rc = field_source(h, levels[k], fields[k], &src);
        if (rc) return rc;
        CUDA_OR_FAIL(cudaMemcpy2DAsync(a[k], (size_t)ld_r[k] * sizeof(double), src, (size_t)L.ld * sizeof(double),
                                       (size_t)(L.nr + L.g) * sizeof(double), (size_t)(L.nz + L.g),
                                       cudaMemcpyDeviceToHost, h->stream));
    }
    CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
    return OLLIN_OK;
}

// The device array that holds ``field`` of grid ``level`` as the reference
// holds it now (derived fields computed first; phi from chi after a t > 0
// ``auxiliary``), element (1-ghost, 1-ghost) first.
static int field_source(ollin_handle* h, int level, int field, const double** out) {
    DLevel& L = h->L[level];
    bool is_aux;
    const int f = internal_field(field, &is_aux);
    if (f < 0) return fail(OLLIN_EINVAL, "unknown field");
    const double* src = nullptr;
    if (is_aux) {
        if (f == X_HAM || f == X_MOMR || f == X_MOMZ || f == X_RSCAL || f == X_KT2 || f == X_LAPLA) {
            int rc = analysis(h, level);
            if (rc) return rc;
        }
        src = L.aux[f];
    } else {
        if (!field_active(h, f)) return fail(OLLIN_EINVAL, "field is not evolved with these parameters");
        src = L.slot[L.cur][f];
        if (f == F_PHI && !L.last_aux_t0) {
            // after a t>0 ``auxiliary`` the reference holds phi = -log(chi)/2
            // (auxiliary_geometry.f90:204)
            launch_phi_from_chi(L.G, base_ptr(L, L.slot[L.cur][F_CHI]), base_ptr(L, L.aux[X_RSCAL]), h->stream);
            int rc = after_launch(h);
            if (rc) return rc;
            src = L.aux[X_RSCAL];
        }
    }
    *out = src;
    return OLLIN_OK;
}

int ollin_gpu_download(ollin_handle* h, int level, int field, double* a, int ld_r) {
    if (!h || !a || level < 0 || level >= h->nlev) return fail(OLLIN_EINVAL, "bad handle, level or pointer");
    DLevel& L = h->L[level];
    if (ld_r < L.nr + L.g) return fail(OLLIN_EINVAL, "ld_r smaller than Nr+ghost");
    const double* src = nullptr;
    int rc = field_source(h, level, field, &src);
    if (rc) return rc;
    CUDA_OR_FAIL(cudaMemcpy2DAsync(a, (size_t)ld_r * sizeof(double), src, (size_t)L.ld * sizeof(double),
                                   (size_t)(L.nr + L.g) * sizeof(double), (size_t)(L.nz + L.g), cudaMemcpyDeviceToHost, h->stream));
    CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
    return OLLIN_OK;
}

int ollin_gpu_interp(ollin_handle* h, int level, int field, const double* rz, int n, double* out) {
    if (!h || level < 0 || level >= h->nlev || n < 0 || (n > 0 && (!rz || !out)))
        return fail(OLLIN_EINVAL, "bad handle, level or pointer");
    if (n == 0) return OLLIN_OK;
    DLevel& L = h->L[level];
    const double* src = nullptr;
    int rc = field_source(h, level, field, &src);
    if (rc) return rc;
    double* d = nullptr;
    if (cudaMalloc(&d, (3 * (size_t)n + 1) * sizeof(double)) != cudaSuccess)
        return fail(OLLIN_ENOMEM, "device allocation failed for the interpolation points");
    struct FreeD { double* p; ~FreeD() { cudaFree(p); } } free_d{d};
    unsigned int* bad = reinterpret_cast<unsigned int*>(d + 3 * (size_t)n);
    CUDA_OR_FAIL(cudaMemcpyAsync(d, rz, 2 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CUDA_OR_FAIL(cudaMemsetAsync(bad, 0, sizeof(unsigned int), h->stream));
    // interp.f90 reads the interpolated array with its ghosts: the base of
    // the level layout, element (1-ghost, 1-ghost) at offset 0
    launch_interp_points(L.G, h->rminl[level], h->rmaxl[level], h->zminl[level], h->zmaxl[level],
                         h->P.interp_bicubic, base_ptr(L, const_cast<double*>(src)), d, n, d + 2 * (size_t)n, bad,
                         h->stream);
    rc = after_launch(h);
    if (rc) return rc;
    unsigned int nbad = 0;
    CUDA_OR_FAIL(cudaMemcpyAsync(out, d + 2 * (size_t)n, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CUDA_OR_FAIL(cudaMemcpyAsync(&nbad, bad, sizeof(nbad), cudaMemcpyDeviceToHost, h->stream));
    CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
    if (nbad) return fail(OLLIN_EINVAL, std::to_string(nbad) + " point(s) outside the grid's interpolation range "
                                        "(interp.f90:146-157); their values are NaN");
    return OLLIN_OK;
}

// The three time levels of an evolved field the next coarse step reads:
// slot 0 the current state, 1 the state at the start of the level's last
// step (the reference's var_bound_*(...,0) on the boundary strips), 2 the
// start of the step before (var_bound_*(...,1)).
static int history_slot(const DLevel& L, int which) {
    return which == 0 ? L.cur : which == 1 ? L.p : which == 2 ? L.pp : -1;
}

int ollin_gpu_download_slot(ollin_handle* h, int level, int field, int which, double* a, int ld_r) {
    if (!h || !a || level < 0 || level >= h->nlev) return fail(OLLIN_EINVAL, "bad handle, level or pointer");
    DLevel& L = h->L[level];
    bool is_aux;
    const int f = internal_field(field, &is_aux);
    if (f < 0 || is_aux || !field_active(h, f)) return fail(OLLIN_EINVAL, "not an evolved field of these parameters");
    const int sl = history_slot(L, which);
    if (sl < 0) return fail(OLLIN_EINVAL, "slot must be 0 (current), 1 or 2 (history)");
    if (ld_r < L.nr + L.g) return fail(OLLIN_EINVAL, "ld_r smaller than Nr+ghost");
    CUDA_OR_FAIL(cudaMemcpy2DAsync(a, (size_t)ld_r * sizeof(double), L.slot[sl][f], (size_t)L.ld * sizeof(double),
                                   (size_t)(L.nr + L.g) * sizeof(double), (size_t)(L.nz + L.g), cudaMemcpyDeviceToHost,
                                   h->stream));
    CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
    return OLLIN_OK;
}

int ollin_gpu_upload_slot(ollin_handle* h, int level, int field, int which, const double* a, int ld_r) {
    if (!h || !a || level < 0 || level >= h->nlev) return fail(OLLIN_EINVAL, "bad handle, level or pointer");
    DLevel& L = h->L[level];
    bool is_aux;
    const int f = internal_field(field, &is_aux);
    if (f < 0 || is_aux || !field_active(h, f)) return fail(OLLIN_EINVAL, "not an evolved field of these parameters");
    const int sl = history_slot(L, which);
    if (sl < 0) return fail(OLLIN_EINVAL, "slot must be 0 (current), 1 or 2 (history)");
    if (ld_r < L.nr + L.g) return fail(OLLIN_EINVAL, "ld_r smaller than Nr+ghost");
    CUDA_OR_FAIL(cudaMemcpy2DAsync(L.slot[sl][f], (size_t)L.ld * sizeof(double), a, (size_t)ld_r * sizeof(double),
                                   (size_t)(L.nr + L.g) * sizeof(double), (size_t)(L.nz + L.g), cudaMemcpyHostToDevice,
                                   h->stream));
    CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
    return OLLIN_OK;
}

int ollin_gpu_get_clocks(ollin_handle* h, int level, double out[4]) {
    if (!h || !out || level < 0 || level >= h->nlev) return fail(OLLIN_EINVAL, "bad handle, level or pointer");
    out[0] = h->t[level];
    out[1] = h->t1[level];
    out[2] = h->t2[level];
    out[3] = (double)h->s[level];
    return OLLIN_OK;
}

int ollin_gpu_set_clocks(ollin_handle* h, int level, const double in[4]) {
    if (!h || !in || level < 0 || level >= h->nlev) return fail(OLLIN_EINVAL, "bad handle, level or pointer");
    if (h->initialized) return fail(OLLIN_ESTATE, "clocks are set before ollin_gpu_initialize (a restart)");
    if (!(in[3] >= 0.0) || in[3] != std::floor(in[3])) return fail(OLLIN_EINVAL, "the step count must be a whole number");
    h->t[level] = in[0];
    h->t1[level] = in[1];
    h->t2[level] = in[2];
    h->s[level] = (long)in[3];
    return OLLIN_OK;
}

int ollin_gpu_initial_data(ollin_handle* h) {
    if (!h) return fail(OLLIN_EINVAL, "null handle");
    // analytic data, or the elliptic solve of idata_scalarpulse.f90 /
    // idata_brillwave.f90 on the device
    return initial_data(h);
}

int ollin_gpu_initialize(ollin_handle* h) {
    if (!h) return fail(OLLIN_EINVAL, "null handle");
    for (int l = 0; l < h->nlev; ++l) {  // evolve.f90:128-142
        int rc = do_symmetry(h, h->L[l], h->L[l].cur, active_fields(h, true));
        if (rc) return rc;
    }
    for (int l = 0; l < h->nlev; ++l) {  // evolve.f90:162-167
        int rc = do_aux(h, h->L[l], h->L[l].cur, h->t[l] == 0.0);
        if (rc) return rc;
    }
    // evolve.f90:174-195: dtbeta = csi Delta for the second-order drivers,
    // unless driverD0
    if ((h->P.shift == OLLIN_SHIFT_GAMMADRIVER2 || h->P.shift == OLLIN_SHIFT_GAMMADRIVERSHOCK2) && !h->P.driverD0) {
        for (int l = 0; l < h->nlev; ++l) {
            DLevel& L = h->L[l];
            launch_gammadriver_init(L.G, base_ptr(L, L.slot[L.cur][F_DTBETAR]), base_ptr(L, L.slot[L.cur][F_DTBETAZ]),
                                    base_ptr(L, L.slot[L.cur][F_DLR]), base_ptr(L, L.slot[L.cur][F_DLZ]), h->P.drivercsi, h->stream);
            int rc = after_launch(h);
            if (rc) return rc;
        }
    }
    for (int level = 1; level <= h->nlmax; ++level) {  // evolve.f90:211-219
        int rc = sync_level(h, level);
        if (rc) return rc;
    }
    CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
    h->initialized = true;
    return OLLIN_OK;
}

int ollin_gpu_resume(ollin_handle* h) {
    if (!h) return fail(OLLIN_EINVAL, "null handle");
    if (h->initialized) return fail(OLLIN_ESTATE, "ollin_gpu_resume replaces ollin_gpu_initialize");
    for (int l = 0; l < h->nlev; ++l)
        if (h->t[l] == 0.0) return fail(OLLIN_EINVAL, "resume needs the clocks of a running evolution (t > 0)");
    // the auxiliary quantities of the uploaded state, which the last
    // ``auxiliary`` call of the suspended evolution already projected
    for (int l = 0; l < h->nlev; ++l) {
        int rc = do_aux(h, h->L[l], h->L[l].cur, false, false);
        if (rc) return rc;
    }
    CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
    h->initialized = true;
    return OLLIN_OK;
}

int ollin_gpu_aux(ollin_handle* h, int level) {
    if (!h || level < 0 || level >= h->nlev) return fail(OLLIN_EINVAL, "bad handle or level");
    DLevel& L = h->L[level];
    int rc = do_aux(h, L, L.cur, h->t[level] == 0.0);
    if (rc) return rc;
    CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
    return OLLIN_OK;
}

int ollin_gpu_coarse_step(ollin_handle* h, double* t_out) {
    if (!h) return fail(OLLIN_EINVAL, "null handle");
    if (!h->initialized) return fail(OLLIN_ESTATE, "ollin_gpu_initialize must run before the first step");
    g_chain_launch = h->chain;
    int rc = h->graphs && !h->ktime ? captured_step(h) : onestep(h, 0);
    g_chain_launch = false;
    if (rc) return rc;
    unsigned int flag = 0;
    CUDA_OR_FAIL(cudaMemcpyAsync(&flag, h->d_flag, sizeof(flag), cudaMemcpyDeviceToHost, h->stream));
    CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
    if (flag) return fail(OLLIN_ENAN, "non-finite value produced by the evolution");
    if (t_out) *t_out = h->t[0];
    return OLLIN_OK;
}

// One coarse step recorded by stream capture into a graph and launched as
// one unit: the kernels, their arguments and their order are those of the
// direct launches, so the results are the same bit for bit; what changes is
// that the driver gets one submission instead of a few hundred.  The step's
// scalars (times, interpolation weights, slot pointers) differ from step to
// step, so each step is captured again and the executable graph updated in
// place; a step whose launch structure differs from the last (the first
// steps, a maximal solve's stale lapse, a syncboxes copy) instantiates anew.
static int captured_step(ollin_handle* h) {
    CUDA_OR_FAIL(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = onestep(h, 0);
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(h->stream, &g);
    if (rc || ec != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return rc ? rc : fail(OLLIN_ECUDA, std::string("step capture: ") + cudaGetErrorString(ec));
    }
    if (h->gexec) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(h->gexec, g, &info) == cudaSuccess) {
            h->graph_updates++;
        } else {
            cudaGetLastError();
            cudaGraphExecDestroy(h->gexec);
            h->gexec = nullptr;
        }
    }
    if (!h->gexec) {
        const cudaError_t ei = cudaGraphInstantiate(&h->gexec, g, 0);
        if (ei != cudaSuccess) {
            h->gexec = nullptr;
            cudaGraphDestroy(g);
            return fail(OLLIN_ECUDA, std::string("graph instantiation: ") + cudaGetErrorString(ei));
        }
        h->graph_instantiations++;
    }
    cudaGraphDestroy(g);
    CUDA_OR_FAIL(cudaGraphLaunch(h->gexec, h->stream));
    return OLLIN_OK;
}

int ollin_gpu_step_begin(ollin_handle* h) {
    if (!h) return fail(OLLIN_EINVAL, "null handle");
    if (!h->initialized) return fail(OLLIN_ESTATE, "ollin_gpu_initialize must run before the first step");
    if (h->step_queued) return fail(OLLIN_ESTATE, "a step is already queued on this handle");
    g_chain_launch = h->chain;
    int rc = h->graphs && !h->ktime ? captured_step(h) : onestep(h, 0);
    g_chain_launch = false;
    // queued work runs to its end whatever happened: the next end waits for it
    h->step_queued = true;
    return rc;
}

int ollin_gpu_step_chaining(ollin_handle* h, int enable) {
    if (!h) return fail(OLLIN_EINVAL, "null handle");
    h->chain = enable != 0;
    return OLLIN_OK;
}

int ollin_gpu_step_graphs(ollin_handle* h, int enable, long long* stats) {
    if (!h) return fail(OLLIN_EINVAL, "null handle");
    if (enable >= 0) h->graphs = enable != 0;
    if (stats) { stats[0] = h->graph_instantiations; stats[1] = h->graph_updates; }
    return OLLIN_OK;
}

int ollin_gpu_step_ready(const ollin_handle* h) {
    if (!h || !h->step_queued) return 1;
    // an error also counts as finished: ollin_gpu_step_end reports it
    return cudaStreamQuery(h->stream) == cudaErrorNotReady ? 0 : 1;
}

int ollin_gpu_step_end(ollin_handle* h, double* t_out) {
    if (!h) return fail(OLLIN_EINVAL, "null handle");
    if (!h->step_queued) return fail(OLLIN_ESTATE, "no step is queued on this handle");
    h->step_queued = false;
    unsigned int flag = 0;
    CUDA_OR_FAIL(cudaMemcpyAsync(&flag, h->d_flag, sizeof(flag), cudaMemcpyDeviceToHost, h->stream));
    CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
    if (flag) return fail(OLLIN_ENAN, "non-finite value produced by the evolution");
    if (t_out) *t_out = h->t[0];
    return OLLIN_OK;
}

int ollin_gpu_footprint(const ollin_params* p, size_t* resident, size_t* transient) {
    if (!p || !resident || !transient) return fail(OLLIN_EINVAL, "null argument");
    int rc = check_params(*p);
    if (rc) return rc;
    ollin_handle tmp;  // the grid list only: no device work
    tmp.P = *p;
    tmp.g = ghost_zones(*p);
    rc = setup_boxes(&tmp);
    if (rc) return rc;
    // a maximal-slicing solve may run whenever the caller asks (maximalevery
    // is the caller's): count its arrays for every run that can have one
    const bool maximal = true;
    const bool elliptic = maximal || p->idata == OLLIN_IDATA_SCALARPULSE || p->idata == OLLIN_IDATA_BRILLWAVE;
    const size_t page = (size_t)2 << 20;  // allocation granularity of large cudaMalloc blocks
    size_t res = 4 * page, tr = 0;
    for (const DLevel& L : tmp.L) {
        const int g = tmp.g, nr = tmp.nrbox[L.box], nz = tmp.nzbox[L.box];
        const size_t n = (size_t)(((nr + g + 31) / 32) * 32) * (size_t)(nz + g);
        const size_t narrays = (size_t)kSlots * NFIELDS + NFIELDS + NAUX;
        res += (narrays * n + (size_t)(nr + g) * 2 + (size_t)(nz + g) + 64) * sizeof(double) + page;
        res += 2 * page;                                  // transfer tables
        if (tmp.nb > 0) res += ((NFIELDS + 3) * n + n) * sizeof(double) + 2 * page;  // syncboxes state and map
        if (maximal) res += n * sizeof(double) + page;  // the lapse of the last auxiliary call
        // the elliptic solver's arrays while a solve runs: 13 arrays of the
        // wave solver's state and sources, 5 of coefficients, and for SOR and
        // the mixed solver their nine-point stencil, residual and correction
        // (3), multigrid hierarchy (below 6) and the 15 Orthomin vectors
        if (elliptic) tr += 56 * n * sizeof(double) + 4 * page;
    }
    *resident = res;
    *transient = tr;
    return OLLIN_OK;
}

int ollin_gpu_coarse_step_many(ollin_handle* const* hs, int n, double* t_out) {
    if (!hs || n < 0) return fail(OLLIN_EINVAL, "bad handle array");
    for (int k = 0; k < n; ++k) {
        if (!hs[k]) return fail(OLLIN_EINVAL, "null handle");
        if (!hs[k]->initialized) return fail(OLLIN_ESTATE, "ollin_gpu_initialize must run before the first step");
    }
    // every evolution's step is queued on its own stream before any is
    // waited for, so the steps of small grids run side by side
    int first = OLLIN_OK;
    std::string first_msg;
    for (int k = 0; k < n && first == OLLIN_OK; ++k) {
        // side by side the evolutions fill the SMs: ordinary launches (a
        // chained successor's waiting blocks would take room from the others)
        g_chain_launch = n == 1 && hs[k]->chain;
        int rc = hs[k]->graphs && !hs[k]->ktime ? captured_step(hs[k]) : onestep(hs[k], 0);
        g_chain_launch = false;
        if (rc) { first = rc; first_msg = g_err; }
    }
    for (int k = 0; k < n; ++k) {
        ollin_handle* h = hs[k];
        unsigned int flag = 0;
        const bool ok = cudaMemcpyAsync(&flag, h->d_flag, sizeof(flag), cudaMemcpyDeviceToHost, h->stream) == cudaSuccess &&
                        cudaStreamSynchronize(h->stream) == cudaSuccess;
        if (first == OLLIN_OK && !ok) { first = OLLIN_ECUDA; first_msg = "stream synchronisation failed"; }
        if (first == OLLIN_OK && flag) {
            first = OLLIN_ENAN;
            first_msg = "non-finite value produced by evolution " + std::to_string(k);
        }
        if (t_out) t_out[k] = h->t[0];
    }
    if (first != OLLIN_OK) return fail(first, first_msg);
    return OLLIN_OK;
}

namespace {

// Host (pinned) and device buffers of the fused launches' argument tables,
// kept between calls and grown on demand.
struct FusedWorkspace {
    std::mutex mu;
    unsigned char* host = nullptr;
    unsigned char* dev = nullptr;
    size_t cap = 0;
    cudaStream_t upload = nullptr;
    cudaEvent_t ready = nullptr;
    // each group's sequence of fused launches recorded once as a CUDA graph,
    // keyed by everything the launches bake in (kernels, shapes, table
    // offsets, the table buffer): a repeated step replays it after uploading
    // that step's tables
    bool graphs = true;
    std::unordered_map<std::string, cudaGraphExec_t> execs;
};
FusedWorkspace g_fused;

void drop_fused_graphs() {
    for (auto& kv : g_fused.execs) cudaGraphExecDestroy(kv.second);
    g_fused.execs.clear();
}

size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

}  // namespace

int ollin_gpu_fused_graphs(int on) {
    std::lock_guard<std::mutex> lock(g_fused.mu);
    g_fused.graphs = on != 0;
    if (!g_fused.graphs) drop_fused_graphs();
    return OLLIN_OK;
}

int ollin_gpu_coarse_step_fused(ollin_handle* const* hs, int n, double* t_out, int* status) {
    if (!hs || n < 0) return fail(OLLIN_EINVAL, "bad handle array");
    if (status)
        for (int k = 0; k < n; ++k) status[k] = OLLIN_OK;
    for (int k = 0; k < n; ++k) {
        if (!hs[k]) return fail(OLLIN_EINVAL, "null handle");
        if (!hs[k]->initialized) return fail(OLLIN_ESTATE, "ollin_gpu_initialize must run before the first step");
    }
    // 1. every evolution's coarse step, recorded instead of launched (the host
    //    logic of onestep runs as usual: slots, clocks, time weights); an
    //    evolution with syncboxes copies (device-to-device copies in its step)
    //    is stepped on its own stream instead
    std::vector<LaunchRecorder> rec(n);
    std::vector<int> direct;
    for (int k = 0; k < n; ++k) {
        ollin_handle* h = hs[k];
        if (!h->sync.empty()) { direct.push_back(k); continue; }
        g_chain_launch = false;
        g_recorder = &rec[k];
        const int rc = onestep(h, 0);
        g_recorder = nullptr;
        if (rc) return rc;
        for (const LaunchRec& r : rec[k].recs)
            if (!multi_for(r.kernel)) return fail(OLLIN_ECUDA, "a step kernel has no fused twin");
    }
    for (int k : direct) {
        g_chain_launch = false;
        const int rc = onestep(hs[k], 0);
        if (rc) return rc;
    }
    // 2. evolutions whose steps launch the same kernels with the same block
    //    shapes in the same order form a group; each position of a group's
    //    sequence becomes one launch over all its members' blocks
    using Sig = std::vector<std::pair<const void*, unsigned>>;
    std::map<Sig, std::vector<int>> groups;
    for (int k = 0; k < n; ++k) {
        Sig sig;
        for (const LaunchRec& r : rec[k].recs) sig.emplace_back(r.kernel, r.block.x | (r.block.y << 16));
        if (!sig.empty()) groups[sig].push_back(k);
    }
    // 3. the argument structs, block offsets and grid widths of every fused
    //    launch in one buffer, uploaded in one copy
    struct Fused { MultiLaunchFn fn; size_t args, boff, gx; int n, total; dim3 block; };
    std::vector<std::vector<Fused>> plan;
    size_t bytes = 0;
    for (auto& [sig, mem] : groups) {
        std::vector<Fused> seq;
        for (size_t p = 0; p < sig.size(); ++p) {
            const LaunchRec& r0 = rec[mem[0]].recs[p];
            Fused f{};
            f.fn = multi_for(r0.kernel);
            f.n = (int)mem.size();
            f.block = r0.block;
            f.args = bytes; bytes = align16(bytes + r0.args.size() * mem.size());
            f.boff = bytes; bytes = align16(bytes + sizeof(int) * (mem.size() + 1));
            f.gx = bytes; bytes = align16(bytes + sizeof(int) * mem.size());
            seq.push_back(f);
        }
        plan.push_back(std::move(seq));
    }
    std::lock_guard<std::mutex> lock(g_fused.mu);
    if (bytes > g_fused.cap) {
        drop_fused_graphs();  // they point into the old buffer
        cudaFreeHost(g_fused.host);
        cudaFree(g_fused.dev);
        g_fused.host = nullptr; g_fused.dev = nullptr; g_fused.cap = 0;
        const size_t cap = bytes + bytes / 2 + 4096;
        if (cudaHostAlloc((void**)&g_fused.host, cap, cudaHostAllocDefault) != cudaSuccess ||
            cudaMalloc((void**)&g_fused.dev, cap) != cudaSuccess)
            return fail(OLLIN_ENOMEM, "allocation of the fused launch tables failed");
        g_fused.cap = cap;
    }
    if (!g_fused.upload) {
        CUDA_OR_FAIL(cudaStreamCreateWithFlags(&g_fused.upload, cudaStreamNonBlocking));
        CUDA_OR_FAIL(cudaEventCreateWithFlags(&g_fused.ready, cudaEventDisableTiming));
    }
    {
        size_t gi = 0;
        for (auto& [sig, mem] : groups) {
            for (size_t p = 0; p < sig.size(); ++p) {
                Fused& f = plan[gi][p];
                int* boff = (int*)(g_fused.host + f.boff);
                int* gx = (int*)(g_fused.host + f.gx);
                int total = 0;
                for (size_t m = 0; m < mem.size(); ++m) {
                    const LaunchRec& r = rec[mem[m]].recs[p];
                    memcpy(g_fused.host + f.args + m * r.args.size(), r.args.data(), r.args.size());
                    boff[m] = total;
                    gx[m] = (int)r.grid.x;
                    total += (int)(r.grid.x * r.grid.y);
                }
                boff[mem.size()] = total;
                f.total = total;
            }
            ++gi;
        }
    }
    if (bytes > 0) {
        CUDA_OR_FAIL(cudaMemcpyAsync(g_fused.dev, g_fused.host, bytes, cudaMemcpyHostToDevice, g_fused.upload));
        CUDA_OR_FAIL(cudaEventRecord(g_fused.ready, g_fused.upload));
    }
    // 4. each group's launches in order on its first member's stream
    {
        size_t gi = 0;
        for (auto& [sig, mem] : groups) {
            cudaStream_t st = hs[mem[0]]->stream;
            CUDA_OR_FAIL(cudaStreamWaitEvent(st, g_fused.ready, 0));
            auto issue = [&](cudaStream_t q) {
                for (const Fused& f : plan[gi]) {
                    if (f.total == 0) continue;
                    f.fn(g_fused.dev + f.args, (const int*)(g_fused.dev + f.boff), (const int*)(g_fused.dev + f.gx),
                         f.n, f.total, f.block, q);
                }
            };
            cudaGraphExec_t exec = nullptr;
            if (g_fused.graphs) {
                std::string key((const char*)&g_fused.dev, sizeof(g_fused.dev));
                for (const Fused& f : plan[gi]) {
                    const long long v[8] = {(long long)(uintptr_t)f.fn, (long long)f.args, (long long)f.boff,
                                            (long long)f.gx, f.n, f.total, (long long)f.block.x, (long long)f.block.y};
                    key.append((const char*)v, sizeof(v));
                }
                auto it = g_fused.execs.find(key);
                if (it != g_fused.execs.end()) {
                    exec = it->second;
                } else {
                    if (g_fused.execs.size() >= 256) drop_fused_graphs();
                    cudaGraph_t graph = nullptr;
                    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
                        issue(st);
                        const cudaError_t ec = cudaStreamEndCapture(st, &graph);
                        if (ec == cudaSuccess && graph &&
                            cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess)
                            g_fused.execs[key] = exec;
                        else
                            exec = nullptr;
                        if (graph) cudaGraphDestroy(graph);
                    }
                    cudaGetLastError();  // a failed capture falls back to direct launches
                }
            }
            if (exec) CUDA_OR_FAIL(cudaGraphLaunch(exec, st));
            else issue(st);
            CUDA_OR_FAIL(cudaGetLastError());
            ++gi;
        }
    }
    // 5. wait for every group and every evolution stepped alone; NaN checks
    int first = OLLIN_OK;
    std::string first_msg;
    for (auto& [sig, mem] : groups)
        if (cudaStreamSynchronize(hs[mem[0]]->stream) != cudaSuccess && first == OLLIN_OK) {
            first = OLLIN_ECUDA;
            first_msg = "fused launches failed";
        }
    for (int k = 0; k < n; ++k) {
        ollin_handle* h = hs[k];
        unsigned int flag = 0;
        const bool ok = cudaStreamSynchronize(h->stream) == cudaSuccess &&
                        cudaMemcpy(&flag, h->d_flag, sizeof(flag), cudaMemcpyDeviceToHost) == cudaSuccess;
        if (status) status[k] = !ok ? OLLIN_ECUDA : flag ? OLLIN_ENAN : OLLIN_OK;
        if (first == OLLIN_OK && !ok) { first = OLLIN_ECUDA; first_msg = "stream synchronisation failed"; }
        if (first == OLLIN_OK && flag) {
            first = OLLIN_ENAN;
            first_msg = "non-finite value produced by evolution " + std::to_string(k);
        }
        if (t_out) t_out[k] = h->t[0];
    }
    if (first != OLLIN_OK) return fail(first, first_msg);
    return OLLIN_OK;
}

namespace {

// The schedule autotuner of ollin_gpu_coarse_step_auto: per batch (the set of
// handles), the wall time per point-update of each schedule, tried on live
// steps (every schedule gives the same results bit for bit, so tuning wastes
// no work), then the fastest one.
enum Schedule { kFusedGraphs = 0, kFusedDirect = 1, kStreams = 2, kSchedules = 3 };
struct TuneEntry {
    double sec_per_pu[kSchedules] = {0, 0, 0};
    int tried[kSchedules] = {0, 0, 0};
    int best = -1;
};
std::mutex g_tune_mu;
std::map<std::vector<const ollin_handle*>, TuneEntry> g_tune;
constexpr int kTrials = 2;  // steps per schedule before choosing

}  // namespace

int ollin_gpu_coarse_step_auto(ollin_handle* const* hs, int n, double* t_out, int* schedule_out) {
    if (!hs || n <= 0) return fail(OLLIN_EINVAL, "bad handle array");
    std::vector<const ollin_handle*> key(hs, hs + n);
    int sched;
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        if (g_tune.size() > 1024) g_tune.clear();
        TuneEntry& e = g_tune[key];
        sched = e.best;
        if (sched < 0) {
            sched = 0;
            while (sched < kSchedules && e.tried[sched] >= kTrials) ++sched;
        }
    }
    double pu0 = 0;
    for (int k = 0; k < n; ++k) pu0 += hs[k]->point_updates;
    const auto t0 = std::chrono::steady_clock::now();
    int rc;
    if (sched == kStreams) {
        rc = ollin_gpu_coarse_step_many(hs, n, t_out);
    } else {
        bool prev;
        {
            std::lock_guard<std::mutex> lock(g_fused.mu);
            prev = g_fused.graphs;
            g_fused.graphs = sched == kFusedGraphs;
        }
        rc = ollin_gpu_coarse_step_fused(hs, n, t_out, nullptr);
        std::lock_guard<std::mutex> lock(g_fused.mu);
        g_fused.graphs = prev;
    }
    if (rc) return rc;
    const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    double pu = -pu0;
    for (int k = 0; k < n; ++k) pu += hs[k]->point_updates;
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        TuneEntry& e = g_tune[key];
        if (e.best < 0 && pu > 0) {
            // the first step of a schedule also pays its set-up (graph
            // recording, table growth): only the later trials count
            if (e.tried[sched] > 0) e.sec_per_pu[sched] += dt / pu;
            e.tried[sched]++;
            bool done = true;
            for (int c = 0; c < kSchedules; ++c) done = done && e.tried[c] >= kTrials;
            if (done) {
                e.best = 0;
                for (int c = 1; c < kSchedules; ++c)
                    if (e.sec_per_pu[c] < e.sec_per_pu[e.best]) e.best = c;
            }
        }
    }
    if (schedule_out) *schedule_out = sched;
    return OLLIN_OK;
}

int ollin_gpu_norms(ollin_handle* h, int level, int field, double out[5]) {
    if (!h || !out || level < 0 || level >= h->nlev) return fail(OLLIN_EINVAL, "bad handle, level or pointer");
    DLevel& L = h->L[level];
    const double* raw = nullptr;
    int rc0 = field_source(h, level, field, &raw);
    if (rc0) return rc0;
    const double* src = base_ptr(L, const_cast<double*>(raw));
    // the origin value only for box 0 (save0Ddata.f90:370-374)
    launch_norms(L.G, src, L.box == 0 ? h->P.interp_bicubic : -1, h->rminl[level], h->zminl[level], h->rmaxl[level],
                 h->zmaxl[level], h->d_norm, norm_partials(h), h->stream);
    int rc = after_launch(h);
    if (rc) return rc;
    double res[6];
    CUDA_OR_FAIL(cudaMemcpyAsync(res, h->d_norm, sizeof(res), cudaMemcpyDeviceToHost, h->stream));
    CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
    if (res[5] != 0.0) return fail(OLLIN_ENAN, "NaN found in the field (save0Ddata.f90:229-264)");
    for (int k = 0; k < 5; ++k) out[k] = res[k];
    return OLLIN_OK;
}

int ollin_gpu_min_lapse(ollin_handle* h, double* out) {
    if (!h || !out) return fail(OLLIN_EINVAL, "null argument");
    // every grid's statistics queued, then one copy and one wait
    for (int l = 0; l < h->nlev; ++l) {
        DLevel& L = h->L[l];
        launch_norms(L.G, base_ptr(L, L.slot[L.cur][F_ALPHA]), -1, 0.0, 0.0, 0.0, 0.0, h->d_norm + 8 * (size_t)l,
                     norm_partials(h), h->stream);
        int rc = after_launch(h);
        if (rc) return rc;
    }
    std::vector<double> res(8 * (size_t)h->nlev);
    CUDA_OR_FAIL(cudaMemcpyAsync(res.data(), h->d_norm, res.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
    double m = HUGE_VAL;
    for (int l = 0; l < h->nlev; ++l) {
        if (res[8 * (size_t)l + 5] != 0.0) return fail(OLLIN_ENAN, "NaN found in the lapse");
        m = std::min(m, res[8 * (size_t)l + 1]);
    }
    *out = m;
    return OLLIN_OK;
}

double ollin_gpu_point_updates(const ollin_handle* h) { return h ? h->point_updates : 0.0; }

double ollin_gpu_fp64_rate(void) { return measure_fp64_dfma_rate(0); }

double ollin_gpu_op_rate(int op) { return measure_op_rate(op, 0); }

int ollin_gpu_kernel_timing(ollin_handle* h, int enable) {
    if (!h) return fail(OLLIN_EINVAL, "null handle");
    CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
    h->ktime = enable != 0;
    h->ev_used = 0;
    h->rhs_point_stages = 0;
    h->rhs_launches = 0;
    return OLLIN_OK;
}

int ollin_gpu_kernel_stats(ollin_handle* h, double* rhs_ms, long long* launches, double* point_stages) {
    if (!h) return fail(OLLIN_EINVAL, "null handle");
    CUDA_OR_FAIL(cudaStreamSynchronize(h->stream));
    double tot = 0;
    for (size_t k = 0; k + 1 < h->ev_used; k += 2) {
        float ms = 0;
        CUDA_OR_FAIL(cudaEventElapsedTime(&ms, h->ev[k], h->ev[k + 1]));
        tot += ms;
    }
    if (rhs_ms) *rhs_ms = tot;
    if (launches) *launches = h->rhs_launches;
    if (point_stages) *point_stages = h->rhs_point_stages;
    return OLLIN_OK;
}

void* ollin_gpu_stream(const ollin_handle* h) { return h ? (void*)h->stream : nullptr; }

int ollin_gpu_maximal_slicing(ollin_handle* h, const double* va_max) {
    if (!h) return fail(OLLIN_EINVAL, "null handle");
    return maximal_slicing(h, va_max);
}

int ollin_gpu_ell_stats(const ollin_handle* h, int steps[2], double* gres) {
    if (!h || !steps) return fail(OLLIN_EINVAL, "null argument");
    steps[0] = h->ell_steps[0];
    steps[1] = h->ell_steps[1];
    if (gres) *gres = h->ell_gres;
    return OLLIN_OK;
}

int ollin_gpu_ell_history(const ollin_handle* h, int level, double* rms, int max, int* n) {
    if (!h || !n || (max > 0 && !rms)) return fail(OLLIN_EINVAL, "null argument");
    if (level < 0 || level >= h->nlev) return fail(OLLIN_EINVAL, "bad level");
    *n = 0;
    if ((int)h->ell_hist.size() != h->nlev) return OLLIN_OK;
    const std::vector<double>& v = h->ell_hist[level];
    *n = (int)v.size();
    for (int k = 0; k < std::min(max, *n); ++k) rms[k] = v[k];
    return OLLIN_OK;
}

long long ollin_gpu_launch_count(const ollin_handle* h) { return h ? h->launches : 0; }

}  // extern "C"
