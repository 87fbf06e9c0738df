// Launch interfaces between the host scheduler (host.cpp) and the CUDA
// kernels (rhs.cu, aux.cu, transfer.cu).  All arguments are passed by value;
// pointers are device pointers pre-offset so that f(i,j) = f[i + j*ld].
#pragma once
#include "ollin_dev.cuh"

namespace ollin {

// Scalar parameters the right-hand side reads (src/base/param.f90 values).
struct PhysParams {
    int slicing;          // OLLIN_SLICING_*
    double gauge_f;
    int shift;            // 1 = the shift is evolved
    int driver;           // which: 2 Gammadriver2 / shock2, 1 Gammadriver1 / shock1, 0 Gammadriver0,
                          // 3 zero or static (zero sources, no boundary)
    int shock;            // the shock-avoiding variant: fdriver evolved
    int driverD0;         // subtract the t = 0 Delta
    int shiftadvect, driveradv;
    double drivercsi, drivereta;
    double eta;           // Delta damping (momentum-constraint multiple)
    double geodiss, scalardiss;
    double ft[8];
    int scalar;           // real scalar field present
    int potential;        // OLLIN_POTENTIAL_*
    double scalar_mass, scalar_lambda;
    int boundtype;        // OLLIN_BOUND_*
};

// ``syncboxes`` sources of one grid on a level (boxes 0..3 share a level; a
// chain of copies can lead back to the grid itself), and the packing of a
// copied point's source and offset into one int
constexpr int kMaxPartners = 4;
// largest par-file ghost accepted (main.f90 sets no bound)
constexpr int kMaxGhost = 8;
constexpr int kPartnerShift = 28;
constexpr int kPartnerOffset = (1 << kPartnerShift) - 1;

// One RK/ICN stage of one level.
struct StageArgs {
    LevelGeom G;
    PhysParams P;
    const double* in[NFIELDS];   // stage input state
    const double* pst[NFIELDS];  // state at the start of the step (var_p)
    double* out[NFIELDS];        // stage output state
    double* acc[NFIELDS];        // RK4 accumulator (var_a)
    const double* aux[NAUX];     // auxiliary quantities of the stage input
    double* auxw[NAUX];          // writable aux (analysis outputs)
    int shift_static;            // zero shift sources this stage: shift zero / static, or
                                 // t(box 0, level 0) < shiftafter (sources_shift.f90:43)
    const double* d0r;           // Delta at t = 0 (driverD0)
    const double* d0z;
    int t0;                      // the level's last ``auxiliary`` ran with time == 0
                                 // (phi-based derivatives, auxiliary_geometry.f90:178-202)
    int evolve_phi;              // level time == 0: phi is evolved (it is recomputed from chi otherwise)
    int level0;                  // level 0 (outer radiative boundary applies)
    int rk4, iter, niter;
    double dtw, weight;
    int analysis;                // 1: write ham/mom/RSCAL/KT2/Lapla_alpha instead of updating
    unsigned int* nanflag;       // set to 1 if a non-finite source is produced
    // The lapse of the level's last ``auxiliary`` call when a maximal-slicing
    // solve has replaced the lapse since (launch_rhs_stale, _stale_sync): the
    // covariant second derivatives, Laplacian, falpha and advective
    // derivatives of the lapse come from it, the lapse itself and the
    // gradient that maximalslicing.f90:156-170 recomputes from the new one.
    const double* alpha_aux;
    // The first stage after ``syncboxes`` copied other boxes' data onto this
    // grid (launch_rhs_sync, _stale_sync): smap[o] >= 0 marks a copied point,
    // its partner k = smap[o] >> kPartnerShift and its offset
    // smap[o] & kPartnerOffset in that partner's state xb[k] (leading
    // dimension xb_ld[k]); the other points read this grid's state before
    // the copy, xa.
    const int* smap;
    const double* xa[NFIELDS];
    const double* xb[kMaxPartners][NFIELDS];
    long xb_ld[kMaxPartners];
    // boundtype = "flat" on level 0: the sources that the outer-edge points
    // take, of the kNBound arrays in their order; per array flat_len values:
    // column Nr-1 (j = jlo..Nz), then row Nz-1 and (no equatorial symmetry)
    // row 2-ghost (i = 1..Nr)
    double* flat;
    int flat_len;
};
// The evolved arrays that simpleboundary.f90 sets (EVOLVE without NOBOUND in
// src/base/arrays.config), in the order of StageArgs::flat: trK, KTA, KTB,
// KTC, Delta_r, Delta_z, dtbeta_r, dtbeta_z, fdriver, scalar_pi
constexpr int kNBound = 10;
// the outer-edge updates of boundtype = "flat" after the stage's right-hand side
void launch_flat_edges(const StageArgs& a, cudaStream_t s);

// Table of a ``syncboxes`` copy onto grid P from grid Q of the same level.
struct SyncTableArgs {
    LevelGeom P, Q;
    double rminl_p, rmaxl_p, zminl_p, zmaxl_p;
    double rminl_q, rmaxl_q, zminl_q, zmaxl_q;
    int bicubic;
};

// Pointwise auxiliary quantities (auxiliary_geometry.f90 pointwise parts).
struct AuxArgs {
    LevelGeom G;
    double* st[NFIELDS];         // state (modified in place: factordet, chi at t=0)
    double* aux[NAUX];
    int t0;
    int scalar;
    // t > 0: 1 projects A, B, C, H onto unit determinant in place (factordet,
    // every ``auxiliary`` call of the reference); 0 takes the state as it is
    // (a resumed state that the last ``auxiliary`` call already projected)
    int project;
    // driverD0: at t = 0 Delta0 = Delta (auxiliary_geometry.f90:1107-1113)
    double* d0r;
    double* d0z;
};

// Parity ghost fill of the evolved fields (generated symmetries_r/_z).
struct SymArgs {
    LevelGeom G;
    double* st[NFIELDS];
    int symr[NFIELDS], symz[NFIELDS];
    int nf;                      // number of fields to fill (first nf slots used)
    int fid[NFIELDS];            // which field slot each entry refers to
    const int* skip;             // optional: the launch does nothing while *skip != 0
};

// One interpolation stencil of a transfer between two levels.  The strip
// and overlap geometry of a level pair never changes, so the stencils are
// built once (by the same interp_weights as a direct evaluation) and every
// transfer launch only applies them.
// o_out of a stencil that writes nothing (offsets of points in rows j <= 0
// are negative, so no negative value can serve)
constexpr int kNoPoint = -2147483647 - 1;

struct XferPt {
    int o_out;           // target element (i + j*ld) in the output level; kNoPoint: none
    int depth;           // prolongation: strip row m (r strip) or n (z strips)
    int i0, j0, mode;    // source base point; 0 copy, 1 bilinear, 2 bicubic
    int cover;           // prolongation: a later strip writes this point when imax >= cover
    double w[16];        // bicubic weights [ii+1][jj+1], or auxr, auxz (bilinear)
};

// Coarse -> fine boundary prolongation (finebound.f90 + bound_interp.inc).
struct ProlongArgs {
    LevelGeom F;                 // fine level
    LevelGeom Cg;                // coarse level
    double* fout[NFIELDS];       // fine stage output (written on the strips)
    const double* fp[NFIELDS];   // fine var_p (border 1) and history level 0
    const double* fpp[NFIELDS];  // fine history level 1 (previous step start)
    const double* cin[NFIELDS];  // coarse current state
    int fid[NFIELDS];
    int nf;
    double rminl_f, rmaxl_f, zminl_f, zmaxl_f;
    double rminl_c, rmaxl_c, zminl_c, zmaxl_c;
    double tp, t0, tm1, tl;
    int imax, border, bicubic;
    const int* skip;             // optional: the launch does nothing while *skip != 0
    // table-driven launch (launch_prolong_tab): stencils of the strips for
    // imax = ghost+2 and the time weights of finebound.f90:118-145
    const XferPt* tab;
    int ntab;
    int tmode;                   // 0: tp == tl (coarse value), 1: linear, 2: quadratic in time
    double wa, wp, wpp;          // weights of the coarse value, var_p and the older history
};

// Fine -> coarse restriction (restrict.f90 + restrict_interp.inc).
struct RestrictArgs {
    LevelGeom F, Cg;
    const double* fin[NFIELDS];
    double* cout[NFIELDS];
    int fid[NFIELDS];
    int nf;
    double rminl_f, rmaxl_f, zminl_f, zmaxl_f;
    double rminl_c, zminl_c;
    int eqsym, bicubic;
    const int* skip;             // optional: the launch does nothing while *skip != 0
    const XferPt* tab;           // table-driven launch (launch_restrict_tab)
    int ntab;
};

// Interpolation of one grid function of a coarser level to every point of a
// finer one (the initial guess of the elliptic solvers on refined levels).
struct InjectArgs {
    LevelGeom F, Cg;
    const double* cin;
    double* fout;
    double rminl_f, zminl_f;
    double rminl_c, rmaxl_c, zminl_c, zmaxl_c;
    int bicubic;
};

// Iteration control of a device-resident elliptic solve: the residual kernel
// of each iteration updates it, and every launch of later iterations returns
// at once when ``done`` is set, so the host can queue iterations in batches.
struct EllCtl {
    int step;      // iterations done in the current phase
    int done;      // stop condition met
    int miniter, maxiter;
    double eps;    // tolerance on the residual
    double gres;   // residual of the last iteration
};

// Coefficients of the physical Laplacian of the conformal metric that both
// elliptic solvers use for maximal slicing (wave_elliptic.f90:781-812,
// sor_elliptic.f90:168-262), at every point of a level; derivatives at the
// ghost points follow the parity fill of derivatives.f90.  hdet = 1 and its
// derivatives vanish after ``initial`` with factorhdet, so the determinant
// terms drop out exactly.
struct MaxCoeffArgs {
    LevelGeom G;
    const double* gA; const double* gB; const double* gC;  // inverse conformal metric
    const double* chi; const double* phi;                  // conformal factor
    const double* trK; const double* KT2; const double* rhos;  // rhos may be null (vacuum)
    int t0;                                                // phi-based conformal factor
    double* S1;                                            // -(K_ij K^ij + 4 pi (rho + S))
    double* P1;                                            // Dr_g_A + r Dz_g_C
    double* P2;                                            // Dz_g_B + r Dr_g_C + g_C
    double* Drphi; double* Dzphi; double* psi4;
    double* vmax;                                          // [2*block]: per-block max sqrt|g^rr/psi4|, sqrt|g^zz/psi4|
    // after ``syncboxes`` (as StageArgs::smap): the derivatives come from the
    // grid's state before the copy (xa) or the partner's (xb[k]) at the copied
    // points; order g_A, g_B, g_C, chi, phi
    const int* smap;
    const double* xa[5];
    const double* xb[kMaxPartners][5];
    long xb_ld[kMaxPartners];
};

// The physical-Laplacian coefficients of one wave stage.
struct WavePhys {
    const double* gA; const double* gB; const double* gC;
    const double* P1; const double* P2;
    const double* Drphi; const double* Dzphi; const double* psi4;
};

// One WaveElliptic stage on one level (wave_elliptic.f90:505-700):
// sources, dissipation, parity, radiative boundary, accumulate and update of
// (u, v) at every point including ghosts.
struct WaveArgs {
    LevelGeom G;
    const double* u_in; const double* v_in;   // stage input
    const double* u_p; const double* v_p;     // start of the step
    double* u_out; double* v_out;
    double* u_acc; double* v_acc;
    const double* S0; const double* S1; const double* S5;
    double eta;        // WE_eta
    double kdiss;      // WE_diss / dt
    double dtw, weight;
    int rk4, iter, niter;
    double* res_partial;   // level 0, last stage: per-block sums of sell_v^2
    const int* skip;
    int physical;          // type = 'physical' (coefficients in ph)
    WavePhys ph;
};

// Scalar-pulse coefficients (idata_scalarpulse.f90:108-170): xi = grad phi,
// pi = 0, S1 = pi (xi_r^2 + xi_z^2), S5 = 2 pi V, S0 = 0.
struct PulseCoeffArgs {
    LevelGeom G;
    const double* sphi;
    double* xir; double* xiz; double* spi;
    double* S0; double* S1; double* S5;
    int potential;
    double mass, lambda;
};

// One red-black pass of the SOR solver (sor_elliptic.f90:640-676) over the
// points (i,j), 2-g <= i <= Nr-1, 2-g <= j <= Nz-1, with (i+j) of one
// parity; flat Laplacian, so only the four axial neighbours couple.
struct SorPassArgs {
    LevelGeom G;
    double* u;
    const double* ca; const double* cb;  // a(i), b(i) per column, indexed [i]
    double cc;                           // c = d = 1/dz^2
    const double* e; const double* f;    // diagonal and source per point
    double omega;
    int parity;
    double* partial;                     // per-block sums of resid^2
    const int* skip;
};

// Per-point coefficients of the SOR stencil for the physical Laplacian
// (sor_elliptic.f90:168-262 on the coarse grid, :371-448 on finer grids,
// which divide by dr and dz in turn): a..d axial, g..j diagonal, e the
// diagonal including S1.
struct SorCoeffArgs {
    LevelGeom G;
    WavePhys ph;
    const double* S1;
    int fine;
    double* a; double* b; double* c; double* d; double* e;
    double* cg; double* ch; double* ci; double* cj;
    unsigned long long* diag_nonzero;  // set when any diagonal coefficient is not zero
};

// A red-black pass with the nine-point stencil of the physical Laplacian.
struct SorPhysPassArgs {
    LevelGeom G;
    double* u;
    const double* a; const double* b; const double* c; const double* d; const double* e; const double* f;
    const double* cg; const double* ch; const double* ci; const double* cj;
    double omega;
    int parity;
    double* partial;
    const int* skip;
};

// End of one SOR iteration (sor_elliptic.f90:678-790): residual norm of the
// two passes, Robin boundary (sequential along each edge, as written), parity
// fill, stop condition.
struct SorFinishArgs {
    LevelGeom G;
    double* u;
    const double* partial1; const double* partial2;
    int nparts;
    int robin;
    double uinf;
    EllCtl* ctl;
};

void launch_sor_e(const LevelGeom& G, double* e, const double* eaux, const double* S5, const double* u,
                  const int* skip, cudaStream_t s);
void launch_sor_pass(const SorPassArgs& a, cudaStream_t s);
int sor_pass_blocks(const LevelGeom& G);
// Dynamic shared memory of the finish kernel with Robin edges; the launch
// returns non-zero if the device cannot provide it.
size_t sor_finish_smem(const LevelGeom& G);
int launch_sor_finish(const SorFinishArgs& a, cudaStream_t s);
void launch_add(const LevelGeom& G, double* out, double c, const double* x, cudaStream_t s);

// Mixed-precision solve of the SOR discretisation (the system that the
// reference's SOR converges to): FP64 residual and update, FP32 multigrid
// for the correction.  ``robin`` selects the coarse problem (Robin
// rows at i = Nr and j = Nz are equations) or a fine one (those rows are
// Dirichlet data).
struct MixArgs {
    LevelGeom G;
    double* u; const double* e64; const double* f64;
    const double* ca; const double* cb; double cc;   // FP64 coefficients
    float* d; float* r32;
    // FP64 correction (ELL_solver = "fp64mg"): when d64 is set the residual
    // goes to r64 and the correction comes from d64 instead of r32/d
    double* d64; double* r64;
    int robin; double uinf;
    double* partial;                                 // per-block sums of squares
    // physical Laplacian (maximal slicing): the per-point nine-point stencil
    // of sor_elliptic.f90 (pa..pj; e64 its diagonal)
    const double* pa; const double* pb; const double* pc; const double* pd;
    const double* pg; const double* ph; const double* pi; const double* pj;
};

void launch_mix_resid(const MixArgs& a, cudaStream_t s);
int mix_blocks(const LevelGeom& G, int robin);

// Orthomin acceleration of the multigrid corrections: up to kOrthoMax stored
// directions (level-layout FP64 vectors) and their coefficients, by value
constexpr int kOrthoMax = 8;
struct OrthoVecs { const double* v[kOrthoMax + 2]; };
struct OrthoCoef { double c[kOrthoMax]; };
void launch_mix_apply(const MixArgs& a, double* z64, double* q, cudaStream_t s);
void launch_mix_dots(const LevelGeom& G, int robin, const double* x, const OrthoVecs& y, int n, double* partial,
                     cudaStream_t s);
void launch_mix_orth(const LevelGeom& G, int robin, double* z, double* q, const OrthoVecs& Zs, const OrthoVecs& Qs,
                     const OrthoCoef& beta, int n, cudaStream_t s);
void launch_mix_step(const LevelGeom& G, int robin, double* u, const double* z, double alpha, cudaStream_t s);

// The FP64 five-point stencil of a level as the multigrid reads it (level
// layout, element (i,j) at [i + j*ld]): per-point east/west/north/south
// coefficients pa..pd, or the flat Laplacian's per-column ca/cb and constant
// cc when pa is null; the diagonal e.
struct MgStencil {
    const double* pa; const double* pb; const double* pc; const double* pd;
    const double* ca; const double* cb; double cc;
    const double* e;
    long ld;
    double dr, dz;
    // the level point of multigrid cell (0, 0), r and z of the lower faces of
    // cell (1, 1), and whether the lower edges are the axis / equator mirrors
    // (else Dirichlet rows of a refinement box off them); rz: row 0 is the
    // lower Robin row of a coarse problem without equatorial symmetry
    int ioff, joff;
    double r0, z0;
    int mr, mz, rz;
};
// Geometric multigrid for the correction equation (multigrid.cu), FP32 or
// FP64 (fp64 = 1); r and d are arrays of that precision
struct MgHierarchy;
MgHierarchy* mg_create(int n, int m, double dr, double dz, int fp64);
void mg_destroy(MgHierarchy* H);
int mg_levels(const MgHierarchy* H);
int mg_launches_per_cycle(const MgHierarchy* H, int robin);
void mg_load_operator(MgHierarchy* H, const MgStencil& S, cudaStream_t s);
void mg_set_rhs(MgHierarchy* H, const void* r, long ld, cudaStream_t s);
void mg_solve(MgHierarchy* H, int robin, int ncycles, void* d, long ld, cudaStream_t s);

void launch_inject(const InjectArgs& a, cudaStream_t s);

// stencil tables of a level pair (built once per handle)
int prolong_table_size(const LevelGeom& F);
void launch_prolong_table(const ProlongArgs& a, XferPt* tab, cudaStream_t s);
void launch_prolong_tab(const ProlongArgs& a, cudaStream_t s);
void launch_restrict_table(const RestrictArgs& a, XferPt* tab, int m_lo, int n_lo, int nm, int nn, cudaStream_t s);
void launch_restrict_tab(const RestrictArgs& a, cudaStream_t s);
void launch_wave_stage(const WaveArgs& a, cudaStream_t s);
int wave_stage_blocks(const LevelGeom& G);
void launch_wave_residual(const double* partial, int nparts, int nr, int nz, EllCtl* ctl, cudaStream_t s);
void launch_pulse_xi(const PulseCoeffArgs& a, cudaStream_t s);
void launch_pulse_coeffs(const PulseCoeffArgs& a, cudaStream_t s);

void launch_rhs(const StageArgs& a, cudaStream_t s);
// KT2 (and rho + trS) on the ghost columns of a grid off the axis; no-op on a
// grid that owns the axis.
void launch_ghost_kt2(const StageArgs& a, cudaStream_t s);
void launch_rhs_stale(const StageArgs& a, cudaStream_t s);
void launch_rhs_sync(const StageArgs& a, cudaStream_t s);
void launch_rhs_stale_sync(const StageArgs& a, cudaStream_t s);
// the same four stage kinds with the order-two stencils (rhs_o2*.cu)
void launch_rhs_o2(const StageArgs& a, cudaStream_t s);
void launch_rhs_o2_stale(const StageArgs& a, cudaStream_t s);
void launch_rhs_o2_sync(const StageArgs& a, cudaStream_t s);
void launch_rhs_o2_stale_sync(const StageArgs& a, cudaStream_t s);
int sync_table_size(const LevelGeom& P);
void launch_sync_table(const SyncTableArgs& a, XferPt* tab, cudaStream_t s);
// maximal slicing (elliptic.cu)
int max_coeff_blocks(const LevelGeom& G);
void launch_max_coeffs(const MaxCoeffArgs& a, cudaStream_t s);
void launch_sor_coeffs(const SorCoeffArgs& a, cudaStream_t s);
void launch_sor_phys_pass(const SorPhysPassArgs& a, cudaStream_t s);
void launch_sor_phys_pass_seq(const SorPhysPassArgs& a, cudaStream_t s);
void launch_aux_point(const AuxArgs& a, cudaStream_t s);
void launch_aux_deriv(const AuxArgs& a, cudaStream_t s);
void launch_symmetry(const SymArgs& a, cudaStream_t s);
void launch_restrict(const RestrictArgs& a, cudaStream_t s);
// 0-D statistics: max, min, max|f|, RMS, origin value, NaN flag into
// dev_out[0..5]; ``partials`` holds 5 doubles per block of the first pass
// (at most kNormMaxBlocks blocks).
constexpr int kNormThreads = 256, kNormMaxBlocks = 4 * 152;
int norm_blocks(const LevelGeom& G);
void launch_norms(const LevelGeom& G, const double* f, int origin_bicubic, double rminl, double zminl,
                  double rmaxl, double zmaxl, double* dev_out, double* partials, cudaStream_t s);
void launch_ham_edges(const LevelGeom& G, double* ham, cudaStream_t s);
// interp.f90 at n points rz = (r0, z0) pairs of one grid (device arrays);
// NaN and a count in *bad where the stencil would leave the grid
void launch_interp_points(const LevelGeom& G, double rminl, double rmaxl, double zminl, double zmaxl, int bicubic,
                          const double* f, const double* rz, int n, double* out, unsigned int* bad, cudaStream_t s);
void launch_gammadriver_init(const LevelGeom& G, double* dtbr, double* dtbz, const double* dlr,
                             const double* dlz, double csi, cudaStream_t s);
// DFMA instructions per second of this GPU (all SMs, independent chains).
double measure_fp64_dfma_rate(cudaStream_t s);
// Operations per second of one entry of the rate table (0 DFMA, 1 DADD, 2 DMUL,
// 3 DDIV, 4 sqrt, 5 cbrt, 6 exp, 7 log, 8 FP32 FMA); -1 on failure.
double measure_op_rate(int op, cudaStream_t s);
void launch_phi_from_chi(const LevelGeom& G, const double* chi, double* out, cudaStream_t s);

}  // namespace ollin
