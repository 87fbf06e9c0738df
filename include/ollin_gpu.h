/*
 * ollin_gpu.h -- C ABI of the GB300 evolution library for OllinAxis-BiB.
 *
 * The reference (malcubi/OllinAxis-BiB, Fortran 90) has no plugin or FFI
 * layer: the evolution is the argument-less recursive subroutine
 * ``onestep(level)`` operating on module arrays.  The seam this ABI replaces is
 * the single call ``call onestep(0)`` in the main loop of
 * ``src/base/evolve.f90:381`` plus the t=0 preparation of
 * ``src/base/evolve.f90:128-195`` (symmetries, ``auxiliary`` on every level,
 * Gamma-driver initialisation).  A Fortran host binds these entry points with
 * ISO_C_BINDING; all arguments are plain pointers,
 * integers and doubles.
 *
 * Conventions
 *  - Every entry point returns 0 on success and a non-zero OLLIN_E* code on
 *    failure; ``ollin_gpu_last_error`` returns a message for the calling
 *    thread.  The Fortran wrapper maps a non-zero code to ``call die``
 *    (src/base/die.f90:3-29).
 *  - Host arrays are the reference's grid functions: ``real(8)`` arrays
 *    dimensioned ``(1-ghost:Nr, 1-ghost:Nz)``, column-major (r fastest).
 *    A pointer argument points at element ``(1-ghost, 1-ghost)``; ``ld_r`` is
 *    the leading dimension in elements (``Nr+ghost`` for an unpadded array).
 *  - One handle = one evolution = one CUDA stream.  Device memory is owned by
 *    the handle.  Handles are independent; several may live at once.
 *  - Refinement boxes Nb = 0..3 (setupboxes.f90); a ``level`` argument is a
 *    grid index: box 0's levels, then each further box's levels.
 */
#ifndef OLLIN_GPU_H
#define OLLIN_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error codes ---------------------------------------------------- */
#define OLLIN_OK            0
#define OLLIN_EINVAL        1   /* bad argument or unsupported parameter combination */
#define OLLIN_ECUDA         2   /* a CUDA runtime call failed */
#define OLLIN_ENAN          3   /* a non-finite value was detected in the state */
#define OLLIN_ENOMEM        4   /* device allocation failed */
#define OLLIN_ESTATE        5   /* call out of order (e.g. step before initialize) */
#define OLLIN_ECONV         6   /* an iterative solve ("mixed", "fp64mg") stopped above its tolerance */

/* ---- enumerated parameter values (param.f90 character parameters) ---- */
#define OLLIN_INTEGRATOR_RK4    0   /* integrator = "rk4" */
#define OLLIN_INTEGRATOR_ICN    1   /* integrator = "icn" */

#define OLLIN_SLICING_1PLUSLOG  0   /* slicing = "1+log"      */
#define OLLIN_SLICING_HARMONIC  1   /* slicing = "harmonic"   */
#define OLLIN_SLICING_SHOCKAVOID 2  /* slicing = "shockavoid" */
#define OLLIN_SLICING_STATIC    3   /* slicing = "static"     */
#define OLLIN_SLICING_MAXIMAL   4   /* slicing = "maximal": no lapse or trK source; the
                                     * host calls ollin_gpu_maximal_slicing after each
                                     * coarse step (evolve.f90:388-393) */

#define OLLIN_SHIFT_NONE        0   /* shift = "none"         */
#define OLLIN_SHIFT_ZERO        1   /* shift = "zero"         */
#define OLLIN_SHIFT_STATIC      2   /* shift = "static"       */
#define OLLIN_SHIFT_GAMMADRIVER2 3  /* shift = "Gammadriver2" */
#define OLLIN_SHIFT_GAMMADRIVER1 4  /* shift = "Gammadriver1": d_t beta = csi Delta - eta beta */
#define OLLIN_SHIFT_GAMMADRIVER0 5  /* shift = "Gammadriver0": d_t beta = csi d_t Delta */
#define OLLIN_SHIFT_GAMMADRIVERSHOCK1 6  /* shift = "Gammadrivershock1": d_t beta = csi fdriver Delta - eta beta,
                                          * d_t fdriver = -2/3 fdriver DIV beta */
#define OLLIN_SHIFT_GAMMADRIVERSHOCK2 7  /* shift = "Gammadrivershock2": d_t dtbeta = csi d_t (fdriver Delta)
                                          * - eta dtbeta */

#define OLLIN_BOUND_RADIATIVE   0   /* boundtype = "radiative" */
#define OLLIN_BOUND_NONE        1   /* boundtype = "none"      */
#define OLLIN_BOUND_STATIC      2   /* boundtype = "static": zero sources on the outer edges */
#define OLLIN_BOUND_FLAT        3   /* boundtype = "flat": the sources of the row inside */

#define OLLIN_MATTER_VACUUM     0   /* mattertype = "vacuum" */
#define OLLIN_MATTER_SCALAR     1   /* mattertype = "scalar" */

#define OLLIN_POTENTIAL_NONE    0   /* scalarpotential = "none" */
#define OLLIN_POTENTIAL_PHI2    1   /* scalarpotential = "phi2" */
#define OLLIN_POTENTIAL_PHI4    2   /* scalarpotential = "phi4" */

#define OLLIN_IDATA_MINKOWSKI       0   /* idata = "minkowski"      */
#define OLLIN_IDATA_SCHWARZSCHILD   1   /* idata = "schwarzschild"  */
#define OLLIN_IDATA_BRILLLINDQUIST  2   /* idata = "BrillLindquist" (one hole) */
#define OLLIN_IDATA_BRILLWAVE       3   /* idata = "BrillWave" (brilltype = "Holz"), elliptic */
#define OLLIN_IDATA_SCALARPULSE     4   /* idata = "scalarpulse" (mattertype = "scalar"), elliptic */

#define OLLIN_ELL_NONE          0   /* ELL_solver = "none" */
#define OLLIN_ELL_WAVE          1   /* ELL_solver = "wave" (WaveElliptic, the default) */
#define OLLIN_ELL_SOR           2   /* ELL_solver = "sor"  */
#define OLLIN_ELL_MIXED         3   /* "mixed": no counterpart in the reference -- the system that "sor"
                                       converges to, solved by FP64 iterative refinement (exactly summed
                                       residuals) whose FP32 multigrid corrections are Orthomin search
                                       directions, to an RMS residual of ELL_epsilon (interior and Robin
                                       rows each) plus two refinements, or the FP64 floor */
#define OLLIN_ELL_FP64MG        4   /* "fp64mg": no counterpart in the reference -- the same solve as "mixed"
                                       with FP64 multigrid corrections: the all-FP64 solve of the system
                                       that the mixed-precision solve's error is measured against */

#define OLLIN_PULSE_SHELL       0   /* scalarpulse_type = "shell"     */
#define OLLIN_PULSE_TORUS       1   /* scalarpulse_type = "torus"     */
#define OLLIN_PULSE_BAUMGARTE   2   /* scalarpulse_type = "Baumgarte" */

#define OLLIN_ILAPSE_ONE        0   /* ilapse = "one"       */
#define OLLIN_ILAPSE_ISOTROPIC  1   /* ilapse = "isotropic" */
#define OLLIN_ILAPSE_PSIMINUS2  2   /* ilapse = "psiminus2" */
#define OLLIN_ILAPSE_PSIMINUS4  3   /* ilapse = "psiminus4" */
#define OLLIN_ILAPSE_MAXIMAL    4   /* ilapse = "maximal": alpha = 1 until the host's
                                     * first ollin_gpu_maximal_slicing (evolve.f90:228) */

/*
 * Parsed parameters, field for field the values of the reference's
 * ``param`` module (src/base/param.f90) that the evolution path reads.
 * ``ollin_params_default`` fills the reference's defaults.
 */
typedef struct ollin_params {
    /* grid: param.f90:95-141 */
    int    nrtotal, nztotal;   /* Nrtotal, Nztotal: points per level (without ghosts) */
    int    nl0;                /* Nl0: refinement levels above the base grid */
    int    ghost;              /* ghost zones: 0 or fewer than the order needs gives 2 (order two) or
                                  3 (order four), a larger value up to 8 is kept (main.f90:286-318) */
    int    eqsym;              /* equatorial symmetry */
    double dr0, dz0;           /* base-grid spacing */
    double dtfac;              /* dt0 = dtfac*min(dr0,dz0) (setupboxes.f90:119) */
    /* time integration: param.f90:410-427 */
    int    integrator;         /* OLLIN_INTEGRATOR_* */
    int    icniter;
    int    order;              /* 2 ("two", the reference's default) or 4 ("four") */
    /* formulation: param.f90:407-438 */
    int    slicing;            /* OLLIN_SLICING_* */
    double gauge_f;
    int    shift;              /* OLLIN_SHIFT_* */
    double drivercsi, drivereta;
    int    driveradv, shiftadvect;
    int    chimethod, chipower;
    int    evolveH, evolveKTH, nolambda;
    int    lagrangian;         /* bssnflavor = "lagrangian" (1) / "eulerian" (0) */
    int    factorhdet;
    double eta;                /* BSSN Delta damping multiple of the momentum constraint */
    double geodiss, scalardiss;
    double ft[8];              /* ft1..ft8 */
    int    boundtype;          /* OLLIN_BOUND_* */
    int    interp_bicubic;     /* interporder = "bicubic" (1) / "bilinear" (0) */
    /* matter: param.f90:612-643 */
    int    mattertype;         /* OLLIN_MATTER_* */
    int    scalarpotential;    /* OLLIN_POTENTIAL_* */
    double scalar_mass, scalar_lambda;
    /* initial data (host side, initial.f90) */
    int    idata;              /* OLLIN_IDATA_* */
    int    ilapse;             /* OLLIN_ILAPSE_* */
    double bh1mass;
    /* elliptic initial data (appended; earlier offsets are unchanged):
     * solver controls param.f90:454-491, Brill waves :573-582, scalar pulse
     * :623-643 */
    int    ell_solver;         /* OLLIN_ELL_* */
    int    ell_maxiter;        /* ELL_maxiter */
    double ell_epsilon;        /* ELL_epsilon */
    int    we_method;          /* WE_method: OLLIN_INTEGRATOR_* */
    int    we_maxiter;         /* WE_maxiter */
    double we_eta, we_diss, we_dtfac, we_epsilon;
    int    scalarpulse_type;   /* OLLIN_PULSE_* */
    int    brilltype;          /* 0 = "Holz" */
    double scalar_a0, scalar_r0, scalar_z0, scalar_sr0, scalar_sz0;
    double brill_a0, brill_sr0, brill_sz0;
    /* refinement boxes (appended; param.f90:115-139, setupboxes.f90): box 0
     * is the base grid with Nl0 levels above it, boxes 1..nb have levels
     * 1..nl[b-1] of nrbox x nzbox points centred at (rbox, zbox) */
    int    nb;                 /* Nb, 0..3 */
    int    nl[3];              /* Nl1, Nl2, Nl3 */
    int    nrbox[3], nzbox[3]; /* Nrbox1..3, Nzbox1..3 */
    double rbox[3], zbox[3];   /* rbox1..3, zbox1..3 (before the alignment of setupboxes.f90:186-206) */
    /* shift options (appended; param.f90:325-352) */
    int    driverD0;           /* subtract the t = 0 Delta in the driver equations */
    double shiftafter;         /* shift sources zero while t(box 0, level 0) < shiftafter */
} ollin_params;

/* Evolved and auxiliary fields addressable by upload/download.  The names are
 * the reference's array names (src/base/arrays.config). */
enum ollin_field {
    OLLIN_F_ALPHA = 0, OLLIN_F_PHI, OLLIN_F_CHI,
    OLLIN_F_A, OLLIN_F_B, OLLIN_F_H, OLLIN_F_C,
    OLLIN_F_TRK, OLLIN_F_KTA, OLLIN_F_KTB, OLLIN_F_KTH, OLLIN_F_KTC,
    OLLIN_F_DELTA_R, OLLIN_F_DELTA_Z,
    OLLIN_F_LAMBDA, OLLIN_F_ALAMBDA,
    OLLIN_F_BETA_R, OLLIN_F_BETA_Z, OLLIN_F_DTBETA_R, OLLIN_F_DTBETA_Z,
    OLLIN_F_SCALAR_PHI, OLLIN_F_SCALAR_XI_R, OLLIN_F_SCALAR_XI_Z, OLLIN_F_SCALAR_PI,
    OLLIN_F_FDRIVER,                      /* evolved by the shock-avoiding drivers (else 1) */
    OLLIN_F_NEVOLVED,                     /* number of evolved-field slots */
    /* derived (read-only) fields, computed on request */
    OLLIN_F_HAM = 64, OLLIN_F_MOM_R, OLLIN_F_MOM_Z,
    OLLIN_F_RSCAL, OLLIN_F_KT2, OLLIN_F_LAPLA_ALPHA
};

/* One level's geometry (box 0): arrays are (1-ghost:nr, 1-ghost:nz). */
typedef struct ollin_level_desc {
    int    level;                   /* refinement level of the grid */
    int    nr, nz, ghost;
    double dr, dz, dt;
    double rmin, rmax, zmin, zmax;  /* rminl/rmaxl/zminl/zmaxl incl. ghosts (evolve.f90:75-92) */
    double time;                    /* t(box,level) */
    int    steps;                   /* s(box,level) */
    int    box;                     /* refinement box (appended) */
    double rbox, zbox;              /* the box centre after setupboxes.f90:186-206 (appended) */
} ollin_level_desc;

typedef struct ollin_handle ollin_handle;

/* Fill ``p`` with the reference defaults of param.f90. */
void ollin_params_default(ollin_params* p);

/* Allocate the level hierarchy on the current CUDA device.
 * Replaces: allocatearrays('on') + setupboxes (src/base/main.f90:333-365). */
int ollin_gpu_create(const ollin_params* p, ollin_handle** out);
void ollin_gpu_destroy(ollin_handle* h);

/* Grid geometry and clocks.  The ``level`` argument of this and every other
 * entry point is a grid index: box 0's levels 0..Nl0 first (so with Nb = 0
 * it is the refinement level), then levels 1..Nl(b) of boxes b = 1..Nb, the
 * order of the reference's ``do box=0,Nb; do level=min(1,box),Nl(box)``
 * loops (e.g. src/base/evolve.f90:157-167).  ollin_gpu_num_levels counts
 * the grids; ollin_level_desc gives each one's box and level. */
int ollin_gpu_level_desc(const ollin_handle* h, int level, ollin_level_desc* out);
int ollin_gpu_num_levels(const ollin_handle* h);

/* The grid's coordinates r(i) for i = 1-ghost..Nr into r[0..Nr+ghost-1] and
 * z(j) into z[0..Nz+ghost-1], the values of evolve.f90:42-70 that the
 * kernels use (the reference's r(i,j) is r(i) on every row). */
int ollin_gpu_coords(const ollin_handle* h, int level, double* r, double* z);

/* Host <-> device copies of one grid function of one level.
 * Replaces direct access to grid(0,level)%<field> (generated mytypes.f90). */
int ollin_gpu_upload(ollin_handle* h, int level, int field, const double* a, int ld_r);
int ollin_gpu_download(ollin_handle* h, int level, int field, double* a, int ld_r);

/* n uploads / downloads in one call: copy k moves ``fields[k]`` of grid
 * ``levels[k]`` from / to the host array a[k] (leading dimension ld_r[k]),
 * as ollin_gpu_upload / ollin_gpu_download do, with one synchronisation for
 * all of them.  Evolved fields only; every copy is checked before any is
 * queued.  A host that moves a whole state per step (a Fortran driver that
 * keeps its arrays) uses these. */
int ollin_gpu_upload_many(ollin_handle* h, int n, const int* levels, const int* fields, const double* const* a,
                          const int* ld_r);
int ollin_gpu_download_many(ollin_handle* h, int n, const int* levels, const int* fields, double* const* a,
                            const int* ld_r);

/* The value of ``field`` at n arbitrary points of grid ``level``: rz holds
 * (r0, z0) pairs, out receives n values (host arrays).  Replaces
 * ``interp(box,level,r0,z0,flag)`` (src/base/interp.f90:2-270: a node is
 * copied, bicubic Lagrange inside, bilinear within one cell of the grid's
 * edge, or bilinear everywhere for interporder = "bilinear"), as the
 * diagonal output of save1Ddata.f90:624-750 and a horizon finder call it.
 * A point whose stencil would leave the grid gets NaN and the call returns
 * OLLIN_EINVAL. */
int ollin_gpu_interp(ollin_handle* h, int level, int field, const double* rz, int n, double* out);

/* Host-side initial data for the supported ``idata`` values, uploaded to
 * every level.  Replaces: call initial (src/base/evolve.f90:124,
 * src/base/initial.f90:59-218, 528-645). */
int ollin_gpu_initial_data(ollin_handle* h);

/* Symmetries, auxiliary quantities on every level at t=0 and the
 * Gamma-driver initialisation.  Replaces src/base/evolve.f90:128-195. */
int ollin_gpu_initialize(ollin_handle* h);

/* Recompute auxiliary quantities of one level after the host changed its
 * state (uploaded arrays).  Replaces: call auxiliary
 * (src/base/auxiliary.f90:26-56) for the current grid. */
int ollin_gpu_aux(ollin_handle* h, int level);

/* One coarse time step of every level: the exact equivalent of
 * ``call onestep(0)`` (src/base/onestep.f90:2-522, called from
 * src/base/evolve.f90:381).  ``t_out`` (may be NULL) receives t(0,0). */
int ollin_gpu_coarse_step(ollin_handle* h, double* t_out);

/* One coarse step of each of ``n`` independent evolutions (handles on the
 * same device).  All steps are queued, each on its handle's stream, before
 * any is waited for, so the kernels of small grids run side by side; the
 * results are those of n ollin_gpu_coarse_step calls.  ``t_out`` (may be
 * NULL) receives each t(0,0).  No counterpart in the reference, which runs
 * one evolution per process (a host batching independent runs calls this
 * in its loop over them). */
int ollin_gpu_coarse_step_many(ollin_handle* const* hs, int n, double* t_out);

/* The smallest lapse over every grid (the minimum of save0Ddata.f90:221-288 on
 * each grid's interior, then over grids): one queued reduction per grid, one
 * copy, one wait.  OLLIN_ENAN if a lapse is NaN. */
int ollin_gpu_min_lapse(ollin_handle* h, double* out);

/* One coarse step split in two, for callers that overlap several evolutions
 * (the request loop below): ollin_gpu_step_begin queues ``onestep(0)`` on the
 * handle's stream and returns without waiting; ollin_gpu_step_end waits for
 * it, checks for non-finite values and gives the coarse time.  Between the
 * two the caller may queue work on other handles.  Every begin needs its end,
 * also when begin failed (the end then waits for what was queued). */
int ollin_gpu_step_begin(ollin_handle* h);
int ollin_gpu_step_end(ollin_handle* h, double* t_out);
/* 1 when ollin_gpu_step_end would not wait (the queued step has finished, or
 * none is queued), 0 while the step runs.  Does not block. */
int ollin_gpu_step_ready(const ollin_handle* h);
/* enable = 1 (the default): the kernels of a coarse step are launched as a
 * programmatic dependent chain -- each may be scheduled while its
 * predecessor runs and waits on the device for it -- which shortens the gaps
 * between the short kernels of small grids; 0: ordinary launches (what the
 * request loop and ollin_gpu_coarse_step_many with n > 1 use: evolutions
 * running side by side fill the SMs already).
 * Results are the same either way. */
int ollin_gpu_step_chaining(ollin_handle* h, int enable);
/* enable = 1: ollin_gpu_step_begin (and ollin_gpu_coarse_step,
 * ollin_gpu_coarse_step_many) records the coarse step by stream capture
 * and launches it as one CUDA graph (same kernels, arguments and order, so
 * the same results); 0: direct launches (the default); -1: leave as is.
 * ``stats`` (may be null) gets the graphs instantiated and updated so far. */
int ollin_gpu_step_graphs(ollin_handle* h, int enable, long long stats[2]);

/* Device bytes an evolution with parameters ``p`` holds from create to
 * destroy (``resident``), and the most its elliptic solves (initial data,
 * maximal slicing) add while they run (``transient``).  An upper bound that
 * includes the 2 MiB granularity of large allocations; no device work.  No
 * counterpart in the reference (one run per process). */
int ollin_gpu_footprint(const ollin_params* p, size_t* resident, size_t* transient);

/* ---------------------------------------------------------------------------
 * Request loop (continuous batching of evolutions; no counterpart in the
 * reference, whose evolve.f90 runs one evolution per process).
 *
 * Requests are submitted as parameter sets with an end time.  Every running
 * evolution always has one coarse step queued on its own stream; no
 * evolution waits for another.  Each call to ollin_server_tick (1) takes
 * every evolution whose step has finished, runs the maximal-slicing solve
 * that follows the step if any, checks the lapse against the request's
 * collapse threshold, and either retires it (end time reached, collapsed or
 * failed) or queues its next step; (2) admits waiting requests, in arrival
 * order and first fit, while their footprint (resident + transient) fits in
 * the device budget next to the running ones' resident bytes and a slot is
 * free -- their initial data, ``initialize`` and any initial maximal-slicing
 * solve run on their own streams while the queued steps run.  A tick that
 * finds nothing to do waits until some step finishes.  A retired
 * evolution's handle is destroyed; its summary is kept for
 * ollin_server_poll.  Each evolution's arithmetic is that of a lone run:
 * running in the mix changes only when its steps happen.
 * ------------------------------------------------------------------------- */
typedef struct ollin_server ollin_server;

#define OLLIN_RESULT_MAXGRIDS 8
typedef struct ollin_result {
    long long id;       /* the caller's request id */
    int    status;      /* OLLIN_OK, or the code that ended the evolution */
    int    collapsed;   /* 1: the smallest lapse fell below the request's threshold */
    int    steps;       /* coarse steps taken */
    int    ngrids;      /* grids of the evolution (norms below for the first OLLIN_RESULT_MAXGRIDS) */
    double t;           /* coarse time reached */
    double min_alpha;   /* smallest lapse at the last check (every coarse step with a threshold, else at the end) */
    double t_submit, t_admit, t_ready, t_done;  /* seconds since ollin_server_create: submitted,
                                                  admitted, set up (initial data done), finished */
    size_t bytes;       /* resident + transient bytes reserved for it */
    double l2[OLLIN_RESULT_MAXGRIDS][4];  /* per grid at the end: L2 norms of alpha, phi, trK, ham (save0Ddata.f90:221-288) */
    double point_updates;                 /* grid points advanced by one full step, summed over its steps */
} ollin_result;

/* ``budget``: device bytes the server's evolutions may hold; ``max_active``:
 * evolutions stepped together (>= 1). */
int ollin_server_create(size_t budget, int max_active, ollin_server** out);
void ollin_server_destroy(ollin_server* s);
/* Queue a request: evolve ``p`` (copied) to coarse time ``t_end`` (rounded to
 * whole coarse steps), with the maximal-slicing solves of evolve.f90:228-230
 * and :388-393 (``maximalevery`` is the par-file value; slicing or ilapse
 * "maximal" in ``p`` also count), stopping early when the smallest lapse over
 * all grids falls below ``collapse_alpha`` (0: no check).  A request that
 * could never fit the budget is rejected at once with OLLIN_ENOMEM; bad
 * parameters give OLLIN_EINVAL. */
int ollin_server_submit(ollin_server* s, long long id, const ollin_params* p, int maximalevery, double t_end,
                        double collapse_alpha);
/* One round of the loop; ``n_active``/``n_waiting`` (may be null) give the
 * counts after it.  Failures of single evolutions end up in their results;
 * the return value is nonzero only for a failure of the loop itself. */
int ollin_server_tick(ollin_server* s, int* n_active, int* n_waiting);
/* Move up to ``max`` finished results, oldest first, into ``out``; ``n_out``
 * gets the number moved. */
int ollin_server_poll(ollin_server* s, ollin_result* out, int max, int* n_out);
/* Whether evolutions admitted from now on step as captured graphs
 * (ollin_gpu_step_graphs; on by default). */
int ollin_server_set_graphs(ollin_server* s, int enable);
/* The loop's schedule: 0 (default) every running evolution keeps its own next
 * coarse step queued on its stream and moves on as soon as that step ends;
 * 1 each tick is one fused coarse step of every running evolution
 * (ollin_gpu_coarse_step_fused: each kernel issued once for all of them),
 * with new requests joining at the next tick.  Results are the same bit for
 * bit.  Changed only while no step is queued (OLLIN_ESTATE otherwise). */
int ollin_server_set_fused(ollin_server* s, int enable);
/* Device bytes reserved now and at most so far by the server's evolutions. */
int ollin_server_usage(const ollin_server* s, size_t* used, size_t* peak);
/* Message for the last failure of an ollin_server_* call on the calling thread. */
const char* ollin_server_last_error(void);

/* Constraint norms and 0-D statistics of one field of one level, the five
 * numbers of save0Dvariable (src/base/save0Ddata.f90:221-288):
 * out[0]=max, out[1]=min, out[2]=nm1 (max |f|), out[3]=nm2 (RMS), out[4]=origin value.
 * Derived fields (OLLIN_F_HAM ...) are computed first (constraints.f90:55-149). */
int ollin_gpu_norms(ollin_handle* h, int level, int field, double out[5]);

/* Maximal slicing on every level: solve lap(alpha) = (K_ij K^ij +
 * 4 pi (rho + S)) alpha with the physical Laplacian of the conformal metric
 * and alpha -> 1 far away, by the solver of ELL_solver (wave or sor), and
 * replace the lapse.  Replaces: call maximalslicing
 * (src/geometry/maximalslicing.f90:3-175), which the host calls at
 * src/base/evolve.f90:228-230 (after ollin_gpu_initialize, when slicing or
 * ilapse is "maximal" or maximalevery /= 0) and :388-393 (after
 * ollin_gpu_coarse_step, when slicing = "maximal" or every maximalevery
 * steps).  ``va_max`` (may be NULL): the largest |va_rp|, |va_zp| over all
 * levels that the host's last analysis_geometry/cfl call left, which
 * wave_elliptic.f90:211-263 folds into its time step; NULL stands for the
 * zero arrays of a run that has not called either.  Like the reference, the
 * call recomputes only the lapse and its first and second derivatives: the
 * next stage of each level still sees the covariant second derivatives,
 * Laplacian, falpha and advective derivatives of the lapse before the solve.
 * ELL_solver = "mixed" solves the same discrete system as "sor" with FP64
 * residuals and FP32 multigrid corrections, "fp64mg" with FP64 ones (no
 * counterpart in the reference); every solver works with refinement boxes
 * and without equatorial symmetry. */
int ollin_gpu_maximal_slicing(ollin_handle* h, const double* va_max);

/* Iterations of the elliptic solve run by ollin_gpu_initial_data for
 * idata = BrillWave / scalarpulse (wave_elliptic.f90:190-262): steps[0] in
 * the coarse-grid phase, steps[1] in the all-level phase (0 with one level);
 * for SOR the iterations on level 0 and level 1; for "mixed" the FP64
 * refinements and the FP32 V-cycles on level 0.  ``gres`` (may be NULL)
 * receives the final residual; after ollin_gpu_maximal_slicing, the numbers
 * of that solve.  No counterpart call in the reference, which prints these
 * numbers. */
int ollin_gpu_ell_stats(const ollin_handle* h, int steps[2], double* gres);

/* The convergence history of the last "mixed" or "fp64mg" solve (initial
 * data or maximal slicing) on ``level``: the larger of the RMS residuals of
 * the interior equations and of the Robin rows (level 0), before each
 * correction and after the last one, up to ``max``
 * values into ``rms``; ``*n`` receives the full count (0 before any such
 * solve).  A non-finite residual ends that solve with OLLIN_ENAN.  No
 * counterpart call in the reference. */
int ollin_gpu_ell_history(const ollin_handle* h, int level, double* rms, int max, int* n);

/* Total point-updates performed by this handle so far (interior points of
 * each level times the steps taken on it). */
double ollin_gpu_point_updates(const ollin_handle* h);

/* The CUDA stream (cudaStream_t) all work of this handle is ordered on,
 * so a caller can record events or synchronise on it. */
void* ollin_gpu_stream(const ollin_handle* h);

/* Number of kernel launches this handle has issued so far. */
long long ollin_gpu_launch_count(const ollin_handle* h);

/* Per-launch timing of the right-hand-side kernel with CUDA events on the
 * handle's stream (for roofline reporting).  Enabling resets the counters.
 * No counterpart in the reference, which has no timers. */
int ollin_gpu_kernel_timing(ollin_handle* h, int enable);
int ollin_gpu_kernel_stats(ollin_handle* h, double* rhs_ms, long long* launches, double* point_stages);

/* Measured FP64 fused-multiply-add instruction rate of the current device
 * (DFMA per second), the ceiling the right-hand-side kernel is held to.
 * No counterpart in the reference. */
double ollin_gpu_fp64_rate(void);

/* Measured rate (operations per second, whole device) of one arithmetic
 * operation: 0 DFMA, 1 DADD, 2 DMUL, 3 DDIV, 4 sqrt, 5 cbrt, 6 exp, 7 log
 * (all FP64), 8 FP32 FMA.  Eight independent chains per thread, 8 blocks of
 * 256 threads per SM.  Returns -1 for an unknown op or on failure.  No
 * counterpart in the reference: it prices the FP64 operations of the
 * right-hand side. */
double ollin_gpu_op_rate(int op);

/*
 * Restart data: replaces checkpointsave / checkpointrestart
 * (src/base/checkpoint.f90:2-328, :338-700).  A reference checkpoint holds,
 * per grid, every evolved array, its boundary history var_bound_{rL,rR,zL,zR}
 * (:253-300) and the clocks t, t1, t2.  On the device the history lives in
 * whole time levels of the state: ``which`` = 0 is the current state, 1 the
 * state at the start of the level's last step (history level 0 on the
 * strips), 2 the start of the step before (history level 1); history level
 * 2 of the reference is never read by finebound's time interpolation.
 * A restart is: ollin_gpu_create, ollin_gpu_upload_slot of every evolved
 * field for which = 0, 1, 2, ollin_gpu_set_clocks of every grid, then
 * ollin_gpu_initialize, which runs what evolve.f90:128-219 runs after
 * checkpointrestart: parity fill, ``auxiliary`` (with the t > 0 branches,
 * since t is no longer 0), the Gamma-driver reset dtbeta = drivercsi Delta
 * (:174-195, as the reference does on a restart) and the t = 0 syncboxes.
 * That ``auxiliary`` call projects A, B, C, H onto unit determinant once
 * more, as the reference's does, which can move them by an ulp; for a
 * continuation bit for bit use ollin_gpu_resume instead of
 * ollin_gpu_initialize.
 * Fields: the ids accepted by ollin_gpu_upload.  ld_r as for ollin_gpu_upload.
 */
int ollin_gpu_download_slot(ollin_handle* h, int level, int field, int which, double* a, int ld_r);
int ollin_gpu_upload_slot(ollin_handle* h, int level, int field, int which, const double* a, int ld_r);
/* Resume a suspended evolution instead of restarting it: after the slots and
 * clocks of a running evolution (t > 0 on every grid) have been uploaded,
 * recompute the auxiliary quantities of that state without projecting it
 * onto unit determinant again and without the Gamma-driver reset, and mark
 * the handle initialized.  The evolution then continues bit for bit as if
 * never interrupted (an ``auxiliary`` call, as ollin_gpu_initialize makes,
 * re-applies factordet and moves A, B, C, H by an ulp).  No counterpart in
 * the reference: it lets a host evict an evolution's state to host memory
 * and bring it back.  Not for a state suspended between a maximal-slicing
 * solve or a syncboxes copy and the next coarse step (their pending stale
 * quantities are not part of the slots). */
int ollin_gpu_resume(ollin_handle* h);
/* out = {t, t1, t2, s} of grid ``level`` (prl/arrays.pl:54-58; s is the
 * level's step count, whose parity decides restriction, onestep.f90:472). */
int ollin_gpu_get_clocks(ollin_handle* h, int level, double out[4]);
/* Sets {t, t1, t2, s} of a grid; only before ollin_gpu_initialize
 * (OLLIN_ESTATE afterwards).  s must be a whole number. */
int ollin_gpu_set_clocks(ollin_handle* h, int level, const double in[4]);

/*
 * One coarse step of n independent evolutions with every kernel of the step
 * issued once for all of them.  Each evolution's step is recorded (the host
 * logic of onestep as usual, the launches kept instead of issued); evolutions
 * whose steps launch the same kernels in the same order form a group, and each
 * kernel of a group's sequence runs as one multi-instance launch whose blocks
 * are the blocks of every member's launch, each block reading its evolution's
 * argument struct from device memory (one upload per call).  The kernels and
 * arguments are those of ollin_gpu_coarse_step, so the results are the same
 * bit for bit; a step is some 150 launches for the whole batch instead of per
 * evolution.  Evolutions with syncboxes copies in their steps are stepped on
 * their own streams.  Returns after every evolution's step has finished,
 * with the first failure; status (may be NULL) receives each evolution's own
 * code (OLLIN_ENAN for the one that produced a non-finite value), so that a
 * caller can retire a failed evolution and keep the others.
 * No counterpart in the reference (it runs one evolution per process).
 */
int ollin_gpu_coarse_step_fused(ollin_handle* const* hs, int n, double* t_out, int* status);

/* Whether ollin_gpu_coarse_step_fused records each group's launch sequence as
 * a CUDA graph the first time it meets it and replays it on later steps of
 * the same batch (1, the default), or issues the launches directly (0).  The
 * kernels, arguments and order are the same either way.  No counterpart in
 * the reference. */
int ollin_gpu_fused_graphs(int on);

/*
 * One coarse step of n independent evolutions under the schedule an
 * autotuner picks for this batch (the same handles in the same order): the
 * fused launches replayed as graphs (0), the fused launches issued directly
 * (1), or every evolution on its own stream (2, ollin_gpu_coarse_step_many).
 * The first calls for a batch try each schedule on live steps, two steps each
 * (results are the same bit for bit under every schedule, so nothing is
 * wasted), timing the second by wall clock per point-update; later calls use
 * the fastest.  *schedule_out (may be NULL) reports the schedule used.  No
 * counterpart in the reference.
 */
int ollin_gpu_coarse_step_auto(ollin_handle* const* hs, int n, double* t_out, int* schedule_out);

/* Message for the last failure on the calling thread ("" if none). */
const char* ollin_gpu_last_error(void);

/*
 * The five 0-D statistics of ollin_gpu_norms (max, min, max|f|, RMS over
 * i = 1..nr-ghost, j = 1..nz-ghost, and the bicubic value at the origin) of a
 * grid function that the caller already holds in device memory, computed
 * without allocating anything.  No counterpart in the reference: it exists
 * for callers that cannot call cudaMalloc -- hosts whose device memory comes
 * from their own allocator or pool, regions where an allocation would
 * synchronise the device, tools that may only read.
 *
 * d_field points at element (1-ghost, 1-ghost) of a column-major
 * (1-ghost:nr, 1-ghost:nz) array with leading dimension ld_r; ghost is the
 * grid's number of ghost zones (2 to 8) and the grid equatorially symmetric (box-0
 * coordinates r = (i-1/2) dr, z = (j-1/2) dz); eqsym = 0 is refused with
 * OLLIN_EINVAL.  ``stream`` is a cudaStream_t or NULL; the call returns after
 * the result has reached ``out`` (host memory), so a capturing stream is
 * refused with OLLIN_EINVAL.  out[4] is the bicubic origin value, which is
 * save0Dvariable's for interporder = "bicubic" (the default) only.
 *
 * Limit: nz - ghost <= 8192 interior rows (larger grids get OLLIN_EINVAL).
 * The intermediate results live in one fixed 320 KiB device array that is
 * part of the library image, so every GPU that loads the library holds it
 * until the process exits.  The first call on a device looks up that array's
 * device address (with the device current) and keeps it for the life of the
 * process, so it must not be called on a device after cudaDeviceReset; make
 * that first call before any stream capture.  All calls share the array and it keeps the last call's
 * contents; every slot a call reads is written earlier in the same call, so
 * no clearing is needed, but calls whose work overlaps on the GPU (other
 * threads or streams, at the same time) race on it and must be serialised by
 * the caller.
 */
int ollin_gpu_norms_noalloc(const double* d_field, int nr, int nz, int ghost, int ld_r, double dr, double dz,
                            int eqsym, void* stream, double out[5]);
/* Message for the last failure of ollin_gpu_norms_noalloc on the calling thread. */
const char* ollin_gpu_noalloc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* OLLIN_GPU_H */
