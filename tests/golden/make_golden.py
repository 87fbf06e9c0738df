"""Generates the golden vectors of tests/golden/*.npz by executing the
reference's own Fortran evolution path (src/base/onestep.f90 and everything
it calls, plus initial.f90 and constraints.f90) through ``ftn_subset``.

Run from the repository root in a container that has the reference checked
out, giving its directory as the first argument or in OLLIN_REFERENCE_DIR:

    python tests/golden/make_golden.py <reference checkout> [case ...]

Each fixture stores, for a small box-in-box configuration, the reference's
grid functions (all points including ghosts, Fortran (i,j) at [i+g-1, j+g-1])
after 0, 1, 2, ... coarse steps, together with the parameters.  The
scalar-field case starts from an analytic Gaussian pulse written into the
arrays after ``initial``.  The ``ell_*`` cases run the reference's elliptic
initial data (idata_scalarpulse.f90 / idata_brillwave.f90 with
wave_elliptic.f90 or sor_elliptic.f90) inside ``initial``.
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from refsim import RefSim  # noqa: E402

BASE = dict(order="four", integrator="rk4", dtfac=0.25, boundtype="radiative", eqsym=True,
            idata="schwarzschild", bh1mass=1.0, ilapse="psiminus2", slicing="1+log",
            gauge_f=2.0, shift="none", geodiss=0.02)

CASES = {
    # Schwarzschild puncture, 1+log, no shift, 2 levels
    "c1_small": dict(BASE, nrtotal=16, nztotal=16, nl0=1, dr0=0.2, dz0=0.2, _steps=[0, 1, 2, 4]),
    # same with the Gamma-driver shift, 3 levels
    "c2_small": dict(BASE, nrtotal=16, nztotal=16, nl0=2, dr0=0.2, dz0=0.2, shift="Gammadriver2",
                     drivercsi=0.75, drivereta=2.0, _steps=[0, 1, 3]),
    # boundtype = "static" and "flat" (the generated simpleboundary.f90) on
    # level 0, the latter without equatorial symmetry (its lower edge too)
    "bound_static": dict(BASE, nrtotal=16, nztotal=16, nl0=1, dr0=0.2, dz0=0.2, boundtype="static",
                         shift="Gammadriver2", drivercsi=0.75, drivereta=2.0, _steps=[0, 1, 2]),
    "bound_flat_noeqsym": dict(BASE, nrtotal=16, nztotal=24, nl0=1, dr0=0.2, dz0=0.2, eqsym=False,
                               boundtype="flat", shift="Gammadriver2", drivercsi=0.75, drivereta=2.0,
                               _steps=[0, 1, 2]),
    # a par-file ghost larger than the order needs (main.f90:298-318 keeps
    # it): four ghost zones in order four, three in order two
    "ghost4_shift": dict(BASE, nrtotal=16, nztotal=16, nl0=2, dr0=0.2, dz0=0.2, ghost=4, shift="Gammadriver2",
                         drivercsi=0.75, drivereta=2.0, _steps=[0, 1, 2]),
    "ghost3_o2_box": dict(BASE, order="two", ghost=3, nrtotal=20, nztotal=20, nl0=1, dr0=0.5, dz0=0.5, Nb=1, Nl1=1,
                          Nrbox1=12, Nzbox1=12, rbox1=2.0, zbox1=2.0, _steps=[0, 1, 2]),
    # the first-order hyperbolic and the parabolic Gamma drivers
    # (sources_shift.f90:62-186, radiative_geometry.f90:195-235); the
    # parabolic one without equatorial symmetry, where the row j = 0 whose
    # shift sources the reference zeroes is an ordinary row
    "gd1_shift": dict(BASE, nrtotal=16, nztotal=16, nl0=2, dr0=0.2, dz0=0.2, shift="Gammadriver1",
                      drivercsi=0.75, drivereta=2.0, _steps=[0, 1, 3]),
    # (a small csi: the parabolic driver is an explicit diffusion of the
    # shift, stable for csi dt/dr^2 below about 0.7)
    "gd0_noeqsym": dict(BASE, nrtotal=16, nztotal=16, nl0=1, dr0=0.25, dz0=0.25, eqsym=False,
                        shift="Gammadriver0", drivercsi=0.1, _steps=[0, 1, 3]),
    # ICN with harmonic slicing and the isotropic lapse, one level
    "icn_harmonic": dict(BASE, nrtotal=16, nztotal=20, nl0=0, dr0=0.25, dz0=0.25, integrator="icn",
                         icniter=3, slicing="harmonic", gauge_f=1.0, ilapse="isotropic", _steps=[0, 1, 3]),
    # massive real scalar field on Minkowski data with the Gamma-driver shift
    "scalar_shift": dict(BASE, nrtotal=16, nztotal=16, nl0=1, dr0=0.25, dz0=0.25, idata="minkowski",
                         ilapse="one", mattertype="scalar", scalarpotential="phi2", scalar_mass=0.5,
                         shift="Gammadriver2", drivercsi=0.75, drivereta=2.0, scalardiss=0.02,
                         _steps=[0, 1, 3]),
    # no equatorial symmetry: the lower z edge is a physical (radiative)
    # boundary on level 0 and a refinement boundary (lower finebound strip)
    # on level 1; Gamma-driver shift for the lopsided stencils at both edges
    "noeqsym_shift": dict(BASE, nrtotal=16, nztotal=16, nl0=1, dr0=0.2, dz0=0.2, eqsym=False,
                          shift="Gammadriver2", drivercsi=0.75, drivereta=2.0, _steps=[0, 1, 2]),
    # elliptic initial data (WaveElliptic, the default ELL_solver): a centred
    # scalar pulse solved to convergence on one level
    "ell_pulse_1lev": dict(BASE, nrtotal=16, nztotal=16, nl0=0, dr0=0.5, dz0=0.5, idata="scalarpulse",
                           ilapse="one", mattertype="scalar", scalar_a0=0.05, scalardiss=0.02,
                           _steps=[0], _elliptic=True),
    # an off-centre shell pulse on two levels (both solver phases: coarse
    # solve, injection, all-level solve), the wave iterations capped at 150
    # per phase so that the run is short; then one evolution step
    "ell_pulse_2lev": dict(BASE, nrtotal=16, nztotal=16, nl0=1, dr0=0.5, dz0=0.5, idata="scalarpulse",
                           ilapse="one", mattertype="scalar", scalar_a0=0.05, scalar_r0=2.0,
                           scalar_z0=2.0, scalardiss=0.02, we_maxiter=150, _steps=[0, 1],
                           _elliptic=True),
    # Holz Brill wave on two levels (factorhdet rescales the metric afterwards)
    "ell_brill_2lev": dict(BASE, nrtotal=16, nztotal=16, nl0=1, dr0=0.25, dz0=0.25, idata="BrillWave",
                           ilapse="one", brill_a0=1.0, we_maxiter=150, _steps=[0], _elliptic=True),
    # the SOR solver (ELL_solver = "sor"): Robin coarse solve, Dirichlet fine
    "ell_sor_2lev": dict(BASE, nrtotal=16, nztotal=16, nl0=1, dr0=0.5, dz0=0.5, idata="scalarpulse",
                         ilapse="one", mattertype="scalar", scalar_a0=0.05, ell_solver="sor",
                         scalardiss=0.02, _steps=[0], _elliptic=True),
    # refinement boxes (Nb > 0) that do not overlap, box 0 the base grid
    # alone: box 1 on the axis above the equator (its lower z edge is a
    # refinement boundary, finebound.f90:361-397) with two levels, box 2 a
    # ring on the equator (lower r edge, finebound.f90:246-285)
    "box_two": dict(BASE, nrtotal=24, nztotal=24, nl0=0, dr0=0.5, dz0=0.5, Nb=2, Nl1=2, Nrbox1=12,
                    Nzbox1=12, zbox1=6.0, Nl2=1, Nrbox2=10, Nzbox2=10, rbox2=8.0, _steps=[0, 1, 2]),
    # a ring off the equator (both lower edges and their corner) with the
    # Gamma-driver shift
    "box_ring_shift": dict(BASE, nrtotal=24, nztotal=24, nl0=0, dr0=0.5, dz0=0.5, Nb=1, Nl1=1, Nrbox1=10,
                           Nzbox1=10, rbox1=5.0, zbox1=5.0, shift="Gammadriver2", drivercsi=0.75,
                           drivereta=2.0, _steps=[0, 1, 2]),
    # elliptic data and maximal slicing without equatorial symmetry (the
    # wave solver's radiative boundary on the lower z edge as well)
    "ell_pulse_noeqsym": dict(BASE, nrtotal=16, nztotal=16, nl0=1, dr0=0.5, dz0=0.5, eqsym=False,
                              idata="scalarpulse", ilapse="one", mattertype="scalar", scalar_a0=0.05,
                              scalar_r0=2.0, scalar_z0=1.0, scalardiss=0.02, we_maxiter=150, _steps=[0, 1],
                              _elliptic=True),
    "max_noeqsym_wave": dict(BASE, nrtotal=16, nztotal=16, nl0=0, dr0=0.25, dz0=0.25, eqsym=False,
                             maximalevery=1, we_maxiter=150, _steps=[0, 1], _elliptic=True),
    # elliptic data with refinement boxes: the wave solver's box loops and its
    # syncboxes of ell_u and ell_v (wave_elliptic.f90:1059-1082), on the
    # overlapping layout below
    "ell_pulse_boxes": dict(BASE, nrtotal=24, nztotal=24, nl0=1, dr0=0.5, dz0=0.5, Nb=1, Nl1=1, Nrbox1=16,
                            Nzbox1=16, zbox1=4.0, idata="scalarpulse", ilapse="one", mattertype="scalar",
                            scalar_a0=0.05, scalar_r0=2.0, scalar_z0=3.0, scalardiss=0.02, we_maxiter=100,
                            _steps=[0, 1], _elliptic=True),
    # the SOR solver with refinement boxes (sor_elliptic.f90:293-521): every
    # box's levels interpolated from their parents in order, then restricted
    # in the same order; box 1 on the axis above box 0's level 1.  The
    # reference sizes its SOR work arrays (sor_elliptic.f90:52) by the grid
    # current at entry, the last box's last level, so the box is as large as
    # box 0 (a smaller one overruns them)
    "ell_sor_boxes": dict(BASE, nrtotal=16, nztotal=16, nl0=1, dr0=0.5, dz0=0.5, Nb=1, Nl1=1, Nrbox1=16,
                          Nzbox1=16, zbox1=3.0, idata="scalarpulse", ilapse="one", mattertype="scalar",
                          scalar_a0=0.05, scalar_r0=2.0, scalar_z0=3.0, ell_solver="sor", scalardiss=0.02,
                          _steps=[0], _elliptic=True),
    # boxes that overlap on level 1 (syncboxes.f90 with intersect_interp.inc):
    # box 0's level 1 around the origin and box 1 on the axis above it
    "box_overlap": dict(BASE, nrtotal=24, nztotal=24, nl0=1, dr0=0.5, dz0=0.5, Nb=1, Nl1=1, Nrbox1=16,
                        Nzbox1=16, zbox1=4.0, _steps=[0, 1, 2]),
    # three grids on level 1 in a column on the axis: box 1 takes copies from
    # box 0's level 1 and from box 2 (two partners), and one copy reads a node
    # that the copy before it wrote (a chain)
    "box_three_chain": dict(BASE, nrtotal=32, nztotal=32, nl0=1, dr0=0.5, dz0=0.5, Nb=2, Nl1=1, Nl2=1,
                            Nrbox1=24, Nzbox1=24, zbox1=6.0, Nrbox2=24, Nzbox2=24, zbox2=10.0, _steps=[0, 1, 2]),
    # maximal slicing (maximalslicing.f90, physical Laplacian).  Time-symmetric
    # vacuum data have K_ij = 0 and a maximal lapse of exactly 1, and so does
    # a static massless scalar field (rho + S = 0), so the cases solve where
    # the source is not zero.  Initial maximal lapse on a massive scalar pulse
    # (rho + S = -2V, a small amplitude: the source then has the sign that
    # makes the damped wave equation grow, and must stay below the lowest
    # eigenvalue of the Laplacian on the grid), then 1+log evolution: the
    # first stage of each level sees the new lapse and its derivatives but
    # the other auxiliary quantities of the old one; WaveElliptic capped
    "max_ilapse_pulse": dict(BASE, nrtotal=16, nztotal=16, nl0=1, dr0=0.5, dz0=0.5, idata="scalarpulse",
                             ilapse="maximal", mattertype="scalar", scalarpotential="phi2", scalar_mass=1.0,
                             scalar_a0=0.02, scalar_r0=2.0, scalar_z0=2.0, scalardiss=0.02, we_maxiter=200,
                             _steps=[0, 1], _elliptic=True),
    # maximalevery = 1 on Schwarzschild data: a (trivial) solve at t = 0, then
    # one after every coarse step, where K_ij is no longer zero
    "max_every_wave": dict(BASE, nrtotal=16, nztotal=16, nl0=1, dr0=0.25, dz0=0.25, maximalevery=1,
                           we_maxiter=120, _steps=[0, 1, 2], _elliptic=True),
    # slicing = maximal with SOR after every coarse step; the Gamma-driver
    # shift makes C, and so the mixed (same-colour) couplings of the SOR
    # stencil, nonzero after the first step
    "max_slicing_sor": dict(BASE, nrtotal=16, nztotal=16, nl0=0, dr0=0.25, dz0=0.25, ilapse="one",
                            slicing="maximal", ell_solver="sor", shift="Gammadriver2", drivercsi=0.75,
                            drivereta=2.0, _steps=[0, 1, 2], _elliptic=True),
    # SOR without equatorial symmetry: the Robin condition on the lower z edge
    # and the lower corner (sor_elliptic.f90:724-756), for the elliptic data
    # (flat Laplacian, two levels) and for maximal slicing every step
    "ell_sor_noeqsym": dict(BASE, nrtotal=16, nztotal=16, nl0=1, dr0=0.5, dz0=0.5, eqsym=False,
                            idata="scalarpulse", ilapse="one", mattertype="scalar", scalar_a0=0.05,
                            scalar_r0=2.0, scalar_z0=1.0, ell_solver="sor", scalardiss=0.02, _steps=[0, 1],
                            _elliptic=True),
    "max_noeqsym_sor": dict(BASE, nrtotal=16, nztotal=16, nl0=0, dr0=0.25, dz0=0.25, eqsym=False,
                            maximalevery=1, ell_solver="sor", _steps=[0, 1], _elliptic=True),
    # the shock-avoiding drivers (sources_shift.f90:141-170, :268-294): fdriver
    # evolved with -2/3 fdriver DIV beta, the advection terms on; the second
    # one with driverD0 (the t = 0 Delta subtracted, no dtbeta initialisation)
    "gds1_shift": dict(BASE, nrtotal=16, nztotal=16, nl0=2, dr0=0.2, dz0=0.2, shift="Gammadrivershock1",
                       drivercsi=0.75, drivereta=2.0, driveradv=True, _steps=[0, 1, 3]),
    "gds2_d0": dict(BASE, nrtotal=16, nztotal=16, nl0=1, dr0=0.2, dz0=0.2, shift="Gammadrivershock2",
                    drivercsi=0.75, drivereta=2.0, driveradv=True, driverD0=True, _steps=[0, 1, 3]),
    # shiftafter: the shift sources are zero until t(0,0) reaches it (dt0 =
    # 0.05: the first two coarse steps), while the dtbeta boundary still acts
    "gd2_shiftafter": dict(BASE, nrtotal=16, nztotal=16, nl0=1, dr0=0.2, dz0=0.2, shift="Gammadriver2",
                           drivercsi=0.75, drivereta=2.0, shiftafter=0.1, _steps=[0, 1, 3, 4]),
    # order two (the reference's default order, two ghost zones): centred
    # second-order differences, second-order one-sided advection and the
    # fourth-difference dissipation (derivatives.f90, derivadvect.f90,
    # dissipation.f90 :121-135), with the hierarchy's strips and margins
    # from ghost = 2: the puncture on 2 levels, the Gamma driver on 3
    "o2_c1": dict(BASE, order="two", nrtotal=16, nztotal=16, nl0=1, dr0=0.2, dz0=0.2, _steps=[0, 1, 2, 4]),
    "o2_shift": dict(BASE, order="two", nrtotal=16, nztotal=16, nl0=2, dr0=0.2, dz0=0.2, shift="Gammadriver2",
                     drivercsi=0.75, drivereta=2.0, _steps=[0, 1, 3]),
    # without equatorial symmetry (the one-sided rows at the lower z edge), a
    # massive scalar field with the shift
    "o2_noeqsym_scalar": dict(BASE, order="two", nrtotal=16, nztotal=16, nl0=1, dr0=0.25, dz0=0.25,
                              eqsym=False, idata="minkowski", ilapse="one", mattertype="scalar",
                              scalarpotential="phi2", scalar_mass=0.5, shift="Gammadriver2", drivercsi=0.75,
                              drivereta=2.0, scalardiss=0.02, _steps=[0, 1, 3]),
    # the wave elliptic solver on order-two stencils, then one step
    "o2_ell_pulse": dict(BASE, order="two", nrtotal=16, nztotal=16, nl0=0, dr0=0.5, dz0=0.5, idata="scalarpulse",
                         ilapse="one", mattertype="scalar", scalar_a0=0.05, scalardiss=0.02, _steps=[0, 1],
                         _elliptic=True),
}

FIELDS = ["alpha", "phi", "chi", "A", "B", "H", "C", "trK", "KTA", "KTB", "KTH", "KTC",
          "Delta_r", "Delta_z", "lambda", "Alambda"]
SHIFT_FIELDS = ["beta_r", "beta_z", "dtbeta_r", "dtbeta_z"]
SCALAR_FIELDS = ["scalar_phi", "scalar_xi_r", "scalar_xi_z", "scalar_pi"]
DERIVED = ["ham", "mom_r", "mom_z", "RSCAL", "KT2", "Lapla_alpha"]


def scalar_pulse(r, z, a0=0.05):
    """phi = a0 exp(-(r^2+z^2)), xi = grad phi, pi = 0 (analytic, so every
    ghost point already has the right parity)."""
    ph = a0 * np.exp(-(r ** 2 + z ** 2))
    return ph, -2.0 * r * ph, -2.0 * z * ph, np.zeros_like(ph)


def run_case(refdir, name, cfg):
    cfg = dict(cfg)
    steps = cfg.pop("_steps")
    elliptic = cfg.pop("_elliptic", False)
    sim = RefSim(refdir, cfg)
    # count the level-0 wave steps of the elliptic solve (one per iteration)
    wave_iters = [0]
    if elliptic and hasattr(sim.prog.F, "wavestep"):
        inner = sim.prog.F.wavestep

        def counted(level, typ, method):
            if level == 0:
                wave_iters[0] += 1
            return inner(level, typ, method)
        sim.prog.F.wavestep = counted
    t_ini = time.time()
    sim.initial()
    if elliptic:
        print("  %s: initial data in %.1fs, %d wave iterations" % (name, time.time() - t_ini, wave_iters[0]),
              flush=True)
    if cfg.get("mattertype") == "scalar" and not elliptic:
        for lev in sim.levels():
            r, z = sim.field(lev, "r"), sim.field(lev, "z")
            ph, xr, xz, pi = scalar_pulse(r, z)
            for nm, v in zip(["scalar_phi", "scalar_xi_r", "scalar_xi_z", "scalar_pi"], [ph, xr, xz, pi]):
                sim.set_field(lev, nm, v)
    ini_iters = wave_iters[0]
    sim.initialize()
    max_iters = [wave_iters[0] - ini_iters]
    names = list(FIELDS)
    if cfg.get("shift", "none") != "none":
        names += SHIFT_FIELDS
    if cfg.get("shift", "none").startswith("Gammadrivershock"):
        names += ["fdriver"]
    if cfg.get("mattertype") == "scalar":
        names += SCALAR_FIELDS
    out = {}
    if elliptic:
        out["wave_iterations"] = np.array(ini_iters)
        out["max_wave_iterations_s0"] = np.array(max_iters[0])
        for lev in sim.levels():
            for nm in ("psi", "ell_u", "ell_S1"):
                out["ell_L%d_%s" % (lev, nm)] = sim.field(lev, nm)
    done = 0
    for target in steps:
        while done < target:
            t0 = time.time()
            sim.step()
            done += 1
            # evolve.f90:388-393
            me = int(cfg.get("maximalevery", 0))
            if cfg.get("slicing") == "maximal" or (me != 0 and done % me == 0):
                before = wave_iters[0]
                sim.maximal_slicing()
                out["max_wave_iterations_s%d" % done] = np.array(wave_iters[0] - before)
            print("  %s: step %d in %.1fs" % (name, done, time.time() - t0), flush=True)
        for lev in sim.levels():
            for nm in names:
                out["s%d_L%d_%s" % (done, lev, nm)] = sim.field(lev, nm)
            if done == steps[-1] or done == 0:
                sim.analysis(lev)
                for nm in DERIVED:
                    out["s%d_L%d_%s" % (done, lev, nm)] = sim.field(lev, nm)
            out["s%d_L%d_time" % (done, lev)] = np.array(sim.time(lev))
    import ftn_subset
    meta = dict(cfg, steps=steps, fields=names, grids=[list(sim.box_level(k)) for k in sim.levels()],
                oob_beyond_reads=ftn_subset.OOB_BEYOND[0])
    ftn_subset.OOB_BEYOND[0] = 0
    out["meta"] = np.array(json.dumps(meta))
    return out


def main():
    refdir = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("OLLIN_REFERENCE_DIR")
    if not refdir or not os.path.isdir(os.path.join(refdir, "src", "base")):
        sys.exit("usage: make_golden.py <reference checkout> [case ...] "
                 "(or set OLLIN_REFERENCE_DIR); the directory must hold src/base/onestep.f90")
    only = sys.argv[2:]
    for name, cfg in CASES.items():
        if only and name not in only:
            continue
        t0 = time.time()
        out = run_case(refdir, name, cfg)
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **out)
        print("%s -> %s (%.0fs, %d KB)" % (name, path, time.time() - t0, os.path.getsize(path) // 1024))


if __name__ == "__main__":
    main()
