"""Elliptic initial data on the GPU (WaveElliptic on the device, C ABI)
against the oracle: the same iteration counts in both solver phases, the
conformal factor and the derived fields to the FP64 parity bound, and the
evolution that starts from them.

The reference's all-level phase measures the residual on level 0, where the
restricted fine solution does not satisfy the coarse discretisation, so with
refinement levels it usually runs to WE_maxiter.  The multi-level cases here
cap WE_maxiter to keep the oracle's run short; the single-level cases
converge to WE_epsilon."""
import numpy as np
import pytest

from oracle_bind import Oracle, ell_stats
from parity_util import field_list, params, rel_diff, tol_for

pytestmark = pytest.mark.gpu

BASE = dict(eqsym=1, order="four", integrator="rk4", ilapse="one", slicing="1+log", gauge_f=2.0,
            geodiss=0.02, dtfac=0.25, boundtype="radiative")

PULSE_1LEV = dict(BASE, nrtotal=32, nztotal=32, nl0=0, dr0=0.4, dz0=0.4, idata="scalarpulse",
                  mattertype="scalar", scalar_a0=0.05, scalardiss=0.02)
PULSE_2LEV = dict(BASE, nrtotal=32, nztotal=32, nl0=1, dr0=0.4, dz0=0.4, idata="scalarpulse",
                  mattertype="scalar", scalar_a0=0.05, scalar_r0=3.0, scalar_z0=3.0, scalardiss=0.02,
                  we_maxiter=200)
BRILL_3LEV = dict(BASE, nrtotal=32, nztotal=32, nl0=2, dr0=0.25, dz0=0.25, idata="BrillWave",
                  brill_a0=1.0, we_maxiter=150)
BRILL_RK4 = dict(BASE, nrtotal=24, nztotal=24, nl0=0, dr0=0.25, dz0=0.25, idata="BrillWave",
                 brill_a0=4.0, we_method="rk4", we_eta=0.5)
# without equatorial symmetry: the pulse off the equator, the radiative
# boundary of the wave solver on the lower z edge too
PULSE_NOEQSYM = dict(BASE, eqsym=0, nrtotal=24, nztotal=24, nl0=1, dr0=0.5, dz0=0.5, idata="scalarpulse",
                     mattertype="scalar", scalar_a0=0.05, scalar_r0=2.0, scalar_z0=1.0, scalardiss=0.02,
                     we_maxiter=200)


def solve_pair(cfg):
    from ollin.gpu import Evolution
    p = params(cfg)
    o = Oracle(p)
    o.initial_data()
    ostats = ell_stats()
    e = Evolution(p)
    e.initial_data()
    return o, e, ostats, e.ell_stats()


def check_fields(o, e, cfg, names, tag):
    for lev in o.levels():
        for nm in names:
            d = rel_diff(e.download(lev, nm), o.get(lev, nm))
            assert d <= tol_for(nm), "%s level %d %s: rel diff %.3e" % (tag, lev, nm, d)


# refinement boxes: box 0's level 1 and a box above it that overlap (the
# wave solver's syncboxes of ell_u and ell_v)
PULSE_BOXES = dict(BASE, nrtotal=24, nztotal=24, nl0=1, dr0=0.5, dz0=0.5, Nb=1, Nl1=1, Nrbox1=16, Nzbox1=16,
                   zbox1=4.0, idata="scalarpulse", mattertype="scalar", scalar_a0=0.05, scalar_r0=2.0,
                   scalar_z0=3.0, scalardiss=0.02, we_maxiter=120)


# a ring off the axis and the equator with two levels: the wave solver's
# lower r and z strips, and the pulse's xi on the ring's ghost columns
PULSE_RING = dict(BASE, nrtotal=24, nztotal=24, nl0=1, dr0=0.5, dz0=0.5, Nb=1, Nl1=2, Nrbox1=12, Nzbox1=12,
                  rbox1=5.0, zbox1=5.0, idata="scalarpulse", mattertype="scalar", scalar_a0=0.05, scalar_r0=4.0,
                  scalar_z0=4.0, scalardiss=0.02, we_maxiter=120)


@pytest.mark.parametrize("cfg", [PULSE_1LEV, PULSE_2LEV, BRILL_3LEV, BRILL_RK4, PULSE_NOEQSYM, PULSE_BOXES,
                                 PULSE_RING, dict(PULSE_2LEV, order="two"),
                                 dict(PULSE_RING, order="two", Nrbox1=13, Nzbox1=13), dict(PULSE_RING, ghost=4)],
                         ids=["pulse_1lev", "pulse_2lev", "brill_3lev", "brill_rk4_damped", "pulse_no_eqsym",
                              "pulse_boxes", "pulse_ring", "pulse_2lev_order_two", "pulse_ring_order_two",
                              "pulse_ring_ghost4"])
def test_elliptic_data_matches_oracle(cfg):
    o, e, (o0, o1, ophases, ogres), (g0, g1, ggres) = solve_pair(cfg)
    assert (g0, g1) == (o0, o1), "iterations gpu %s oracle %s" % ((g0, g1), (o0, o1))
    assert abs(ggres - ogres) <= 1e-6 * ogres
    names = ["phi", "chi", "A", "B", "H", "C", "alpha"]
    if cfg.get("mattertype") == "scalar":
        names += ["scalar_phi", "scalar_xi_r", "scalar_xi_z", "scalar_pi"]
    check_fields(o, e, cfg, names, "initial data")
    if cfg["nl0"] == 0 and "we_maxiter" not in cfg:
        assert ggres <= 1e-8  # converged to WE_epsilon


def test_evolution_from_scalar_pulse_data():
    """Evolve the scalar pulse (two levels) from its elliptic initial data."""
    cfg = dict(PULSE_2LEV, we_maxiter=120)
    o, e, *_ = solve_pair(cfg)
    o.initialize()
    e.initialize()
    for k in range(3):
        assert o.step() == e.step()
    check_fields(o, e, cfg, field_list(cfg), "step 3")


SOR_2LEV = dict(BASE, nrtotal=24, nztotal=24, nl0=1, dr0=0.4, dz0=0.4, idata="scalarpulse",
                mattertype="scalar", scalar_a0=0.05, scalar_r0=2.0, scalar_z0=2.0, scalardiss=0.02,
                ell_solver="sor")
SOR_POTENTIAL = dict(BASE, nrtotal=24, nztotal=24, nl0=0, dr0=0.25, dz0=0.25, idata="scalarpulse",
                     mattertype="scalar", scalarpotential="phi2", scalar_mass=1.0, scalar_a0=0.1,
                     scalardiss=0.02, ell_solver="sor")
SOR_BRILL = dict(BASE, nrtotal=32, nztotal=32, nl0=2, dr0=0.25, dz0=0.25, idata="BrillWave",
                 brill_a0=1.0, ell_solver="sor")


# SOR with refinement boxes (sor_elliptic.f90:293-521): the layout of the
# executed-reference fixture (a box as large as box 0), and a smaller box
# off the axis, where the reference's work arrays (sized by the last box)
# would be overrun and only the oracle's restatement defines the result
SOR_BOXES = dict(BASE, nrtotal=16, nztotal=16, nl0=1, dr0=0.5, dz0=0.5, Nb=1, Nl1=1, Nrbox1=16, Nzbox1=16,
                 zbox1=3.0, idata="scalarpulse", mattertype="scalar", scalar_a0=0.05, scalar_r0=2.0,
                 scalar_z0=3.0, scalardiss=0.02, ell_solver="sor")
SOR_RING = dict(BASE, nrtotal=24, nztotal=24, nl0=1, dr0=0.5, dz0=0.5, Nb=1, Nl1=2, Nrbox1=12, Nzbox1=12,
                rbox1=5.0, zbox1=5.0, idata="scalarpulse", mattertype="scalar", scalar_a0=0.05, scalar_r0=4.0,
                scalar_z0=4.0, scalardiss=0.02, ell_solver="sor")


# without equatorial symmetry: the Robin condition on the lower z edge and
# the lower corner (sor_elliptic.f90:724-756), the layout of the
# executed-reference fixture ell_sor_noeqsym and a Brill wave on three levels
SOR_NOEQSYM = dict(BASE, nrtotal=16, nztotal=16, nl0=1, dr0=0.5, dz0=0.5, eqsym=0, idata="scalarpulse",
                   mattertype="scalar", scalar_a0=0.05, scalar_r0=2.0, scalar_z0=1.0, scalardiss=0.02,
                   ell_solver="sor")
SOR_BRILL_NOEQSYM = dict(SOR_BRILL, eqsym=0, nztotal=48)


@pytest.mark.parametrize("cfg", [SOR_2LEV, SOR_POTENTIAL, SOR_BRILL, SOR_BOXES, SOR_RING, SOR_NOEQSYM,
                                 SOR_BRILL_NOEQSYM, dict(SOR_RING, ghost=4), dict(SOR_NOEQSYM, ghost=4)],
                         ids=["sor_pulse_2lev", "sor_pulse_potential", "sor_brill_3lev", "sor_boxes",
                              "sor_ring_two_levels", "sor_pulse_no_eqsym", "sor_brill_no_eqsym",
                              "sor_ring_ghost4", "sor_no_eqsym_ghost4"])
def test_sor_data_matches_oracle(cfg):
    """SOR (sor_elliptic.f90): the red-black sweeps and the sequential Robin
    boundary reproduce the reference's arithmetic; the residual norm that
    decides when to stop is summed in another order, so the iteration counts
    agree unless it lands within rounding of ELL_epsilon."""
    o, e, (o0, o1, _, _), (g0, g1, _) = solve_pair(cfg)
    assert (g0, g1) == (o0, o1), "iterations gpu %s oracle %s" % ((g0, g1), (o0, o1))
    names = ["phi", "chi", "A", "B", "H", "C", "alpha"]
    if cfg.get("mattertype") == "scalar":
        names += ["scalar_phi", "scalar_xi_r", "scalar_xi_z"]
    check_fields(o, e, cfg, names, "sor initial data")



MIXED_2LEV = dict(SOR_2LEV, ell_solver="mixed", ell_epsilon=1e-12)
MIXED_BRILL = dict(SOR_BRILL, ell_solver="mixed", ell_epsilon=1e-12)
FP64MG_2LEV = dict(MIXED_2LEV, ell_solver="fp64mg")
FP64MG_BRILL = dict(MIXED_BRILL, ell_solver="fp64mg")
# refinement boxes: a box on the axis above box 0's level 1, and a ring off
# the axis and the equator (Dirichlet rows on all its edges, its ghost
# columns and rows unknowns as SOR sweeps them)
MIXED_BOXES = dict(SOR_BOXES, ell_solver="mixed", ell_epsilon=1e-12)
MIXED_RING = dict(SOR_RING, ell_solver="mixed", ell_epsilon=1e-12)
# without equatorial symmetry: the lower z edge of the coarse problem is a
# Robin row (and its corner), the finer levels' lower edge a Dirichlet row
MIXED_NOEQSYM = dict(SOR_NOEQSYM, ell_solver="mixed", ell_epsilon=1e-12)
MIXED_BRILL_NOEQSYM = dict(SOR_BRILL_NOEQSYM, ell_solver="mixed", ell_epsilon=1e-12)


@pytest.mark.parametrize("cfg", [MIXED_2LEV, MIXED_BRILL, FP64MG_2LEV, FP64MG_BRILL, MIXED_BOXES, MIXED_RING,
                                 MIXED_NOEQSYM, MIXED_BRILL_NOEQSYM, dict(MIXED_RING, ghost=4),
                                 dict(MIXED_NOEQSYM, ghost=4)],
                         ids=["mixed_pulse_2lev", "mixed_brill_3lev", "fp64mg_pulse_2lev", "fp64mg_brill_3lev",
                              "mixed_boxes", "mixed_ring", "mixed_no_eqsym", "mixed_brill_no_eqsym",
                              "mixed_ring_ghost4", "mixed_no_eqsym_ghost4"])
def test_mixed_precision_solve_matches_fp64_sor(cfg):
    """ELL_solver = "mixed" (FP64 iterative refinement, FP32 multigrid
    corrections) and "fp64mg" (the same with FP64 multigrid corrections)
    solve the discrete system that SOR converges to.  The reference's SOR
    stop test at ELL_epsilon = 1e-8 corresponds to an RMS residual near
    N * 1e-16, so the oracle's FP64 SOR solution is the FP64 solve to compare
    with: the conformal factor agrees to 1e-10 once the FP64 residual of the
    solve is below 1e-12."""
    from ollin.gpu import Evolution
    o = Oracle(params(dict(cfg, ell_solver="sor", ell_epsilon=1e-8)))
    o.initial_data()
    e = Evolution(params(cfg))
    e.initial_data()
    outer, cycles, rms = e.ell_stats()
    assert rms < 1e-12 and outer >= 1 and cycles >= outer
    for lev in o.levels():
        chi = rel_diff(e.download(lev, "chi"), o.get(lev, "chi"))
        dphi = float(abs(e.download(lev, "phi") - o.get(lev, "phi")).max())
        assert chi <= 1e-10 and dphi <= 1e-10, "level %d: chi rel %.2e, phi abs %.2e" % (lev, chi, dphi)
        for nm in ("A", "B", "H", "C", "alpha"):
            assert rel_diff(e.download(lev, nm), o.get(lev, nm)) <= 1e-10


@pytest.mark.parametrize("a0", [1.0, 4.0, 5.0])
def test_precision_pattern_against_fp64_solve(a0):
    """The Brill-wave precision configuration at reduced size (2 levels of
    256^2, dr0 = 0.16, so the same physical extent as 4 levels of 1024^2 at
    0.04 on the coarse level): the conformal factor of the mixed solver
    against the all-FP64 multigrid solve of the same system, then the
    maximal-slicing lapse after one coarse step, every solve by each solver;
    both agree to 1e-10 (max abs)."""
    from ollin.gpu import Evolution
    base = dict(eqsym=1, order="four", integrator="rk4", ilapse="one", idata="BrillWave", brill_a0=a0,
                brill_sr0=1.0, brill_sz0=1.0, nrtotal=256, nztotal=256, nl0=1, dr0=0.16, dz0=0.16,
                ell_epsilon=1e-12, maximalevery=1, slicing="1+log", gauge_f=2.0)
    res = {}
    for solver in ("mixed", "fp64mg"):
        e = Evolution(params(dict(base, ell_solver=solver)))
        e.initial_data()
        assert e.ell_stats()[2] < 1e-11
        chi = [e.download(lev, "chi") for lev in e.levels()]
        e.initialize()
        e.maximal_slicing()
        e.step()
        e.maximal_slicing()
        rms = e.ell_stats()[2]
        print("a0 = %g, %s: maximal-slicing RMS residual %.2e" % (a0, solver, rms))
        assert rms < 1e-10, (solver, rms)
        alpha = [e.download(lev, "alpha") for lev in e.levels()]
        res[solver] = (chi, alpha)
        e.close()
    for k, nm in enumerate(("chi", "alpha")):
        err = max(float(abs(a - b).max()) for a, b in zip(res["mixed"][k], res["fp64mg"][k]))
        print("a0 = %g: max |%s_mixed - %s_fp64| = %.2e" % (a0, nm, nm, err))
        assert err <= 1e-10, (nm, err)


# a massless scalar shell phi = a exp(-(r - 5)^2), a = 0.089, on one 1024^2
# level over a 16 M square: the zeroth-order term pi |grad phi|^2 of its
# Hamiltonian constraint has the Helmholtz sign, on which plain multigrid
# cycles diverge at this resolution (the RMS residual grew from 0.42 to 1.0
# within two refinements)
SHELL_1024 = dict(eqsym=1, order="four", integrator="rk4", ilapse="one", slicing="1+log", gauge_f=2.0,
                  idata="scalarpulse", mattertype="scalar", scalarpotential="none", scalarpulse_type="shell",
                  scalar_a0=0.0888, scalar_r0=5.0, scalar_sr0=1.0, scalar_sz0=1.0, nrtotal=1024, nztotal=1024,
                  nl0=0, dr0=16.0 / 1024, dz0=16.0 / 1024, ell_epsilon=1e-12)


def test_krylov_accelerated_solve_of_a_helmholtz_sign_problem():
    """Each multigrid correction is a search direction of an Orthomin
    iteration (the step that minimises the residual along its image, kept
    orthogonal to the last few): the residual of the interior rows falls
    to the FP64 floor, and the mixed (FP32 multigrid) and fp64mg solves of
    the system agree to 1e-10."""
    from ollin.gpu import Evolution
    chi = {}
    for solver in ("mixed", "fp64mg"):
        e = Evolution(params(dict(SHELL_1024, ell_solver=solver)))
        e.initial_data()
        h = e.ell_history(0)
        print(solver, "refinements", len(h) - 1, "RMS", ["%.1e" % x for x in h])
        assert h[-1] < 1e-11 and h[-1] < 1e-9 * h[0], (solver, h[-1])
        # the minimising step never lets the full residual grow; the RMS
        # over the interior rows (without the Robin rows) follows it to the
        # floor within a factor of two
        assert all(h[k + 1] <= 2.0 * h[k] for k in range(len(h) - 1)), (solver, h)
        chi[solver] = e.download(0, "chi")
        assert np.all(np.isfinite(chi[solver])) and chi[solver].min() > 0.0
        e.close()
    err = float(abs(chi["mixed"] - chi["fp64mg"]).max())
    print("max |chi_mixed - chi_fp64mg| = %.2e" % err)
    assert err <= 1e-10
