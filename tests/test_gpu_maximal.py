"""Maximal slicing on the GPU (ollin_gpu_maximal_slicing, C ABI) against the
oracle's restatement of maximalslicing.f90: the lapse after each solve, the
iteration counts of the wave solver, and the evolution that follows, whose
first stage on each level reads the lapse quantities of the last
``auxiliary`` call as the reference's does.

The host sequence is that of evolve.f90: a solve after ``initialize`` when
slicing or ilapse is "maximal" or maximalevery /= 0 (:228-230), and after a
coarse step when slicing is "maximal" or every maximalevery steps
(:388-393).

Bound: the lapse of a solve agrees to rounding (about 1e-13; the device
forms the coefficient derivatives with folded stencil constants) and the
wave iteration counts are equal.  Fields after a solve are held to 1e-9
normwise: trK starts from zero, so the relative difference of the small
trK a step later amplifies the rounding of the lapse's second derivatives
(observed 2e-10)."""
import pytest

from oracle_bind import Oracle, ell_stats
from parity_util import field_list, params, rel_diff, tol_for

pytestmark = pytest.mark.gpu

BASE = dict(eqsym=1, order="four", integrator="rk4", slicing="1+log", gauge_f=2.0, geodiss=0.02, dtfac=0.25,
            boundtype="radiative")

# initial maximal lapse on a massive scalar pulse (source 4 pi (rho + S) =
# -8 pi V: small, since with this sign a larger source makes the damped wave
# equation grow), wave solver on two levels, then 1+log evolution
PULSE = dict(BASE, nrtotal=24, nztotal=24, nl0=1, dr0=0.5, dz0=0.5, idata="scalarpulse", ilapse="maximal",
             mattertype="scalar", scalarpotential="phi2", scalar_mass=1.0, scalar_a0=0.02, scalar_r0=2.0,
             scalar_z0=2.0, scalardiss=0.02, we_maxiter=200)
# a solve after every coarse step of a Schwarzschild puncture (K_ij /= 0
# after the first step)
EVERY = dict(BASE, nrtotal=24, nztotal=24, nl0=1, dr0=0.25, dz0=0.25, idata="schwarzschild", bh1mass=1.0,
             ilapse="psiminus2", maximalevery=1, we_maxiter=150)
# slicing = maximal with SOR and the Gamma-driver shift: C /= 0 after the
# first step, so the SOR stencil couples points of one colour
SOR_SHIFT = dict(BASE, nrtotal=20, nztotal=20, nl0=0, dr0=0.25, dz0=0.25, idata="schwarzschild", bh1mass=1.0,
                 ilapse="one", slicing="maximal", ell_solver="sor", shift="Gammadriver2", drivercsi=0.75,
                 drivereta=2.0)
# SOR on two levels with C = 0 (the colours decouple), scalar pulse
SOR_PULSE = dict(PULSE, nrtotal=20, nztotal=20, ell_solver="sor", we_maxiter=100000)


def maximal_due(cfg, step):
    me = int(cfg.get("maximalevery", 0))
    if step == 0:
        return cfg.get("slicing") == "maximal" or cfg.get("ilapse") == "maximal" or me != 0
    return cfg.get("slicing") == "maximal" or (me != 0 and step % me == 0)


def solve_both(o, e, cfg, va_max, tag):
    o.maximal_slicing(va_max)
    e.maximal_slicing(va_max)
    o0, o1, _, _ = ell_stats()
    g0, g1, _ = e.ell_stats()
    if cfg.get("ell_solver", "wave") == "wave":
        assert (g0, g1) == (o0, o1), "%s: iterations gpu %s oracle %s" % (tag, (g0, g1), (o0, o1))
    for lev in o.levels():
        d = rel_diff(e.download(lev, "alpha"), o.get(lev, "alpha"))
        assert d <= tol_for("alpha"), "%s level %d alpha: rel diff %.3e" % (tag, lev, d)


TOL = 1e-9


def compare(o, e, cfg, tag):
    for lev in o.levels():
        for nm in field_list(cfg):
            d = rel_diff(e.download(lev, nm), o.get(lev, nm))
            assert d <= max(TOL, tol_for(nm)), "%s level %d %s: rel diff %.3e" % (tag, lev, nm, d)


def run(cfg, steps, va_max=None):
    from ollin.gpu import Evolution
    p = params(cfg)
    o, e = Oracle(p), Evolution(p)
    o.initial_data()
    e.initial_data()
    o.initialize()
    e.initialize()
    assert maximal_due(cfg, 0)
    solve_both(o, e, cfg, va_max, "t=0")
    for k in range(1, steps + 1):
        assert o.step() == e.step()
        compare(o, e, cfg, "step %d" % k)
        if maximal_due(cfg, k):
            solve_both(o, e, cfg, va_max, "after step %d" % k)
    return o, e


def test_initial_maximal_lapse_scalar_pulse():
    o, e = run(PULSE, 2)
    a = e.download(0, "alpha")
    assert a.max() > 1.001  # the source is not zero: a nontrivial lapse


def test_maximal_every_step_wave():
    run(EVERY, 3)


@pytest.mark.parametrize("solver", ["wave", "sor"])
def test_maximal_every_step_without_equatorial_symmetry(solver):
    """Without equatorial symmetry: the wave solver's radiative lower edge, or
    SOR's Robin lower edge and lower corner (sor_elliptic.f90:724-756)."""
    run(dict(EVERY, eqsym=0, nl0=0, ell_solver=solver), 2)


@pytest.mark.parametrize("solver", ["wave", "sor"])
def test_maximal_every_step_order_two(solver):
    """Order two: the wave solver's second-order physical Laplacian and
    fourth-difference dissipation, and the coefficient derivatives of either
    solver on second-order stencils."""
    run(dict(EVERY, order="two", ell_solver=solver), 2)


def test_maximal_every_step_with_refinement_boxes():
    """Box 0's level 1 and an overlapping box above it: the wave solver's box
    loops and syncboxes, then the stale lapse of the next stage on each grid."""
    run(dict(EVERY, nl0=1, Nb=1, Nl1=1, Nrbox1=16, Nzbox1=16, zbox1=2.0), 2)


def test_initial_maximal_lapse_scalar_pulse_with_refinement_boxes():
    """The solve right after ``initialize`` (whose t = 0 syncboxes is still
    pending) on a scalar pulse: the first stage on the box grids reads the
    kept pre-copy state and the solved lapse together."""
    run(dict(PULSE, Nb=1, Nl1=1, Nrbox1=16, Nzbox1=16, zbox1=4.0), 1)


@pytest.mark.parametrize("solver", ["wave", "sor"])
def test_maximal_every_step_on_a_ring(solver):
    """A ring off the axis and the equator: the coefficient derivatives on its
    ghost columns (r derivatives unset, so zero) and ghost rows (one-sided z
    stencils), with either solver's box handling.  SOR sweeps the ring's
    ghost columns (sor_elliptic.f90:648, i = 2..imax-1), so its source
    S1 = -K2 is needed there too: K_ij K^ij on the ghost columns of a grid
    off the axis (omitting it moves the level-0 lapse by 5.7e-8).  SOR stops when a residual
    norm summed in another order crosses ELL_epsilon, so at the default 1e-8
    the iteration counts can differ by one on level 0 and then by many on the
    ring, which starts from level 0's values (the lapses then agree to about
    the solver's tolerance, 1e-6); with ELL_epsilon = 1e-12 both converge to
    the same discrete solution."""
    cfg = dict(EVERY, nl0=0, Nb=1, Nl1=1, Nrbox1=12, Nzbox1=12, rbox1=2.5, zbox1=2.5, ell_solver=solver)
    if solver == "sor":
        cfg["ell_epsilon"] = 1e-12
    run(cfg, 2)


def test_maximal_every_step_with_speeds():
    """The slicing speeds of the host's last analysis enter the wave
    solver's time step (wave_elliptic.f90:211-263)."""
    run(dict(EVERY, nl0=0), 2, va_max=(1.7, 1.3))


def test_maximal_slicing_sor_with_shift():
    o, e = run(SOR_SHIFT, 3)
    # maximal slicing keeps trK = 0 (strK = 0, no radiative boundary)
    assert abs(e.download(0, "trK")).max() == 0.0


def test_maximal_lapse_sor_two_levels():
    run(SOR_PULSE, 1)


def test_maximal_slicing_sor_with_refinement_boxes():
    """SOR's box loops (sor_elliptic.f90:293-521) for the physical
    Laplacian: box 0's level 1 and an overlapping box above it, a solve after
    every step (so right after each syncboxes)."""
    run(dict(EVERY, nl0=1, Nb=1, Nl1=1, Nrbox1=16, Nzbox1=16, zbox1=2.0, ell_solver="sor"), 2)


@pytest.mark.parametrize("cfg", [EVERY, dict(SOR_SHIFT, slicing="1+log", maximalevery=1),
                                 dict(EVERY, nl0=1, Nb=1, Nl1=1, Nrbox1=16, Nzbox1=16, zbox1=2.0),
                                 dict(EVERY, eqsym=0)],
                         ids=["schwarzschild_two_levels", "shift_c_nonzero", "refinement_box", "no_eqsym"])
def test_maximal_lapse_mixed_precision_matches_fp64_sor(cfg):
    """ELL_solver = "mixed" for the physical Laplacian: FP64 residual of the
    nine-point SOR system, FP32 multigrid corrections of the flat operator
    applied to psi^4 times the residual.  It converges to the system SOR
    converges to, so after a coarse step (K_ij /= 0) the lapse agrees with the
    oracle's FP64 SOR solve."""
    from ollin.gpu import Evolution
    o = Oracle(params(dict(cfg, ell_solver="sor", ell_epsilon=1e-8)))
    e = Evolution(params(dict(cfg, ell_solver="mixed", ell_epsilon=1e-12)))
    for x in (o, e):
        x.initial_data()
        x.initialize()
        x.maximal_slicing()
        x.step()
    compare(o, e, cfg, "step 1")
    o.maximal_slicing()
    e.maximal_slicing()
    outer, cycles, rms = e.ell_stats()
    assert rms < 1e-11 and outer >= 1
    for lev in o.levels():
        d = rel_diff(e.download(lev, "alpha"), o.get(lev, "alpha"))
        assert d <= 1e-10, "level %d alpha: rel diff %.3e" % (lev, d)
    a = e.download(0, "alpha")
    assert a.min() < 0.999  # K_ij /= 0: a nontrivial lapse
