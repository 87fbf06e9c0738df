"""Several independent evolutions stepped together
(ollin_gpu_coarse_step_many): each gives, bit for bit, what it gives when
stepped alone, and a non-finite value in one of them is reported."""
import numpy as np
import pytest

from parity_util import C1, field_list, params

pytestmark = pytest.mark.gpu

CFGS = [
    dict(C1, nrtotal=32, nztotal=32, nl0=1),
    dict(C1, nrtotal=24, nztotal=40, nl0=2, shift="Gammadriver2", drivercsi=0.75, drivereta=2.0),
    dict(C1, nrtotal=40, nztotal=24, nl0=0, integrator="icn", icniter=3, slicing="harmonic", gauge_f=1.0),
]


def make(cfg):
    from ollin.gpu import Evolution
    e = Evolution(params(cfg))
    e.initial_data()
    e.initialize()
    return e


def test_batched_steps_equal_single_steps():
    from ollin.gpu import step_many
    alone = [make(c) for c in CFGS]
    batch = [make(c) for c in CFGS]
    for _ in range(3):
        t_alone = [e.step() for e in alone]
        t_batch = step_many(batch)
        assert t_alone == t_batch
    for cfg, a, b in zip(CFGS, alone, batch):
        for lev in a.levels():
            for nm in field_list(cfg):
                assert np.array_equal(a.download(lev, nm), b.download(lev, nm)), (lev, nm)


def test_batched_step_reports_nan():
    from ollin.gpu import OllinError, step_many
    es = [make(c) for c in CFGS[:2]]
    a = es[1].download(0, "alpha")
    a[5, 5] = np.nan
    es[1].upload(0, "alpha", a)
    with pytest.raises(OllinError) as ex:
        step_many(es)
    assert ex.value.code == 3


# a mix for the fused step: groups of identical launch sequences (two 3-level
# punctures of different sizes, two scalar shells), evolutions alone in their
# group (shift; ICN), a ring box without syncboxes, an overlapping box (its
# syncboxes copies put it on its own stream) and a maximal-slicing evolution
# whose first stage after each solve reads the stale lapse
FUSED_CFGS = CFGS + [
    dict(C1, nrtotal=48, nztotal=48, nl0=2),
    dict(C1, nrtotal=32, nztotal=32, nl0=1, dr0=0.25, dz0=0.25, idata="minkowski", ilapse="one",
         mattertype="scalar", scalarpotential="phi2", scalar_mass=0.5, scalardiss=0.02),
    dict(C1, nrtotal=24, nztotal=24, nl0=1, dr0=0.5, dz0=0.5, idata="minkowski", ilapse="one",
         mattertype="scalar", scalarpotential="phi2", scalar_mass=0.5, scalardiss=0.02),
    dict(C1, nrtotal=24, nztotal=24, nl0=0, dr0=0.5, dz0=0.5, Nb=1, Nl1=1, Nrbox1=10, Nzbox1=10, rbox1=5.0,
         zbox1=5.0, shift="Gammadriver2", drivercsi=0.75, drivereta=2.0),
    dict(C1, nrtotal=24, nztotal=24, nl0=1, dr0=0.25, dz0=0.25, Nb=1, Nl1=1, Nrbox1=16, Nzbox1=16, zbox1=2.0),
    dict(C1, nrtotal=24, nztotal=24, nl0=1, dr0=0.25, dz0=0.25, maximalevery=1, we_maxiter=150),
]


@pytest.mark.parametrize("graphs", [True, False], ids=["graphs", "direct"])
def test_fused_steps_equal_single_steps(graphs):
    """ollin_gpu_coarse_step_fused: every kernel of the step once for all the
    evolutions of a group, replayed as a recorded graph from the second step
    of a group on, or issued directly; the fields of every evolution equal,
    bit for bit, those of stepping it alone."""
    from ollin.gpu import fused_graphs, step_fused
    from parity_util import scalar_pulse
    fused_graphs(graphs)
    alone, fused = [], []
    for cfg in FUSED_CFGS:
        for lst in (alone, fused):
            from ollin.gpu import Evolution
            e = Evolution(params(cfg))
            e.initial_data()
            if cfg.get("mattertype") == "scalar":
                for lev in e.levels():
                    d = e.desc(lev)
                    i = np.arange(1 - d.ghost, d.nr + 1)
                    j = np.arange(1 - d.ghost, d.nz + 1)
                    r, z = np.meshgrid((i - 0.5) * d.dr, (j - 0.5) * d.dz, indexing="ij")
                    for nm, v in zip(["scalar_phi", "scalar_xi_r", "scalar_xi_z", "scalar_pi"], scalar_pulse(r, z)):
                        e.upload(lev, nm, v)
            e.initialize()
            if cfg.get("maximalevery"):
                e.maximal_slicing()
            lst.append(e)
    for step in range(4):
        t_alone = [e.step() for e in alone]
        t_fused = step_fused(fused)
        assert t_alone == t_fused
        for cfg, a, b in zip(FUSED_CFGS, alone, fused):
            if cfg.get("maximalevery"):
                a.maximal_slicing()
                b.maximal_slicing()
    for cfg, a, b in zip(FUSED_CFGS, alone, fused):
        for lev in a.levels():
            for nm in field_list(cfg):
                assert np.array_equal(a.download(lev, nm), b.download(lev, nm)), (cfg, lev, nm)
    for e in alone + fused:
        e.close()
    fused_graphs(True)


def test_fused_step_reports_nan():
    from ollin.gpu import OllinError, step_fused
    es = [make(c) for c in (CFGS[0], CFGS[0], CFGS[1])]
    a = es[1].download(0, "alpha")
    a[5, 5] = np.nan
    es[1].upload(0, "alpha", a)
    with pytest.raises(OllinError) as ex:
        step_fused(es)
    assert ex.value.code == 3


def test_autotuned_steps_equal_single_steps():
    """ollin_gpu_coarse_step_auto: two live steps under each schedule (fused
    with graphs, fused direct, one stream per evolution), then the fastest;
    every step gives the fields of stepping each evolution alone."""
    from ollin.gpu import step_auto
    cfgs = FUSED_CFGS[:4]
    alone = [make(c) for c in cfgs]
    auto = [make(c) for c in cfgs]
    used = []
    for _ in range(8):
        t_alone = [e.step() for e in alone]
        t_auto, sched = step_auto(auto)
        used.append(sched)
        assert t_alone == t_auto
    assert used[:6] == [0, 0, 1, 1, 2, 2]
    assert used[6] == used[7] and used[6] in (0, 1, 2)
    for cfg, a, b in zip(cfgs, alone, auto):
        for lev in a.levels():
            for nm in field_list(cfg):
                assert np.array_equal(a.download(lev, nm), b.download(lev, nm)), (lev, nm)
