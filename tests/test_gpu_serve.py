"""The request loop (ollin_server_*) on the device: every request's result is
the one it gives alone, the device-byte budget bounds what runs at once, the
footprint bounds what an evolution holds, and the collapse threshold stops a
run early."""
import numpy as np
import pytest

from parity_util import C1, params

pytestmark = pytest.mark.gpu

BASE = dict(eqsym=1, order="four", integrator="rk4", ilapse="one", slicing="1+log", gauge_f=2.0,
            geodiss=0.02, dtfac=0.25, boundtype="radiative")
PULSE = dict(BASE, nrtotal=32, nztotal=32, nl0=1, dr0=0.4, dz0=0.4, idata="scalarpulse", mattertype="scalar",
             scalar_a0=0.05, scalar_r0=3.0, scalar_z0=3.0, scalardiss=0.02, we_maxiter=200)
BRILL = dict(BASE, nrtotal=32, nztotal=32, nl0=2, dr0=0.25, dz0=0.25, idata="BrillWave", brill_a0=1.0,
             we_maxiter=150)
# (parameters, maximalevery, t_end, collapse threshold)
MIX = [
    (dict(C1, nrtotal=32, nztotal=32, nl0=1), 0, 0.5, 0.0),
    (PULSE, 0, 1.2, 0.05),
    (BRILL, 0, 0.5, 0.0),
    (dict(C1, nrtotal=24, nztotal=24, nl0=1, dr0=0.25, dz0=0.25, ilapse="psiminus2", we_maxiter=150), 2, 0.25, 0.0),
    (dict(C1, nrtotal=40, nztotal=24, nl0=2, shift="Gammadriver2", drivercsi=0.75, drivereta=2.0), 0, 0.4, 0.0),
    (dict(C1, nrtotal=24, nztotal=24, nl0=1, dr0=0.25, dz0=0.25, Nb=1, Nl1=1, Nrbox1=16, Nzbox1=16, zbox1=2.0), 0,
     0.4, 0.0),
]


def submit_all(s, reqs, ids=None):
    for k, (cfg, me, t_end, col) in enumerate(reqs):
        s.submit(k if ids is None else ids[k], params(cfg), t_end, col, me)


@pytest.mark.parametrize("fused", [False, True], ids=["streams", "fused_ticks"])
def test_each_result_is_the_same_alone_and_in_the_mix(fused):
    """Alone versus in the mix, with each evolution on its own stream or with
    every tick one fused step of all running evolutions."""
    from ollin.gpu import Server
    alone = {}
    for k, req in enumerate(MIX):
        s = Server(1 << 36, max_active=1)
        submit_all(s, [req], ids=[k])
        (r,) = s.drain()
        assert r.status == 0, (k, r.status)
        alone[k] = r
        s.close()
    s = Server(1 << 36, max_active=len(MIX), fused=fused)
    submit_all(s, MIX)
    mixed = {r.id: r for r in s.drain()}
    assert sorted(mixed) == list(range(len(MIX)))
    for k, a in alone.items():
        b = mixed[k]
        assert b.status == 0 and (a.steps, a.t, a.collapsed) == (b.steps, b.t, b.collapsed), k
        assert a.steps > 0
        assert np.array_equal(a.norms(), b.norms()), k
        assert a.min_alpha == b.min_alpha, k
        assert np.all(np.isfinite(a.norms())) and a.norms()[:, 0].min() > 0
    # the mix ran together: some request was admitted before another finished
    spans = sorted((r.t_admit, r.t_done) for r in mixed.values())
    assert any(spans[i + 1][0] < spans[i][1] for i in range(len(spans) - 1))


def test_budget_bounds_what_runs_at_once():
    from ollin.gpu import Server, footprint
    cfg = dict(C1, nrtotal=32, nztotal=32, nl0=1)
    res, tr = footprint(params(cfg))
    budget = 2 * res + tr
    s = Server(budget, max_active=16)
    submit_all(s, [(cfg, 0, 0.3, 0.0)] * 5)
    most, out = 0, []
    while True:
        a, w = s.tick()
        most = max(most, a)
        out += s.poll()
        if a == 0 and w == 0:
            break
    assert most == 2
    used, peak = s.usage()
    assert used == 0 and peak <= budget
    assert len(out) == 5 and all(r.status == 0 for r in out)
    ref = out[0].norms()
    assert all(np.array_equal(r.norms(), ref) for r in out)


@pytest.mark.parametrize("cfg", [dict(C1, nrtotal=128, nztotal=128, nl0=2), dict(PULSE, nrtotal=96, nztotal=96)],
                         ids=["schwarzschild_3x128", "pulse_2x96"])
def test_footprint_bounds_the_device_bytes(cfg):
    import torch
    from ollin.gpu import Evolution, footprint
    torch.cuda.init()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    e = Evolution(params(cfg))
    e.initial_data()
    e.initialize()
    free1, _ = torch.cuda.mem_get_info()
    res, _ = footprint(params(cfg))
    held = free0 - free1
    assert 0 < held <= res, (held, res)
    e.close()


def test_collapse_threshold_stops_early():
    from ollin.gpu import Server
    s = Server(1 << 36, max_active=4)
    # the precollapsed puncture lapse is below 0.05 next to the puncture
    s.submit(0, params(dict(C1, nrtotal=32, nztotal=32, nl0=1)), 2.0, 0.05)
    # a weak pulse on a flat slice stays far from collapse
    s.submit(1, params(PULSE), 0.8, 0.05)
    out = {r.id: r for r in s.drain()}
    assert out[0].status == 0 and out[0].collapsed == 1 and out[0].steps == 1 and out[0].min_alpha < 0.05
    assert out[1].status == 0 and out[1].collapsed == 0 and out[1].min_alpha > 0.5
    assert out[1].steps == int(np.ceil(0.8 / (0.25 * 0.4) - 1e-9))


@pytest.mark.parametrize("fused", [False, True], ids=["streams", "fused_ticks"])
def test_a_failing_request_ends_alone(fused):
    """An unstable Courant factor (dtfac = 3) makes the evolution overflow
    within a few steps: its request ends with OLLIN_ENAN, and the request
    running beside it (in the same fused steps, with fused ticks) is
    unaffected."""
    from ollin.gpu import Server
    good = (dict(C1, nrtotal=32, nztotal=32, nl0=1), 0, 0.5, 0.0)
    s = Server(1 << 36, max_active=1)
    submit_all(s, [good])
    (alone,) = s.drain()
    s = Server(1 << 36, max_active=4, fused=fused)
    submit_all(s, [(dict(C1, nrtotal=24, nztotal=24, nl0=0, dtfac=3.0), 0, 5.0, 0.0), good])
    out = {r.id: r for r in s.drain()}
    assert out[0].status == 3 and 0 < out[0].steps < 10
    assert out[1].status == 0 and np.array_equal(out[1].norms(), alone.norms())
    assert s.usage()[0] == 0


def test_min_lapse_is_the_smallest_level_minimum():
    """ollin_gpu_min_lapse (one copy for all grids) against the minima of the
    per-grid statistics, on a box hierarchy and after steps."""
    from ollin.gpu import Evolution
    cfg = dict(C1, nrtotal=24, nztotal=24, nl0=1, dr0=0.25, dz0=0.25, Nb=1, Nl1=1, Nrbox1=16, Nzbox1=16, zbox1=2.0)
    e = Evolution(params(cfg))
    e.initial_data()
    e.initialize()
    for _ in range(3):
        e.step()
        m = min(e.norms(lev, "alpha")[1] for lev in e.levels())
        assert e.min_lapse() == m
