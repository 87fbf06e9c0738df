"""Output and restart compatibility of the GPU path (C ABI).

* 0-D records (src/base/save0Ddata.f90:297-403): the ``(2ES20.8E3)`` lines
  written from ollin_gpu_norms of the evolved state equal, character for
  character, the lines computed from the reference-executed fixture c1_small.
* Restart (src/base/checkpoint.f90): every evolved field's three time levels
  (current state and the two step starts that hold the boundary history of
  :253-300) and the clocks t, t1, t2, s are downloaded after some coarse
  steps and uploaded into a new handle.  ollin_gpu_resume continues the
  evolution bit for bit; ollin_gpu_initialize runs the reference's
  post-restart sequence instead (``auxiliary`` re-projects the metric, and
  with the Gamma-driver shift dtbeta = drivercsi Delta, evolve.f90:174-195),
  which stays within rounding of the uninterrupted evolution.
* 1-D and 2-D records (save1Ddata.f90, save2Ddata.f90) of the GPU state
  against the same writers fed by the oracle after the same steps, and the
  point interpolation behind the diagonals (ollin_gpu_interp, interp.f90)."""
import numpy as np
import pytest

from ollin.output import Save0D, header, lines, lines_1d, lines_2d
from oracle_bind import Oracle
from output_util import OUT_NAMES, OracleView, fixture_stats, load_fixture
from parity_util import C1, params

pytestmark = pytest.mark.gpu

EVOLVED = ["alpha", "chi", "phi", "A", "B", "H", "C", "trK", "KTA", "KTB", "KTC", "Delta_r", "Delta_z"]
SHIFT = ["beta_r", "beta_z", "dtbeta_r", "dtbeta_z"]


def test_gpu_records_match_reference_fixture(tmp_path):
    from ollin.gpu import Evolution
    d, meta, cfg = load_fixture("c1_small")
    e = Evolution(params(cfg))
    e.initial_data()
    e.initialize()
    writer = Save0D(str(tmp_path), OUT_NAMES)
    expect = {}
    done = 0
    for target in meta["steps"]:
        while done < target:
            e.step()
            done += 1
        wrote = all(("s%d_L%d_ham" % (done, lev)) in d for lev in e.levels())
        if wrote:
            writer.write(e)
        for lev in e.levels():
            t = float(d["s%d_L%d_time" % (done, lev)])
            assert e.clocks(lev)[0] == t
            for nm in OUT_NAMES:
                key = "s%d_L%d_%s" % (done, lev, nm)
                if key not in d:  # constraints are stored at the first and last snapshot
                    continue
                ref = lines(t, fixture_stats(d[key]))
                assert lines(t, e.norms(lev, nm)) == ref, (done, lev, nm)
                if wrote:
                    for kind, rec in ref.items():
                        expect.setdefault((nm, lev, kind), []).append(rec)
    for (nm, lev, kind), recs in expect.items():
        text = (tmp_path / ("%s_b0l%d_%s.tl" % (nm, lev, kind))).read_text().splitlines()
        assert text == [header(nm, kind)] + recs
    e.close()


def _restart_copy(src, cfg, names, resume):
    from ollin.gpu import Evolution
    dst = Evolution(params(cfg))
    for lev in src.levels():
        for nm in names:
            for which in (0, 1, 2):
                dst.upload_slot(lev, nm, which, src.download_slot(lev, nm, which))
        dst.set_clocks(lev, src.clocks(lev))
    if resume:
        dst.resume()
    else:
        dst.initialize()
    return dst


def _worst(a, b, names, tag, exact):
    worst = 0.0
    for lev in a.levels():
        assert np.array_equal(a.clocks(lev), b.clocks(lev)), (tag, lev)
        for nm in names:
            if nm == "phi":
                # phi is evolved during a level's first step only; afterwards
                # its slots hold values nothing reads (download recomputes
                # phi = -log(chi)/2), so it is compared that way
                assert np.array_equal(a.download(lev, "phi"), b.download(lev, "phi")) or not exact
                continue
            for which in (0, 1, 2):
                x, y = a.download_slot(lev, nm, which), b.download_slot(lev, nm, which)
                if exact:
                    assert np.array_equal(x, y), "%s level %d %s slot %d: max diff %.3e" % (
                        tag, lev, nm, which, float(np.abs(x - y).max()))
                else:
                    worst = max(worst, float(np.abs(x - y).max()) / max(float(np.abs(x).max()), 1e-300))
    return worst


def _run(shift):
    from ollin.gpu import Evolution
    cfg = dict(C1, nrtotal=48, nztotal=48)
    names = list(EVOLVED)
    if shift:
        cfg.update(shift="Gammadriver2", drivercsi=0.75, drivereta=2.0)
        names += SHIFT
    x = Evolution(params(cfg))
    x.initial_data()
    x.initialize()
    for _ in range(5):
        x.step()
    return x, cfg, names


@pytest.mark.parametrize("shift", [False, True], ids=["puncture", "puncture_gammadriver2"])
def test_resume_continues_bit_for_bit(shift):
    """ollin_gpu_resume: the suspended evolution's three time levels and
    clocks in a new handle continue bit for bit, shift included."""
    x, cfg, names = _run(shift)
    y = _restart_copy(x, cfg, names, resume=True)
    _worst(x, y, names, "after resume", exact=True)
    for _ in range(7):
        assert x.step() == y.step()
    _worst(x, y, names, "7 coarse steps after resume", exact=True)
    for lev in x.levels():
        assert np.array_equal(x.norms(lev, "ham"), y.norms(lev, "ham"))
    x.close()
    y.close()


@pytest.mark.parametrize("shift", [False, True], ids=["puncture", "puncture_gammadriver2"])
def test_restart_follows_the_reference(shift):
    """A reference-style restart (ollin_gpu_initialize after the upload):
    ``auxiliary`` projects A, B, C, H onto unit determinant once more, which
    moves them by an ulp, and with the Gamma driver dtbeta is reset to
    drivercsi Delta (evolve.f90:174-195), as in the reference.  With dtbeta
    uploaded again the restarted evolution stays within 1e-12 (normwise) of
    the uninterrupted one over the next 7 coarse steps."""
    x, cfg, names = _run(shift)
    y = _restart_copy(x, cfg, names, resume=False)
    if shift:
        for lev in x.levels():
            for db, dl in (("dtbeta_r", "Delta_r"), ("dtbeta_z", "Delta_z")):
                assert np.array_equal(y.download_slot(lev, db, 0), 0.75 * y.download_slot(lev, dl, 0))
            for db in ("dtbeta_r", "dtbeta_z"):
                y.upload_slot(lev, db, 0, x.download_slot(lev, db, 0))
    for _ in range(7):
        assert x.step() == y.step()
    w = _worst(x, y, names, "7 coarse steps after restart", exact=False)
    assert w <= 1e-12, w
    x.close()
    y.close()


def test_clocks_only_before_initialize():
    from ollin.gpu import Evolution, OllinError
    e = Evolution(params(dict(C1, nl0=0)))
    e.initial_data()
    e.initialize()
    with pytest.raises(OllinError):
        e.set_clocks(0, [1.0, 0.5, 0.0, 2.0])
    e.close()


def _numbers(rec, width):
    return [float(rec[k:k + width]) for k in range(0, len(rec), width)]


@pytest.mark.parametrize("eqsym", [1, 0], ids=["eqsym", "no_eqsym"])
def test_1d_2d_records_match_oracle(eqsym):
    from ollin.gpu import Evolution
    cfg = dict(C1, nrtotal=24, nztotal=24, nl0=1, eqsym=eqsym)
    o = Oracle(params(cfg))
    e = Evolution(params(cfg))
    for x in (o, e):
        x.initial_data()
        x.initialize()
    for _ in range(2):
        assert o.step() == e.step()
    v = OracleView(o, cfg)
    for lev in o.levels():
        for nm in ("alpha", "trK"):
            got, ref = lines_1d(e, lev, nm, eqsym), lines_1d(v, lev, nm, eqsym)
            assert sorted(got) == sorted(ref)
            for ext in got:
                assert got[ext][0] == ref[ext][0] and len(got[ext]) == len(ref[ext]), ext
                a = np.array([_numbers(x, 20) for x in got[ext][1:-1]])
                b = np.array([_numbers(x, 20) for x in ref[ext][1:-1]])
                assert np.array_equal(a[:, 0], b[:, 0]), ext
                scale = max(np.abs(b[:, 1]).max(), 1e-6)
                assert np.abs(a[:, 1] - b[:, 1]).max() <= 1e-9 * scale, (lev, nm, ext)
            g2, r2 = lines_2d(e, lev, nm, True), lines_2d(v, lev, nm, True)
            assert g2[0] == r2[0] and len(g2) == len(r2)
            a = np.array([_numbers(x, 23) for x in g2[1:] if x])
            b = np.array([_numbers(x, 23) for x in r2[1:] if x])
            assert np.array_equal(a[:, :2], b[:, :2])
            assert np.abs(a[:, 2] - b[:, 2]).max() <= 1e-9 * max(np.abs(b[:, 2]).max(), 1e-6)


def test_interp_points_match_oracle():
    """ollin_gpu_interp against the oracle's interp.f90 at random points of
    each level (bicubic inside, bilinear next to the edges), at nodes (a
    copy), and a point outside the grid refused."""
    from ollin.gpu import Evolution, OllinError
    cfg = dict(C1, nrtotal=24, nztotal=24, nl0=1)
    o = Oracle(params(cfg))
    e = Evolution(params(cfg))
    for x in (o, e):
        x.initial_data()
        x.initialize()
    assert o.step() == e.step()
    rng = np.random.default_rng(5)
    for lev in o.levels():
        r, z = e.coords(lev)
        rr = rng.uniform(r[0], r[-1], 200)
        zz = rng.uniform(z[0], z[-1], 200)
        for nm in ("alpha", "KTA"):
            a, b = e.interp(lev, nm, rr, zz), o.interp(lev, nm, rr, zz)
            assert np.abs(a - b).max() <= 1e-10 * max(np.abs(b).max(), 1e-6), (lev, nm)
            # at nodes: the node's value (copied when r0 - r(1-ghost) divides
            # by dr exactly, else a Lagrange stencil whose weights are 0 and 1)
            node = e.interp(lev, nm, r[5:8], z[4:7])
            arr = e.download(lev, nm)
            want = np.array([arr[5, 4], arr[6, 5], arr[7, 6]])
            assert np.abs(node - want).max() <= 1e-13 * max(np.abs(want).max(), 1e-6), (lev, nm)
            assert np.abs(node - o.interp(lev, nm, r[5:8], z[4:7])).max() <= 1e-13 * max(np.abs(want).max(), 1e-6)
        with pytest.raises(OllinError):
            e.interp(lev, "alpha", [r[-1] + 10.0], [z[3]])
