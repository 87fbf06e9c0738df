"""Benchmark: FP64 BSSN point-updates/s of the OllinAxis-BiB evolution path.

Workload (one "step" = one coarse step, ``call onestep(0)``): the large plain
configuration -- a Schwarzschild puncture (M=1, psi = 1 + M/2r, lapse psi^-2)
with 1+log slicing and the Gamma-driver-2 shift (drivereta = 2/M), 6
box-in-box levels of 512x512 points (finest dr = dz = 0.00625), RK4, 4th-order
differences, Kreiss-Oliger eps = 0.02, Courant factor 0.25, FP64.  One coarse
step advances level l by 2^l steps: 63 x 512^2 = 16.5 M point-updates.  Data
are synthetic (analytic initial data); the state (~1.5 GB) is far larger than
the 129 MB L2, so no L2 flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

``value`` is device-resident throughput timed with CUDA events on the
library's stream.  ``e2e`` is measured through the C ABI as a host-resident
caller would use it: every step copies the evolved state of all levels from
pinned host memory to the device, runs the coarse step and copies it back.
``--impl reference`` times the CPU restatement of the reference (oracle/,
the reference Fortran itself cannot be compiled on these hosts) on the host
cores.  With N > 1 (torchrun) every rank evolves an independent replica.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "ollinaxis-bib_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

WORKLOAD = dict(nrtotal=512, nztotal=512, nl0=5, dr0=0.2, dz0=0.2, eqsym=1, idata="schwarzschild",
                bh1mass=1.0, ilapse="psiminus2", slicing="1+log", gauge_f=2.0, shift="Gammadriver2",
                drivercsi=0.75, drivereta=2.0, integrator="rk4", order="four", geodiss=0.02,
                dtfac=0.25, boundtype="radiative")
METRIC = "FP64 BSSN point-updates/s"
UNIT = "point-updates/s"
F_EVOLVED = 16          # fields with non-zero sources (12 BSSN + 4 shift)
ALG_BYTES_PER_PU = 136 * F_EVOLVED  # compulsory FP64 traffic per point-update (3-register RK4)


def config_dict(args):
    nlev, n = args.levels, args.size
    return {"workload": "schwarzschild puncture, %d box-in-box levels of %dx%d, Gammadriver2, 1+log, RK4, FP64" % (nlev, n, n),
            "levels": nlev, "points_per_level": "%dx%d" % (n, n), "finest_dr": 0.2 / 2 ** (nlev - 1),
            "coarse_steps_per_step": 1, "point_updates_per_step": (2 ** nlev - 1) * n * n,
            "integrator": "rk4", "order": 4,
            "l2": "inputs larger than L2 (1.5 GB state), no flush", "parallelism": "replicas" if args.gpus > 1 else "single"}


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, x):
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(pg, x):
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def oracle_hierarchy(cfg):
    """The oracle (CPU restatement of the reference, C++ -O2, OpenMP loops)
    set up on ``cfg`` through the reference's sequence: initial data,
    ``initialize``."""
    from oracle_bind import Oracle
    from ollin.params import params_from_dict
    o = Oracle(params_from_dict(cfg))
    o.initial_data()
    o.initialize()
    return o


def time_oracle_steps(o, min_seconds, min_steps=1, max_steps=None):
    """Coarse steps of ``o`` until at least ``min_seconds`` and ``min_steps``
    have passed (or ``max_steps``); returns (steps, seconds, point-updates)."""
    pu0 = o.point_updates()
    t0 = time.perf_counter()
    n = 0
    while True:
        o.step()
        n += 1
        dt = time.perf_counter() - t0
        if (dt >= min_seconds and n >= min_steps) or (max_steps is not None and n >= max_steps):
            break
    return n, dt, o.point_updates() - pu0


def cpu_baseline(seconds=10.0):
    """The oracle on the host cores: the whole benchmarked hierarchy (6
    levels of 512^2, every level's steps, prolongation, restriction and
    recursion of onestep) with all cores, timed over whole coarse steps after
    one untimed coarse step; beside it one core on one 512^2 level of the same
    physics (a whole coarse step on one core takes minutes)."""
    from oracle_bind import set_threads
    cores = set_threads(host_cores())
    o = oracle_hierarchy(dict(WORKLOAD))
    o.step()  # untimed: the first step's time == 0 branches
    n, dt, pu = time_oracle_steps(o, seconds)
    del o
    one = set_threads(1)
    s = oracle_hierarchy(dict(WORKLOAD, nl0=0))
    s.step()
    n1, dt1, pu1 = time_oracle_steps(s, seconds / 2.0, min_steps=2)
    del s
    set_threads(cores)
    nlev = WORKLOAD["nl0"] + 1
    return {"value": pu / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d whole coarse step(s) of the %d-level %dx%d hierarchy (Gammadriver2, 1+log, RK4, FP64), "
                      "%.1f s, after one untimed coarse step" % (n, nlev, WORKLOAD["nrtotal"], WORKLOAD["nztotal"], dt),
            "single_thread": {"value": pu1 / dt1, "unit": UNIT, "cores": one,
                              "sample": "%d RK4 steps of one %dx%d level of the same physics on one core, %.1f s"
                                        % (n1, WORKLOAD["nrtotal"], WORKLOAD["nztotal"], dt1)}}


# Largest number of coarse steps the reference arm times (one coarse step of
# the 6-level hierarchy takes several seconds on the host cores).
REFERENCE_MAX_STEPS = 30


def run_reference(args):
    """The reference's CPU path (the oracle restatement; the Fortran cannot be
    built on these hosts) on the same workload as the GPU arm: whole coarse
    steps of the 6-level hierarchy with every host core.  One untimed coarse
    step stands in for the warm-up (a CPU needs no more); the timed steps are
    the requested ones, up to REFERENCE_MAX_STEPS."""
    world, rank, _, pg = dist_setup(args)
    if rank != 0:
        return
    from oracle_bind import set_threads
    threads = set_threads(host_cores())
    o = oracle_hierarchy(dict(WORKLOAD))
    warm = min(args.warmup, 1)
    for _ in range(warm):
        o.step()
    timed = min(args.steps, REFERENCE_MAX_STEPS)
    n, dt, pu = time_oracle_steps(o, 0.0, min_steps=timed, max_steps=timed)
    v = pu / dt
    nlev = WORKLOAD["nl0"] + 1
    sample = ("%d whole coarse steps of the %d-level %dx%d hierarchy per timed region, after %d untimed"
              % (n, nlev, WORKLOAD["nrtotal"], WORKLOAD["nztotal"], warm))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": n, "warmup": args.warmup, "ms_per_step": 1000.0 * dt / n,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (analytic Schwarzschild initial data)", "config": config_dict(args),
            "timed_seconds": dt, "warmup_steps_run": warm,
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if n != args.steps:
        line["steps_note"] = "timed %d of the %d requested coarse steps (cap %d)" % (n, args.steps,
                                                                                  REFERENCE_MAX_STEPS)
    print(json.dumps(line))


def run_gpu(args):
    world, rank, local, pg = dist_setup(args)
    import torch
    torch.cuda.set_device(local)
    from ollin.gpu import Evolution, load, field_id
    from ollin.params import params_from_dict
    L = load()
    p = params_from_dict(WORKLOAD)
    e = Evolution(p)
    e.initial_data()
    e.initialize()
    stream = torch.cuda.ExternalStream(e.stream())
    for _ in range(args.warmup):
        e.step()
    torch.cuda.synchronize()
    # ---- device-resident throughput -------------------------------------
    e.kernel_timing(True)
    launches0 = e.launch_count()
    pu0 = e.point_updates()
    sampler = ClockSampler(local)
    sampler.start()
    barrier(pg)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        e.step()
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(pg)
    clocks = sampler.stop()
    ms_local = ev0.elapsed_time(ev1)
    launches = e.launch_count() - launches0
    pu = e.point_updates() - pu0
    rhs_ms, rhs_n, rhs_pts = e.kernel_stats()
    e.kernel_timing(False)
    ms = max_over_ranks(pg, ms_local)
    pu_all = sum_over_ranks(pg, pu)
    value = pu_all / (ms * 1e-3)
    # ---- end to end through the C ABI with host-resident state -----------
    names = ["alpha", "chi", "A", "B", "H", "C", "trK", "KTA", "KTB", "KTC", "Delta_r", "Delta_z",
             "beta_r", "beta_z", "dtbeta_r", "dtbeta_z"]
    host = {}
    for lev in e.levels():
        d = e.desc(lev)
        for nm in names:
            host[(lev, nm)] = torch.empty((d.nz + d.ghost, d.nr + d.ghost), dtype=torch.float64).pin_memory()
            e.L.ollin_gpu_download(e.h, lev, field_id(nm), ctypes.c_void_p(host[(lev, nm)].data_ptr()),
                                   d.nr + d.ghost)
    bytes_per_dir = sum(t.numel() * 8 for t in host.values())
    # the whole state in one ollin_gpu_upload_many / download_many call per
    # direction and step: every array of the reference's layout, one
    # synchronisation each way
    nq = len(host)
    q_lev = (ctypes.c_int * nq)(*[lev for (lev, _) in host])
    q_fld = (ctypes.c_int * nq)(*[field_id(nm) for (_, nm) in host])
    q_ptr = (ctypes.c_void_p * nq)(*[t.data_ptr() for t in host.values()])
    q_ld = (ctypes.c_int * nq)(*[t.shape[1] for t in host.values()])
    e2e_steps = max(2, args.steps // 2)
    barrier(pg)
    t0 = time.perf_counter()
    pu1 = e.point_updates()
    for _ in range(e2e_steps):
        assert e.L.ollin_gpu_upload_many(e.h, nq, q_lev, q_fld, q_ptr, q_ld) == 0
        e.step()
        assert e.L.ollin_gpu_download_many(e.h, nq, q_lev, q_fld, q_ptr, q_ld) == 0
    torch.cuda.synchronize()
    dt_e2e = max_over_ranks(pg, time.perf_counter() - t0)
    e2e_value = sum_over_ranks(pg, e.point_updates() - pu1) / dt_e2e
    # ---- roofline of the right-hand-side kernel --------------------------
    # algorithmic bytes per launch = 136 F / 4 bytes per point-stage x points
    avg_launch_s = rhs_ms * 1e-3 / max(rhs_n, 1)
    alg_bytes_per_launch = (ALG_BYTES_PER_PU / 4.0) * rhs_pts / max(rhs_n, 1)
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    hbm_peak, peak_note = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        with open(peaks_path) as f:
            hbm_peak = float(json.load(f).get("hbm_gbs", hbm_peak))
            peak_note = "measured"
    achieved = alg_bytes_per_launch / avg_launch_s / 1e9
    dfma_rate = L.ollin_gpu_fp64_rate()
    traffic = None
    prof = os.path.join(ROOT, "profiles", "rhs_kernel_traffic.json")
    if os.path.exists(prof):
        with open(prof) as f:
            pj = json.load(f)
        traffic = pj.get("dram_bytes_per_point_stage", None)
        if traffic is not None:
            traffic = traffic * rhs_pts / max(rhs_n, 1)
        dp_per_pt = pj.get("dp_instructions_per_point_stage", None)
    else:
        dp_per_pt = None
    fp64 = {"peak_dfma_per_s": dfma_rate, "peak_note": "measured live (DFMA chains on all SMs)"}
    if dp_per_pt:
        achieved_dp = dp_per_pt * rhs_pts / (rhs_ms * 1e-3)
        fp64.update({"dp_instructions_per_point_stage": dp_per_pt, "achieved_dp_per_s": achieved_dp,
                     "frac": achieved_dp / dfma_rate})
    e.close()
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (analytic Schwarzschild initial data)", "config": config_dict(args),
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": bytes_per_dir,
                        "d2h_bytes_per_step": bytes_per_dir, "steps": e2e_steps},
                "gpu_launches": launches,
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                             "frac": achieved / hbm_peak, "traffic": traffic,
                             "kernel": "rhs_kernel (fused RHS + RK stage)", "peak_source": peak_note,
                             "binding_ceiling": "fp64", "fp64": fp64,
                             "rhs_launches": rhs_n, "rhs_avg_launch_ms": avg_launch_s * 1e3,
                             "rhs_share_of_step": (rhs_ms / max(ms_local, 1e-9))},
                "clocks": clocks}
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(seconds=args.cpu_seconds)
        if not args.no_elliptic:
            line["elliptic"] = elliptic_precision()
        if not args.no_batch:
            line["batch"] = batch_throughput()
        if not args.no_serve:
            line["serving"] = serving()
            line["plain_small"] = plain_small()
        print(json.dumps(line))
    if pg is not None:
        pg.destroy_process_group()


def elliptic_precision():
    """The precision pattern of the Brill-wave configuration (Holz data,
    sigma = 1, dr0 = 0.04, 4 box-in-box levels of 1024^2) for a0 = 1, 4, 5:
      * the conformal factor by the mixed solver (FP32 multigrid corrections,
        FP64 residual refinement) and by the all-FP64 solve of the same
        system (ELL_solver = fp64mg: FP64 multigrid corrections), timed
        through the C ABI; the error is max |chi_mixed - chi_fp64| over all
        levels;
      * after one coarse step (K_ij no longer zero), the maximal-slicing
        lapse by both, and max |alpha_mixed - alpha_fp64|;
    and on one 256^2 level, where the reference's FP64 SOR converges, the
    mixed and FP64 multigrid solves against that SOR."""
    import numpy as np
    from ollin.gpu import Evolution
    from ollin.params import params_from_dict
    base = dict(eqsym=1, order="four", integrator="rk4", ilapse="one", idata="BrillWave", brill_a0=1.0,
                brill_sr0=1.0, brill_sz0=1.0, dr0=0.04, dz0=0.04, ell_epsilon=1e-12)
    c3 = dict(nrtotal=1024, nztotal=1024, nl0=3)
    one = dict(nrtotal=256, nztotal=256, nl0=0)

    def solve(cfg):
        e = Evolution(params_from_dict(dict(base, **cfg)))
        t = time.perf_counter()
        e.initial_data()
        dt = time.perf_counter() - t
        chi = [e.download(lev, "chi") for lev in e.levels()]
        stats = e.ell_stats()
        e.close()
        return dt, stats, chi

    def maximal(cfg):
        """Brill data, the maximal lapse, one coarse step, then the
        maximal-slicing lapse again (maximalslicing.f90), every solve by the
        solver of cfg: the whole precision pattern against the all-FP64 one."""
        e = Evolution(params_from_dict(dict(base, maximalevery=1, slicing="1+log", gauge_f=2.0, **cfg)))
        e.initial_data()
        e.initialize()
        e.maximal_slicing()
        e.step()
        t = time.perf_counter()
        e.maximal_slicing()
        dt = time.perf_counter() - t
        alpha = [e.download(lev, "alpha") for lev in e.levels()]
        stats = e.ell_stats()
        e.close()
        return dt, stats, alpha

    def maxdiff(x, y):
        return float(max(np.max(np.abs(a - b)) for a, b in zip(x, y)))

    solve(dict(nrtotal=64, nztotal=64, nl0=0, ell_solver="mixed"))  # warm-up
    out = {"workload": "Holz Brill wave, sigma = 1, dr0 = 0.04, 4 levels of 1024x1024; mixed solver (FP32 multigrid "
                       "corrections, FP64 residual) against the FP64 solve of the same system (FP64 multigrid "
                       "corrections), each to an RMS residual of 1e-12 or its FP64 floor",
           "cases": []}
    for a0 in (1.0, 4.0, 5.0):
        cfg = dict(c3, brill_a0=a0)
        tm, sm, chim = solve(dict(cfg, ell_solver="mixed"))
        tf, sf, chif = solve(dict(cfg, ell_solver="fp64mg"))
        mtm, msm, am = maximal(dict(cfg, ell_solver="mixed"))
        mtf, msf, af = maximal(dict(cfg, ell_solver="fp64mg"))
        out["cases"].append({
            "a0": a0,
            "psi": {"mixed_seconds": tm, "fp64_seconds": tf, "mixed_refinements_level0": sm[0],
                    "mixed_vcycles_level0": sm[1], "mixed_rms_residual": sm[2], "fp64_rms_residual": sf[2],
                    "max_abs_chi_error": maxdiff(chim, chif)},
            "maximal_lapse": {"mixed_seconds": mtm, "fp64_seconds": mtf, "mixed_rms_residual": msm[2],
                              "fp64_rms_residual": msf[2], "max_abs_alpha_error": maxdiff(am, af),
                              "min_alpha": float(min(a.min() for a in am))}})
    t_mx, _, chi_mx = solve(dict(one, ell_solver="mixed"))
    t_64, _, chi_64 = solve(dict(one, ell_solver="fp64mg"))
    t_sor, st_sor, chi_sor = solve(dict(one, ell_solver="sor", ell_epsilon=1e-8))
    out["vs_fp64_sor_256"] = {"mixed_seconds": t_mx, "fp64mg_seconds": t_64, "sor_seconds": t_sor,
                              "sor_iterations": st_sor[0], "mixed_max_abs_chi_diff": maxdiff(chi_mx, chi_sor),
                              "fp64mg_max_abs_chi_diff": maxdiff(chi_64, chi_sor)}
    out["max_abs_error"] = max(max(c["psi"]["max_abs_chi_error"], c["maximal_lapse"]["max_abs_alpha_error"])
                               for c in out["cases"])
    return out


def ceiling_rate(cfg, size=1024, levels=3, steps=2):
    """Point-updates/s of one large evolution of ``cfg``'s physics alone
    (size^2 x levels, one untimed coarse step, then ``steps`` timed): a grid
    that large fills the device, so its rate is the ceiling any batch of that
    physics can reach."""
    from ollin.gpu import Evolution
    from ollin.params import params_from_dict
    c = dict(cfg, nrtotal=size, nztotal=size, nl0=levels - 1, dr0=cfg["dr0"] * cfg["nrtotal"] / size,
             dz0=cfg["dz0"] * cfg["nztotal"] / size)
    e = Evolution(params_from_dict(c))
    e.initial_data()
    e.initialize()
    e.step()
    p0 = e.point_updates()
    t = time.perf_counter()
    for _ in range(steps):
        e.step()
    dt = time.perf_counter() - t
    rate = (e.point_updates() - p0) / dt
    e.close()
    return rate


def c4_configs(n, seed):
    """The batching configuration's seeded mix: massless scalar-field shells
    phi = a exp(-(r - 5)^2) (r0 = 5, s = 1), a log-uniform in [0.01, 0.1],
    grids of 64^2 to 512^2 per level (multiples of 64) with 2-5 levels, a
    16 M square coarse domain (dr0 = 16/N), elliptic data by the mixed solver."""
    import numpy as np
    rng = np.random.default_rng(seed)
    cfgs = []
    for _ in range(n):
        size = int(64 * rng.integers(1, 9))
        cfgs.append(dict(nrtotal=size, nztotal=size, nl0=int(rng.integers(1, 5)), dr0=16.0 / size, dz0=16.0 / size,
                         eqsym=1, order="four", integrator="rk4", dtfac=0.25, boundtype="radiative",
                         idata="scalarpulse", mattertype="scalar", scalarpotential="none", scalarpulse_type="shell",
                         scalar_a0=float(np.exp(rng.uniform(np.log(0.01), np.log(0.1)))), scalar_r0=5.0,
                         scalar_sr0=1.0, scalar_sz0=1.0, ilapse="one", slicing="1+log", gauge_f=2.0,
                         geodiss=0.02, scalardiss=0.02, ell_solver="mixed", ell_epsilon=1e-12))
    return cfgs


def batch_throughput(n=256, steps=1, seed=7):
    """The batching configuration (256 seeded scalar-field shells, 64^2-512^2
    per level, 2-5 levels), t_end cut to ``steps`` coarse steps per run:
      * plain: each evolution alone, set up, then its steps timed by
        themselves (host wall clock, launches included);
      * batched: all n set up, then every coarse step of all of them queued
        together (ollin_gpu_coarse_step_many, one stream each).
    The bound: batching cannot beat the FP64 ceiling of the device, the rate
    R of the large single instance; plain run i at rate r_i leaves the rest
    of the device idle, so batched/plain <= sum(t_i) / (sum(pu_i) / R)."""
    import numpy as np
    from ollin.gpu import SCHEDULES, Evolution, step_auto, step_fused, step_many
    from ollin.params import params_from_dict
    cfgs = c4_configs(n, seed)

    def setup(c):
        e = Evolution(params_from_dict(c))
        e.initial_data()
        e.initialize()
        return e

    w = setup(cfgs[0])  # warm-up: kernel loading
    w.step()
    w.close()
    t_plain, pu_plain, digest_plain = [], [], []
    t_setup = time.perf_counter()
    for c in cfgs:
        e = setup(c)
        p0 = e.point_updates()
        t = time.perf_counter()
        for _ in range(steps):
            e.step()
        t_plain.append(time.perf_counter() - t)
        pu_plain.append(e.point_updates() - p0)
        digest_plain.append(e.norms(0, "trK"))
        e.close()
    t_setup = time.perf_counter() - t_setup - sum(t_plain)
    es = [setup(c) for c in cfgs]
    p0 = sum(e.point_updates() for e in es)
    t = time.perf_counter()
    for _ in range(steps):
        step_many(es)
    t_bat = time.perf_counter() - t
    pu_bat = sum(e.point_updates() for e in es) - p0
    same = all(np.array_equal(a, e.norms(0, "trK")) for a, e in zip(digest_plain, es))
    # the same evolutions' next steps with every kernel fused over all of them
    step_fused(es)  # warm-up: the fused launch tables
    p0 = sum(e.point_updates() for e in es)
    t = time.perf_counter()
    for _ in range(steps):
        step_fused(es)
    t_fused = time.perf_counter() - t
    pu_fused = sum(e.point_updates() for e in es) - p0
    # the schedule autotuner on the same batch: two live steps under each
    # schedule, then its choice, timed
    for _ in range(6):
        step_auto(es)
    p0 = sum(e.point_updates() for e in es)
    t = time.perf_counter()
    for _ in range(steps):
        _, sched = step_auto(es)
    t_auto = time.perf_counter() - t
    pu_auto = sum(e.point_updates() for e in es) - p0
    for e in es:
        e.close()
    t_plain = np.array(t_plain)
    pu = float(sum(pu_plain))
    rate_plain = np.array(pu_plain) / t_plain
    # the ceiling of this physics (scalar field, no shift): one large shell
    # evolution alone (1024^2 x 3 levels) fills the device
    ceiling = ceiling_rate(cfgs[0])
    bound = float(t_plain.sum()) / (pu / ceiling)
    return {"workload": "%d massless scalar shells (a log-uniform in [0.01, 0.1], seeded), 64^2-512^2 per level x 2-5 "
                        "levels, elliptic data by the mixed solver; t_end cut to %d coarse step(s) per run"
                        % (n, steps),
            "plain_runs_per_s": n / float(t_plain.sum()), "batched_runs_per_s": n / t_bat,
            "speedup": float(t_plain.sum()) / t_bat,
            "plain_point_updates_per_s": pu / float(t_plain.sum()), "batched_point_updates_per_s": pu_bat / t_bat,
            "fused_point_updates_per_s": pu_fused / t_fused,
            "fused_speedup": float(t_plain.sum()) / t_fused * (pu_fused / pu),
            "fused_runs_per_s": n / t_fused * (pu_fused / pu),
            "autotuned_schedule": SCHEDULES[sched], "autotuned_point_updates_per_s": pu_auto / t_auto,
            "autotuned_speedup": float(t_plain.sum()) / t_auto * (pu_auto / pu),
            "plain_run_seconds_p50": float(np.percentile(t_plain, 50)),
            "plain_run_seconds_p99": float(np.percentile(t_plain, 99)),
            "plain_rate_p50": float(np.percentile(rate_plain, 50)),
            "setup_seconds_per_run": t_setup / n,
            "ceiling_point_updates_per_s": ceiling,
            "ceiling_note": "one scalar shell of 1024^2 x 3 levels stepped alone",
            "speedup_bound_from_plain_occupancy": bound,
            "identical_results": bool(same)}


def plain_small():
    """The plain-method small configuration end to end on the device: the
    Schwarzschild puncture on 3 levels of 64^2 (finest dr 0.05), RK4, evolved
    to t = 10M (200 coarse steps) through ollin_gpu_coarse_step, with direct
    launches and with each step launched as a captured graph (the same
    kernels and arguments: the final norms agree bit for bit)."""
    import numpy as np
    from ollin.gpu import Evolution
    from ollin.params import params_from_dict
    cfg = dict(nrtotal=64, nztotal=64, nl0=2, dr0=0.2, dz0=0.2, eqsym=1, idata="schwarzschild", bh1mass=1.0,
               ilapse="psiminus2", slicing="1+log", gauge_f=2.0, shift="none", integrator="rk4", order="four",
               geodiss=0.02, dtfac=0.25, boundtype="radiative")
    out, norms = {}, []
    for graphs in (False, True):
        e = Evolution(params_from_dict(cfg))
        e.initial_data()
        e.initialize()
        e.step_graphs(graphs)
        for _ in range(3):  # warm-up: first steps and kernel loading
            e.step()
        t = time.perf_counter()
        for _ in range(197):
            e.step()
        dt = time.perf_counter() - t
        out["graphs" if graphs else "direct"] = {"seconds_for_197_steps": dt, "ms_per_coarse_step": 1e3 * dt / 197}
        norms.append(np.array([e.norms(lev, "alpha") for lev in e.levels()]))
        e.close()
    out["workload"] = "Schwarzschild puncture, 3 levels of 64^2, RK4 to t = 10M (3 warm-up + 197 timed coarse steps)"
    out["identical_results"] = bool(np.array_equal(norms[0], norms[1]))
    return out


def serving_requests(rng, n):
    """A seeded mix of the serving configuration's request types: Schwarzschild
    punctures (the plain-method configuration's physics), Brill waves
    (A in {1, 4, 5}) and massless scalar shells (a log-uniform in
    [0.01, 0.1]), both with elliptic data by the mixed solver; grids of 64^2
    to 1024^2 per level with 2-6 levels; t_end uniform in [5, 40]."""
    import numpy as np
    common = dict(eqsym=1, order="four", integrator="rk4", dtfac=0.25, boundtype="radiative", slicing="1+log",
                  gauge_f=2.0, geodiss=0.02, ell_solver="mixed", ell_epsilon=1e-12)
    out = []
    for _ in range(n):
        kind = int(rng.integers(0, 3))
        size = int(rng.choice([64, 128, 256, 512, 1024]))
        nl0 = int(rng.integers(1, 6))
        t_end = float(rng.uniform(5.0, 40.0))
        if kind == 0:
            cfg = dict(common, nrtotal=size, nztotal=size, nl0=nl0, dr0=12.8 / size, dz0=12.8 / size,
                       idata="schwarzschild", bh1mass=1.0, ilapse="psiminus2")
        elif kind == 1:
            cfg = dict(common, nrtotal=size, nztotal=size, nl0=nl0, dr0=40.96 / size, dz0=40.96 / size,
                       idata="BrillWave", brill_a0=float(rng.choice([1.0, 4.0, 5.0])), brill_sr0=1.0, brill_sz0=1.0,
                       ilapse="one")
        else:
            cfg = dict(common, nrtotal=size, nztotal=size, nl0=nl0, dr0=16.0 / size, dz0=16.0 / size,
                       idata="scalarpulse", mattertype="scalar", scalarpotential="none", scalarpulse_type="shell",
                       scalar_a0=float(np.exp(rng.uniform(np.log(0.01), np.log(0.1)))), scalar_r0=5.0,
                       scalar_sr0=1.0, scalar_sz0=1.0, ilapse="one", scalardiss=0.02)
        out.append((kind, cfg, t_end))
    return out


def request_point_updates(cfg, t_end):
    """Point-updates of a request evolved to t_end (RK4 steps of every level)."""
    import numpy as np
    dt0 = cfg["dtfac"] * min(cfg["dr0"], cfg["dz0"])
    steps = max(1, int(np.ceil(t_end / dt0 - 1e-9)))
    return steps * cfg["nrtotal"] * cfg["nztotal"] * (2 ** (cfg["nl0"] + 1) - 1)


def serving(n=24, chain=4, seed=11, budget=150e9, load=0.8, work=1.5e9):
    """The serving pattern through the request loop (ollin_server_*) on the
    serving configuration's mix, coarse steps launched as captured graphs
    unless stated.  Every t_end is multiplied by one factor chosen so that the
    mix totals ``work`` point-updates (stated in the result):
      * plain: the requests one at a time (max_active = 1), all queued at 0;
      * batched: the same requests with up to 64 running together (and again
        with direct launches);
      * served: Poisson arrivals (seeded) at ``load`` x the batched rate, plus a
        bisection chain on the shell amplitude whose next request is submitted
        when the previous one finishes (collapse = smallest lapse < 0.05).
    Latency is finish minus submission, host wall clock.  Every request's
    norms must agree between the plain and the served runs.  The bound on
    batched/plain is the plain runs' step time over the time the fastest
    request's rate (a large grid alone fills the device) needs for their
    point-updates."""
    import numpy as np
    from ollin.gpu import Server
    from ollin.params import params_from_dict
    rng = np.random.default_rng(seed)
    raw = serving_requests(rng, n)
    full = sum(request_point_updates(c, t) for _, c, t in raw)
    scale = work / full
    reqs = [(k, c, t * scale) for k, c, t in raw]

    def closed(max_active, graphs=True, reqs=reqs, fused=False):
        s = Server(budget, max_active=max_active, graphs=graphs, fused=fused)
        for k, (_, cfg, t_end) in enumerate(reqs):
            s.submit(k, params_from_dict(cfg), t_end, 0.05 if cfg.get("mattertype") == "scalar" else 0.0)
        t = time.perf_counter()
        res = s.drain()
        dt = time.perf_counter() - t
        s.close()
        return dt, {r.id: r for r in res}

    t_plain, plain = closed(1)
    t_bat, bat = closed(64)
    t_direct, _ = closed(64, graphs=False)
    t_fus, fus = closed(64, fused=True)
    pu = sum(r.point_updates for r in plain.values())
    step_time = sum(plain[k].t_done - plain[k].t_ready for k in range(n))
    # the ceiling of each request type: one large evolution of its physics
    # alone (1024^2 x 3 levels); batched time >= sum over requests of their
    # point-updates at their type's ceiling
    ceil = {kd: ceiling_rate(next(c for k2, c, _ in reqs if k2 == kd)) for kd in sorted(set(k for k, _, _ in reqs))}
    t_min = sum(plain[k].point_updates / ceil[reqs[k][0]] for k in range(n))
    bound = step_time / t_min
    # the small end of the mix alone: 32 punctures of 3 levels of 64^2 (the
    # plain-method configuration's grids), where one evolution fills a few
    # SMs and the plain path is bound by kernel latency
    small_cfg = dict(next(c for kd, c, _ in reqs if kd == 0), nrtotal=64, nztotal=64, nl0=2, dr0=0.2, dz0=0.2)
    small = [(0, small_cfg, 2.0)] * 32
    t_sp, sp = closed(1, reqs=small)
    t_sb, _ = closed(64, reqs=small)
    t_sd, _ = closed(64, graphs=False, reqs=small)
    t_sf, sf = closed(64, reqs=small, fused=True)
    pu_s = sum(r.point_updates for r in sp.values())
    rate = load * n / t_bat
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=n))
    chain_cfg = dict(next(c for kd, c, _ in reqs if kd == 2))
    chain_t = float(np.median([t for kd, _, t in reqs if kd == 2]))
    lo, hi = 0.01, 0.1
    s = Server(budget, max_active=64)
    res, nxt, t0, pending_chain, chain_done = {}, 0, time.perf_counter(), None, 0
    peak_run = 0
    while len(res) < n + chain:
        now = time.perf_counter() - t0
        while nxt < n and arrivals[nxt] <= now:
            _, cfg, t_end = reqs[nxt]
            s.submit(nxt, params_from_dict(cfg), t_end, 0.05 if cfg.get("mattertype") == "scalar" else 0.0)
            nxt += 1
        if pending_chain is None and chain_done < chain:
            a = float(np.sqrt(lo * hi))
            pending_chain = (1000 + chain_done, a)
            s.submit(1000 + chain_done, params_from_dict(dict(chain_cfg, scalar_a0=a)), chain_t, 0.05)
        a_run, _ = s.tick()
        peak_run = max(peak_run, a_run)
        for r in s.poll():
            res[r.id] = r
            if pending_chain and r.id == pending_chain[0]:
                if r.collapsed:
                    hi = pending_chain[1]
                else:
                    lo = pending_chain[1]
                pending_chain, chain_done = None, chain_done + 1
        if a_run == 0 and nxt < n and pending_chain is None and chain_done >= chain:
            time.sleep(max(0.0, min(0.01, arrivals[nxt] - (time.perf_counter() - t0))))
    t_served = time.perf_counter() - t0
    used, peak = s.usage()
    s.close()
    lat = np.array([res[k].t_done - res[k].t_submit for k in range(n)])
    svc = np.array([plain[k].t_done - plain[k].t_admit for k in range(n)])
    setup = np.array([plain[k].t_ready - plain[k].t_admit for k in range(n)])
    same = all(np.array_equal(plain[k].norms(), res[k].norms()) and plain[k].steps == res[k].steps
               and np.array_equal(plain[k].norms(), fus[k].norms()) for k in range(n))
    same = same and all(np.array_equal(sp[k].norms(), sf[k].norms()) for k in range(32))
    ok = all(r.status == 0 for r in list(res.values()) + list(plain.values()) + list(bat.values()))
    kinds = [kd for kd, _, _ in reqs]
    return {"workload": "%d requests (%d punctures, %d Brill waves, %d scalar shells), 64^2-1024^2 x 2-6 levels "
                        "(seeded), t_end in [5, 40] x %.2e (the mix scaled to %.2g point-updates); + a %d-step "
                        "bisection chain on the shell amplitude" % (n, kinds.count(0), kinds.count(1), kinds.count(2),
                                                                     scale, work, chain),
            "t_end_scale": scale, "budget_bytes": budget, "peak_reserved_bytes": peak, "most_running": peak_run,
            "plain_runs_per_s": n / t_plain, "batched_runs_per_s": n / t_bat, "batched_vs_plain": t_plain / t_bat,
            "batched_direct_launch_runs_per_s": n / t_direct,
            "fused_ticks_runs_per_s": n / t_fus, "fused_ticks_vs_plain": t_plain / t_fus,
            "plain_point_updates_per_s": pu / t_plain, "batched_point_updates_per_s": pu / t_bat,
            "ceiling_point_updates_per_s": {["puncture", "brill", "shell"][k]: v for k, v in ceil.items()},
            "ceiling_note": "one evolution of each request type's physics, 1024^2 x 3 levels, stepped alone",
            "speedup_bound_from_plain_occupancy": bound,
            "small_grids": {"workload": "32 Schwarzschild punctures, 3 levels of 64^2, t_end 2 (40 coarse steps)",
                            "plain_runs_per_s": 32 / t_sp, "batched_runs_per_s": 32 / t_sb,
                            "batched_vs_plain": t_sp / t_sb, "batched_direct_launch_runs_per_s": 32 / t_sd,
                            "fused_ticks_runs_per_s": 32 / t_sf, "fused_ticks_vs_plain": t_sp / t_sf,
                            "batched_point_updates_per_s": pu_s / t_sb},
            "served": {"arrival_rate_per_s": rate, "runs_per_s": (n + chain) / t_served,
                       "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99))},
            "plain_service": {"p50_s": float(np.percentile(svc, 50)), "p99_s": float(np.percentile(svc, 99)),
                              "setup_share": float(setup.sum() / svc.sum())},
            "bisection_bracket": [lo, hi], "all_ok": bool(ok), "identical_results": bool(same)}


OP_NAMES = ["DFMA", "DADD", "DMUL", "DDIV", "sqrt", "cbrt", "exp", "log", "FFMA (FP32)"]


def probe(args):
    """Stand-alone measurements behind the committed profile summaries:
    ``fp64`` prints the operation-rate table (ollin_gpu_op_rate);
    ``norms`` runs ollin_gpu_norms on the lapse of one 1024x1024
    Schwarzschild level five times (the launches an ncu capture of
    norms_partial_kernel selects from); ``rhs-shapes`` rebuilds rhs.cu for
    several launch shapes and register budgets (threads per block, blocks per
    SM of __launch_bounds__), links each with the other objects and times the
    6-level step with each library."""
    if args.probe == "rhs-shapes":
        from ollin import build as B
        B.build()
        objs = [os.path.join(B.BUILD, os.path.splitext(x)[0] + ".o") for x in B.SOURCES if x != "rhs.cu"]
        out = {}
        shapes = [(128, 3), (64, 6), (64, 5), (96, 4), (128, 2), (32, 12)]

        def make(shape):  # one library per launch shape, compiled side by side
            thr, mb = shape
            obj = os.path.join(B.BUILD, "rhs_%d_%d.o" % shape)
            lib = os.path.join(B.BUILD, "libollin_gpu_rhs_%d_%d.so" % shape)
            subprocess.run([B.nvcc()] + B.ARCH + B.COMMON + ["-DOLLIN_RHS_THREADS=%d" % thr,
                            "-DOLLIN_RHS_MINBLOCKS=%d" % mb, "-c", os.path.join(B.CSRC, "rhs.cu"), "-o", obj],
                           check=True)
            subprocess.run([B.nvcc()] + B.ARCH + ["-shared", "-o", lib] + objs + [obj, "-lcudart"], check=True)
            return lib

        import concurrent.futures
        with concurrent.futures.ThreadPoolExecutor(max_workers=len(shapes)) as ex:
            libs = dict(zip(shapes, ex.map(make, shapes)))
        for thr, mb in shapes:
            tag = "%d_%d" % (thr, mb)
            lib = libs[(thr, mb)]
            r = subprocess.run([sys.executable, os.path.abspath(__file__), "--steps", "6", "--warmup", "3",
                                "--no-elliptic", "--no-batch", "--no-serve", "--no-cpu-baseline"],
                               env=dict(os.environ, OLLIN_GPU_LIB=lib), capture_output=True, text=True)
            if r.returncode != 0:
                out[tag] = {"error": r.stderr[-400:]}
                continue
            d = json.loads(r.stdout.strip().splitlines()[-1])
            out[tag] = {"threads": thr, "min_blocks": mb, "ms_per_step": d["ms_per_step"],
                        "rhs_avg_launch_ms": d["roofline"]["rhs_avg_launch_ms"], "clocks": d["clocks"]}
        print(json.dumps({"probe": "rhs-shapes", "shapes": out}))
        return
    import torch
    from ollin.gpu import Evolution, load
    from ollin.params import params_from_dict
    L = load()
    L.ollin_gpu_op_rate.argtypes = [ctypes.c_int]
    L.ollin_gpu_op_rate.restype = ctypes.c_double
    if args.probe == "fp64":
        rates = {nm: L.ollin_gpu_op_rate(k) for k, nm in enumerate(OP_NAMES)}
        dfma = rates["DFMA"]
        print(json.dumps({"probe": "fp64", "ops_per_s": rates,
                          "cost_vs_dfma": {nm: dfma / v if v > 0 else None for nm, v in rates.items()}}))
    else:
        e = Evolution(params_from_dict(dict(WORKLOAD, nl0=0, nrtotal=1024, nztotal=1024, shift="none")))
        e.initial_data()
        e.initialize()
        out = [e.norms(0, "alpha") for _ in range(5)]
        torch.cuda.synchronize()
        e.close()
        print(json.dumps({"probe": "norms", "alpha_norms": [float(x) for x in out[-1]]}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-elliptic", action="store_true", help="skip the mixed-precision elliptic measurement")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched small-evolution measurement")
    ap.add_argument("--no-serve", action="store_true", help="skip the request-loop measurement")
    ap.add_argument("--levels", type=int, default=6, help="box-in-box levels (profiling a smaller case)")
    ap.add_argument("--size", type=int, default=512, help="points per level per direction")
    ap.add_argument("--probe", choices=["fp64", "norms", "rhs-shapes"], default=None,
                    help="print a stand-alone measurement (operation rates, or the norms launches) and exit")
    args = ap.parse_args()
    WORKLOAD.update(nl0=args.levels - 1, nrtotal=args.size, nztotal=args.size)
    if args.probe:
        probe(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
