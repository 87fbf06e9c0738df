"""Self-convergence runs shared by the CPU (oracle) and GPU convergence tests:
smooth data on one level (no refinement interfaces), three resolutions
h, h/2, h/4 evolved to the same time, and the value at the origin from the
reference's bicubic interpolation (save0Ddata.f90:370-374, 4th-order
accurate).  The factor (Q(h) - Q(h/2)) / (Q(h/2) - Q(h/4)) is 2^p."""
import numpy as np

from parity_util import params, scalar_pulse

RESOLUTIONS = ((20, 0.4), (40, 0.2), (80, 0.1))
T_END = 0.8


def config(n, h, matter, order="four"):
    cfg = dict(nrtotal=n, nztotal=n, nl0=0, dr0=h, dz0=h, eqsym=1, idata="minkowski", ilapse="one",
               slicing="1+log", gauge_f=2.0, shift="none", integrator="rk4", order=order, geodiss=0.02,
               dtfac=0.25, boundtype="radiative")
    if matter:
        cfg.update(mattertype="scalar", scalardiss=0.02)
    return cfg


def prepare(sim, matter, get, put):
    """Gauge pulse in the lapse (vacuum) or a Gaussian scalar pulse."""
    r, z = get("r"), get("z")
    if matter:
        for nm, v in zip(["scalar_phi", "scalar_xi_r", "scalar_xi_z", "scalar_pi"], scalar_pulse(r, z, a0=0.05)):
            put(nm, v)
    else:
        put("alpha", 1.0 + 0.05 * np.exp(-(r ** 2 + z ** 2)))


def factors(values):
    v = np.asarray(values)
    return (v[0] - v[1]) / (v[1] - v[2])
