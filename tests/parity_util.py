"""Shared helpers for the GPU-versus-oracle parity tests."""
import numpy as np

from ollin.params import params_from_dict

C1 = dict(nrtotal=64, nztotal=64, nl0=2, dr0=0.2, dz0=0.2, eqsym=1, idata="schwarzschild",
          bh1mass=1.0, ilapse="psiminus2", slicing="1+log", gauge_f=2.0, shift="none",
          integrator="rk4", order="four", geodiss=0.02, dtfac=0.25, boundtype="radiative")

BASE_FIELDS = ["alpha", "chi", "A", "B", "H", "C", "trK", "KTA", "KTB", "KTC", "Delta_r", "Delta_z",
               "KTH", "lambda", "Alambda", "phi"]
SHIFT_FIELDS = ["beta_r", "beta_z", "dtbeta_r", "dtbeta_z"]
SCALAR_FIELDS = ["scalar_phi", "scalar_xi_r", "scalar_xi_z", "scalar_pi"]

# FP64 parity bound between the GPU path and the oracle: max |gpu - oracle|
# over a level's points (ghosts included), divided by max |oracle| of that
# field on that level.  FMA contraction and reordered arithmetic in the fused
# GPU kernel make the results differ at the 1e-15 level per step.
REL_TOL = 1e-10

# Auxiliary (non-evolved) quantities recomputed from the state each stage:
# lambda = (A - H)/r^2 and Alambda = (KTA - KTH)/r^2 subtract two O(1) numbers
# that agree to ~1e-8 next to the axis and divide by r^2 ~ 1e-4 on the finest
# levels, so last-bit differences in A and H are amplified ~1e6 there.
AUX_FIELDS = ("lambda", "Alambda", "KTH")
AUX_TOL = 1e-8


def tol_for(name):
    return AUX_TOL if name in AUX_FIELDS else REL_TOL


def field_list(cfg):
    names = list(BASE_FIELDS)
    if cfg.get("shift", "none") != "none":
        names += SHIFT_FIELDS
    if str(cfg.get("shift", "none")).startswith("Gammadrivershock"):
        names += ["fdriver"]
    if cfg.get("mattertype") == "scalar":
        names += SCALAR_FIELDS
    return names


def rel_diff(a, b):
    scale = max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(a - b))) / scale


# Pointwise relative difference: |gpu - oracle| / max(|oracle|, floor), with
# the floor POINT_FLOOR x max|oracle| of that field on that level, so that
# points where a field crosses zero (C, KTC, Delta_z, beta_z are zero on the
# axis and the equator and tiny far out) are measured against a millionth of
# the field's scale instead of their own vanishing value.
POINT_FLOOR = 1e-6


def point_rel_diff(a, b, floor=POINT_FLOOR):
    scale = max(float(np.max(np.abs(b))), 1e-300)
    den = np.maximum(np.abs(b), floor * scale)
    return float(np.max(np.abs(a - b) / den))


def scalar_pulse(r, z, a0=0.05):
    ph = a0 * np.exp(-(r ** 2 + z ** 2))
    return ph, -2.0 * r * ph, -2.0 * z * ph, np.zeros_like(ph)


def coords(nr, nz, g, dr, dz):
    i = np.arange(1 - g, nr + 1)
    j = np.arange(1 - g, nz + 1)
    r = ((i.astype(np.float64)) - 0.5) * dr
    z = ((j.astype(np.float64)) - 0.5) * dz
    return np.meshgrid(r, z, indexing="ij")


def params(cfg):
    return params_from_dict(cfg)
