"""The evolution parameters as the reference's ``param`` module holds them.

``Params`` is the ctypes mirror of ``ollin_params`` (include/ollin_gpu.h);
``default_params`` fills the defaults of src/base/param.f90 and
``params_from_par`` applies a reference par file (``name = value`` lines,
src/base/parse.f90 semantics: case-sensitive names, ``!`` comments, numbers
read as real(8)).  Character-valued parameters are mapped to the enumerations
of the C ABI.
"""
import ctypes
import re

import numpy as np


class Params(ctypes.Structure):
    _fields_ = [
        ("nrtotal", ctypes.c_int), ("nztotal", ctypes.c_int), ("nl0", ctypes.c_int),
        ("ghost", ctypes.c_int), ("eqsym", ctypes.c_int),
        ("dr0", ctypes.c_double), ("dz0", ctypes.c_double), ("dtfac", ctypes.c_double),
        ("integrator", ctypes.c_int), ("icniter", ctypes.c_int), ("order", ctypes.c_int),
        ("slicing", ctypes.c_int), ("gauge_f", ctypes.c_double),
        ("shift", ctypes.c_int), ("drivercsi", ctypes.c_double), ("drivereta", ctypes.c_double),
        ("driveradv", ctypes.c_int), ("shiftadvect", ctypes.c_int),
        ("chimethod", ctypes.c_int), ("chipower", ctypes.c_int),
        ("evolveH", ctypes.c_int), ("evolveKTH", ctypes.c_int), ("nolambda", ctypes.c_int),
        ("lagrangian", ctypes.c_int), ("factorhdet", ctypes.c_int),
        ("eta", ctypes.c_double), ("geodiss", ctypes.c_double), ("scalardiss", ctypes.c_double),
        ("ft", ctypes.c_double * 8),
        ("boundtype", ctypes.c_int), ("interp_bicubic", ctypes.c_int),
        ("mattertype", ctypes.c_int), ("scalarpotential", ctypes.c_int),
        ("scalar_mass", ctypes.c_double), ("scalar_lambda", ctypes.c_double),
        ("idata", ctypes.c_int), ("ilapse", ctypes.c_int), ("bh1mass", ctypes.c_double),
        ("ell_solver", ctypes.c_int), ("ell_maxiter", ctypes.c_int), ("ell_epsilon", ctypes.c_double),
        ("we_method", ctypes.c_int), ("we_maxiter", ctypes.c_int),
        ("we_eta", ctypes.c_double), ("we_diss", ctypes.c_double), ("we_dtfac", ctypes.c_double),
        ("we_epsilon", ctypes.c_double),
        ("scalarpulse_type", ctypes.c_int), ("brilltype", ctypes.c_int),
        ("scalar_a0", ctypes.c_double), ("scalar_r0", ctypes.c_double), ("scalar_z0", ctypes.c_double),
        ("scalar_sr0", ctypes.c_double), ("scalar_sz0", ctypes.c_double),
        ("brill_a0", ctypes.c_double), ("brill_sr0", ctypes.c_double), ("brill_sz0", ctypes.c_double),
        ("nb", ctypes.c_int), ("nl", ctypes.c_int * 3),
        ("nrbox", ctypes.c_int * 3), ("nzbox", ctypes.c_int * 3),
        ("rbox", ctypes.c_double * 3), ("zbox", ctypes.c_double * 3),
        ("driverD0", ctypes.c_int), ("shiftafter", ctypes.c_double),
    ]


INTEGRATOR = {"rk4": 0, "icn": 1}
SLICING = {"1+log": 0, "harmonic": 1, "shockavoid": 2, "static": 3, "maximal": 4}
SHIFT = {"none": 0, "zero": 1, "static": 2, "Gammadriver2": 3, "Gammadriver1": 4, "Gammadriver0": 5,
         "Gammadrivershock1": 6, "Gammadrivershock2": 7}
BOUND = {"radiative": 0, "none": 1, "static": 2, "flat": 3}
MATTER = {"vacuum": 0, "scalar": 1}
POTENTIAL = {"none": 0, "phi2": 1, "phi4": 2}
IDATA = {"minkowski": 0, "schwarzschild": 1, "BrillLindquist": 2, "BrillWave": 3, "scalarpulse": 4}
ELL_SOLVER = {"none": 0, "wave": 1, "sor": 2, "mixed": 3, "fp64mg": 4}
PULSE = {"shell": 0, "torus": 1, "Baumgarte": 2}
BRILLTYPE = {"Holz": 0}
ILAPSE = {"one": 0, "isotropic": 1, "psiminus2": 2, "psiminus4": 3, "maximal": 4}

# field ids of enum ollin_field
FIELDS = ["alpha", "phi", "chi", "A", "B", "H", "C", "trK", "KTA", "KTB", "KTH", "KTC",
          "Delta_r", "Delta_z", "lambda", "Alambda", "beta_r", "beta_z", "dtbeta_r",
          "dtbeta_z", "scalar_phi", "scalar_xi_r", "scalar_xi_z", "scalar_pi", "fdriver"]
FIELD_ID = {n: k for k, n in enumerate(FIELDS)}
DERIVED_ID = {"ham": 64, "mom_r": 65, "mom_z": 66, "RSCAL": 67, "KT2": 68, "Lapla_alpha": 69}


def _single(x):
    """A default written without a d-exponent in param.f90 is a default
    (single precision) real converted to real(8)."""
    return float(np.float32(x))


def default_params():
    """src/base/param.f90 defaults for every field of ollin_params."""
    p = Params()
    p.nrtotal, p.nztotal, p.nl0, p.ghost, p.eqsym = 10, 10, 0, 0, 0
    p.dr0, p.dz0, p.dtfac = 1.0, 1.0, 0.5
    p.integrator, p.icniter, p.order = INTEGRATOR["icn"], 3, 2
    p.slicing, p.gauge_f = SLICING["harmonic"], 1.0
    p.shift, p.drivercsi, p.drivereta = SHIFT["none"], 0.75, 0.0
    p.driveradv, p.shiftadvect = 0, 1
    p.chimethod, p.chipower = 1, 2
    p.evolveH, p.evolveKTH, p.nolambda = 1, 0, 1
    p.lagrangian, p.factorhdet = 1, 1
    p.eta = 2.0
    p.geodiss, p.scalardiss = _single(0.01), _single(0.01)
    for k in range(8):
        p.ft[k] = 0.0
    p.boundtype, p.interp_bicubic = BOUND["radiative"], 1
    p.mattertype, p.scalarpotential = MATTER["vacuum"], POTENTIAL["none"]
    p.scalar_mass, p.scalar_lambda = 0.0, 0.0
    p.idata, p.ilapse, p.bh1mass = IDATA["minkowski"], ILAPSE["one"], 1.0
    p.ell_solver, p.ell_maxiter, p.ell_epsilon = ELL_SOLVER["wave"], 100000, 1.0e-8
    p.we_method, p.we_maxiter = INTEGRATOR["icn"], 100000
    p.we_eta, p.we_diss, p.we_dtfac, p.we_epsilon = 0.0, 0.1, 0.6, 1.0e-8
    p.scalarpulse_type, p.brilltype = PULSE["shell"], BRILLTYPE["Holz"]
    p.scalar_a0, p.scalar_r0, p.scalar_z0 = _single(0.0), _single(0.0), _single(0.0)
    p.scalar_sr0, p.scalar_sz0 = _single(1.0), _single(1.0)
    p.brill_a0, p.brill_sr0, p.brill_sz0 = _single(0.0), _single(1.0), _single(1.0)
    p.nb = 0
    for k in range(3):
        p.nl[k], p.nrbox[k], p.nzbox[k], p.rbox[k], p.zbox[k] = 0, 1, 1, 0.0, 0.0
    p.driverD0, p.shiftafter = 0, 0.0
    return p


_ENUMS = {"integrator": INTEGRATOR, "slicing": SLICING, "shift": SHIFT, "boundtype": BOUND,
          "mattertype": MATTER, "scalarpotential": POTENTIAL, "idata": IDATA, "ilapse": ILAPSE,
          "ell_solver": ELL_SOLVER, "we_method": INTEGRATOR, "scalarpulse_type": PULSE,
          "brilltype": BRILLTYPE}
_RENAME = {"Nrtotal": "nrtotal", "Nztotal": "nztotal", "Nl0": "nl0", "BH1mass": "bh1mass",
           "ELL_solver": "ell_solver", "ELL_maxiter": "ell_maxiter", "ELL_epsilon": "ell_epsilon",
           "WE_method": "we_method", "WE_maxiter": "we_maxiter", "WE_eta": "we_eta",
           "WE_diss": "we_diss", "WE_dtfac": "we_dtfac", "WE_epsilon": "we_epsilon"}
_IGNORED = {"Nt", "maximalevery", "Ninfo", "ELL_verbose", "ELL_Noutput", "WE_verbose", "WE_Noutput", "Noutput0D", "Noutput1D", "Noutput2D", "outvars0D", "outvars1D",
            "outvars2D", "directory", "checkpoint", "outparallel", "commenttype"}


def set_param(p, name, value):
    """Assign one parameter by its reference name (case-sensitive)."""
    name = _RENAME.get(name, name)
    if name in _IGNORED:
        return
    if name == "order":
        p.order = {"two": 2, "four": 4}[str(value)]
        return
    if name == "bssnflavor":
        p.lagrangian = 1 if str(value) == "lagrangian" else 0
        return
    if name == "interporder":
        p.interp_bicubic = 1 if str(value) == "bicubic" else 0
        return
    if name in _ENUMS:
        table = _ENUMS[name]
        if value not in table:
            raise ValueError("%s = %s is not supported by this library" % (name, value))
        setattr(p, name, table[value])
        return
    m = re.match(r"^ft([1-8])$", name)
    if m:
        p.ft[int(m.group(1)) - 1] = float(value)
        return
    if name == "Nb":
        p.nb = int(float(str(value)))
        return
    # the per-box parameters Nl1..3, Nrbox1..3, Nzbox1..3, rbox1..3, zbox1..3
    m = re.match(r"^(Nl|Nrbox|Nzbox|rbox|zbox)([1-3])$", name)
    if m:
        arr = getattr(p, m.group(1).lower())
        v = str(value).strip().replace("d", "e").replace("D", "e")
        arr[int(m.group(2)) - 1] = float(v) if m.group(1) in ("rbox", "zbox") else int(float(v))
        return
    if not hasattr(p, name):
        raise ValueError("unknown parameter %s" % name)
    cur = getattr(p, name)
    if isinstance(value, str):
        v = value.strip()
        if v.lower() in (".true.", "true"):
            value = 1
        elif v.lower() in (".false.", "false"):
            value = 0
        else:
            value = float(v.replace("d", "e").replace("D", "e")) if not isinstance(cur, int) else int(v)
    setattr(p, name, int(value) if isinstance(cur, int) else float(value))


def params_from_dict(d, base=None):
    p = base if base is not None else default_params()
    for k, v in d.items():
        set_param(p, k, v)
    return p


def params_from_par(text, base=None):
    """Parse a reference par file (src/base/parse.f90 conventions)."""
    d = {}
    for line in text.splitlines():
        line = line.split("!", 1)[0].strip()
        if not line or "=" not in line:
            continue
        k, v = line.split("=", 1)
        d[k.strip()] = v.strip().strip("\"'")
    return params_from_dict(d, base)
