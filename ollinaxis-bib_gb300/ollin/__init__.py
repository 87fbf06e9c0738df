"""Host-side mirror of the OllinAxis-BiB evolution interface over the GB300
C ABI (include/ollin_gpu.h).

``params`` holds the reference's parameters (src/base/param.f90) as the
``ollin_params`` struct; ``gpu.Evolution`` is the driver of
src/base/evolve.f90 over the CUDA library; ``build`` compiles csrc/ for
sm_103a.
"""
from .params import (Params, default_params, params_from_dict, params_from_par, set_param,
                     FIELDS, FIELD_ID, DERIVED_ID)

__all__ = ["Params", "default_params", "params_from_dict", "params_from_par", "set_param",
           "FIELDS", "FIELD_ID", "DERIVED_ID"]
