"""The C ABI library loads on a host without a GPU, exports every symbol
include/ollin_gpu.h declares, and reports a missing device as an error code."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if not fn.endswith(".h"):
            continue
        with open(os.path.join(ROOT, "include", fn)) as f:
            text = f.read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(ollin_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    from ollin import gpu
    lib = gpu.load()
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_default_parameters_match_param_module():
    from ollin import gpu
    from ollin.params import Params, default_params
    lib = gpu.load()
    p = Params()
    lib.ollin_params_default(ctypes.byref(p))
    q = default_params()
    for f, _ in Params._fields_:
        a, b = getattr(p, f), getattr(q, f)
        if f in ("ft", "nl", "nrbox", "nzbox", "rbox", "zbox"):
            a, b = list(a), list(b)
        assert a == b, f
    # a literal without a d-exponent in param.f90 is single precision
    assert p.geodiss == float(ctypes.c_float(0.01).value)


def test_struct_layout_matches_header(tmp_path):
    """ctypes mirror of ollin_params against the C compiler's layout."""
    import subprocess
    from ollin.params import Params
    fields = [f for f, _ in Params._fields_]
    src = ['#include <stdio.h>', '#include <stddef.h>', '#include "ollin_gpu.h"', "int main(void){",
           'printf("%zu\\n", sizeof(ollin_params));']
    for f in fields:
        src.append('printf("%%zu\\n", offsetof(ollin_params, %s));' % f)
    src.append("return 0;}")
    c = tmp_path / "layout.c"
    c.write_text("\n".join(src))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(c), "-o", str(exe)], check=True)
    out = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert out[0] == ctypes.sizeof(Params)
    for f, off in zip(fields, out[1:]):
        assert getattr(Params, f).offset == off, f


def test_unsupported_parameters_are_rejected_before_any_device_work():
    from ollin import gpu
    from ollin.params import params_from_dict
    lib = gpu.load()
    # a negative number of ghost zones
    p = params_from_dict(dict(order="four", ghost=-1, eqsym=1))
    h = ctypes.c_void_p()
    rc = lib.ollin_gpu_create(ctypes.byref(p), ctypes.byref(h))
    assert rc == 1 and b"ghost" in lib.ollin_gpu_last_error()


@pytest.mark.skipif(os.path.exists("/dev/nvidia0"), reason="host has a GPU")
def test_missing_device_is_an_error_code():
    from ollin import gpu
    from ollin.params import params_from_dict
    lib = gpu.load()
    p = params_from_dict(dict(order="four", eqsym=1, nrtotal=16, nztotal=16))
    h = ctypes.c_void_p()
    rc = lib.ollin_gpu_create(ctypes.byref(p), ctypes.byref(h))
    assert rc == 2
