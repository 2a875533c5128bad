"""Host-side checks that need no GPU: the C ABI library loads and exports
every declared entry point, the param-file reader and the FP64 tables."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in ("colore_cuda.h", "colore_host.h"):
        txt = open(os.path.join(ROOT, "include", h)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names.update(re.findall(r"\b(cg(?:64)?_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_library_exports_every_declared_symbol(built):
    import colore_gb300 as cg
    lib = C.CDLL(cg.LIB_PATH)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    assert set(cg.exported_symbols()) <= set(declared_symbols())


def test_create_without_gpu_fails_loudly(built):
    import colore_gb300 as cg
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    from colore_gb300 import inputs
    import tempfile
    d = tempfile.mkdtemp()
    f = inputs.write_inputs(d, inputs.scaled("c1", 64))
    with pytest.raises(cg.CGError):
        cg.Mock.from_param_file(f)


def test_memory_estimate(built):
    import colore_gb300 as cg
    from colore_gb300 import inputs
    import tempfile
    f = inputs.write_inputs(tempfile.mkdtemp(), inputs.scaled("c1", 64))
    p = cg.Params(f)
    b = C.c_ulonglong()
    assert cg.lib().cg_memory_estimate(C.byref(p.config), C.byref(b)) == 0
    assert b.value >= 2 * 64 * 64 * 33 * 8


def test_unsupported_grid_is_rejected(built):
    import colore_gb300 as cg
    from colore_gb300 import inputs
    import tempfile
    f = inputs.write_inputs(tempfile.mkdtemp(), inputs.scaled("c1", 100))
    p = cg.Params(f)
    b = C.c_ulonglong()
    assert cg.lib().cg_memory_estimate(C.byref(p.config), C.byref(b)) == 1
