"""Known-answer tests and checks of the shared scalar arithmetic (CPU)."""
import ctypes as C
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "kat.json")))


def test_philox_known_answers(built):
    """Philox4x32-10 vectors published with the Random123 library."""
    import oracle as orc
    for v in GOLD["philox4x32_10"]:
        out = orc.philox([int(x, 16) for x in v["ctr"]], [int(x, 16) for x in v["key"]])
        assert ["%08x" % x for x in out] == v["out"]


class _Cos(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("om", "ol", "ob", "ok", "h", "w0")] + \
               [("ksign", C.c_int), ("normal_de", C.c_int)] + \
               [(n, C.c_double) for n in ("a_eq", "phorizon", "growth0")]


def test_cosmology_matches_reference_run_log(built):
    """Values printed by the reference's example run (notebook log): a_eq,
    chi_H(0), D_0, r_min, r_max, L_box, dx and dk for its cosmology."""
    import colore_gb300 as cg
    L = cg.lib()
    k = GOLD["notebook_run"]
    c = _Cos()
    L.cg_cosmo_init.argtypes = [C.POINTER(_Cos)] + [C.c_double] * 5
    assert L.cg_cosmo_init(C.byref(c), k["omega_M"], k["omega_L"], k["omega_B"], k["w"], k["h"]) == 0
    L.cg_cosmo_chi.restype = C.c_double
    L.cg_cosmo_chi.argtypes = [C.POINTER(_Cos), C.c_double]
    rmax = L.cg_cosmo_chi(C.byref(c), 1 / (1 + k["z_max"]))
    rmin = L.cg_cosmo_chi(C.byref(c), 1 / (1 + k["z_min"]))
    lbox = 2 * rmax * (1 + 2.0 / k["n_grid"])
    assert "%.5f" % c.a_eq == k["a_eq"]
    assert "%.3E" % c.phorizon == k["chi_H0"]
    assert "%.3f" % c.growth0 == k["D_0"]
    assert "%.3f" % rmax == k["r_max"]
    assert "%.3f" % rmin == k["r_min"]
    assert "%.3f" % lbox == k["L_box"]
    assert "%.3E" % (lbox / k["n_grid"]) == k["dx"]
    assert "%.3E" % (2 * np.pi / lbox) == k["dk"]


def _ulps(got, ref):
    got = got.astype(np.float64)
    r32 = ref.astype(np.float32)
    sp = np.abs(np.spacing(r32)).astype(np.float64)
    return np.abs(got - ref) / sp


def test_math_functions_within_4_ulp(built):
    import oracle as orc
    rng = np.random.default_rng(1)
    x = rng.uniform(-87, 88, 200000).astype(np.float32)
    assert _ulps(orc.vec("expf", x), np.exp(x.astype(np.float64))).max() <= 2
    x = np.exp(rng.uniform(-80, 80, 200000)).astype(np.float32)
    assert _ulps(orc.vec("logf", x), np.log(x.astype(np.float64))).max() <= 2
    x = rng.uniform(-0.99, 10, 200000).astype(np.float32)
    ref = np.log1p(x.astype(np.float64))
    ok = np.abs(ref) > 1e-30
    assert _ulps(orc.vec("log1pf", x)[ok], ref[ok]).max() <= 4
    y = rng.normal(size=200000).astype(np.float32)
    xx = rng.normal(size=200000).astype(np.float32)
    assert _ulps(orc.vec("atan2f", y, xx), np.arctan2(y.astype(np.float64), xx.astype(np.float64))).max() <= 4
    c = rng.uniform(-1, 1, 200000).astype(np.float32)
    assert _ulps(orc.vec("acosf", c), np.arccos(c.astype(np.float64))).max() <= 4
    t = rng.uniform(0, 2 * np.pi, 200000).astype(np.float32)
    s, co = orc.vec("sincosf", t)
    assert np.abs(s - np.sin(t.astype(np.float64))).max() < 3e-7
    assert np.abs(co - np.cos(t.astype(np.float64))).max() < 3e-7


@pytest.mark.parametrize("lam", [0.05, 0.7, 3.0, 9.9, 10.0, 17.0, 150.0, 4000.0])
def test_poisson_moments(built, lam):
    import oracle as orc
    n = 400000
    k = orc.poisson(np.full(n, lam, np.float32), 11, 22)
    m, v = k.mean(), k.var()
    assert abs(m - lam) < 6 * np.sqrt(lam / n)
    assert abs(v / lam - 1) < 6 * np.sqrt(2.0 / n) + 0.01
    assert k.min() >= 0


def test_poisson_pmf_small_lambda(built):
    import oracle as orc
    from math import exp, factorial
    lam, n = 2.5, 1000000
    k = orc.poisson(np.full(n, lam, np.float32), 5, 6)
    h = np.bincount(k, minlength=12)[:12] / n
    pmf = np.array([exp(-lam) * lam ** i / factorial(i) for i in range(12)])
    assert np.all(np.abs(h - pmf) < 6 * np.sqrt(pmf / n) + 1e-5)
