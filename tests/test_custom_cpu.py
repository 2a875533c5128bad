"""Custom maps on the CPU: the custom%d sections of the parameter file
(io.c:344-364), the K(z) and b(z) tables (cosmo.c:631-662), and the two
oracle restatements of cstm_get_beam_properties (cstm.c:68-145) on fields
whose ray integral is known in closed form."""
import os
import sys
import tempfile

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _spec(**custom):
    from colore_gb300 import inputs
    spec = inputs.scaled("c1", 64)
    spec["custom"] = [dict(kz=("gauss", 0.3, 0.06), bias=("const", 1.4), nside=8),
                      dict(kz=("flat", 0.2, 0.35), bias=("1+z",), nside=4, amp=-3.0)]
    spec.update(custom)
    return spec


def _oracle():
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
    import oracle as orc
    return orc


def test_custom_sections(built):
    """Two custom sections give two maps with their nside; K(z) and b(z) are
    sampled on the r table from the spline of the files; a K(z) file that
    does not cover [z_min, z_max] is rejected with the reference's message."""
    import colore_gb300 as cg
    from colore_gb300 import inputs
    d = tempfile.mkdtemp()
    prm = cg.Params(inputs.write_inputs(d, _spec()))  # owns the tables the config points to
    c = prm.config
    assert c.n_cstm == 2 and (c.nside_cstm[0], c.nside_cstm[1]) == (8, 4) and c.need_beaming > 0
    z = np.array([c.z_arr_r2z[i] for i in range(cg.NA)])
    kz0 = np.array([c.cstm_kz_arr[0][i] for i in range(cg.NA)])
    bz1 = np.array([c.cstm_bz_arr[1][i] for i in range(cg.NA)])
    inside = (z > 0.1) & (z < 0.5)
    np.testing.assert_allclose(kz0[inside], np.exp(-0.5 * ((z[inside] - 0.3) / 0.06) ** 2), atol=1e-6)
    np.testing.assert_allclose(bz1[inside], 1 + z[inside], rtol=1e-8)
    zs = np.linspace(0.2, 0.4, 20)
    np.savetxt(os.path.join(d, "kzc_1.txt"), np.transpose([zs, np.ones_like(zs)]))
    with pytest.raises(cg.CGError, match="K\\(z\\) z-range is too small"):
        cg.Params(os.path.join(d, "run.cfg"))


def test_custom_support(built):
    """The integration range is where |K/H| exceeds 1e-4 of its maximum
    (cstm.c:98-116): the flat kernel between z = 0.2 and 0.35 covers the
    steps whose centres lie in that range."""
    import colore_gb300 as cg
    from colore_gb300 import inputs
    orc = _oracle()
    prm = cg.Params(inputs.write_inputs(tempfile.mkdtemp(), _spec()))
    c = prm.config
    kz, bz, lo, hi, rc = orc.cstm_steps(c, 1)
    assert rc == 0 and 0 < lo < hi < c.n_grid // 2 - 1
    nr = c.n_grid // 2
    rm = (np.arange(nr) + 0.5) * c.r_max / nr
    r_arr = np.array([c.r_arr_r2z[i] for i in range(cg.NA)])
    z_arr = np.array([c.z_arr_r2z[i] for i in range(cg.NA)])
    zm = np.interp(rm, r_arr, z_arr)
    assert zm[lo] > 0.17 and zm[hi] < 0.38  # the tanh edges are 0.005 wide
    assert np.all(kz[lo:hi + 1] < 0)  # amp = -3
    assert np.all(np.abs(kz[:lo]) <= 1e-4 * np.abs(kz).max())


@pytest.mark.parametrize("delta", [0.0, 0.25])
def test_custom_oracles_on_a_uniform_density(built, delta):
    """For a uniform density delta and a constant normalisation n, every pixel
    of custom map p is dr * sum over the support of kz (bias(delta, bz) n - 1);
    the FP64 restatement matches to 1e-12, the FP32 one to 1e-5."""
    import colore_gb300 as cg
    from colore_gb300 import inputs
    orc = _oracle()
    prm = cg.Params(inputs.write_inputs(tempfile.mkdtemp(), _spec()))
    c = prm.config
    n = c.n_grid
    nr = n // 2
    dr = c.r_max / nr
    nrm = 1.1
    tab = np.full(cg.NA, nrm)
    for ip in range(c.n_cstm):
        kz, bz, lo, hi, _ = orc.cstm_steps(c, ip)
        assert c.bias_model == 1  # (1 + d)^b, common.h:429
        b = (1 + delta) ** bz
        want = dr * np.sum(kz[lo:hi + 1] * (b[lo:hi + 1] * nrm - 1))
        m64 = orc.cstm64(c, ip, np.full((n, n, n), delta), tab, (nrm, nrm))
        m32 = orc.cstm32(c, ip, np.full((n, n, 2 * (n // 2 + 1)), delta, np.float32), tab.astype(np.float32),
                         np.array([nrm, nrm], np.float32))
        assert m64.shape == (12 * c.nside_cstm[ip] ** 2,)
        np.testing.assert_allclose(m64, want, rtol=1e-12)
        np.testing.assert_allclose(m32, want, rtol=1e-5, atol=1e-7 * abs(want))


def test_custom_oracles_agree_on_a_random_field(built):
    """On a lognormal-like random field the FP32 restatement (the GPU kernel's
    arithmetic) stays within 1e-5 rms of the FP64 one."""
    import colore_gb300 as cg
    from colore_gb300 import inputs
    orc = _oracle()
    prm = cg.Params(inputs.write_inputs(tempfile.mkdtemp(), _spec()))
    c = prm.config
    n = c.n_grid
    rng = np.random.default_rng(5)
    dens = np.exp(rng.normal(0, 0.5, (n, n, n))) - 1
    pad = np.zeros((n, n, 2 * (n // 2 + 1)), np.float32)
    pad[:, :, :n] = dens
    tab = np.linspace(0.9, 1.2, cg.NA)
    for ip in range(c.n_cstm):
        m64 = orc.cstm64(c, ip, dens, tab, (0.9, 1.2))
        m32 = orc.cstm32(c, ip, pad, tab.astype(np.float32), np.array([0.9, 1.2], np.float32))
        assert np.sqrt(np.mean((m32 - m64) ** 2) / np.mean(m64 ** 2)) < 1e-5
        assert np.std(m64) > 0
