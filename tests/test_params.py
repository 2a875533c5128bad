"""The libconfig-grammar reader and read_run_params (io.c:246-563)."""
import os
import tempfile

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _write_tables(d):
    from colore_gb300 import inputs
    spec = inputs.scaled("c1", 64)
    return inputs.write_inputs(d, spec)


def test_grammar_features(built):
    """Comments of three kinds, ':' and '=', groups, arrays, lists, adjacent
    strings, hex and L-suffixed ints, optional separators."""
    import colore_gb300 as cg
    d = tempfile.mkdtemp()
    base = open(_write_tables(d)).read()
    txt = open(os.path.join(HERE, "golden", "grammar.cfg")).read().replace("@DIR@", d)
    f = os.path.join(d, "g.cfg")
    open(f, "w").write(txt)
    p = cg.Params(f)
    c = p.config
    assert c.n_grid == 64 and c.seed == 1001 and c.n_srcs == 1
    assert c.do_kappa == 1 and c.n_kappa == 2 and c.nside_kappa == 16
    assert abs(c.r2_smooth - 4.0) < 1e-12 and c.do_smoothing == 1
    assert c.bias_model == 2 and c.need_beaming == 1
    assert base  # the generated file parses too
    cg.Params(os.path.join(d, "run.cfg"))


@pytest.mark.parametrize("drop", ["n_grid", "omega_M", "seed", "pk_filename"])
def test_missing_key_is_an_error(built, drop):
    import colore_gb300 as cg
    d = tempfile.mkdtemp()
    f = _write_tables(d)
    lines = [l for l in open(f).read().split("\n") if not l.strip().startswith(drop + "=")]
    open(f, "w").write("\n".join(lines))
    with pytest.raises(cg.CGError, match="Couldn't read variable"):
        cg.Params(f)


def test_short_redshift_table_is_an_error(built):
    import colore_gb300 as cg
    d = tempfile.mkdtemp()
    f = _write_tables(d)
    z = np.linspace(0.2, 0.3, 10)
    np.savetxt(os.path.join(d, "bz_1.txt"), np.transpose([z, 1 + z]))
    with pytest.raises(cg.CGError, match="z-range is too small"):
        cg.Params(f)


def test_missing_file_is_an_error(built):
    import colore_gb300 as cg
    with pytest.raises(cg.CGError, match="Couldn't open"):
        cg.Params("/nonexistent/run.cfg")


def test_syntax_error_reports_line(built):
    import colore_gb300 as cg
    d = tempfile.mkdtemp()
    f = os.path.join(d, "bad.cfg")
    open(f, "w").write("global:\n{\n  z_min = ;\n}\n")
    with pytest.raises(cg.CGError, match="line 3"):
        cg.Params(f)


def test_isw_section(built):
    """isw { z_out; nside } (io.c:421-426): plane distances from the
    cosmology, as the kappa planes (cosmo.c:831-845); planes beyond z_max are
    rejected with the reference's message."""
    import colore_gb300 as cg
    from colore_gb300 import inputs
    d = tempfile.mkdtemp()
    spec = inputs.scaled("c1", 64)
    spec["kappa"] = dict(z_out=[0.3, 0.45], nside=16)
    spec["isw"] = dict(z_out=[0.45, 0.3], nside=8)
    prm = cg.Params(inputs.write_inputs(d, spec))  # owns the tables the config points to
    c = prm.config
    assert (c.do_isw, c.n_isw, c.nside_isw) == (1, 2, 8) and c.need_beaming > 0
    assert c.isw_r[0] == c.kappa_r[1] and c.isw_r[1] == c.kappa_r[0]
    spec["isw"] = dict(z_out=[0.9], nside=8)
    with pytest.raises(cg.CGError, match="Source plane 1 outside redshift range"):
        cg.Params(inputs.write_inputs(tempfile.mkdtemp(), spec))


def test_isw_oracles_on_a_constant_potential(built):
    """For a uniform potential c the ISW map of plane p is c * sum of
    2 PD(r) dr over the steps up to that plane, in both restatements."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
    import oracle as orc
    import colore_gb300 as cg
    from colore_gb300 import inputs
    spec = inputs.scaled("c1", 64)
    spec["isw"] = dict(z_out=[0.2, 0.45], nside=4)
    prm = cg.Params(inputs.write_inputs(tempfile.mkdtemp(), spec))  # owns the tables
    c = prm.config
    n = c.n_grid
    nr = n // 2
    dr = c.r_max / nr
    pd = np.array([c.growth_pd_arr[i] for i in range(cg.NA)])
    r_arr = np.array([c.r_arr_r2z[i] for i in range(cg.NA)])
    rm = (np.arange(nr) + 0.5) * dr
    fac = 2 * np.interp(rm, r_arr, pd) * dr
    rp = sorted(np.float32(c.isw_r[i]) for i in range(c.n_isw))
    irmax = [min(int(r / dr + 0.5), nr - 1) for r in rp]
    want = [3.0 * fac[:k + 1].sum() for k in irmax]
    m64 = orc.isw64(c, np.full((n, n, n), 3.0))
    m32 = orc.isw32(c, np.full((n, n, 2 * (n // 2 + 1)), 3.0, np.float32))
    for pl in range(c.n_isw):
        np.testing.assert_allclose(m64[pl], want[pl], rtol=1e-12)
        np.testing.assert_allclose(m32[pl], want[pl], rtol=2e-6)
