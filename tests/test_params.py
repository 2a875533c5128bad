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
