"""Integer outputs at larger sizes: the c4 configuration at 256^3 (1LPT,
one population with an nside 512 count map; its 64-shell intensity map at
nside 64, so that forcing every sub-sample into the double pass fits that
pass's queue) and the c2 configuration at 512^3 (lognormal, two
populations with nside 256 count maps), each run twice on the device, once as the kernels decide (single
precision with proven margins, float-float for the intensity-map samples
those margins leave open, double for the rest) and once with every decision
taken in the device's double arithmetic (cg_set_decisions_in_double).  The
source counts, catalogue positions and pixels, the count map and every
intensity-map hit count must be the same: over ~4e7 sources and ~2e7
sub-samples, the margins never keep a decision the double arithmetic takes
differently (srcs.c:156-183, healpix_extra.c:141-172, imap.c:179-231)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _spec(name):
    from colore_gb300 import inputs
    if name == "c4":
        spec = inputs.scaled("c4", 256)
        spec["imap"] = [dict(spec["imap"][0], nside=64)]
    else:
        spec = inputs.scaled("c2", 512)
    spec.pop("kappa", None)
    return spec


def _run(tmp_path, name, double):
    import colore_gb300 as cg
    from colore_gb300 import inputs
    spec = _spec(name)
    m = cg.Mock(cg.Params(inputs.write_inputs(str(tmp_path), spec)))
    m.set_decisions_in_double(double)
    m.create_cartesian_fields()
    m.compute_physical_density_field()
    m.compute_density_normalization()
    m.exact_stats(reset=True)
    nsrc = list(m.srcs_set_cartesian())
    imap = bool(spec.get("imap"))
    if imap:
        m.imap_set_cartesian()
    st = m.exact_stats()
    out = dict(nsrc=nsrc, stats=st, cats=[], cmaps=[])
    for ip in range(len(nsrc)):
        cat = m.catalog(ip, pos=True, ipix=True, src=False)
        out["cats"].append((cat["pos"].copy(), cat["ipix"].copy()))
        out["cmaps"].append(m.count_map(ip).copy())
    if imap:
        out["nadd"] = m.imap(0, with_nadd=True)[1].copy()
        out["samples"] = m.imap_samples(0)
    m.close()
    return out


@pytest.mark.parametrize("name", ["c4", "c2"])
def test_decisions_equal_forced_double_at_size(tmp_path_factory, name):
    a = _run(tmp_path_factory.mktemp("margins"), name, False)
    b = _run(tmp_path_factory.mktemp("double"), name, True)
    print(name, "decided in double with the margins:", a["stats"], "forced:", b["stats"])
    assert a["nsrc"] == b["nsrc"] and a["nsrc"][0] > 10 ** 7
    for (pa, ia), (pb, ib) in zip(a["cats"], b["cats"]):
        assert np.array_equal(pa, pb)
        assert np.array_equal(ia, ib)
    for ca, cb in zip(a["cmaps"], b["cmaps"]):
        assert np.array_equal(ca, cb)
    assert a["stats"]["count_cells"] < 1e-3 * b["stats"]["count_cells"]
    if "nadd" not in a:
        return
    assert a["samples"] == b["samples"] and a["samples"] > 10 ** 6
    assert np.array_equal(a["nadd"], b["nadd"]), int((a["nadd"] != b["nadd"]).sum())
    # the forced run took every sample in double; the margins left few
    assert b["stats"]["imap_samples"] == b["samples"]
    assert a["stats"]["imap_samples"] < 1e-3 * a["samples"]
