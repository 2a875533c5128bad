"""Integer outputs at a larger size: the c4 configuration at 256^3 (1LPT,
one population with an nside 512 count map; its 64-shell intensity map at
nside 64, so that forcing every sub-sample into the double pass fits that
pass's queue) run twice on the device, once as the kernels decide (single
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


def _run(tmp_path, double):
    import colore_gb300 as cg
    from colore_gb300 import inputs
    spec = inputs.scaled("c4", 256)
    spec.pop("kappa", None)
    spec["imap"] = [dict(spec["imap"][0], nside=64)]
    m = cg.Mock(cg.Params(inputs.write_inputs(str(tmp_path), spec)))
    m.set_decisions_in_double(double)
    m.create_cartesian_fields()
    m.compute_physical_density_field()
    m.compute_density_normalization()
    m.exact_stats(reset=True)
    nsrc = list(m.srcs_set_cartesian())
    m.imap_set_cartesian()
    st = m.exact_stats()
    cat = m.catalog(0, pos=True, ipix=True, src=False)
    out = dict(nsrc=nsrc, pos=cat["pos"].copy(), ipix=cat["ipix"].copy(), cmap=m.count_map(0).copy(),
               nadd=m.imap(0, with_nadd=True)[1].copy(), samples=m.imap_samples(0), stats=st)
    m.close()
    return out


def test_c4_256_decisions_equal_forced_double(tmp_path_factory):
    a = _run(tmp_path_factory.mktemp("margins"), False)
    b = _run(tmp_path_factory.mktemp("double"), True)
    print("decided in double with the margins:", a["stats"], "forced:", b["stats"])
    assert a["nsrc"] == b["nsrc"] and a["nsrc"][0] > 10 ** 7
    assert np.array_equal(a["pos"], b["pos"])
    assert np.array_equal(a["ipix"], b["ipix"])
    assert np.array_equal(a["cmap"], b["cmap"])
    assert a["samples"] == b["samples"] and a["samples"] > 10 ** 6
    assert np.array_equal(a["nadd"], b["nadd"]), int((a["nadd"] != b["nadd"]).sum())
    # the forced run took every sample in double; the margins left few
    assert b["stats"]["imap_samples"] == b["samples"]
    assert a["stats"]["imap_samples"] < 1e-3 * a["samples"]
