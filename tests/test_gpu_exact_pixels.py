"""The intensity maps' RING pixel decision on the GPU, against the oracle's
double restatement of he_ang2pix (healpix_extra.c:141-172).

The device evaluates the single-precision decision with its approximate
reciprocal and reciprocal square root, whose errors the CPU mirror cannot
reproduce; here millions of directions -- at random and within 1e-9..1e-4 of
every kind of pixel edge -- go through the device's own arithmetic, with exact
float coordinates and with coordinates carrying a relative error.  Every
decision the device keeps in single precision must be the double one, and
the share it leaves to double must stay small.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ns", [16, 256, 512, 1024, 2048])
def test_device_pixel_margins_never_disagree_with_double(built, ns):
    import colore_gb300 as cg
    import oracle as orc
    import test_exact_cpu as tx
    rng = np.random.default_rng(ns)
    for kind in ("random", "edges"):
        v = rng.normal(size=(2_000_000, 3)) if kind == "random" else tx._edge_points(ns, 200_000)
        v *= rng.uniform(10, 4000, (len(v), 1))
        v32 = v.astype(np.float32)
        got = cg.ring_pixels_checked(ns, v32, 0.0)
        ref = orc.pix64(ns, v32.astype(np.float64))
        ok = got >= 0
        assert np.array_equal(got[ok], ref[ok]), (ns, kind, int((got[ok] != ref[ok]).sum()))
        if kind == "random":
            assert 1 - ok.mean() < 4e-6 * ns + 1e-4, (ns, 1 - ok.mean())
        pert = (v * (1 + rng.uniform(-1, 1, v.shape) * 2.0 ** -24)).astype(np.float32)
        got = cg.ring_pixels_checked(ns, pert, 2.0 ** -23)
        ref = orc.pix64(ns, v)
        ok = got >= 0
        assert np.array_equal(got[ok], ref[ok]), (ns, kind, "perturbed")
