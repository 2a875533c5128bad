"""The stand-alone driver (colore_gpu, the main() of the reference on the GPU)
against the same run through the Python binding: every file it writes holds
what the library computes.  Catalogue, count map, density grids and
convergence are deterministic and compared exactly; the intensity maps sum
floats with atomics in an unspecified order and are compared to 1e-5."""
import os
import subprocess

import numpy as np
import pytest

from test_output_formats import read_fits

pytestmark = pytest.mark.gpu


def _spec(fmt):
    return dict(n_grid=64, z_min=0.05, z_max=0.6, r_smooth=2.0, seed=53, dens_type=0, bias_model=2,
                output_format=fmt, output_density=True,
                srcs=[dict(nz=("gauss", 0.3, 0.1), density=50.0, bias=("1+z",), nside_count=8, lensing=True,
                           skewers=True)],
                imap=[dict(tz=0.1, bias=("const", 1.0), z_range=(0.1, 0.5), nbands=3, nside=8)],
                kappa=dict(z_out=[0.3, 0.5], nside=8),
                isw=dict(z_out=[0.4], nside=8),
                custom=[dict(kz=("gauss", 0.3, 0.1), bias=("const", 1.2), nside=8)])


@pytest.mark.parametrize("fmt", ["FITS", "ASCII"])
def test_driver_outputs_match_library(built, tmp_path, fmt):
    import colore_gb300 as cg
    from colore_gb300 import build, inputs
    pfile = inputs.write_inputs(str(tmp_path), _spec(fmt))
    r = subprocess.run([build.DRIVER, pfile], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    prefix = str(tmp_path / "run")
    m = cg.Mock.from_param_file(pfile)
    m.create_cartesian_fields()
    g0 = m.grid(0).copy()
    m.compute_physical_density_field()
    m.compute_density_normalization()
    g1 = m.grid(0).copy()
    m.srcs_set_cartesian()
    m.imap_set_cartesian()
    m.get_beam_properties()
    n = 64
    for tag, g in (("gaussian", g0), ("lightcone", None)):
        raw = open("%s_dens_%s_0.dat" % (prefix, tag), "rb").read()
        body = np.frombuffer(raw[28:], np.float32).reshape(n, n, n)
        if g is not None:
            assert np.array_equal(body, g[:, :, :n])
        else:
            assert np.array_equal(body, g1[:, :, :n])
    src = m.catalog(0, pos=False, ipix=False)["src"]
    if fmt == "FITS":
        hdus = read_fits(prefix + "_srcs_s1_0.fits")
        (h, d) = hdus[1]
        rows = np.frombuffer(d, np.dtype([("t", ">i4"), ("c", ">f4", (9,))]))
        assert h["NAXIS2"] == len(src) and h["TFIELDS"] == 10
        assert np.array_equal(rows["c"], src)
        sd, sv = m.skewers(0)
        assert hdus[2][0]["CONTENTS"] == "density skewers" and hdus[3][0]["CONTENTS"] == "velocity skewers"
        assert np.array_equal(np.frombuffer(hdus[2][1], ">f4").reshape(sd.shape), sd)
        assert np.array_equal(np.frombuffer(hdus[3][1], ">f4").reshape(sv.shape), sv)
        assert hdus[4][0]["NAXIS2"] == n // 2
    else:
        a = np.loadtxt(prefix + "_srcs_s1_0.txt", ndmin=2)
        assert a.shape[0] == len(src)
        np.testing.assert_allclose(a[:, 1:10], src, rtol=1e-6, atol=1e-12)
    (_, _), (h, d) = read_fits(prefix + "_srcs_s1_counts.fits")
    assert np.array_equal(np.frombuffer(d, ">f4"), m.count_map(0).astype(np.float32))
    im = m.imap(0)
    for ir in range(im.shape[0]):
        (_, _), (h, d) = read_fits("%s_imap_s1_nu%03d.fits" % (prefix, ir))
        assert h["NSIDE"] == 8
        np.testing.assert_allclose(np.frombuffer(d, ">f4"), im[ir], rtol=1e-5, atol=1e-12)
    k = m.kappa()
    for ir in range(k.shape[0]):
        (_, _), (h, d) = read_fits("%s_kappa_z%03d.fits" % (prefix, ir))
        assert np.array_equal(np.frombuffer(d, ">f4"), k[ir])
    (_, _), (h, d) = read_fits("%s_isw_z000.fits" % prefix)
    assert np.array_equal(np.frombuffer(d, ">f4"), m.isw()[0])
    (_, _), (h, d) = read_fits("%s_custom_s1.fits" % prefix)
    assert h["NSIDE"] == 8 and h["NAXIS2"] == 12 * 64
    assert np.array_equal(np.frombuffer(d, ">f4"), m.custom(0))
    m.close()
