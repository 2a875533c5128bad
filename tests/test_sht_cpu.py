"""The oracle's FP64 angular power spectrum (oracle/sht.py), the checker of
the maps' C_ell, pinned on the CPU:

  geometry   every RING pixel centre it produces maps back to its own index
             through the oracle's restatement of he_ang2pix
             (healpix_extra.c:141-172), nside 1..64;
  transform  a_lm equal to the definition (4 pi / Npix) sum_p map_p Y*_lm,
             summed directly with scipy's spherical harmonics, to 1e-13,
             for the C Legendre sums (or_sht.c) and the numpy transform; the
             two agree to 1e-13 at nside 64;
  spectrum   he_alm2cl's weighting (healpix_extra.c:437-465): a map that is
             one real harmonic has all its power at that l.
"""
import numpy as np
import pytest


def _sht():
    import oracle  # noqa: F401  (puts oracle/ on the path)
    import sht
    return sht


@pytest.mark.parametrize("ns", [1, 2, 4, 16, 64])
def test_ring_geometry_is_he_ang2pix(ns):
    import oracle as orc
    sht = _sht()
    cth, phi = sht.pixel_centres(ns)
    s = np.sqrt(1 - cth ** 2)
    v = np.stack([s * np.cos(phi), s * np.sin(phi), cth], 1)
    assert np.array_equal(orc.pix64(ns, v), np.arange(12 * ns * ns))


@pytest.mark.parametrize("ns", [2, 8])
def test_alm_equals_direct_sum(ns):
    special = pytest.importorskip("scipy.special")
    if not hasattr(special, "sph_harm_y"):
        pytest.skip("scipy without sph_harm_y")
    sht = _sht()
    rng = np.random.default_rng(ns)
    maps = rng.normal(size=(2, 12 * ns * ns))
    alm = sht.map2alm(maps, ns)
    alm_py = sht.map2alm_py(maps, ns)
    cth, phi = sht.pixel_centres(ns)
    th = np.arccos(cth)
    om = 4 * np.pi / (12 * ns * ns)
    for l in range(3 * ns):
        for m in range(l + 1):
            direct = (maps * np.conj(special.sph_harm_y(l, m, th, phi))[None]).sum(1) * om
            assert np.abs(direct - alm[:, l, m]).max() < 1e-13, (l, m)
            assert np.abs(direct - alm_py[:, l, m]).max() < 1e-13, (l, m)


def test_c_and_numpy_transforms_agree():
    sht = _sht()
    ns = 64
    maps = np.random.default_rng(5).normal(size=(3, 12 * ns * ns))
    a, b = sht.map2alm(maps, ns), sht.map2alm_py(maps, ns)
    assert np.abs(a - b).max() < 1e-13


def test_single_harmonic_spectrum():
    special = pytest.importorskip("scipy.special")
    if not hasattr(special, "sph_harm_y"):
        pytest.skip("scipy without sph_harm_y")
    sht = _sht()
    ns = 32
    cth, phi = sht.pixel_centres(ns)
    th = np.arccos(cth)
    for l, m in ((0, 0), (3, 0), (10, 4), (40, 17)):
        y = special.sph_harm_y(l, m, th, phi)
        mp = y.real if m == 0 else np.sqrt(2) * y.real  # unit-norm real harmonic
        cl = sht.anafast(mp, ns)[0]
        # all the power at l, 1/(2l+1) of the unit norm, to the quadrature's accuracy
        assert abs(cl[l] * (2 * l + 1) - 1) < 1e-3, (l, m, cl[l])
        other = np.delete(cl, l)
        assert other.max() < 1e-5 * cl[l], (l, m)
