"""Source lensing and skewers on the CPU: the srcs sections' flags
(io.c:331-339), the two oracle restatements of the line-of-sight integrals
at the sources (srcs.c:452-625, 715-733) on fields with known answers, and
the catalogue writer's lensing columns and skewer extensions
(io.c:1069-1236)."""
import os
import sys
import tempfile

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))


def _cfg(**src):
    import colore_gb300 as cg
    from colore_gb300 import inputs
    spec = inputs.scaled("c1", 64)
    s = dict(spec["srcs"][0])
    s.update(src)
    spec["srcs"] = [s]
    prm = cg.Params(inputs.write_inputs(tempfile.mkdtemp(), spec))
    return prm


def _steps(c):
    import colore_gb300 as cg
    nr = c.n_grid // 2
    dr = c.r_max / nr
    rm = (np.arange(nr) + 0.5) * dr
    r_arr = np.array([c.r_arr_r2z[i] for i in range(cg.NA)])

    def tab(name):
        return np.interp(rm, r_arr, np.array([getattr(c, name)[i] for i in range(cg.NA)]))
    return nr, dr, rm, tab


def test_srcs_flags(built):
    prm = _cfg(lensing=True, skewers=True, gaussian_skewers=True)
    c = prm.config
    assert (c.lensing_srcs[0], c.skw_srcs[0], c.skw_gauss[0]) == (1, 1, 1) and c.need_beaming > 0
    prm = _cfg(skewers=True)
    c = prm.config
    assert (c.lensing_srcs[0], c.skw_srcs[0], c.skw_gauss[0]) == (0, 1, 0)


def test_lensing_plane_wave_on_axis(built):
    """phi = A cos(2 pi m x / N) and a source on the +z axis: the ray stays in
    one x column, so kappa = e1 = idx^2/r t_xx sum(rm pg dr (r - rm)), e2 = 0,
    the deflection along x only, dra = 0."""
    import oracle as orc
    prm = _cfg(lensing=True)
    c = prm.config
    n = c.n_grid
    nr, dr, rm, tab = _steps(c)
    m, amp = 3, 2e-3
    x = np.arange(n)
    col = amp * np.cos(2 * np.pi * m * x / n)
    phi = np.broadcast_to(col[None, None, :], (n, n, n)).copy()
    zs = 0.37 * c.r_max
    pos = np.array([[0, 0, zs, 0]], np.float32)
    out = orc.lens64(c, phi, pos)[0]
    idx = n / c.l_box
    x0 = int((0 * rm[0] + c.pos_obs[0]) * idx + 0.5) % n
    txx = col[(x0 + 1) % n] + col[x0 - 1] - 2 * col[x0]
    vx = col[(x0 + 1) % n] - col[x0 - 1]
    r = float(np.float32(zs))
    kmax = min(int(r / dr + 0.5), nr - 1)
    pg = tab("growth_d_arr") * (1 + tab("z_arr_r2z"))
    fr = (rm * pg * dr * r - rm * rm * pg * dr)[:kmax + 1]
    frm = 2 * (pg * dr * r - rm * pg * dr)[:kmax + 1]
    kappa = idx * idx / r * txx * fr.sum()
    np.testing.assert_allclose(out[2], kappa, rtol=1e-6)
    np.testing.assert_allclose(out[0], kappa, rtol=1e-6)
    assert out[1] == 0 and out[3] == 0
    np.testing.assert_allclose(out[4], 180 / np.pi * 0.5 * idx / r * vx * frm.sum(), rtol=1e-6)
    pad = np.zeros((n, n, 2 * (n // 2 + 1)), np.float32)
    pad[:, :, :n] = phi
    o32 = orc.lens32(c, pad, pos, np.zeros((1, 9), np.float32))[0]
    np.testing.assert_allclose(o32[4:9], out, rtol=2e-5, atol=1e-9 * np.abs(out).max())


def test_lensing_fp32_vs_fp64_and_linearity(built):
    """On a smooth random potential the FP32 restatement follows the FP64 one
    (rms 1e-3: the nearest cell of a step can differ), and doubling the
    potential doubles every output bit for bit."""
    import oracle as orc
    prm = _cfg(lensing=True)
    c = prm.config
    n = c.n_grid
    rng = np.random.default_rng(3)
    k = np.fft.fftfreq(n)
    kk = k[:, None, None] ** 2 + k[None, :, None] ** 2 + k[None, None, :] ** 2
    phi = np.real(np.fft.ifftn(np.fft.fftn(rng.normal(size=(n, n, n))) * np.exp(-kk * 200))) * 1e-2
    pad = np.zeros((n, n, 2 * (n // 2 + 1)), np.float32)
    pad[:, :, :n] = phi
    u = rng.normal(size=(400, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    r = rng.uniform(0.05, 1.0, 400) * c.r_max
    pos = np.zeros((400, 4), np.float32)
    pos[:, :3] = u * r[:, None]
    o64 = orc.lens64(c, pad[:, :, :n].astype(np.float64), pos)
    o32 = orc.lens32(c, pad, pos, np.zeros((400, 9), np.float32))[:, 4:9]
    for j in range(5):
        assert np.sqrt(np.mean((o32[:, j] - o64[:, j]) ** 2) / np.mean(o64[:, j] ** 2)) < 1e-3, j
    o32b = orc.lens32(c, 2 * pad, pos, np.zeros((400, 9), np.float32))[:, 4:9]
    assert np.array_equal(o32b, 2 * o32)


@pytest.mark.parametrize("gauss", [0, 1])
def test_skewers_uniform_density(built, gauss):
    """A uniform density d0 and potential: density skewers read d0 (Gaussian
    ones log(1 + d0)/D + D sigma^2/2 with D at the corner cells), velocity
    skewers 0, and every step past the source 0."""
    import oracle as orc
    prm = _cfg(skewers=True, gaussian_skewers=bool(gauss))
    c = prm.config
    n = c.n_grid
    nr, dr, rm, tab = _steps(c)
    d0, s2 = 0.3, 0.8
    dens = np.full((n, n, n), d0)
    phi = np.full((n, n, n), 5.0)
    pos = np.array([[0.1 * c.r_max, 0.2 * c.r_max, -0.3 * c.r_max, 0], [0, 0, 0.999 * c.r_max, 0]], np.float32)
    d64, v64 = orc.skw64(c, dens, phi, gauss, s2, pos)
    pad = np.zeros((n, n, 2 * (n // 2 + 1)), np.float32)
    pad[:, :, :n] = d0
    padp = np.full((n, n, 2 * (n // 2 + 1)), 5.0, np.float32)
    d32, v32 = orc.skw32(c, pad, padp, gauss, s2, pos)
    r0 = float(np.linalg.norm(pos[0, :3].astype(np.float64)))
    kmax = min(int(r0 / dr + 0.5), nr - 1)
    assert np.all(v64 == 0) and np.all(v32 == 0)
    assert np.all(d64[0, kmax + 1:] == 0) and np.all(d32[0, kmax + 1:] == 0)
    assert np.all(d64[1] != 0)  # the second source reaches the last step
    if not gauss:
        np.testing.assert_allclose(d64[0, :kmax + 1], d0, rtol=1e-14)
        np.testing.assert_allclose(d32[0, :kmax + 1], d0, rtol=1e-6)
    else:
        dg = tab("growth_d_arr")[:kmax + 1]
        want = np.log(1 + d0) / dg + dg * s2 * 0.5
        np.testing.assert_allclose(d64[0, :kmax + 1], want, rtol=2e-3)  # corners at other radii
        np.testing.assert_allclose(d32[0], d64[0], rtol=2e-5, atol=1e-7)


def test_skewers_fp32_vs_fp64(built):
    import oracle as orc
    prm = _cfg(skewers=True)
    c = prm.config
    n = c.n_grid
    rng = np.random.default_rng(9)
    dens = np.exp(rng.normal(0, 0.4, (n, n, n))) - 1
    phi = rng.normal(0, 1e-2, (n, n, n))
    pad = np.zeros((n, n, 2 * (n // 2 + 1)), np.float32)
    padp = pad.copy()
    pad[:, :, :n] = dens
    padp[:, :, :n] = phi
    u = rng.normal(size=(200, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    pos = np.zeros((200, 4), np.float32)
    pos[:, :3] = u * rng.uniform(0.05, 1.0, 200)[:, None] * c.r_max
    d64, v64 = orc.skw64(c, pad[:, :, :n].astype(np.float64), padp[:, :, :n].astype(np.float64), 0, 0.0, pos)
    d32, v32 = orc.skw32(c, pad, padp, 0, 0.0, pos)
    assert np.sqrt(np.mean((d32 - d64) ** 2) / np.mean(d64 ** 2)) < 1e-5
    assert np.sqrt(np.mean((v32 - v64) ** 2) / np.mean(v64 ** 2)) < 1e-5


def test_catalog_writer_lensing_and_skewers(built, tmp_path):
    """The 10-column table with lensing, the ASCII lensing header, and the
    two skewer images plus the background table after the catalogue."""
    import colore_gb300 as cg
    from test_output_formats import read_fits
    rng = np.random.default_rng(2)
    n, nr = 37, 16
    src = rng.normal(size=(n, 9)).astype(np.float32)
    sk = dict(dens=rng.normal(size=(n, nr)), vel=rng.normal(size=(n, nr)), r=np.arange(nr) + 0.5,
              z=np.linspace(0, 1, nr), d1=np.linspace(1, 0.5, nr), v1=np.linspace(1, 2, nr), sigma_g=0.75, gauss=True)
    prefix = str(tmp_path / "o")
    cg.write_catalog(prefix, 0, src, cg.OUT_FITS, lensing=True, skewers=sk)
    hdus = read_fits(prefix + "_srcs_s1_0.fits")
    assert len(hdus) == 5
    h1, d1 = hdus[1]
    assert h1["TFIELDS"] == 10 and h1["NAXIS1"] == 40
    assert [h1["TTYPE%d" % i] for i in range(6, 11)] == ["E1", "E2", "KAPPA", "DRA", "DDEC"]
    rows = np.frombuffer(d1, np.dtype([("t", ">i4"), ("c", ">f4", (9,))]))
    assert np.array_equal(rows["c"], src)
    for k, (key, want) in enumerate((("gaussian skewers", sk["dens"]), ("velocity skewers", sk["vel"]))):
        h, d = hdus[2 + k]
        assert (h["XTENSION"], h["BITPIX"], h["NAXIS1"], h["NAXIS2"], h["CONTENTS"]) == ("IMAGE", -32, nr, n, key)
        assert np.array_equal(np.frombuffer(d, ">f4").reshape(n, nr), want.astype(np.float32))
    hb, db = hdus[4]
    assert hb["CONTENTS"] == "Background cosmology" and abs(float(hb["SIGMA_G"]) - 0.75) < 1e-7
    bg = np.frombuffer(db, ">f4").reshape(nr, 4)
    assert np.array_equal(bg[:, 1], sk["z"].astype(np.float32))
    cg.write_catalog(prefix, 0, src, cg.OUT_ASCII, lensing=True)
    lines = open(prefix + "_srcs_s1_0.txt").read().splitlines()
    assert lines[0] == "#[1]type [2]RA, [3]dec, [4]z0, [5]dz_RSD #[6]e1, [7]e2 [8]kappa [9]d_ra [10]d_dec"
    a = np.array([[float(x) for x in ln.split()] for ln in lines[1:]])
    np.testing.assert_allclose(a[:, 1:], src, rtol=1e-6, atol=1e-12)
