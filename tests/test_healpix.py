"""HEALPix identities of the shared pixel functions (CPU)."""
import numpy as np
import pytest


@pytest.mark.parametrize("nside", [1, 2, 4, 16, 64])
def test_nest_ring_bijection(built, nside):
    import oracle as orc
    npix = 12 * nside * nside
    ip = np.arange(npix)
    r = orc.nest2ring(nside, ip)
    assert np.array_equal(np.sort(r), ip)
    assert np.array_equal(orc.ring2nest(nside, r), ip)


@pytest.mark.parametrize("nside", [1, 2, 8, 64, 512])
def test_pixel_centres_map_to_themselves(built, nside):
    import oracle as orc
    npix = 12 * nside * nside
    ip = np.arange(npix) if npix < 200000 else np.random.default_rng(0).integers(0, npix, 200000)
    v = orc.pix2vec_nest(nside, ip).astype(np.float64)
    assert np.allclose(np.linalg.norm(v, axis=1), 1, atol=1e-6)
    phi = np.arctan2(v[:, 1], v[:, 0])
    phi[phi < 0] += 2 * np.pi
    ring = orc.ang2pix(nside, v[:, 2].astype(np.float32), phi.astype(np.float32))
    assert np.array_equal(ring, orc.nest2ring(nside, ip))


def _ang2pix_ring_f64(nside, z, phi):
    """Independent FP64 restatement (Gorski et al. 2005) for comparison."""
    za = np.abs(z)
    tt = np.mod(phi, 2 * np.pi) * 2 / np.pi
    out = np.empty(len(z), np.int64)
    eq = za <= 2.0 / 3
    t1 = nside * (0.5 + tt[eq])
    t2 = nside * z[eq] * 0.75
    jp = (t1 - t2).astype(np.int64)
    jm = (t1 + t2).astype(np.int64)
    ir = nside + 1 + jp - jm
    ks = 1 - (ir & 1)
    ip = (jp + jm - nside + ks + 1) // 2
    ip = np.mod(ip, 4 * nside)
    out[eq] = nside * (nside - 1) * 2 + (ir - 1) * 4 * nside + ip
    pc = ~eq
    tp = tt[pc] - np.floor(tt[pc])
    tmp = nside * np.sqrt(3 * (1 - za[pc]))
    jp = (tp * tmp).astype(np.int64)
    jm = ((1 - tp) * tmp).astype(np.int64)
    ir = jp + jm + 1
    ip = np.mod((tt[pc] * ir).astype(np.int64), 4 * ir)
    out[pc] = np.where(z[pc] > 0, 2 * ir * (ir - 1) + ip, 12 * nside * nside - 2 * ir * (ir + 1) + ip)
    return out


@pytest.mark.parametrize("nside", [4, 64, 1024])
def test_ang2pix_agrees_with_fp64_away_from_edges(built, nside):
    import oracle as orc
    rng = np.random.default_rng(3)
    z = rng.uniform(-1, 1, 300000)
    phi = rng.uniform(0, 2 * np.pi, 300000)
    p32 = orc.ang2pix(nside, z.astype(np.float32), phi.astype(np.float32))
    p64 = _ang2pix_ring_f64(nside, z.astype(np.float32).astype(np.float64),
                            phi.astype(np.float32).astype(np.float64))
    frac = np.mean(p32 != p64)
    assert frac < 2e-4 * max(1, nside / 64), frac


def _ang2pix_ring_f32_modulo(nside, z, phi):
    """The FP32 RING pixel with the textbook modulo (Gorski et al. 2005), in
    numpy float32 arithmetic: every product, sum and square root rounded
    once, as the shared C function does them."""
    f = np.float32
    z = z.astype(f)
    phi = phi.astype(f)
    za = np.abs(z)
    tt = phi * f(0.636619772367581343)
    ns = f(nside)
    out = np.empty(len(z), np.int64)
    eq = za <= f(0.666666666666666667)
    t1 = ns * (f(0.5) + tt[eq])
    t2 = (ns * z[eq]) * f(0.75)
    jp = (t1 - t2).astype(np.int64)
    jm = (t1 + t2).astype(np.int64)
    ir = nside + 1 + jp - jm
    ks = 1 - (ir & 1)
    ip = np.trunc((jp + jm - nside + ks + 1) / 2).astype(np.int64)
    ip = np.mod(ip, 4 * nside)
    out[eq] = nside * (nside - 1) * 2 + (ir - 1) * 4 * nside + ip
    pc = ~eq
    tq = tt[pc]
    tp = tq - tq.astype(np.int64).astype(f)
    tmp = ns * np.sqrt(f(3.0) * (f(1.0) - za[pc]))
    jp = (tp * tmp).astype(np.int64)
    jm = ((f(1.0) - tp) * tmp).astype(np.int64)
    ir = jp + jm + 1
    ip = np.mod((tq * ir.astype(f)).astype(np.int64), 4 * ir)
    out[pc] = np.where(z[pc] > 0, 2 * ir * (ir - 1) + ip, 12 * nside * nside - 2 * ir * (ir + 1) + ip)
    return out


@pytest.mark.parametrize("nside", [1, 3, 5, 64, 96, 512, 1000, 8192])
def test_ang2pix_wrap_is_the_modulo(built, nside):
    """The pixel index within a ring is reduced by one conditional
    subtraction instead of a modulo; the two agree bit for bit, including
    phi just below 2 pi (where tt * ir rounds up to 4 ir) and z at the
    equatorial/polar boundary."""
    import oracle as orc
    rng = np.random.default_rng(11)
    n = 200000
    z = rng.uniform(-1, 1, n).astype(np.float32)
    phi = rng.uniform(0, 2 * np.pi, n).astype(np.float32)
    top = np.float32(2 * np.pi)
    edge_phi = np.array([0.0, np.nextafter(top, np.float32(0)), np.nextafter(np.nextafter(top, np.float32(0)),
                                                                              np.float32(0)),
                         np.float32(np.pi / 2), np.float32(np.pi), np.float32(3 * np.pi / 2)], np.float32)
    edge_z = np.array([-1, -2.0 / 3, -0.5, 0, 0.5, 2.0 / 3, 1, np.nextafter(np.float32(2.0 / 3), np.float32(1)),
                       np.nextafter(np.float32(-2.0 / 3), np.float32(-1))], np.float32)
    ez, ep = np.meshgrid(edge_z, edge_phi)
    z = np.concatenate([z, ez.ravel()])
    phi = np.concatenate([phi, ep.ravel()])
    got = orc.ang2pix(nside, z, phi)
    want = _ang2pix_ring_f32_modulo(nside, z, phi)
    assert np.array_equal(got, want)
    assert got.min() >= 0 and got.max() < 12 * nside * nside
