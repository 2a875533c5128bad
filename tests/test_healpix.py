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
