"""The CPU oracle checked on its own (no GPU): its FFT against numpy's
pocketfft, and the Gaussian field against the input power spectrum."""
import numpy as np
import pytest


@pytest.mark.parametrize("n", [16, 24, 32, 48])
def test_oracle_c2r_matches_numpy_irfftn(built, n):
    import oracle as orc
    rng = np.random.default_rng(n)
    X = rng.normal(size=(n, n, n // 2 + 1)) + 1j * rng.normal(size=(n, n, n // 2 + 1))
    out = np.empty((n, n, n))
    orc.lib().or_c2r_3d(n, orc.P(X), orc.P(out))
    ref = np.fft.irfftn(X, s=(n, n, n), axes=(0, 1, 2), norm="forward")
    assert np.abs(out - ref).max() < 1e-9 * np.abs(ref).max()


@pytest.mark.parametrize("n", [16, 24])
def test_oracle_r2c_matches_numpy_rfftn(built, n):
    import oracle as orc
    x = np.random.default_rng(1).normal(size=(n, n, n))
    out = np.empty((n, n, n // 2 + 1), np.complex128)
    orc.lib().or_r2c_3d(n, orc.P(x), orc.P(out))
    ref = np.fft.rfftn(x, axes=(0, 1, 2))
    assert np.abs(out - ref).max() < 1e-9 * np.abs(ref).max()


def test_oracle_field_power_spectrum(built, tmp_path):
    """P(k) of the oracle's Gaussian field follows the input P(k) e^{-k^2 R^2}
    (the statistical check the reference relies on, predictions.c)."""
    import colore_gb300 as cg
    from colore_gb300 import inputs
    import oracle as orc
    f = inputs.write_inputs(str(tmp_path), inputs.scaled("c1", 64))
    prm = cg.Params(f)  # owns the tables cfg points at
    cfg = prm.config
    dk, _ = orc.fill64(cfg)
    n = cfg.n_grid
    kf = 2 * np.pi / cfg.l_box
    kx = np.arange(n // 2 + 1) * kf
    ky = np.fft.fftfreq(n, 1.0 / n) * kf
    kk = np.sqrt(kx[None, None, :] ** 2 + ky[None, :, None] ** 2 + ky[:, None, None] ** 2)
    sel = (kk > 0) & (kk < 0.5 * n * kf)
    pk = np.ctypeslib.as_array(cfg.pkarr, (cfg.numk,))
    lk = cfg.logkmin + np.arange(cfg.numk) / cfg.idlogk
    model = np.interp(np.log10(kk[sel]), lk, pk) * np.exp(-cfg.r2_smooth * kk[sel] ** 2) / kf ** 3
    ratio = np.abs(dk[sel]) ** 2 / model
    assert abs(ratio.mean() - 1) < 0.02


@pytest.mark.parametrize("scheme", [0, 1, 2])
def test_oracle_lpt_deposits_conserve_mass(built, tmp_path, scheme):
    """pos_2_ngp / pos_2_cic / pos_2_tsc (density.c:37-176): the weights of
    each particle sum to one, so the mean of 1 + delta is exactly 1; NGP puts
    whole particles in cells."""
    import oracle as orc
    import colore_gb300 as cg
    from colore_gb300 import inputs
    spec = inputs.scaled("c1", 32)
    spec.update(dens_type=1, lpt_interp_type=scheme)
    prm = cg.Params(inputs.write_inputs(str(tmp_path), spec))
    c = prm.config
    assert c.lpt_interp_type == scheme
    d, _, _ = orc.field64(c)
    out, disp = orc.lpt64(c, d)
    assert abs(np.mean(out + 1) - 1) < 1e-12
    assert np.all(out >= -1 - 1e-12)
    if scheme == 0:
        assert np.allclose(out + 1, np.round(out + 1), atol=1e-12)


def test_oracle_2lpt_matches_numpy(built, tmp_path):
    """The 2LPT restatement (density.c:646-1031) against the same steps with
    numpy's FFTs: r2c of the Gaussian field, the six second derivatives, the
    source, its r2c and the second-order displacements (unnormalised
    transforms, positive Nyquist wavenumbers as the reference takes them)."""
    import colore_gb300 as cg
    from colore_gb300 import inputs
    import oracle as orc
    spec = inputs.scaled("c1", 64)
    spec.update(dens_type=2, n_grid=64)
    prm = cg.Params(inputs.write_inputs(str(tmp_path), spec))
    c = prm.config
    n = 64
    rng = np.random.default_rng(12)
    k = np.fft.fftfreq(n) * n
    kk = np.sqrt(k[:, None, None] ** 2 + k[None, :, None] ** 2 + k[None, None, :] ** 2)
    dg = np.real(np.fft.ifftn(np.fft.fftn(rng.normal(size=(n, n, n))) * np.exp(-(kk / 8.0) ** 2)))
    dens, d1, d2 = orc.lpt2_64(c, dg)
    dkk = 2 * np.pi / c.l_box
    idx = np.arange(n)
    kf = np.where(2 * idx <= n, idx, idx - n) * dkk
    kx = np.arange(n // 2 + 1)[None, None, :] * dkk
    ky = kf[None, :, None]
    kz = kf[:, None, None]
    kv = [kx, ky, kz]
    k2 = n ** 3 * (kx ** 2 + ky ** 2 + kz ** 2)
    k2[0, 0, 0] = 1.0
    dk = np.fft.rfftn(dg)
    cdisp = [1j * kv[a] * dk / k2 for a in range(3)]
    for c_ in cdisp:
        c_[0, 0, 0] = 0
    pairs = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    dig = [np.fft.irfftn(1j * kv[j] * cdisp[i], s=(n, n, n), axes=(0, 1, 2), norm="forward") for i, j in pairs]
    src = dig[0] * dig[3] + dig[0] * dig[5] + dig[3] * dig[5] - dig[1] ** 2 - dig[2] ** 2 - dig[4] ** 2
    sk = np.fft.rfftn(src)
    for a in range(3):
        c2 = -1j * kv[a] * sk / k2
        c2[0, 0, 0] = 0
        want2 = np.fft.irfftn(c2, s=(n, n, n), axes=(0, 1, 2), norm="forward")
        want1 = np.fft.irfftn(cdisp[a], s=(n, n, n), axes=(0, 1, 2), norm="forward")
        assert np.abs(d2[a] - want2).max() <= 1e-10 * np.abs(want2).max()
        assert np.abs(d1[a] - want1).max() <= 1e-10 * np.abs(want1).max()
    assert np.std(d2[0]) > 1e-3 * np.std(d1[0])  # the second order is not empty
    assert abs(dens.mean()) < 1e-12  # mass conservation: mean of 1 + delta is 1
