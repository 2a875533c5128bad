"""Theory predictions (write_predictions, predictions.c:26-173) and the
FFTLog transforms behind them (fftlog.c:93-157), on the CPU.

The C transform is pinned to a numpy restatement of the reference's steps
(low-ringing k_c r_c, the u_m coefficients, the FFT convolution and its
reversal).  That reversal (b[j] <-> b[N-1-j]) leaves the values one log-step
off the grid the reference reports, so against an analytic pair the
transform is good to ~2e-3 where a one-step-shifted reversal would give
4e-5; the files reproduce the reference's numbers, quirk included."""
import numpy as np
import pytest


def _grid(n=10000):
    return 1e-4 * (1e6) ** (np.arange(n) / (n - 1))


def _reference_steps(k, pk):
    """pk2xi as fftlog.c does it, in numpy."""
    from scipy.special import loggamma
    n = len(k)
    a = k ** 1.5 * pk
    mu = 0.5
    L = np.log(k[-1] / k[0]) * n / (n - 1)
    x = (mu + 1) / 2
    y = np.pi * n / (2 * L)
    arg = np.log(2.0) * n / L + 2 * loggamma(x + 1j * y).imag / np.pi
    kr = np.exp((arg - np.round(arg)) * L / n) if arg != np.round(arg) else 1.0
    y = np.pi / L
    k0r0 = kr * np.exp(-L)
    t = -2 * y * np.log(k0r0 / 2)
    m = np.arange(n // 2 + 1)
    u = np.exp(1j * (m * t + 2 * loggamma(x + 1j * m * y).imag))
    uu = np.empty(n, complex)
    uu[:n // 2 + 1] = u
    uu[n // 2 + 1:] = np.conj(u[1:n // 2][::-1])
    uu[n // 2] = uu[n // 2].real
    b = np.fft.ifft(np.fft.fft(a) * uu)[::-1]
    r = k0r0 / k[0] * np.exp(np.arange(n) * L / n)
    return r, ((2 * np.pi * r) ** -1.5 * b).real


def test_fftlog_matches_the_reference_steps(built):
    pytest.importorskip("scipy")
    import colore_gb300 as cg
    k = _grid(4096)
    pk = k / (1 + (k / 0.02) ** 2.5)  # a P(k)-like shape
    r, xi = cg.pk2xi(k, pk)
    r2, xi2 = _reference_steps(k, pk)
    np.testing.assert_allclose(r, r2, rtol=1e-12)
    assert np.abs(xi - xi2).max() <= 1e-10 * np.abs(xi2).max()


def test_fftlog_round_trip_and_analytic_pair(built):
    """xi2pk(pk2xi(P)) returns P; a Gaussian P(k) gives the Gaussian xi(r)
    within the reference's one-step offset (3e-3 of the peak)."""
    import colore_gb300 as cg
    k = _grid()
    s = 5.0
    pk = np.exp(-k ** 2 * s ** 2 / 2)
    r, xi = cg.pk2xi(k, pk)
    k2, pk2 = cg.xi2pk(r, xi)
    assert np.abs(k2 / k - 1).max() < 1e-12
    m = (k > 1e-3) & (k < 0.5)
    assert np.abs(pk2[m] / pk[m] - 1).max() < 1e-10
    want = (2 * np.pi * s ** 2) ** -1.5 * np.exp(-r ** 2 / (2 * s ** 2))
    mr = (r > 0.5) & (r < 30)
    assert np.abs(xi[mr] - want[mr]).max() < 3e-3 * want.max()


def test_prediction_files(built, tmp_path):
    """write_predictions: the bias table and, per redshift and tracer, the
    spectra and correlation functions with the reference's names, headers
    and columns; the linear columns are P_lin g^2 times the smoothing
    kernels of predictions.c:43-45."""
    import colore_gb300 as cg
    from colore_gb300 import inputs
    spec = inputs.scaled("c1", 64)
    spec["pred"] = dict(dz=0.25, just=True)
    spec["imap"] = [dict(tz=0.1, bias=("const", 1.0), z_range=(0.1, 0.5), nbands=2, nside=8)]
    prm = cg.Params(inputs.write_inputs(str(tmp_path), spec))
    c = prm.config
    cg.write_predictions(prm)
    prefix = str(tmp_path / "run")
    g = open(prefix + "_gbias.txt").read().splitlines()
    assert g[0] == "#1-z 2-r(z) 3-g(z) 4-bg_1(z) 5-bi_1(z) "
    rows = [list(map(float, ln.split())) for ln in g[1:]]
    z, want_z = 0.0, []  # z <= z_max (0.5 for c1) in steps of 0.25, accumulated as in the reference
    while z <= spec["z_max"]:
        want_z.append(z)
        z += 0.25
    assert [r[0] for r in rows] == pytest.approx(want_z)
    assert all(abs(r[3] - 1.5) < 1e-9 for r in rows)  # c1: constant bias 1.5
    for zz in want_z:
        fpk = "%s_pk_srcs_pop0_z%.3f.txt" % (prefix, zz)
        fxi = "%s_xi_imap_pop0_z%.3f.txt" % (prefix, zz)
        lines = open(fpk).read().splitlines()
        assert lines[0] == "# k[h/Mpc] P_tt P_tl P_ll"
        a = np.loadtxt(fpk)
        assert a.shape[1] == 4 and 9990 <= len(a) <= 10000
        assert open(fxi).readline() == "# k[Mpc/h] xi_tt xi_ll*b^2 xi_ll\n"
        assert open("%s_xi_srcs_pop0_z%.3f.txt" % (prefix, zz)).readline() == "# r[Mpc/h] xi_tt xi_ll*b^2 xi_ll\n"
        # P_tl / P_ll = b exp(-(rsm2_gm - rsm2_mm) k^2)
        dx = c.l_box / c.n_grid
        d_gm_mm = (2.0 - 1.88) * dx ** 2 / 6
        ok = (a[:, 3] > 1e-250) & (a[:, 2] > 1e-250)  # away from the %g-printed underflow
        ratio = a[ok, 2] / a[ok, 3]
        # k is printed to 6 digits: exp(-d k^2) carries 2 d k^2 * 5e-7 of it
        np.testing.assert_allclose(ratio, 1.5 * np.exp(-d_gm_mm * a[ok, 0] ** 2), rtol=2e-4)
