"""Integer outputs equal to the reference's double arithmetic, on the CPU.

The kernels decide Poisson counts and HEALPix pixels in single precision
where a bound on the distance to the double value proves the decision, and
in double otherwise (colore_gb300/csrc/cg_exact.h).  These tests run the
same functions on the CPU (the oracle's dev32 mirror) against the oracle's
independent double restatement of the reference (or_ref64.c):

  pixels   directions at random and next to every kind of RING pixel edge
           (equatorial edge lines, polar-cap lines, the phi = k pi/2 lines,
           |cos theta| = 2/3), exact float inputs and inputs carrying a
           relative error; every decision kept in single precision must be
           the double one;
  counts   every cell's Poisson count of 64^3 mocks (three bias models, a
           population dense enough near the observer to take PTRS) equals
           the double restatement's;
  sources  positions, base pixels and count maps equal; RA, Dec, z within
           single-precision tolerance.
"""
import numpy as np
import pytest

rng = np.random.default_rng(7)


def _dirs(z, tt):
    phi = tt * np.pi / 2
    s = np.sqrt(np.maximum(0, 1 - z * z))
    return np.stack([s * np.cos(phi), s * np.sin(phi), z], 1)


def _edge_points(ns, n):
    """Directions within 1e-9..1e-4 of RING pixel edges at nside ns."""
    zs, ts = [], []
    z = rng.uniform(-2 / 3, 2 / 3, n)
    k = rng.integers(0, 4 * ns + 2, n)
    sgn = rng.choice([-1, 1], n)
    zs.append(z)
    ts.append((k / ns - 0.5 - sgn * 0.75 * z) % 4)
    z = rng.uniform(2 / 3, 1, n) * rng.choice([-1, 1], n)
    tmp = ns * np.sqrt(3 * (1 - np.abs(z)))
    k = np.floor(rng.uniform(0, 1, n) * tmp)
    tp = np.where(rng.uniform(size=n) < 0.5, k / np.maximum(tmp, 1e-9), 1 - k / np.maximum(tmp, 1e-9))
    zs.append(z)
    ts.append((rng.integers(0, 4, n) + np.clip(tp, 0, 1)) % 4)
    ir = rng.integers(1, ns + 1, n)
    kk = rng.integers(0, 4 * ir)
    zs.append((1 - (ir / ns) ** 2 / 3 * rng.uniform(0.9, 1.0, n)) * rng.choice([-1, 1], n))
    ts.append((kk / ir) % 4)
    zs.append(rng.uniform(-1, 1, n))
    ts.append(rng.integers(0, 4, n).astype(float))
    zs.append(rng.choice([-2 / 3, 2 / 3], n))
    ts.append(rng.uniform(0, 4, n))
    z = np.concatenate(zs)
    tt = np.concatenate(ts)
    sc = 10 ** rng.uniform(-9, -4, len(z))
    z = np.clip(z + rng.normal(size=len(z)) * sc, -1, 1)
    tt = (tt + rng.normal(size=len(z)) * sc) % 4
    return _dirs(z, tt)


@pytest.mark.parametrize("ns", [1, 2, 16, 256, 512, 1024])
def test_pixel_margins_never_disagree_with_double(ns):
    import oracle as orc
    for kind in ("random", "edges"):
        v = rng.normal(size=(100000, 3)) if kind == "random" else _edge_points(ns, 20000)
        v *= rng.uniform(10, 4000, (len(v), 1))
        v32 = v.astype(np.float32)
        fast = orc.pix_checked(ns, v32, 0.0)
        ref = orc.pix64(ns, v32.astype(np.float64))
        ok = fast >= 0
        assert np.array_equal(fast[ok], ref[ok]), (ns, kind)
        # the kernels' own double restatement agrees with the oracle's
        assert np.array_equal(orc.pix64(ns, v32.astype(np.float64), shared=True), ref)
        if kind == "random":
            assert 1 - ok.mean() < 5e-6 * ns + 1e-4, (ns, 1 - ok.mean())
        # float coordinates within a relative 2^-24 of the double point
        pert = (v * (1 + rng.uniform(-1, 1, v.shape) * 2.0 ** -24)).astype(np.float32)
        fast = orc.pix_checked(ns, pert, 2.0 ** -23)
        ref = orc.pix64(ns, v)
        ok = fast >= 0
        assert np.array_equal(fast[ok], ref[ok]), (ns, kind, "perturbed")


def _edge_points_tight(ns, n, seed):
    """Directions within 1e-15..1e-8 (in quarter turns) of equatorial RING
    edge lines: far inside the single-precision margins."""
    r = np.random.default_rng(seed)
    z = r.uniform(-2 / 3, 2 / 3, n)
    k = r.integers(0, 4 * ns + 2, n)
    tt = (k / ns - 0.5 - r.choice([-1, 1], n) * 0.75 * z) % 4
    tt = (tt + r.normal(size=n) * 10 ** r.uniform(-15, -8, n)) % 4
    return _dirs(z, tt) * r.uniform(10, 4000, (n, 1))


@pytest.mark.parametrize("ns", [1, 16, 512, 1024, 4096])
def test_float_float_pixels_never_disagree_with_double(ns):
    """The float-float tier (cg_pix_ff) that the samples left open by the
    single-precision margins take before double: every pixel it keeps is the
    double one, at random, next to every kind of edge, and within 1e-15 of
    equatorial edges; it leaves only the poles and what lies within ~1e-12
    of an edge."""
    import oracle as orc
    for kind in ("random", "edges", "tight"):
        if kind == "random":
            v = rng.normal(size=(100000, 3)) * rng.uniform(10, 4000, (100000, 1))
        elif kind == "edges":
            v = _edge_points(ns, 20000) * rng.uniform(10, 4000, (100000, 1))
        else:
            v = _edge_points_tight(ns, 100000, ns)
        ref = orc.pix64(ns, v, shared=True)
        ff = orc.pix_ff(ns, v)
        ok = ff >= 0
        assert np.array_equal(ff[ok], ref[ok]), (ns, kind, int((ff[ok] != ref[ok]).sum()))
        r = np.sqrt((v * v).sum(1))
        pole = np.hypot(v[:, 0], v[:, 1]) < 1e-6 * r
        if kind == "random":
            assert ok[~pole].all(), (ns, kind, int((~ok[~pole]).sum()))
        elif kind == "edges":
            # offsets 1e-9..1e-4 times a normal draw: a few land within 1e-12
            assert (~ok[~pole]).mean() < 1e-3, (ns, kind, int((~ok[~pole]).sum()))
        else:
            # offsets log-uniform over 1e-15..1e-8: all beyond ~1e-12 decided
            assert ok.mean() > 0.55, ok.mean()
            assert (orc.pix_checked(ns, v.astype(np.float32)) < 0).mean() > 0.99


@pytest.mark.parametrize("op,bound", [(0, 4), (1, 5), (2, 16), (3, 4), (4, 2)])
def test_float_float_operations_within_their_bounds(op, bound):
    """cg_ff.h's sum, product, quotient, square root and product by a float
    on random normalised pairs (both signs, magnitudes 1e-3..1e4, so sums
    cancel) against exact rational arithmetic: the relative error stays
    within the u^2 = 2^-48 multiples the float-float pixel bounds use."""
    from decimal import Decimal, getcontext
    from fractions import Fraction
    import oracle as orc
    getcontext().prec = 80
    r = np.random.default_rng(100 + op)

    def pairs(n):
        h = (r.choice([-1, 1], n) * 10 ** r.uniform(-3, 4, n)).astype(np.float32)
        l = (r.uniform(-0.5, 0.5, n) * np.spacing(np.abs(h)).astype(np.float64)).astype(np.float32)
        return h, l

    n = 4000
    (xh, xl), (yh, yl) = pairs(n), pairs(n)
    if op == 3:
        xl = np.where(xh < 0, -xl, xl).astype(np.float32)
        xh = np.abs(xh)
    if op == 4:
        yl = np.zeros(n, np.float32)
    oh, ol = orc.ff_ops(op, (xh, xl), (yh, yl))
    u2 = Fraction(1, 2 ** 48)
    worst = 0.0
    for i in range(n):
        X = Fraction(float(xh[i])) + Fraction(float(xl[i]))
        Y = Fraction(float(yh[i])) + Fraction(float(yl[i]))
        R = Fraction(float(oh[i])) + Fraction(float(ol[i]))
        if op == 3:
            s = (Decimal(X.numerator) / Decimal(X.denominator)).sqrt()
            rel = float(abs((Decimal(R.numerator) / Decimal(R.denominator) - s) / s) * Decimal(2 ** 48))
        else:
            E = X + Y if op == 0 else (X / Y if op == 2 else X * Y)
            rel = float(abs((R - E) / E) / u2) if E != 0 else 0.0
        worst = max(worst, rel)
    assert worst <= bound, (op, worst)


def test_quarter_turn_atan_exhaustive():
    """The polynomial behind every float direction's quarter-turn angle
    (cg_atan01_q) is within 8.2e-8 of atan(t) / (pi/2) for every float t in
    [0, 1]: the accuracy the pixel margins assume."""
    import oracle as orc
    assert orc.lib().or_atan_q_maxerr() < 8.2e-8


def _spec(bias_model):
    return dict(n_grid=64, z_min=0.05, z_max=0.6, r_smooth=2.0, seed=11 + bias_model, dens_type=0,
                bias_model=bias_model,
                srcs=[dict(nz=("gauss", 0.3, 0.1), density=40.0, bias=("1+z",), nside_count=64),
                      dict(nz=("flat", 0.0, 0.5), density=30.0, bias=("const", 2.0), nside_count=512)])


@pytest.mark.parametrize("bias_model", [1, 2, 3])
def test_counts_and_sources_equal_double(tmp_path, bias_model):
    import oracle as orc
    from colore_gb300 import inputs
    prm = orc.Params(inputs.write_inputs(str(tmp_path), _spec(bias_model)))
    cfg = prm.config
    n = cfg.n_grid
    d64, p64, st = orc.field64(cfg)
    dens = orc.density64(cfg, d64, st[3])
    d32 = dens.astype(np.float32)
    phi32 = p64.astype(np.float32)
    tabs, e0f, _ = orc.norm_tables64(cfg, d32.astype(np.float64))
    pad = lambda a: np.ascontiguousarray(np.pad(a, ((0, 0), (0, 0), (0, 2 * (n // 2 + 1) - n))))
    for ip in range(cfg.n_srcs):
        t64, e64 = tabs[ip], np.asarray(e0f[ip], np.float64)
        t32, e32 = t64.astype(np.float32), e64.astype(np.float32)
        c32, tot32, fb = orc.counts32(cfg, ip, pad(d32), t32, e32, t64, e64)
        c64, tot64 = orc.counts64(cfg, ip, d32, t64, e64)
        assert tot64 > 1000
        assert np.array_equal(c32, c64), (ip, int((c32 != c64).sum()))
        # the flat population's tails hold ~5e3 cells whose density is within
        # its bound of zero: decided by the inversion with lambda 0, not in
        # double
        assert fb < 1e-3 * n ** 3, (ip, fb)
        if ip == 1:
            assert c64.max() >= 10  # the dense cells near the observer take PTRS
        o32 = orc.emit32(cfg, ip, pad(d32), pad(phi32), t32, e32, t64, e64, cap=tot64 + 16)
        o64 = orc.emit64(cfg, ip, phi32, c64, cap=tot64 + 16)
        assert np.array_equal(o32["pos"][:, :3].view(np.uint32), o64["pos"][:, :3].view(np.uint32))
        assert np.array_equal(o32["ipix"], o64["ipix"])
        assert np.array_equal(o32["cmap"], o64["cmap"])
        np.testing.assert_allclose(o32["pos"][:, 3], o64["pos"][:, 3], rtol=1e-4, atol=1e-3)
        s32, s64 = o32["src"], o64["src"]
        dra = np.abs(s32[:, 0] - s64[:, 0])
        assert np.all(np.minimum(dra, 360 - dra) < 2e-4)
        assert np.max(np.abs(s32[:, 1] - s64[:, 1])) < 2e-4
        np.testing.assert_allclose(s32[:, 2], s64[:, 2], rtol=2e-6, atol=1e-7)


def _imap_spec(case):
    base = dict(n_grid=64, z_min=0.05, z_max=0.6, r_smooth=2.0, seed=41, dens_type=0, bias_model=2,
                imap=[dict(tz=0.1, bias=("const", 1.0), z_range=(0.05, 0.5), nbands=12, nside=64)])
    if case == "fine":
        base["imap"] = [dict(tz=0.1, bias=("1+z",), z_range=(0.2, 0.55), nbands=24, nside=256)]
        base["seed"] = 43
        base["bias_model"] = 1
    return base


@pytest.mark.parametrize("case", ["coarse", "fine"])
def test_imap_hits_equal_double(tmp_path, case):
    """Every sub-sample's shell and RING pixel (imap.c:179-231), decided as
    the GPU decides them, equals the oracle's double restatement: hit counts
    exactly; brightness (float sums) to 2e-6 relative."""
    import oracle as orc
    from colore_gb300 import inputs
    prm = orc.Params(inputs.write_inputs(str(tmp_path), _imap_spec(case)))
    cfg = prm.config
    n = cfg.n_grid
    d64, p64, st = orc.field64(cfg)
    dens = orc.density64(cfg, d64, st[3])
    d32 = dens.astype(np.float32)
    phi32 = p64.astype(np.float32)
    tabs, e0f, _ = orc.norm_tables64(cfg, d32.astype(np.float64))
    pad = lambda a: np.ascontiguousarray(np.pad(a, ((0, 0), (0, 0), (0, 2 * (n // 2 + 1) - n))))
    t64, e64 = tabs[0], np.asarray(e0f[0], np.float64)
    data32, nadd32, stats = orc.imap32(cfg, 0, pad(d32), pad(phi32), t64.astype(np.float32),
                                       e64.astype(np.float32), t64, e64)
    data64, nadd64 = orc.imap64(cfg, 0, d32.astype(np.float64), phi32.astype(np.float64), t64, e64)
    assert nadd64.sum() > 10 ** 6
    assert np.array_equal(nadd32, nadd64), int((nadd32 != nadd64).sum())
    np.testing.assert_allclose(data32, data64, rtol=2e-6, atol=1e-12)
    # the double path is the exception: the float margins leave ~2e-3 of
    # the samples open, the float-float tier settles their pixels, and what
    # remains are shells within the float radial shift's bound of an edge
    print("imap %s: %d of %d samples in double, %d cells" % (case, stats[1], stats[2], stats[0]))
    assert stats[1] < 1e-4 * stats[2], stats


# (128, 3.0): dx = 3 2^-7 and the observer at 1.5, so every sum is exact in
# double and often falls exactly half-way between two floats -- a tie the
# single-precision check leaves to double
@pytest.mark.parametrize("n_grid,l_box,fall", [(64, 874.993, 1e-4), (1024, 7727.3, 1e-4), (2048, 14401.7, 1e-4),
                                               (128, 3.0, 5e-2)])
def test_source_offset_in_single_precision(n_grid, l_box, fall):
    """The emission's source coordinate (float)(x0 + dx (u - 1/2)) of the
    double arithmetic (srcs.c:261-263), formed in single precision: whenever
    it claims certainty it equals the double expression rounded to float,
    including corners next to the observer (x0 near 0) and uniforms at the
    cell edges; it falls back for a few in a million (the margin is 2^-44
    of the corner against half a float ulp)."""
    import oracle as orc
    r = np.random.default_rng(n_grid)
    dx = l_box / n_grid
    pos_obs = 0.5 * l_box
    n = 400000
    i = r.integers(0, n_grid, n)
    x0 = i * dx - pos_obs
    bits = r.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    bits[:1000] = np.arange(1000) << 8                  # u near 0
    bits[1000:2000] = (2 ** 24 - 1 - np.arange(1000)) << 8  # u near 1
    x0[2000:3000] = (n_grid // 2) * dx - pos_obs        # the observer's cell
    out, ok, ref = orc.src_offset_checked(x0, dx, bits)
    assert np.array_equal(out[ok].view(np.uint32), ref[ok].view(np.uint32))
    assert 1 - ok.mean() < fall, 1 - ok.mean()


def test_ptrs_in_single_precision():
    """PTRS (Hormann 1993) for lambda >= 10 in single precision: wherever it
    decides, the count equals the double PTRS of the reference's mean, for
    float means anywhere within their bound of it; below lambda = 100 (where
    nearly all such cells are) 99.9 % of draws decide in single precision,
    88 % above 1000 (the logarithmic test's terms grow with lambda)."""
    import oracle as orc
    r = np.random.default_rng(3)
    n = 300000
    lam64 = np.exp(r.uniform(np.log(10.5), np.log(5e4), n))
    elam = (lam64 * 8 * 2.0 ** -24).astype(np.float32)
    lam = (lam64 * (1 + r.uniform(-1, 1, n) * 6 * 2.0 ** -24)).astype(np.float32)
    cid = r.integers(0, 2 ** 40, n)
    got, ref = orc.ptrs_checked(lam, elam, lam64, cid, 12345, 678)
    ok = got >= 0
    assert np.array_equal(got[ok], ref[ok])
    low = lam64 < 100
    assert ok[low].mean() > 0.99 and ok.mean() > 0.9, (ok[low].mean(), ok.mean())
