"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Integer results (Poisson counts, catalogue order, HEALPix ids, hit counts)
are compared bit for bit with the oracle's double restatement of the
reference (ref64), fed the same intermediate grids; the catalogue's float
columns and the other single-precision outputs also with the oracle evaluated
in the GPU's single-precision arithmetic (dev32).  Floating-point fields are compared with the FP64
restatement of the reference (ref64) within the stated tolerances:

  Gaussian field, potential     relative rms error <= 2e-6
  sigma^2 of the field          relative error <= 1e-5
  P(k) of the field per bin     relative error <= 1e-4
  lognormal field               bit-exact vs dev32 given the GPU Gaussian field
  1LPT displacements            relative rms error <= 2e-5 (literal r2c path)
  1LPT density                  relative rms error <= 1e-4
  redshift-bin sums             cell counts exact, sums relative 1e-6
  normalisation tables          relative 2e-4 vs FP64 (FP32 bin edges)
  intensity maps                hit counts equal the double arithmetic's,
                                brightness relative 2e-5
  convergence maps              bit-exact vs dev32; relative rms 1e-3 vs FP64
  custom maps                   bit-exact vs dev32; relative rms 1e-4 vs FP64
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_SMALL = 64


def _spec(kind):
    from colore_gb300 import inputs
    base = dict(n_grid=N_SMALL, z_min=0.05, z_max=0.6, r_smooth=2.0, seed=7, dens_type=0, bias_model=2,
                srcs=[dict(nz=("gauss", 0.3, 0.1), density=200.0, bias=("1+z",), nside_count=16, lensing=True,
                           skewers=True),
                      dict(nz=("flat", 0.1, 0.5), density=4.0, bias=("const", 2.0), nside_count=8)],
                imap=[dict(tz=0.1, bias=("const", 1.0), z_range=(0.1, 0.5), nbands=6, nside=16)],
                kappa=dict(z_out=[0.2, 0.4, 0.55], nside=16),
                isw=dict(z_out=[0.55, 0.3], nside=16),
                custom=[dict(kz=("gauss", 0.3, 0.08), bias=("const", 1.5), nside=16),
                        dict(kz=("flat", 0.2, 0.45), bias=("1+z",), nside=8, amp=-2.0)])
    if kind == "nobeam":
        base.pop("kappa")
        base["bias_model"] = 1
        base["seed"] = 11
    elif kind == "lpt":
        base["dens_type"] = 1
        base["seed"] = 13
        base["srcs"] = base["srcs"][:1]
    elif kind == "n96":
        base["n_grid"] = 96
        base["seed"] = 17
        base["bias_model"] = 3
        base.pop("kappa")
    elif kind == "ptrs":
        base["seed"] = 19
        base["srcs"] = [dict(nz=("gauss", 0.3, 0.15), density=30.0, bias=("const", 1.3), nside_count=16)]
        base.pop("imap")
        base.pop("kappa")
    elif kind == "lpt2":
        base["dens_type"] = 2
        base["seed"] = 47
        base["srcs"] = base["srcs"][:1]
        base.pop("kappa")
    elif kind in ("lpt_ngp", "lpt_tsc"):
        base["dens_type"] = 1
        base["lpt_interp_type"] = 0 if kind == "lpt_ngp" else 2
        base["seed"] = 37
        base["srcs"] = base["srcs"][:1]
        base.pop("kappa")
    elif kind == "heavy":
        # nside 64 from z = 0.05: the inner shells have nsub ~ 21 (heavy-cell
        # pass), the outer ones nsub ~ 3 (painted in place)
        base["seed"] = 29
        base["imap"] = [dict(tz=0.1, bias=("const", 1.0), z_range=(0.05, 0.5), nbands=6, nside=64)]
        base.pop("kappa")
    elif kind == "skwg":
        # Gaussian skewers and lensing on the second population
        base["seed"] = 31
        base["srcs"] = [base["srcs"][1]]
        base["srcs"][0].update(lensing=True, skewers=True, gaussian_skewers=True, density=30.0)
        base.pop("kappa")
    elif kind == "clip":
        base["dens_type"] = 3
        base["seed"] = 23
        base.pop("kappa")
    return base


class Run:
    """One GPU run with every intermediate downloaded.  A failing stage is
    recorded and re-raised by the tests that need it, so earlier stages are
    still checked."""

    def __init__(self, kind, tmpdir):
        self.error = None
        try:
            self._run(kind, tmpdir)
        except Exception as e:  # noqa: BLE001
            self.error = e

    def need(self, attr):
        if not hasattr(self, attr):
            raise self.error if self.error else AttributeError(attr)
        return getattr(self, attr)

    def _run(self, kind, tmpdir):
        import colore_gb300 as cg
        from colore_gb300 import inputs
        self.kind = kind
        self.params = cg.Params(inputs.write_inputs(tmpdir, _spec(kind)))
        self.cfg = self.params.config
        m = cg.Mock(self.params)
        self.m = m
        m.create_cartesian_fields()
        self.dG = m.grid(0).copy()
        self.phi = m.grid(1).copy()
        self.s2, self.mean = m.sigma2()
        m.compute_physical_density_field()
        if self.cfg.dens_type in (1, 2):
            self.disp = [m.grid(w).copy() for w in (2, 3, 4)]
        if self.cfg.dens_type == 2:
            self.disp2 = [m.grid(w).copy() for w in (5, 6, 7)]
        m.compute_density_normalization()
        self.d = m.grid(0).copy()
        self.norm_s = [m.norm_table(0, i) for i in range(self.cfg.n_srcs)]
        self.norm_s64 = [m.norm_table64(0, i) for i in range(self.cfg.n_srcs)]
        self.norm_i64 = [m.norm_table64(1, i) for i in range(self.cfg.n_imap)]
        self.norm_i = [m.norm_table(1, i) for i in range(self.cfg.n_imap)]
        self.norm_c = [m.norm_table(2, i) for i in range(self.cfg.n_cstm)]
        m.exact_stats(reset=True)
        self.nsrc = m.srcs_set_cartesian()
        self.xstats_srcs = m.exact_stats(reset=True)
        self.cats = [m.catalog(i) for i in range(self.cfg.n_srcs)]
        self.cmaps = [m.count_map(i) if self.cfg.nside_count[i] > 0 else None for i in range(self.cfg.n_srcs)]
        m.imap_set_cartesian()
        self.xstats_imap = m.exact_stats(reset=True)
        self.imaps = [m.imap(i, with_nadd=True) for i in range(self.cfg.n_imap)]
        m.get_beam_properties()
        self.cats_beam = [m.catalog(i, pos=False, ipix=False) for i in range(self.cfg.n_srcs)]
        self.kappa = m.kappa() if self.cfg.do_kappa else None
        self.isw = m.isw() if self.cfg.do_isw else None
        self.cstm = [m.custom(i) for i in range(self.cfg.n_cstm)]
        self.skw = [m.skewers(i) if self.cfg.skw_srcs[i] else None for i in range(self.cfg.n_srcs)]


_RUNS = {}


@pytest.fixture(scope="module")
def runs(built, tmp_path_factory):
    def get(kind):
        if kind not in _RUNS:
            _RUNS[kind] = Run(kind, str(tmp_path_factory.mktemp(kind)))
        return _RUNS[kind]
    return get


def unpad(g):
    return g[:, :, :g.shape[0]]


def rel_rms(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.sqrt(np.mean((a - b) ** 2) / np.mean(b ** 2))


def pk_bins(f, lbox, nb=12):
    n = f.shape[0]
    fk = np.fft.rfftn(f)
    kf = 2 * np.pi / lbox
    kx = np.arange(n // 2 + 1)
    ky = np.fft.fftfreq(n, 1.0 / n)
    kk = np.sqrt(kx[None, None, :] ** 2 + ky[None, :, None] ** 2 + ky[:, None, None] ** 2)
    b = np.minimum((kk / (n / 2) * nb).astype(int), nb)
    p = np.bincount(b.ravel(), weights=(np.abs(fk) ** 2).ravel(), minlength=nb + 1)
    c = np.bincount(b.ravel(), minlength=nb + 1)
    return (p / np.maximum(c, 1))[1:nb]


@pytest.mark.parametrize("n", [64, 96, 128, 192, 256])
def test_field_transform_all_sizes(built, tmp_path, n):
    """create_cartesian_fields alone at every supported size up to 256^3:
    radix 2, 4, 8, 16, 32 and 3 (96, 192) plans against the FP64 oracle."""
    import colore_gb300 as cg
    from colore_gb300 import inputs
    import oracle as orc
    spec = dict(n_grid=n, z_min=0.05, z_max=0.6, r_smooth=2.0, seed=3 + n, dens_type=0, bias_model=2)
    prm = cg.Params(inputs.write_inputs(str(tmp_path), spec))
    m = cg.Mock(prm)
    m.create_cartesian_fields()
    g = m.grid(0)
    p = m.grid(1)
    s2, _ = m.sigma2()
    d64, p64, st = orc.field64(prm.config)
    assert rel_rms(unpad(g), d64) < 2e-6
    assert rel_rms(unpad(p), p64) < 2e-6
    assert abs(s2 / st[3] - 1) < 1e-5


@pytest.mark.parametrize("kind", ["full", "n96"])
def test_gaussian_field_vs_fp64(runs, kind):
    import oracle as orc
    r = runs(kind)
    d64, p64, st = orc.field64(r.cfg)
    assert rel_rms(unpad(r.dG), d64) < 2e-6
    assert rel_rms(unpad(r.phi), p64) < 2e-6
    assert abs(r.s2 / st[3] - 1) < 1e-5
    pg = pk_bins(unpad(r.dG).astype(np.float64), r.cfg.l_box)
    po = pk_bins(d64, r.cfg.l_box)
    assert np.max(np.abs(pg / po - 1)) <= 1e-4


@pytest.mark.parametrize("kind", ["full", "nobeam", "n96", "clip"])
def test_physical_density_bitexact(runs, kind):
    import oracle as orc
    r = runs(kind)
    mode = {0: 1, 3: 2}[r.cfg.dens_type]
    ref = orc.density32(r.cfg, r.dG, np.float32(r.s2), mode)
    assert np.array_equal(unpad(ref), unpad(r.need('d')))


def test_lognormal_vs_fp64(runs):
    import oracle as orc
    r = runs("full")
    ref = orc.density64(r.cfg, unpad(r.dG).astype(np.float64), r.s2)
    assert rel_rms(unpad(r.need('d')), ref) < 5e-6


def test_lpt_vs_fp64_literal_path(runs):
    """The GPU builds Psi_k from the regenerated modes; the oracle takes the
    reference's route: r2c of the Gaussian grid, then Psi_k (density.c:392-440)."""
    import oracle as orc
    r = runs("lpt")
    d64, _, _ = orc.field64(r.cfg)
    out, disp = orc.lpt64(r.cfg, d64)
    for a in range(3):
        assert rel_rms(unpad(r.need('disp')[a]), disp[a]) < 2e-5, a
    assert rel_rms(unpad(r.need('d')), out) < 1e-4


def test_2lpt_vs_fp64(runs):
    """2LPT (density.c:646-1031): first- and second-order displacements and
    the deposited density against the FP64 restatement, which takes the
    reference's literal route (r2c of the Gaussian field and of the source).
    The second order goes through an FP32 r2c of a source made of products
    of FP32 derivatives: relative rms 1e-4."""
    import oracle as orc
    r = runs("lpt2")
    d64, _, _ = orc.field64(r.cfg)
    out, d1, d2 = orc.lpt2_64(r.cfg, d64)
    for a in range(3):
        assert rel_rms(unpad(r.need('disp')[a]), d1[a]) < 2e-5, a
        assert rel_rms(unpad(r.need('disp2')[a]), d2[a]) < 1e-4, (a, rel_rms(unpad(r.need('disp2')[a]), d2[a]))
    assert rel_rms(unpad(r.need('d')), out) < 1e-4
    assert np.std(d2[0]) > 1e-3 * np.std(d1[0])


@pytest.mark.parametrize("kind", ["lpt_ngp", "lpt_tsc"])
def test_lpt_deposit_schemes_vs_fp64(runs, kind):
    """NGP and TSC mass assignment (density.c:37-62, 107-176) against the FP64
    restatement.  The mass is conserved (mean of 1 + delta is 1).  TSC is
    continuous, so it agrees like CIC; NGP moves a whole particle when an FP32
    position and an FP64 one fall on either side of a cell edge, so for NGP
    the test counts the cells that differ."""
    import oracle as orc
    r = runs(kind)
    d64, _, _ = orc.field64(r.cfg)
    out, _ = orc.lpt64(r.cfg, d64)
    got = unpad(r.need('d')).astype(np.float64)
    assert abs(np.mean(got + 1.0) - 1.0) < 1e-6 and abs(np.mean(out + 1.0) - 1.0) < 1e-12
    if kind == "lpt_tsc":
        assert rel_rms(got, out) < 1e-4
    else:
        diff = np.abs(got - out) > 1e-3
        assert diff.mean() < 1e-3, diff.mean()
        assert np.all(np.abs(np.round(got + 1.0) - (got + 1.0)) < 1e-4)  # whole particles per cell


@pytest.mark.parametrize("kind", ["full", "lpt"])
def test_redshift_bin_sums(runs, kind):
    import oracle as orc
    r = runs(kind)
    zmax = np.interp(0.5 * r.cfg.l_box, np.ctypeslib.as_array(r.cfg.r_arr_r2z, (5001,)),
                     np.ctypeslib.as_array(r.cfg.z_arr_r2z, (5001,)))
    nz = int(zmax / 0.05) + 2
    idz = (nz - 2) / zmax
    import ctypes as C
    import colore_gb300 as cg
    nt = r.cfg.n_srcs + r.cfg.n_imap
    narr = np.empty(nz, np.uint64)
    zarr = np.empty(nz)
    bs = np.empty((r.cfg.n_srcs, nz))
    bi = np.empty((max(r.cfg.n_imap + r.cfg.n_cstm, 1), nz))
    rc = cg.lib().cg_collect_density_normalization(
        r.m._c, nz, idz, zarr.ctypes.data_as(C.POINTER(C.c_double)),
        narr.ctypes.data_as(C.POINTER(C.c_ulonglong)), bs.ctypes.data_as(C.POINTER(C.c_double)),
        bi.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == 0
    n32, z32, b32 = orc.bins32(r.cfg, r.need('d'), nz, idz)
    assert np.array_equal(n32, narr)
    ok = narr > 0
    assert np.allclose(zarr[ok], z32[ok], rtol=1e-6)
    gb = np.concatenate([bs, bi[:r.cfg.n_imap + r.cfg.n_cstm]])
    assert np.allclose(gb[:, ok], b32[:, ok], rtol=1e-6)


@pytest.mark.parametrize("kind", ["full", "nobeam", "lpt", "n96", "ptrs", "clip"])
def test_norm_tables_vs_fp64(runs, kind):
    """compute_density_normalization (density.c:1227-1355): the FP32 tables the
    kernels use against the FP64 oracle's, from the same physical field.

    The GPU places each cell in a redshift bin from its FP32 radius and z(r),
    so a few cells within ~1e-7 of a bin edge land in the neighbouring bin;
    with 64^3 cells and bins of a few hundred cells that moves a table entry by
    up to ~1e-4 relative (5e-5 seen).  The bins themselves are checked exactly
    against the FP32 restatement in test_redshift_bin_sums."""
    import oracle as orc
    r = runs(kind)
    tabs, e0f, nz = orc.norm_tables64(r.cfg, unpad(r.need('d')).astype(np.float64))
    got = r.need('norm_s') + r.need('norm_i') + r.need('norm_c')
    assert len(got) == r.cfg.n_srcs + r.cfg.n_imap + r.cfg.n_cstm
    for t, (tab, e) in enumerate(got):
        assert np.all(np.isfinite(tab)), (t, tab[~np.isfinite(tab)][:5])
        assert np.allclose(tab, tabs[t], rtol=2e-4), (t, np.max(np.abs(tab / tabs[t] - 1)))
        assert np.allclose(e, e0f[t], rtol=2e-4)


@pytest.mark.parametrize("kind", ["full", "nobeam", "lpt", "n96", "ptrs", "clip"])
def test_sources_equal_double_arithmetic(runs, kind):
    """Counts of every cell, positions, base-pixel ids and count maps equal
    the oracle's double restatement of the reference (srcs.c:156-283,
    386-416) on the same density, potential and normalisation table, bit for
    bit; RA, Dec, z and the RSD shift agree to single-precision accuracy."""
    import oracle as orc
    r = runs(kind)
    for ip in range(r.cfg.n_srcs):
        t64, e64 = r.need('norm_s64')[ip]
        c64, tot64 = orc.counts64(r.cfg, ip, r.need('d'), t64, e64)
        assert tot64 == r.need('nsrc')[ip], (tot64, r.need('nsrc')[ip])
        o = orc.emit64(r.cfg, ip, r.phi, c64, cap=tot64 + 16)
        g = r.need('cats')[ip]
        assert np.array_equal(o["pos"][:, :3].view(np.uint32), g["pos"][:, :3].view(np.uint32))
        assert np.array_equal(o["ipix"], g["ipix"])
        if r.need('cmaps')[ip] is not None:
            assert np.array_equal(o["cmap"], r.need('cmaps')[ip])
        np.testing.assert_allclose(g["pos"][:, 3], o["pos"][:, 3], rtol=1e-4, atol=1e-3)
        if not r.cfg.need_beaming:
            dra = np.abs(g["src"][:, 0] - o["src"][:, 0])
            assert np.all(np.minimum(dra, 360 - dra) < 2e-4)
            assert np.max(np.abs(g["src"][:, 1] - o["src"][:, 1])) < 2e-4
            np.testing.assert_allclose(g["src"][:, 2], o["src"][:, 2], rtol=2e-6, atol=1e-7)
    print(kind, "decisions in double:", r.need('xstats_srcs'))


def test_sources_all_decisions_in_double(runs, tmp_path):
    """With every count and pixel decided by the device's double arithmetic
    the catalogue is the same: the double restatement on the device agrees
    with the float margins everywhere."""
    import colore_gb300 as cg
    from colore_gb300 import inputs
    r = runs("full")
    m = cg.Mock(cg.Params(inputs.write_inputs(str(tmp_path), _spec("full"))))
    m.set_decisions_in_double(True)
    m.create_cartesian_fields()
    m.compute_physical_density_field()
    m.compute_density_normalization()
    m.exact_stats(reset=True)
    nsrc = m.srcs_set_cartesian()
    st = m.exact_stats()
    assert list(nsrc) == list(r.need('nsrc'))
    assert st["count_cells"] > 1000 and st["src_pixels"] >= 2 * sum(nsrc)
    for ip in range(r.cfg.n_srcs):
        g = m.catalog(ip)
        for k in ("pos", "ipix"):
            assert np.array_equal(g[k], r.need('cats')[ip][k]), k
    m.close()


@pytest.mark.parametrize("kind", ["full", "nobeam", "lpt", "n96", "ptrs", "clip"])
def test_sources_bitexact(runs, kind):
    """Counts, catalogue order, positions, base-pixel ids, ra/dec/z, RSD and
    the count map equal the dev32 restatement (the CPU mirror of the kernels'
    arithmetic) bit for bit."""
    import oracle as orc
    r = runs(kind)
    for ip in range(r.cfg.n_srcs):
        tab, e = r.need('norm_s')[ip]
        t64, e64 = r.need('norm_s64')[ip]
        ref = orc.emit32(r.cfg, ip, r.need('d'), r.phi, tab, e, t64, e64, cap=int(r.need('nsrc')[ip] * 1.2) + 100)
        g = r.need('cats')[ip]
        assert len(ref["pos"]) == r.need('nsrc')[ip]
        assert np.array_equal(ref["pos"].view(np.uint32), g["pos"].view(np.uint32))
        assert np.array_equal(ref["ipix"], g["ipix"])
        assert np.array_equal(ref["src"].view(np.uint32), g["src"].view(np.uint32))
        if r.need('cmaps')[ip] is not None:
            assert np.array_equal(ref["cmap"], r.need('cmaps')[ip])
            assert r.need('cmaps')[ip].sum() == r.need('nsrc')[ip]


@pytest.mark.parametrize("kind", ["full", "lpt", "skwg"])
def test_beam_rsd_bitexact(runs, kind):
    """RSD at the sources, and with include_lensing the shear, convergence and
    deflection integrated to each source, bit for bit."""
    import oracle as orc
    r = runs(kind)
    assert r.cfg.need_beaming
    for ip in range(r.cfg.n_srcs):
        pos = r.need('cats')[ip]["pos"]
        s = orc.beam_rsd32(r.cfg, r.phi, pos, r.need('cats')[ip]["src"])
        if r.cfg.lensing_srcs[ip]:
            s = orc.lens32(r.cfg, r.phi, pos, s)
        assert np.array_equal(s.view(np.uint32), r.need('cats_beam')[ip]["src"].view(np.uint32))


@pytest.mark.parametrize("kind", ["full", "skwg"])
def test_source_lensing_vs_fp64(runs, kind):
    """Source lensing (srcs.c:536-625) against the FP64 restatement of the
    reference on the same potential: relative rms 2e-3 per quantity (the
    nearest cell of a step can differ between FP32 and FP64 positions)."""
    import oracle as orc
    r = runs(kind)
    ip = [i for i in range(r.cfg.n_srcs) if r.cfg.lensing_srcs[i]][0]
    got = r.need('cats_beam')[ip]["src"][:, 4:9].astype(np.float64)
    assert len(got) > 100
    ref = orc.lens64(r.cfg, unpad(r.phi).astype(np.float64), r.need('cats')[ip]["pos"])
    for j in range(5):
        assert rel_rms(got[:, j], ref[:, j]) < 2e-3, (j, rel_rms(got[:, j], ref[:, j]))


@pytest.mark.parametrize("kind", ["full", "skwg"])
def test_skewers_bitexact_and_fp64(runs, kind):
    """Density (or Gaussian) and velocity skewers (srcs.c:509-536, 725-733):
    bit-exact against the FP32 restatement.  Against FP64, a source whose
    r/dr + 1/2 lies within rounding of an integer ends one step earlier or
    later (a few in 1e6); the others agree to relative rms 2e-5."""
    import oracle as orc
    r = runs(kind)
    ip = [i for i in range(r.cfg.n_srcs) if r.cfg.skw_srcs[i]][0]
    gauss = r.cfg.skw_gauss[ip]
    assert gauss == (kind == "skwg")
    d, v = r.need('skw')[ip]
    pos = r.need('cats')[ip]["pos"]
    assert d.shape == (len(pos), r.cfg.n_grid // 2) and np.all(np.isfinite(d))
    d32, v32 = orc.skw32(r.cfg, r.need('d'), r.phi, gauss, np.float32(r.s2), pos)
    assert np.array_equal(d32.view(np.uint32), d.view(np.uint32))
    assert np.array_equal(v32.view(np.uint32), v.view(np.uint32))
    d64, v64 = orc.skw64(r.cfg, unpad(r.need('d')).astype(np.float64), unpad(r.phi).astype(np.float64), gauss,
                         r.s2, pos)
    same_end = np.all((d != 0) == (d64 != 0), axis=1)
    assert (~same_end).sum() <= 1e-5 * len(pos) + 4, (~same_end).sum()
    assert rel_rms(d[same_end], d64[same_end]) < 2e-5 and rel_rms(v[same_end], v64[same_end]) < 2e-5


@pytest.mark.parametrize("kind", ["full", "nobeam", "lpt", "ptrs"])
def test_source_counts_vs_fp64_mean(runs, kind):
    """The FP64 Poisson means summed over cells predict the GPU count."""
    import oracle as orc
    r = runs(kind)
    for ip in range(r.cfg.n_srcs):
        tab, e = r.need('norm_s')[ip]
        lam = orc.lambda64(r.cfg, ip, unpad(r.need('d')).astype(np.float64), tab.astype(np.float64), e)
        mu = lam.sum()
        assert abs(r.need('nsrc')[ip] - mu) < 5 * np.sqrt(mu) + 5, (r.need('nsrc')[ip], mu)


def _imap64(r, ip):
    import oracle as orc
    t64, e64 = r.need('norm_i64')[ip]
    data, nadd = orc.imap64(r.cfg, ip, unpad(r.need('d')).astype(np.float64), unpad(r.phi).astype(np.float64),
                            t64, e64)
    return np.where(nadd > 0, data / np.maximum(nadd, 1), 0), nadd


@pytest.mark.parametrize("kind", ["full", "nobeam", "lpt", "n96", "heavy"])
def test_imap_equal_double_arithmetic(runs, kind):
    """Every sub-sample's shell and RING pixel (imap.c:179-231) as the
    reference's double arithmetic decides it, on the same density, potential
    and normalisation table: hit counts equal the oracle's double
    restatement's exactly; the brightness per pixel (float sums of the
    cells' float brightness) within 2e-5 relative."""
    r = runs(kind)
    for ip in range(r.cfg.n_imap):
        ref, nadd = _imap64(r, ip)
        gm, gn = r.need('imaps')[ip]
        assert gn.sum() > 0
        assert np.array_equal(gn, nadd), int((gn != nadd).sum())
        np.testing.assert_allclose(gm, ref, rtol=2e-5, atol=1e-12)


def test_imap_all_decisions_in_double(runs, tmp_path):
    """With every cell and sample decided by the device's double arithmetic
    (the queue of the double pass takes them all) the maps are the same."""
    import colore_gb300 as cg
    from colore_gb300 import inputs
    r = runs("heavy")
    m = cg.Mock(cg.Params(inputs.write_inputs(str(tmp_path), _spec("heavy"))))
    m.set_decisions_in_double(True)
    m.create_cartesian_fields()
    m.compute_physical_density_field()
    m.compute_density_normalization()
    m.exact_stats(reset=True)
    m.imap_set_cartesian()
    st = m.exact_stats()
    assert st["imap_samples"] == m.imap_samples(0) and st["imap_cells"] > 1000
    gm, gn = m.imap(0, with_nadd=True)
    rm, rn = r.need('imaps')[0]
    assert np.array_equal(gn, rn)
    np.testing.assert_allclose(gm, rm, rtol=1e-5, atol=1e-12)
    m.close()


@pytest.mark.parametrize("cap", [1, 3000])
def test_imap_list_overflow(runs, cap):
    """With the cell list bounded, the cells past the bound are painted by the
    listing kernel itself (the path a run takes when the list would not fit
    in device memory): the same hit counts as the double arithmetic, the same
    sample count, brightness within float rounding."""
    r = runs("full")
    want_n = [r.m.imap_samples(ip) for ip in range(r.cfg.n_imap)]
    r.m.set_imap_list_cap(cap)
    try:
        r.m.imap_set_cartesian()
        got = [r.m.imap(ip, with_nadd=True) for ip in range(r.cfg.n_imap)]
        got_n = [r.m.imap_samples(ip) for ip in range(r.cfg.n_imap)]
    finally:
        r.m.set_imap_list_cap(0)
    assert got_n == want_n
    for ip in range(r.cfg.n_imap):
        ref, nadd = _imap64(r, ip)
        gm, gn = got[ip]
        assert np.array_equal(gn, nadd)
        np.testing.assert_allclose(gm, ref, rtol=2e-5, atol=1e-12)


@pytest.mark.parametrize("kind", ["full", "heavy"])
def test_imap_sample_count(runs, kind):
    """Sub-samples drawn (cells in range x nsub^3, imap.c:184-231) equal the
    count of the double arithmetic from the geometry."""
    import oracle as orc
    r = runs(kind)
    r.need('imaps')
    for ip in range(r.cfg.n_imap):
        want = orc.lib().or_imap_samples(orc.cfgp(r.cfg), ip)
        got = r.m.imap_samples(ip)
        assert want > 0 and got == want, (got, want)


@pytest.mark.parametrize("kind", ["full", "lpt"])
def test_kappa_bitexact_and_fp64(runs, kind):
    import oracle as orc
    r = runs(kind)
    ref32 = orc.kappa32(r.cfg, r.phi)
    assert np.array_equal(ref32.view(np.uint32), r.need('kappa').view(np.uint32))
    ref64 = orc.kappa64(r.cfg, unpad(r.phi).astype(np.float64))
    assert rel_rms(r.need('kappa'), ref64) < 1e-3


def test_isw_bitexact_and_fp64(runs):
    """ISW maps (isw.c:78-147): bit-exact against the FP32 restatement fed the
    GPU potential; against the FP64 reference within 1e-3 rms (the nearest
    cell of a ray step can differ between FP32 and FP64 positions)."""
    import oracle as orc
    r = runs("full")
    got = r.need('isw')
    assert got.shape == (2, 12 * 16 * 16) and np.all(np.isfinite(got))
    ref32 = orc.isw32(r.cfg, r.phi)
    assert np.array_equal(ref32.view(np.uint32), got.view(np.uint32))
    ref64 = orc.isw64(r.cfg, unpad(r.phi).astype(np.float64))
    assert rel_rms(got, ref64) < 1e-3
    # maps come in order of distance (isw_beams_preproc sorts the planes) and
    # are cumulative along the ray, so the two differ
    assert not np.allclose(got[0], got[1])


def test_custom_maps_bitexact_and_fp64(runs):
    """Custom maps (cstm.c:68-145): bit-exact against the FP32 restatement fed
    the GPU density and normalisation table; against the FP64 restatement of
    the reference fed the same density within 1e-4 rms (FP32 positions and
    step tables).  Maps are in NEST order, as the reference writes them."""
    import oracle as orc
    r = runs("full")
    assert r.cfg.n_cstm == 2
    for ip in range(2):
        got = r.need('cstm')[ip]
        ns = r.cfg.nside_cstm[ip]
        assert got.shape == (12 * ns * ns,) and np.all(np.isfinite(got)) and np.any(got != 0)
        tab, e = r.norm_c[ip]
        ref32 = orc.cstm32(r.cfg, ip, r.need('d'), tab, e)
        assert np.array_equal(ref32.view(np.uint32), got.view(np.uint32)), ip
        ref64 = orc.cstm64(r.cfg, ip, unpad(r.need('d')).astype(np.float64), tab.astype(np.float64),
                           e.astype(np.float64))
        assert rel_rms(got, ref64) < 1e-4, ip
    # kernel 2 has the opposite sign and another support
    assert np.corrcoef(r.cstm[0], np.repeat(r.cstm[1], 4))[0, 1] < 0.5


def test_rerun_is_deterministic(runs, tmp_path):
    import colore_gb300 as cg
    r = runs("full")
    m = cg.Mock(r.params)
    m.run()
    assert np.array_equal(unpad(m.grid(0)), unpad(r.need('d')))
    for ip in range(r.cfg.n_srcs):
        assert np.array_equal(m.catalog(ip, src=False)["pos"], r.need('cats')[ip]["pos"])
    assert np.array_equal(m.kappa(), r.kappa)
    assert m.launches() > 0
    # the normalisation sums do not depend on the order the blocks finish
    m2 = cg.Mock(r.params)
    m2.run()
    for kind, npop in ((0, r.cfg.n_srcs), (1, r.cfg.n_imap)):
        for ip in range(npop):
            for a, b in zip(m.norm_table64(kind, ip), m2.norm_table64(kind, ip)):
                assert np.array_equal(a.view(np.uint64), b.view(np.uint64)), (kind, ip)
    m2.close()


def test_stage_order_is_enforced(runs):
    import colore_gb300 as cg
    r = runs("full")
    m = cg.Mock(r.params)
    with pytest.raises(cg.CGError, match="stage out of order"):
        m.srcs_set_cartesian()
    with pytest.raises(cg.CGError, match="stage out of order"):
        m.compute_physical_density_field()
