"""Graph-captured sequence and batches of realisations (cg_graph_*,
cg_batch_*): a replay gives the plain run's catalogue bit for bit, and so
does every realisation of a batch whose graphs run side by side on several
streams.  The whole sequence is captured, intensity maps and line-of-sight
quantities included: a replay gives the plain run's catalogue (with RSD,
lensing and skewer columns), count maps, convergence and ISW maps bit for
bit, the intensity maps' hit counts exactly and their brightness sums to
float atomics' rounding (2e-6)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _spec(n, seed, zmax=0.5):
    return dict(n_grid=n, z_min=0.05, z_max=zmax, r_smooth=2.0, seed=seed, dens_type=0, bias_model=2,
                srcs=[dict(nz=("flat", 0.05, zmax), density=60.0, bias=("const", 1.5), nside_count=16)])


def _params(tmp_path, spec, tag):
    import colore_gb300 as cg
    from colore_gb300 import inputs
    return cg.Params(inputs.write_inputs(str(tmp_path / tag), spec))


def _catalog(m):
    c = m.catalog(0)
    return c["pos"], c["ipix"], c["src"], m.count_map(0)


def test_graph_replay_matches_plain_run(built, tmp_path):
    import colore_gb300 as cg
    import oracle as orc
    prm = _params(tmp_path, _spec(64, 71), "g")
    m = cg.Mock(prm)
    m.run()
    ref = _catalog(m)
    n0 = m.num_sources(0)
    m.graph_capture()
    l0 = m.launches()
    for _ in range(2):
        m.graph_launch()
        assert m.num_sources(0) == n0
        got = _catalog(m)
        for a, b in zip(ref, got):
            assert np.array_equal(a, b)
    assert m.launches() > l0
    # the replayed pipeline against the oracle: emit from the replay's own
    # density and normalisation table
    tab, e = m.norm_table(0, 0)
    t64, e64 = m.norm_table64(0, 0)
    o = orc.emit32(prm.config, 0, m.grid(0), m.grid(1), tab, e, t64, e64, cap=n0 + 100)
    assert np.array_equal(o["pos"].view(np.uint32), ref[0].view(np.uint32))
    m.close()


def _c4_style(n, seed):
    spec = _spec(n, seed, zmax=0.45)
    spec["dens_type"] = 1
    spec["srcs"][0]["lensing"] = True
    spec["srcs"][0]["skewers"] = True
    spec["imap"] = [dict(tz=0.1, bias=("const", 1.0), z_range=(0.1, 0.4), nbands=6, nside=32)]
    spec["kappa"] = dict(z_out=[0.2, 0.4], nside=16)
    spec["isw"] = dict(z_out=[0.3], nside=16)
    return spec


def _all_outputs(m):
    out = list(_catalog(m))
    out += list(m.skewers(0))
    out += [m.kappa(), m.isw()]
    data, nadd = m.imap(0, with_nadd=True)
    return out, data, nadd


def test_graph_replay_with_maps_and_beams(built, tmp_path):
    import colore_gb300 as cg
    m = cg.Mock(_params(tmp_path, _c4_style(64, 72), "k"))
    m.run()
    ref, rdata, rnadd = _all_outputs(m)
    n0 = m.num_sources(0)
    assert n0 > 0 and rnadd.sum() > 0
    m.graph_capture()
    for _ in range(2):
        m.graph_launch()
        assert m.num_sources(0) == n0
        got, data, nadd = _all_outputs(m)
        for k, (a, b) in enumerate(zip(ref, got)):
            assert np.array_equal(a, b), k
        assert np.array_equal(nadd, rnadd)
        np.testing.assert_allclose(data, rdata, rtol=2e-6, atol=0)
        assert m.imap_samples(0) > 0
    m.close()


def test_batch_of_c4_style_realisations(built, tmp_path):
    """Intensity maps, convergence and 1LPT in a batch: each realisation's
    outputs equal those of the same configuration run alone."""
    import colore_gb300 as cg
    prms = [_params(tmp_path, _c4_style(n, 120 + i), "c%d" % i) for i, n in enumerate([64, 96, 64])]
    b = cg.Batch(prms, nstreams=2)
    b.run()
    for i, p in enumerate(prms):
        m = cg.Mock(p)
        m.run()
        ref, rdata, rnadd = _all_outputs(m)
        got, data, nadd = _all_outputs(b.mocks[i])
        for k, (x, y) in enumerate(zip(ref, got)):
            assert np.array_equal(x, y), (i, k)
        assert np.array_equal(nadd, rnadd), i
        np.testing.assert_allclose(data, rdata, rtol=2e-6, atol=0)
        m.close()
    b.close()


def test_batch_matches_separate_runs(built, tmp_path):
    """Six realisations of three grid sizes, graphs over autotuned streams:
    each catalogue equals the one of the same configuration run alone."""
    import colore_gb300 as cg
    specs = [_spec(n, 80 + i, zmax=0.3 + 0.05 * i) for i, n in enumerate([64, 96, 128, 64, 96, 128])]
    prms = [_params(tmp_path, s, "b%d" % i) for i, s in enumerate(specs)]
    b = cg.Batch(prms)
    assert b.streams in (1, 2, 4, 8, 16) and len(b.tuning()) == 5
    for _ in range(2):
        ms = b.run()
        assert ms > 0
    for i, p in enumerate(prms):
        m = cg.Mock(p)
        m.run()
        ref = _catalog(m)
        got = _catalog(b.mocks[i])
        assert b.mocks[i].num_sources(0) == m.num_sources(0) > 0
        for x, y in zip(ref, got):
            assert np.array_equal(x, y), i
        m.close()
    b.close()


def test_batch_fixed_streams(built, tmp_path):
    import colore_gb300 as cg
    prms = [_params(tmp_path, _spec(64, 90 + i), "f%d" % i) for i in range(3)]
    b = cg.Batch(prms, nstreams=2)
    assert b.streams == 2 and b.tuning() == []
    b.run()
    assert all(m.num_sources(0) > 0 for m in b.mocks)
    b.close()


def _pinned(shape, dtype):
    torch = pytest.importorskip("torch")
    t = torch.empty(shape, dtype={np.float32: torch.float32, np.int64: torch.int64}[dtype], pin_memory=True)
    return t, t.numpy()


def test_batch_host_catalogs(built, tmp_path):
    """cg_batch_set_host_catalog: each pass copies every realisation's Src
    array into page-locked host memory behind its graph; the copies equal
    the catalogues downloaded afterwards, a short buffer receives its first
    cap sources and the full count, and pageable memory is refused."""
    import colore_gb300 as cg
    prms = [_params(tmp_path, _spec(n, 110 + i), "h%d" % i) for i, n in enumerate([64, 96, 128, 64])]
    b = cg.Batch(prms, nstreams=2)
    b.run()
    ns = [m.num_sources(0) for m in b.mocks]
    keep = []
    outs = []
    for i, n in enumerate(ns):
        cap = n + 64 if i != 3 else n // 2  # the last one too short
        ts, src = _pinned((cap, 9), np.float32)
        tn, cnt = _pinned((1,), np.int64)
        src[:] = -7.0
        cnt[0] = -1
        keep += [ts, tn]
        b.set_host_catalog(i, 0, src, cnt)
        outs.append((src, cnt, cap))
    for _ in range(2):
        b.run()
        for i, (src, cnt, cap) in enumerate(outs):
            n = b.mocks[i].num_sources(0)
            assert cnt[0] == n == ns[i]
            ref = b.mocks[i].catalog(0, pos=False, ipix=False)["src"]
            k = min(n, cap)
            assert np.array_equal(src[:k], ref[:k]), i  # records past the count are unspecified
    with pytest.raises(cg.CGError, match="pinned"):
        b.set_host_catalog(0, 0, np.zeros((10, 9), np.float32), np.zeros(1, np.int64))
    b.set_host_catalog(1, 0, None, None)
    b.close()
