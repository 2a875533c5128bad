"""Graph-captured sequence and batches of realisations (cg_graph_*,
cg_batch_*): a replay gives the plain run's catalogue bit for bit, and so
does every realisation of a batch whose graphs run side by side on several
streams; configurations with intensity maps or line-of-sight quantities are
refused."""
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


def test_graph_refuses_maps_and_beams(built, tmp_path):
    import colore_gb300 as cg
    spec = _spec(64, 72)
    spec["kappa"] = dict(z_out=[0.3], nside=8)
    m = cg.Mock(_params(tmp_path, spec, "k"))
    with pytest.raises(cg.CGError, match="graph capture covers"):
        m.graph_capture()
    m.close()


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
