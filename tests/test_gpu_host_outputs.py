"""Host outputs (cg_set_host_catalog / _imap / _kappa): the stages copy each
output into page-locked host memory as it becomes final, on a copy stream
that overlaps the later stages.  After cg_sync the host arrays equal what
the download calls give, run after run; short catalogue buffers get their
first cap sources and the full count; pageable memory is refused."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pinned(shape, dtype):
    torch = pytest.importorskip("torch")
    t = torch.empty(shape, dtype={np.float32: torch.float32, np.int64: torch.int64}[dtype], pin_memory=True)
    return t, t.numpy()


def _spec():
    return dict(n_grid=64, z_min=0.05, z_max=0.6, r_smooth=2.0, seed=31, dens_type=1, bias_model=2,
                srcs=[dict(nz=("gauss", 0.3, 0.1), density=200.0, bias=("1+z",), nside_count=16, lensing=True),
                      dict(nz=("flat", 0.1, 0.5), density=20.0, bias=("const", 2.0), nside_count=8)],
                imap=[dict(tz=0.1, bias=("const", 1.0), z_range=(0.1, 0.5), nbands=6, nside=16)],
                kappa=dict(z_out=[0.2, 0.4, 0.55], nside=16))


def test_host_outputs_match_downloads(built, tmp_path):
    import colore_gb300 as cg
    from colore_gb300 import inputs
    prm = cg.Params(inputs.write_inputs(str(tmp_path), _spec()))
    cfg = prm.config
    m = cg.Mock(prm)
    m.run()
    m.sync()
    ns = [m.num_sources(i) for i in range(cfg.n_srcs)]
    keep = []
    cats = {}
    for i, n in enumerate(ns):
        cap = n + 100 if i == 0 else max(n // 3, 1)  # the second buffer too short
        ts, src = _pinned((cap, 9), np.float32)
        tn, cnt = _pinned((1,), np.int64)
        src[:] = -5.0
        keep += [ts, tn]
        cats[i] = (src, cnt)
    ti, im = _pinned((cfg.imap_nr[0], 12 * cfg.nside_imap[0] ** 2), np.float32)
    tk, ka = _pinned((cfg.n_kappa, 12 * cfg.nside_kappa ** 2), np.float32)
    keep += [ti, tk]
    m.set_host_outputs(catalogs=cats, imaps={0: im}, kappa=ka)
    for _ in range(2):
        im[:] = np.nan
        ka[:] = np.nan
        for i in cats:
            cats[i][1][0] = -1
        m.run()
        m.sync()
        for i, (src, cnt) in cats.items():
            n = m.num_sources(i)
            assert cnt[0] == n == ns[i]
            ref = m.catalog(i, pos=False, ipix=False)["src"]
            k = min(n, src.shape[0])
            assert np.array_equal(src[:k], ref[:k]), i
            if src.shape[0] > n:
                assert np.all(src[n:] == -5.0)
        assert np.array_equal(im, m.imap(0))
        assert np.array_equal(ka, m.kappa())
    with pytest.raises(cg.CGError):
        m.set_host_outputs(catalogs={0: (np.zeros((4, 9), np.float32), np.zeros(1, np.int64))})
    m.set_host_outputs(catalogs={0: None, 1: None}, imaps={0: None})
    m.run()
    m.sync()
    m.close()
