"""The allocation-free bins entry, cg_collect_density_normalization_static,
against the allocating cg_collect_density_normalization through the C ABI.

The file name makes it the last GPU test collected, so it runs both alone in
a fresh process (its first call does the per-device scratch set-up) and
after every other GPU test of a session.  Cell counts must be equal; the
FP64 redshift and bias sums are accumulated with atomics in an unspecified
order, so they are compared to a relative 1e-12.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

_dp = C.POINTER(C.c_double)


def _spec():
    return dict(n_grid=64, z_min=0.05, z_max=0.6, r_smooth=2.0, seed=31, dens_type=0, bias_model=2,
                srcs=[dict(nz=("gauss", 0.3, 0.1), density=200.0, bias=("1+z",), nside_count=0),
                      dict(nz=("flat", 0.1, 0.5), density=4.0, bias=("const", 2.0), nside_count=0)],
                imap=[dict(tz=0.1, bias=("const", 1.0), z_range=(0.1, 0.5), nbands=6, nside=16)])


def _collect(fn, m, nz, idz):
    import colore_gb300 as cg
    nts, nti = m.cfg.n_srcs, m.cfg.n_imap
    z = np.full(nz, np.nan)
    n = np.zeros(nz, np.uint64)
    bs = np.full(max(nts, 1) * nz, np.nan)
    bi = np.full(max(nti, 1) * nz, np.nan)
    rc = fn(m._c, nz, idz, z.ctypes.data_as(_dp), n.ctypes.data_as(C.POINTER(C.c_ulonglong)),
            bs.ctypes.data_as(_dp), bi.ctypes.data_as(_dp))
    assert rc == 0, cg.lib().cg_last_error(m._c)
    return n, z, bs[:nts * nz], bi[:nti * nz]


def _free_bytes():
    import torch
    torch.cuda.synchronize(0)
    return torch.cuda.mem_get_info(0)[0]


@pytest.fixture
def mock(built, tmp_path):
    import colore_gb300 as cg
    from colore_gb300 import inputs
    params = cg.Params(inputs.write_inputs(str(tmp_path), _spec()))
    m = cg.Mock(params)
    m.create_cartesian_fields()
    m.compute_physical_density_field()
    yield m
    m.close()


def test_static_bins_match_allocating_entry(mock):
    import colore_gb300 as cg
    L = cg.lib()
    nz = 14
    idz = (nz - 2) / 0.6
    # the first call also applies the pending lognormal transform in place
    ref = _collect(L.cg_collect_density_normalization, mock, nz, idz)
    assert ref[0].sum() > 0
    free = []
    for _ in range(3):
        got = _collect(L.cg_collect_density_normalization_static, mock, nz, idz)
        assert np.array_equal(got[0], ref[0])
        for a, b in zip(got[1:], ref[1:]):
            assert np.all(np.isfinite(a))
            np.testing.assert_allclose(a, b, rtol=1e-12, atol=0)
        free.append(_free_bytes())
    # after the first call (which looks up the scratch array once per
    # device) the entry takes no device memory: free memory stays put
    assert free[1] == free[0] and free[2] == free[0], free


def test_static_bins_rejects_more_bins_than_its_scratch(mock):
    import colore_gb300 as cg
    L = cg.lib()
    nz = 1025
    z = np.zeros(nz)
    n = np.zeros(nz, np.uint64)
    b = np.zeros(3 * nz)
    rc = L.cg_collect_density_normalization_static(mock._c, nz, 1.0, z.ctypes.data_as(_dp),
                                                     n.ctypes.data_as(C.POINTER(C.c_ulonglong)),
                                                     b.ctypes.data_as(_dp), b.ctypes.data_as(_dp))
    assert rc == 1  # CG_EINVAL
    assert b"1024" in L.cg_last_error(mock._c)
