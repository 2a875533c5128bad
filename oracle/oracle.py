"""ORACLE Python binding (test infrastructure only).

ctypes wrappers around oracle/_lib/liboracle.so, the CPU restatement of
CoLoRe's hot path.  Imported by tests/, the smoke check and the CPU-baseline
leg of bench.py; never by the product package.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build_oracle  # noqa: E402

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        vp, d, i, f = C.c_void_p, C.c_double, C.c_int, C.c_float
        sig = {
            "or_fill64": [vp, vp, vp], "or_field64": [vp, vp, vp, vp], "or_density64": [vp, vp, d],
            "or_lpt64": [vp, vp, vp, vp], "or_lpt2_64": [vp, vp, vp, vp, vp], "or_bins64": [vp, vp, i, d, vp, vp, vp],
            "or_norm_tables64": [vp, vp, vp, vp, vp, vp, vp, vp],
            "or_lambda64": [vp, i, vp, vp, d, d, vp], "or_kappa64": [vp, vp, vp],
            "or_imap64": [vp, i, vp, vp, vp, d, d, vp, vp, i], "or_run_mock64": [vp, i, vp, vp],
            "or_imap64_part": [vp, i, vp, vp, vp, d, d, i, vp, vp, vp, i], "or_imap_samples": [vp, i],
            "or_kappa64_part": [vp, vp, i, vp], "or_poisson_total64": [vp, i, vp],
            "or_density32": [vp, vp, f, i], "or_bins32": [vp, vp, i, d, vp, vp, vp],
            "or_counts32": [vp, i, vp, vp, vp, vp, vp, vp],
            "or_emit32": [vp, i, vp, vp, vp, vp, C.c_longlong, vp, vp, vp, vp, vp, vp],
            "or_counts64": [vp, i, vp, vp, vp, vp],
            "or_emit64": [vp, i, vp, vp, C.c_longlong, vp, vp, vp, vp, vp],
            "or_beam_rsd32": [vp, vp, C.c_longlong, vp, vp], "or_imap32": [vp, i, vp, vp, vp, vp, vp, vp, vp],
            "or_kappa32": [vp, vp, vp], "or_isw32": [vp, vp, vp], "or_isw64": [vp, vp, vp],
            "or_cstm_steps": [vp, i, vp, vp, vp, vp], "or_cstm64": [vp, i, vp, vp, d, d, vp],
            "or_cstm32": [vp, i, vp, vp, f, f, vp],
            "or_lens64": [vp, vp, C.c_longlong, vp, vp], "or_lens32": [vp, vp, C.c_longlong, vp, vp],
            "or_skw64": [vp, vp, vp, i, d, C.c_longlong, vp, vp, vp],
            "or_skw32": [vp, vp, vp, i, f, C.c_longlong, vp, vp, vp], "or_c2r_3d": [i, vp, vp], "or_r2c_3d": [i, vp, vp],
            "or_vec_expf": [vp, vp, C.c_long], "or_vec_logf": [vp, vp, C.c_long],
            "or_vec_log1pf": [vp, vp, C.c_long], "or_vec_acosf": [vp, vp, C.c_long],
            "or_vec_atan2f": [vp, vp, vp, C.c_long], "or_vec_sincosf": [vp, vp, vp, C.c_long],
            "or_philox": [vp, vp, vp], "or_poisson": [vp, vp, C.c_long, C.c_uint32, C.c_uint32],
            "or_ang2pix": [C.c_long, vp, vp, vp, C.c_long], "or_nest2ring": [C.c_long, vp, vp, C.c_long],
            "or_ring2nest": [C.c_long, vp, vp, C.c_long], "or_pix2vec_nest": [C.c_long, vp, vp, C.c_long],
            "or_shell_index": [vp, vp, i, vp, vp, vp, C.c_long],
            "or_pix_checked": [C.c_long, vp, C.c_long, f, vp], "or_pix_cgx": [C.c_long, vp, C.c_long, vp],
            "or_pix64": [C.c_long, vp, C.c_long, vp], "or_pix_ff": [C.c_long, vp, vp, C.c_long, vp],
            "or_atan_q_maxerr": [], "or_ff_ops": [i, vp, vp, vp, vp, C.c_long, vp, vp],
            "or_sht_legendre": [i, i, i, vp, vp, vp, d, vp],
            "or_src_offset_checked": [C.c_long, vp, d, vp, vp, vp, vp],
            "or_ptrs_checked": [C.c_long, vp, vp, vp, vp, C.c_uint32, C.c_uint32, vp, vp],
        }
        void = ("or_philox", "or_poisson", "or_ang2pix", "or_nest2ring", "or_ring2nest", "or_pix2vec_nest",
                "or_shell_index", "or_pix_checked", "or_pix_cgx", "or_pix64", "or_pix_ff", "or_ff_ops", "or_src_offset_checked",
                "or_ptrs_checked")
        for k, a in sig.items():
            fn = getattr(L, k)
            fn.argtypes = a
            if k in ("or_imap_samples", "or_poisson_total64"):
                fn.restype = C.c_longlong
            elif k == "or_atan_q_maxerr":
                fn.restype = C.c_double
            elif k.startswith("or_vec") or k in void:
                fn.restype = None
            else:
                fn.restype = C.c_int
        _lib = L
    return _lib


def P(a):
    return a.ctypes.data if a is not None else None


class Params:
    """Run parameters and FP64 tables read by the oracle library's own build
    of the host C side (no GPU library loaded): the same param-file reader
    and table builder, for the CPU reference arm."""

    def __init__(self, fname):
        from colore_gb300 import Config  # the ctypes mirror of cg_config only
        L = lib()
        for name, res, args in (("cg_read_run_params", C.c_int, [C.c_char_p, C.POINTER(C.c_void_p), C.c_char_p,
                                                                  C.c_size_t]),
                                ("cg_params_free", None, [C.c_void_p]),
                                ("cg_params_to_config", C.c_int, [C.c_void_p, C.POINTER(Config)])):
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        self._p = C.c_void_p()
        err = C.create_string_buffer(1024)
        if L.cg_read_run_params(os.fsencode(fname), C.byref(self._p), err, 1024):
            raise RuntimeError("read_run_params(%s): %s" % (fname, err.value.decode()))
        self.config = Config()
        L.cg_params_to_config(self._p, C.byref(self.config))
        self.config._owner = self

    def __del__(self):
        if getattr(self, "_p", None) and _lib is not None:
            _lib.cg_params_free(self._p)
            self._p = None


def cfgp(cfg):
    return C.cast(C.pointer(cfg), C.c_void_p)


def unpad(g):
    """Padded [N][N][2(N/2+1)] grid -> unpadded [N][N][N] view."""
    n = g.shape[0]
    return g[:, :, :n]


# ---- ref64 ----
def field64(cfg):
    n = cfg.n_grid
    d = np.empty((n, n, n)), np.empty((n, n, n))
    st = np.empty(4)
    assert lib().or_field64(cfgp(cfg), P(d[0]), P(d[1]), P(st)) == 0
    return d[0], d[1], st


def fill64(cfg):
    n = cfg.n_grid
    dk = np.empty((n, n, n // 2 + 1), np.complex128)
    pk = np.empty_like(dk)
    lib().or_fill64(cfgp(cfg), P(dk), P(pk))
    return dk, pk


def density64(cfg, dens, sigma2):
    dens = np.ascontiguousarray(dens, np.float64).copy()
    lib().or_density64(cfgp(cfg), P(dens), sigma2)
    return dens


def lpt64(cfg, dens_gauss):
    n = cfg.n_grid
    dg = np.ascontiguousarray(dens_gauss, np.float64)
    out = np.empty((n, n, n))
    disp = np.empty((3, n, n, n))
    assert lib().or_lpt64(cfgp(cfg), P(dg), P(out), P(disp)) == 0
    return out, disp


def lpt2_64(cfg, dens_gauss):
    """2LPT in double: (density, first-order displacements, second-order ones)."""
    n = cfg.n_grid
    dg = np.ascontiguousarray(dens_gauss, np.float64)
    out = np.empty((n, n, n))
    d1 = np.empty((3, n, n, n))
    d2 = np.empty((3, n, n, n))
    assert lib().or_lpt2_64(cfgp(cfg), P(dg), P(out), P(d1), P(d2)) == 0
    return out, d1, d2


def norm_tables64(cfg, dens):
    nt = cfg.n_srcs + cfg.n_imap + cfg.n_cstm
    tabs = np.empty((max(nt, 1), 5001))
    e0f = np.empty((max(nt, 1), 2))
    nz = C.c_int()
    narr = np.empty(4096, np.uint64)
    zarr = np.empty(4096)
    bsum = np.empty((max(nt, 1), 4096))
    dd = np.ascontiguousarray(dens, np.float64)
    lib().or_norm_tables64(cfgp(cfg), P(tabs), P(e0f), C.byref(nz), P(narr), P(zarr), P(bsum), P(dd))
    return tabs, e0f, nz.value


def bins64(cfg, dens, nz, idz):
    nt = cfg.n_srcs + cfg.n_imap + cfg.n_cstm
    narr = np.empty(nz, np.uint64)
    zarr = np.empty(nz)
    bsum = np.empty((max(nt, 1), nz))
    dd = np.ascontiguousarray(dens, np.float64)
    lib().or_bins64(cfgp(cfg), P(dd), nz, idz, P(narr), P(zarr), P(bsum))
    return narr, zarr, bsum[:nt]


def lambda64(cfg, ipop, dens, tab, e):
    n = cfg.n_grid
    lam = np.empty((n, n, n))
    dd = np.ascontiguousarray(dens, np.float64)
    lib().or_lambda64(cfgp(cfg), ipop, P(dd), P(np.ascontiguousarray(tab, np.float64)), float(e[0]), float(e[1]),
                      P(lam))
    return lam


def kappa64(cfg, npot):
    ns = cfg.nside_kappa
    m = np.empty((cfg.n_kappa, 12 * ns * ns))
    lib().or_kappa64(cfgp(cfg), P(np.ascontiguousarray(npot, np.float64)), P(m))
    return m


def imap64(cfg, ipop, dens, npot, tab, e, sprec=True):
    """Intensity map in double (imap.c:135-245): (summed brightness, hits).
    sprec: the reference built with _SPREC (float shells and potential
    differences), which the FP32 path matches; False: the double build, which
    the FP64 baseline path matches."""
    ns, nr = cfg.nside_imap[ipop], cfg.imap_nr[ipop]
    data = np.empty((nr, 12 * ns * ns))
    nadd = np.empty((nr, 12 * ns * ns), np.int32)
    lib().or_imap64(cfgp(cfg), ipop, P(np.ascontiguousarray(dens, np.float64)),
                    P(np.ascontiguousarray(npot, np.float64)), P(np.ascontiguousarray(tab, np.float64)),
                    float(e[0]), float(e[1]), P(data), P(nadd), 1 if sprec else 0)
    return data, nadd

def run_mock64(cfg):
    n = C.c_longlong()
    cs = C.c_double()
    assert lib().or_run_mock64(cfgp(cfg), 0, C.byref(n), C.byref(cs)) == 0
    return n.value, cs.value


# ---- dev32 (padded float32 grids as downloaded from the GPU) ----
def density32(cfg, dens, s2f, mode):
    d = np.array(dens, np.float32, copy=True)
    lib().or_density32(cfgp(cfg), P(d), float(s2f), mode)
    return d


def bins32(cfg, dens, nz, idz):
    nt = cfg.n_srcs + cfg.n_imap + cfg.n_cstm
    narr = np.empty(nz, np.uint64)
    zarr = np.empty(nz)
    bsum = np.empty((max(nt, 1), nz))
    lib().or_bins32(cfgp(cfg), P(np.ascontiguousarray(dens, np.float32)), nz, idz, P(narr), P(zarr), P(bsum))
    return narr, zarr, bsum[:nt]


def _norm_pair(tab32, e32, tab64, e64):
    """The float and double normalisation tables with their edges appended
    (CG_NA + 2 values each), as the kernels hold them."""
    t32 = np.concatenate([np.asarray(tab32, np.float32), np.asarray(e32, np.float32)])
    t64 = np.concatenate([np.asarray(tab64, np.float64), np.asarray(e64, np.float64)])
    return t32, t64


def counts32(cfg, ipop, dens, tab32, e32, tab64, e64):
    """Counts as the GPU computes them (float margins, double where they do
    not hold): (counts [N][N][N], total, cells decided in double)."""
    n = cfg.n_grid
    cnt = np.empty((n, n, n), np.int32)
    tot = C.c_longlong()
    fb = C.c_longlong()
    t32, t64 = _norm_pair(tab32, e32, tab64, e64)
    lib().or_counts32(cfgp(cfg), ipop, P(np.ascontiguousarray(dens, np.float32)), P(t32), P(t64), P(cnt),
                      C.byref(tot), C.byref(fb))
    return cnt, tot.value, fb.value


def emit32(cfg, ipop, dens, npot, tab32, e32, tab64, e64, cap):
    """The catalogue as the GPU writes it; 'fallbacks': pixels decided in
    double."""
    pos = np.empty((cap, 4), np.float32)
    ipix = np.empty(cap, np.int32)
    src = np.empty((cap, 9), np.float32)
    ns = cfg.nside_count[ipop]
    cmap = np.zeros(12 * ns * ns, np.int32) if ns > 0 else None
    n = C.c_longlong()
    fb = C.c_longlong()
    t32, t64 = _norm_pair(tab32, e32, tab64, e64)
    rc = lib().or_emit32(cfgp(cfg), ipop, P(np.ascontiguousarray(dens, np.float32)),
                         P(np.ascontiguousarray(npot, np.float32)), P(t32), P(t64), cap, P(pos), P(ipix), P(src),
                         P(cmap), C.byref(n), C.byref(fb))
    assert rc == 0
    k = n.value
    return dict(pos=pos[:k], ipix=ipix[:k], src=src[:k], cmap=cmap, fallbacks=fb.value)


def counts64(cfg, ipop, dens, tab64, e64):
    """Counts in double (srcs.c:156-183) from the float density (any float
    grid, padded or not, is read as its N^3 cells): (counts, total)."""
    n = cfg.n_grid
    d = np.ascontiguousarray(np.asarray(dens)[:, :, :n], np.float64)
    cnt = np.empty((n, n, n), np.int32)
    tot = C.c_longlong()
    t64 = np.concatenate([np.asarray(tab64, np.float64), np.asarray(e64, np.float64)])
    assert lib().or_counts64(cfgp(cfg), ipop, P(d), P(t64), P(cnt), C.byref(tot)) == 0
    return cnt, tot.value


def emit64(cfg, ipop, npot, counts, cap):
    """The catalogue in double (srcs.c:238-276, 386-416) from the counts and
    the float potential: pos, ipix, src, cmap."""
    n = cfg.n_grid
    ph = np.ascontiguousarray(np.asarray(npot)[:, :, :n], np.float64)
    pos = np.empty((cap, 4), np.float32)
    ipix = np.empty(cap, np.int32)
    src = np.empty((cap, 9), np.float32)
    ns = cfg.nside_count[ipop]
    cmap = np.zeros(12 * ns * ns, np.int32) if ns > 0 else None
    k = C.c_longlong()
    assert lib().or_emit64(cfgp(cfg), ipop, P(ph), P(np.ascontiguousarray(counts, np.int32)), cap, P(pos), P(ipix),
                           P(src), P(cmap), C.byref(k)) == 0
    k = k.value
    return dict(pos=pos[:k], ipix=ipix[:k], src=src[:k], cmap=cmap)


def beam_rsd32(cfg, npot, pos, src):
    s = np.array(src, np.float32, copy=True)
    lib().or_beam_rsd32(cfgp(cfg), P(npot), len(pos), P(np.ascontiguousarray(pos, np.float32)), P(s))
    return s


def imap32(cfg, ipop, dens, npot, tab32, e32, tab64, e64):
    """The intensity map as the GPU paints it: (summed brightness, hit
    counts, stats) with stats = (cells and samples decided in double,
    samples drawn)."""
    ns, nr = cfg.nside_imap[ipop], cfg.imap_nr[ipop]
    data = np.empty((nr, 12 * ns * ns), np.float32)
    nadd = np.empty((nr, 12 * ns * ns), np.int32)
    st = np.zeros(3, np.int64)
    t32, t64 = _norm_pair(tab32, e32, tab64, e64)
    lib().or_imap32(cfgp(cfg), ipop, P(np.ascontiguousarray(dens, np.float32)),
                    P(np.ascontiguousarray(npot, np.float32)), P(t32), P(t64), P(data), P(nadd), P(st))
    return data, nadd, st

def isw64(cfg, npot):
    ns = cfg.nside_isw
    m = np.empty((cfg.n_isw, 12 * ns * ns))
    lib().or_isw64(cfgp(cfg), P(np.ascontiguousarray(npot, np.float64)), P(m))
    return m


def isw32(cfg, npot):
    ns = cfg.nside_isw
    m = np.empty((cfg.n_isw, 12 * ns * ns), np.float32)
    lib().or_isw32(cfgp(cfg), P(npot), P(m))
    return m


def cstm_steps(cfg, ipop):
    """(kz, bz, ir_min, ir_max): the custom-map step tables in double."""
    nr = cfg.n_grid // 2
    kz = np.empty(nr)
    bz = np.empty(nr)
    lo, hi = C.c_int(), C.c_int()
    rc = lib().or_cstm_steps(cfgp(cfg), ipop, P(kz), P(bz), C.byref(lo), C.byref(hi))
    return kz, bz, lo.value, hi.value, rc


def cstm64(cfg, ipop, dens, tab, e):
    ns = cfg.nside_cstm[ipop]
    m = np.empty(12 * ns * ns)
    assert lib().or_cstm64(cfgp(cfg), ipop, P(np.ascontiguousarray(dens, np.float64)),
                           P(np.ascontiguousarray(tab, np.float64)), float(e[0]), float(e[1]), P(m)) == 0
    return m


def cstm32(cfg, ipop, dens, tab, e):
    ns = cfg.nside_cstm[ipop]
    m = np.empty(12 * ns * ns, np.float32)
    assert lib().or_cstm32(cfgp(cfg), ipop, P(dens), P(np.ascontiguousarray(tab, np.float32)), float(e[0]),
                           float(e[1]), P(m)) == 0
    return m


def lens64(cfg, npot, pos4):
    """(n, 5): e1, e2, kappa, dra, ddec of each source in double precision."""
    pos4 = np.ascontiguousarray(pos4, np.float32).reshape(-1, 4)
    out = np.empty((len(pos4), 5))
    assert lib().or_lens64(cfgp(cfg), P(np.ascontiguousarray(npot, np.float64)), len(pos4), P(pos4), P(out)) == 0
    return out


def lens32(cfg, npot, pos4, src9):
    """src9 with columns 4..8 replaced by the FP32 lensing restatement."""
    pos4 = np.ascontiguousarray(pos4, np.float32).reshape(-1, 4)
    out = np.array(src9, np.float32, copy=True).reshape(-1, 9)
    assert lib().or_lens32(cfgp(cfg), P(npot), len(pos4), P(pos4), P(out)) == 0
    return out


def skw64(cfg, dens, npot, gauss, sigma2, pos4):
    pos4 = np.ascontiguousarray(pos4, np.float32).reshape(-1, 4)
    nr = cfg.n_grid // 2
    d = np.empty((len(pos4), nr))
    v = np.empty((len(pos4), nr))
    assert lib().or_skw64(cfgp(cfg), P(np.ascontiguousarray(dens, np.float64)), P(np.ascontiguousarray(npot, np.float64)),
                          int(gauss), float(sigma2), len(pos4), P(pos4), P(d), P(v)) == 0
    return d, v


def skw32(cfg, dens, npot, gauss, sigma2f, pos4):
    pos4 = np.ascontiguousarray(pos4, np.float32).reshape(-1, 4)
    nr = cfg.n_grid // 2
    d = np.empty((len(pos4), nr), np.float32)
    v = np.empty((len(pos4), nr), np.float32)
    assert lib().or_skw32(cfgp(cfg), P(dens), P(npot), int(gauss), float(sigma2f), len(pos4), P(pos4), P(d),
                          P(v)) == 0
    return d, v


def kappa32(cfg, npot):
    ns = cfg.nside_kappa
    m = np.empty((cfg.n_kappa, 12 * ns * ns), np.float32)
    lib().or_kappa32(cfgp(cfg), P(npot), P(m))
    return m


# ---- scalar checks ----
def vec(name, *arrs):
    out = [np.empty_like(arrs[0]) for _ in range(2 if name == "sincosf" else 1)]
    args = [P(np.ascontiguousarray(a, np.float32)) for a in arrs] + [P(o) for o in out] + [len(arrs[0])]
    getattr(lib(), "or_vec_" + name)(*args)
    return out if len(out) > 1 else out[0]


def philox(ctr, key):
    c = np.array(ctr, np.uint32)
    k = np.array(key, np.uint32)
    o = np.empty(4, np.uint32)
    lib().or_philox(P(c), P(k), P(o))
    return o


def poisson(lam, k0=1, k1=2):
    lam = np.ascontiguousarray(lam, np.float32)
    k = np.empty(len(lam), np.int32)
    lib().or_poisson(P(lam), P(k), len(lam), k0, k1)
    return k


def ang2pix(nside, cth, phi):
    cth = np.ascontiguousarray(cth, np.float32)
    phi = np.ascontiguousarray(phi, np.float32)
    p = np.empty(len(cth), np.int64)
    lib().or_ang2pix(nside, P(cth), P(phi), P(p), len(cth))
    return p


def shell_index(r0, rf, r):
    """Shell of each radius r: the walk from shell 0 and its bisection form
    (both from the shared cell header)."""
    r0 = np.ascontiguousarray(r0, np.float32)
    rf = np.ascontiguousarray(rf, np.float32)
    r = np.ascontiguousarray(r, np.float32)
    w = np.empty(len(r), np.int32)
    b = np.empty(len(r), np.int32)
    lib().or_shell_index(P(r0), P(rf), len(r0), P(r), P(w), P(b), len(r))
    return w, b


def nest2ring(nside, ip):
    ip = np.ascontiguousarray(ip, np.int64)
    o = np.empty_like(ip)
    lib().or_nest2ring(nside, P(ip), P(o), len(ip))
    return o


def ring2nest(nside, ip):
    ip = np.ascontiguousarray(ip, np.int64)
    o = np.empty_like(ip)
    lib().or_ring2nest(nside, P(ip), P(o), len(ip))
    return o


def pix2vec_nest(nside, ip):
    ip = np.ascontiguousarray(ip, np.int64)
    v = np.empty((len(ip), 3), np.float32)
    lib().or_pix2vec_nest(nside, P(ip), P(v), len(ip))
    return v


def imap64_part(cfg, ipop, dens, npot, tab, e, iz_stride):
    ns, nr = cfg.nside_imap[ipop], cfg.imap_nr[ipop]
    data = np.empty((nr, 12 * ns * ns))
    nadd = np.empty((nr, 12 * ns * ns), np.int32)
    nsamp = C.c_longlong()
    lib().or_imap64_part(cfgp(cfg), ipop, P(np.ascontiguousarray(dens, np.float64)),
                         P(np.ascontiguousarray(npot, np.float64)), P(np.ascontiguousarray(tab, np.float64)),
                         float(e[0]), float(e[1]), iz_stride, P(data), P(nadd), C.byref(nsamp), 1)
    return nsamp.value


def imap_samples(cfg, ipop):
    return lib().or_imap_samples(cfgp(cfg), ipop)


def kappa64_part(cfg, npot, pix_stride):
    ns = cfg.nside_kappa
    m = np.zeros((cfg.n_kappa, 12 * ns * ns))
    lib().or_kappa64_part(cfgp(cfg), P(np.ascontiguousarray(npot, np.float64)), pix_stride, P(m))
    return m


def poisson_total64(cfg, ipop, lam):
    return lib().or_poisson_total64(cfgp(cfg), ipop, P(np.ascontiguousarray(lam, np.float64)))


def pix_checked(nside, xyz32, ein=0.0):
    """Margin-checked float RING pixels of float directions (-1: deferred)."""
    a = np.ascontiguousarray(xyz32, np.float32)
    out = np.empty(len(a), np.int64)
    lib().or_pix_checked(nside, P(a), len(a), float(ein), P(out))
    return out


def pix_ff(nside, xyz, rel=2.0 ** -47):
    """RING pixels of double positions by the float-float tier
    (cg_pix_ff, -1: deferred to double): each coordinate split into a float
    pair, declared within rel |p| of the double position."""
    a = np.ascontiguousarray(xyz, np.float64)
    h = a.astype(np.float32)
    lo = (a - h.astype(np.float64)).astype(np.float32)
    q = np.ascontiguousarray(np.stack([h, lo], 2).reshape(len(a), 6), np.float32)
    eP = (rel * np.sqrt((a * a).sum(1))).astype(np.float32)
    out = np.empty(len(a), np.int64)
    lib().or_pix_ff(nside, P(q), P(eP), len(a), P(out))
    return out


def ff_ops(op, x, y=None):
    """cg_ff.h's operation op (0 sum, 1 product, 2 quotient, 3 root of x,
    4 product by a float) on float-float operands given as (h, l) arrays."""
    xh, xl = (np.ascontiguousarray(a, np.float32) for a in x)
    yh, yl = (np.ascontiguousarray(a, np.float32) for a in (y if y is not None else (xh, xl)))
    oh = np.empty_like(xh)
    ol = np.empty_like(xh)
    lib().or_ff_ops(op, P(xh), P(xl), P(yh), P(yl), len(xh), P(oh), P(ol))
    return oh, ol


def pix64(nside, xyz, shared=False):
    """RING pixels of double directions by the oracle's restatement (or the
    kernels' double restatement with shared=True)."""
    a = np.ascontiguousarray(xyz, np.float64)
    out = np.empty(len(a), np.int64)
    (lib().or_pix_cgx if shared else lib().or_pix64)(nside, P(a), len(a), P(out))
    return out


def src_offset_checked(x0, dx, bits):
    """The emission's single-precision source coordinate (cg_src_offset_checked)
    for corners x0 (double) and uniform words bits: (out, ok, ref) with ref
    the double expression rounded to float."""
    x0 = np.ascontiguousarray(x0, np.float64)
    bits = np.ascontiguousarray(bits, np.uint32)
    n = len(x0)
    out = np.empty(n, np.float32)
    ok = np.empty(n, np.int32)
    ref = np.empty(n, np.float32)
    lib().or_src_offset_checked(n, P(x0), C.c_double(dx), P(bits), P(out), P(ok), P(ref))
    return out, ok.astype(bool), ref


def ptrs_checked(lam, elam, lam64, cid, k0, k1):
    """Single-precision PTRS (-1 where left to double) and the double PTRS."""
    lam = np.ascontiguousarray(lam, np.float32)
    elam = np.ascontiguousarray(elam, np.float32)
    lam64 = np.ascontiguousarray(lam64, np.float64)
    cid = np.ascontiguousarray(cid, np.int64)
    n = len(lam)
    got = np.empty(n, np.int32)
    ref = np.empty(n, np.int32)
    lib().or_ptrs_checked(n, P(lam), P(elam), P(lam64), P(cid), k0, k1, P(got), P(ref))
    return got, ref
