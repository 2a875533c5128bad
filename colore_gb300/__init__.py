"""colore_gb300: CoLoRe's mock-generation path on one GB300 (sm_103a).

The product is the C library colore_gb300/lib/libcolore_cuda.so (C ABI in
include/colore_cuda.h and include/colore_host.h).  This module binds it with
ctypes for Python users, tests and the benchmark:

    from colore_gb300 import Mock
    m = Mock.from_param_file("run.cfg")
    m.run()                      # main.c stage sequence on the GPU
    ra_dec = m.catalog(0)["src"]

There is no CPU fallback: importing works without a GPU, but creating a Mock
without the built library or without a CUDA device raises.
"""
import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "lib", "libcolore_cuda.so")

NPOP_MAX = 10
NPLANES_MAX = 100
NA = 5001
PREC_F32, PREC_F64 = 0, 1
DENS_LGNR, DENS_1LPT, DENS_CLIP = 0, 1, 3
ERRORS = {0: "ok", 1: "invalid argument", 2: "out of memory", 3: "CUDA error", 4: "device error flag",
          5: "stage out of order"}

_dp = C.POINTER(C.c_double)


class Config(C.Structure):
    """Mirror of cg_config (include/colore_cuda.h)."""
    _fields_ = [
        ("precision", C.c_int), ("n_grid", C.c_int), ("l_box", C.c_double), ("pos_obs", C.c_double * 3),
        ("seed", C.c_uint64),
        ("omega_m", C.c_double), ("hubble_0", C.c_double), ("fgrowth_0", C.c_double),
        ("prefac_lensing", C.c_double), ("r_max", C.c_double),
        ("r2_smooth", C.c_double), ("do_smoothing", C.c_int), ("smooth_potential", C.c_int),
        ("dens_type", C.c_int), ("bias_model", C.c_int),
        ("numk", C.c_int), ("logkmin", C.c_double), ("logkmax", C.c_double), ("idlogk", C.c_double),
        ("n_scal", C.c_double), ("pkarr", _dp),
        ("glob_idr", C.c_double),
        ("r_arr_r2z", _dp), ("z_arr_r2z", _dp), ("growth_d_arr", _dp), ("growth_d2_arr", _dp),
        ("growth_v_arr", _dp), ("growth_pd_arr", _dp), ("ihub_arr", _dp), ("a_arr_a2r", _dp), ("r_arr_a2r", _dp),
        ("n_srcs", C.c_int), ("srcs_nz_arr", _dp * NPOP_MAX), ("srcs_bz_arr", _dp * NPOP_MAX),
        ("nside_base", C.c_int), ("nside_count", C.c_int * NPOP_MAX),
        ("n_imap", C.c_int), ("imap_tz_arr", _dp * NPOP_MAX), ("imap_bz_arr", _dp * NPOP_MAX),
        ("nside_imap", C.c_int * NPOP_MAX), ("imap_nr", C.c_int * NPOP_MAX),
        ("imap_r0", _dp * NPOP_MAX), ("imap_rf", _dp * NPOP_MAX),
        ("do_kappa", C.c_int), ("n_kappa", C.c_int), ("nside_kappa", C.c_int),
        ("kappa_r", C.c_double * NPLANES_MAX),
        ("need_beaming", C.c_int),
        ("do_isw", C.c_int), ("n_isw", C.c_int), ("nside_isw", C.c_int),
        ("isw_r", C.c_double * NPLANES_MAX),
        ("lpt_interp_type", C.c_int),
        ("n_cstm", C.c_int),
        ("cstm_kz_arr", _dp * NPOP_MAX),
        ("cstm_bz_arr", _dp * NPOP_MAX),
        ("nside_cstm", C.c_int * NPOP_MAX),
        ("lensing_srcs", C.c_int * NPOP_MAX),
        ("skw_srcs", C.c_int * NPOP_MAX),
        ("skw_gauss", C.c_int * NPOP_MAX),
    ]


_lib = None


def lib():
    """The loaded libcolore_cuda.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libcolore_cuda.so is not built: run colore_gb300.build.build() "
                               "(python -c 'import __graft_entry__ as g; g.build()')")
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        sigs = {
            "cg_create": (C.c_int, [C.POINTER(vp), C.POINTER(Config), C.c_int]),
            "cg_destroy": (None, [vp]),
            "cg_last_error": (C.c_char_p, [vp]),
            "cg_set_stream": (C.c_int, [vp, vp]),
            "cg_sync": (C.c_int, [vp]),
            "cg_graph_capture": (C.c_int, [vp]),
            "cg_graph_launch": (C.c_int, [vp, vp]),
            "cg_batch_create": (C.c_int, [C.POINTER(vp), C.c_int, vp, C.c_int, C.c_int]),
            "cg_batch_run": (C.c_int, [vp, C.POINTER(C.c_float)]),
            "cg_batch_streams": (C.c_int, [vp]),
            "cg_batch_tuning": (C.c_int, [vp, C.POINTER(C.c_float), C.c_int]),
            "cg_batch_context": (vp, [vp, C.c_int]),
            "cg_batch_set_host_catalog": (C.c_int, [vp, C.c_int, C.c_int, vp, C.c_longlong, vp]),
            "cg_batch_last_error": (C.c_char_p, [vp]),
            "cg_batch_destroy": (None, [vp]),
            "cg_memory_estimate": (C.c_int, [C.POINTER(Config), C.POINTER(C.c_ulonglong)]),
            "cg_upload_tables": (C.c_int, [vp, C.POINTER(Config)]),
            "cg_create_cartesian_fields": (C.c_int, [vp]),
            "cg_get_sigma2": (C.c_int, [vp, _dp, _dp]),
            "cg_compute_physical_density_field": (C.c_int, [vp]),
            "cg_compute_density_normalization": (C.c_int, [vp]),
            "cg_collect_density_normalization": (C.c_int, [vp, C.c_int, C.c_double, _dp,
                                                           C.POINTER(C.c_ulonglong), _dp, _dp]),
            "cg_collect_density_normalization_static": (C.c_int, [vp, C.c_int, C.c_double, _dp,
                                                                  C.POINTER(C.c_ulonglong), _dp, _dp]),
            "cg_set_norm_tables": (C.c_int, [vp, _dp, _dp, _dp, _dp]),
            "cg_srcs_set_cartesian": (C.c_int, [vp, C.POINTER(C.c_longlong)]),
            "cg_imap_set_cartesian": (C.c_int, [vp]),
            "cg_imap_samples": (C.c_int, [vp, C.c_int, C.POINTER(C.c_ulonglong)]),
            "cg_set_imap_list_cap": (C.c_int, [vp, C.c_longlong]),
            "cg_set_host_catalog": (C.c_int, [vp, C.c_int, vp, C.c_longlong, vp]),
            "cg_set_host_imap": (C.c_int, [vp, C.c_int, vp]),
            "cg_set_host_kappa": (C.c_int, [vp, vp]),
            "cg_get_beam_properties": (C.c_int, [vp]),
            "cg_run_mock": (C.c_int, [vp]),
            "cg_download_grid": (C.c_int, [vp, C.c_int, vp]),
            "cg_num_sources": (C.c_longlong, [vp, C.c_int]),
            "cg_download_catalog": (C.c_int, [vp, C.c_int, vp, vp, vp]),
            "cg_download_count_map": (C.c_int, [vp, C.c_int, vp]),
            "cg_download_imap": (C.c_int, [vp, C.c_int, vp, vp]),
            "cg_download_kappa": (C.c_int, [vp, vp]),
            "cg_download_isw": (C.c_int, [vp, vp]),
            "cg_download_custom": (C.c_int, [vp, C.c_int, vp]),
            "cg_download_norm": (C.c_int, [vp, C.c_int, C.c_int, vp, vp]),
            "cg_download_norm64": (C.c_int, [vp, C.c_int, C.c_int, vp, vp]),
            "cg_set_decisions_in_double": (C.c_int, [vp, C.c_int]),
            "cg_exact_stats": (C.c_int, [vp, vp, C.c_int]),
            "cg_ring_pixels_checked": (C.c_int, [C.c_int, C.c_int, vp, C.c_longlong, C.c_float, vp]),
            "cg_kernel_launches": (C.c_longlong, [vp]),
            "cg_set_profiling": (C.c_int, [vp, C.c_int]),
            "cg_set_field_variant": (C.c_int, [vp, C.c_int, C.c_int]),
            "cg_field_plan": (C.c_int, [vp, C.c_char_p, C.c_size_t]),
            "cg_kernel_times": (C.c_int, [vp, C.c_char_p, C.c_size_t, C.POINTER(C.c_float), C.c_int,
                                          C.POINTER(C.c_int)]),
            "cg64_create": (C.c_int, [C.POINTER(vp), C.POINTER(Config), C.c_int]),
            "cg64_destroy": (None, [vp]),
            "cg64_last_error": (C.c_char_p, [vp]),
            "cg64_run_mock": (C.c_int, [vp, C.POINTER(C.c_float)]),
            "cg64_create_cartesian_fields": (C.c_int, [vp]),
            "cg64_num_sources": (C.c_longlong, [vp, C.c_int]),
            "cg64_download": (C.c_int, [vp, C.c_int, C.c_int, vp]),
            "cg_write_healpix_map": (C.c_int, [C.c_char_p, vp, C.c_long]),
            "cg_write_catalog": (C.c_int, [C.c_char_p, C.c_int, C.c_int, vp, C.c_longlong, C.c_int, vp]),
            "cg_download_skewers": (C.c_int, [vp, C.c_int, vp, vp]),
            "cg_write_predictions": (C.c_int, [vp]),
            "cg_pk_linear0": (C.c_double, [vp, C.c_double]),
            "cg_pk2xi": (None, [C.c_int, vp, vp, vp, vp]),
            "cg_xi2pk": (None, [C.c_int, vp, vp, vp, vp]),
            "cg_write_density_grid": (C.c_int, [C.c_char_p, C.c_char_p, vp, C.c_int, C.c_double]),
            "cg_read_run_params": (C.c_int, [C.c_char_p, C.POINTER(vp), C.c_char_p, C.c_size_t]),
            "cg_params_free": (None, [vp]),
            "cg_params_to_config": (C.c_int, [vp, C.POINTER(Config)]),
        }
        for name, (res, args) in sigs.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    """Names of the C-ABI entry points this binding expects in the library."""
    return ["cg_create", "cg_destroy", "cg_last_error", "cg_set_stream", "cg_sync", "cg_memory_estimate",
            "cg_upload_tables", "cg_create_cartesian_fields", "cg_get_sigma2",
            "cg_compute_physical_density_field", "cg_compute_density_normalization",
            "cg_collect_density_normalization", "cg_collect_density_normalization_static", "cg_set_norm_tables", "cg_srcs_set_cartesian",
            "cg_imap_set_cartesian", "cg_imap_samples", "cg_set_imap_list_cap", "cg_set_host_catalog",
            "cg_set_host_imap", "cg_set_host_kappa", "cg_get_beam_properties", "cg_run_mock", "cg_download_grid",
            "cg_num_sources", "cg_download_catalog", "cg_download_count_map", "cg_download_imap",
            "cg_download_kappa", "cg_download_isw", "cg_download_custom", "cg_download_skewers", "cg_download_norm", "cg_download_norm64", "cg_set_decisions_in_double",
            "cg_exact_stats", "cg_ring_pixels_checked", "cg_kernel_launches", "cg_set_profiling", "cg_kernel_times", "cg_set_field_variant", "cg_field_plan", "cg_read_run_params",
            "cg_params_free", "cg_params_to_config", "cg_write_healpix_map", "cg_write_catalog",
            "cg_write_density_grid", "cg_graph_capture", "cg_graph_launch", "cg_batch_create", "cg_batch_run",
            "cg_batch_streams", "cg_batch_tuning", "cg_batch_context", "cg_batch_set_host_catalog",
            "cg_batch_last_error", "cg_batch_destroy",
            "cg_skewer_background", "cg_write_predictions", "cg_pk_linear0", "cg_pk2xi", "cg_xi2pk",
            "cg64_create", "cg64_destroy", "cg64_last_error",
            "cg64_run_mock", "cg64_create_cartesian_fields", "cg64_num_sources", "cg64_download"]


class CGError(RuntimeError):
    pass


def ring_pixels_checked(nside, xyz, ein=0.0, device=0):
    """RING pixels of float directions (n x 3) decided on the GPU by the
    margin-checked single precision of the intensity maps; -1 where only the
    double arithmetic can decide."""
    a = np.ascontiguousarray(xyz, np.float32)
    out = np.empty(len(a), np.int64)
    rc = lib().cg_ring_pixels_checked(device, nside, a.ctypes.data, len(a), float(ein), out.ctypes.data)
    if rc:
        raise CGError("cg_ring_pixels_checked: %s" % ERRORS.get(rc, rc))
    return out


OUT_ASCII, OUT_FITS = 0, 1


def write_healpix_map(fname, m, nside):
    """One RING map as a FITS binary table (he_write_healpix_map)."""
    m = np.ascontiguousarray(m, np.float32)
    if m.size != 12 * nside * nside:
        raise ValueError("map has %d pixels, nside %d needs %d" % (m.size, nside, 12 * nside * nside))
    if lib().cg_write_healpix_map(os.fsencode(fname), m.ctypes.data, nside):
        raise CGError("cannot write %s" % fname)


def write_predictions(params):
    """The theory-prediction files of write_predictions for these parameters."""
    if lib().cg_write_predictions(params._p):
        raise CGError("write_predictions failed (write_pred and pred_dz set?)")


def pk2xi(k, pk):
    """FFTLog P(k) -> xi(r) on log-spaced k (the reference's pk2xi): (r, xi)."""
    k = np.ascontiguousarray(k, np.float64)
    pk = np.ascontiguousarray(pk, np.float64)
    r = np.empty_like(k)
    xi = np.empty_like(k)
    lib().cg_pk2xi(len(k), k.ctypes.data, pk.ctypes.data, r.ctypes.data, xi.ctypes.data)
    return r, xi


def xi2pk(r, xi):
    """FFTLog xi(r) -> P(k) on log-spaced r (the reference's xi2pk): (k, pk)."""
    r = np.ascontiguousarray(r, np.float64)
    xi = np.ascontiguousarray(xi, np.float64)
    k = np.empty_like(r)
    pk = np.empty_like(r)
    lib().cg_xi2pk(len(r), r.ctypes.data, xi.ctypes.data, k.ctypes.data, pk.ctypes.data)
    return k, pk


class SkewerSet(C.Structure):
    """Mirror of cg_skewer_set (include/colore_host.h)."""
    _fields_ = [("nr", C.c_int), ("gauss", C.c_int), ("dens", C.c_void_p), ("vel", C.c_void_p),
                ("r", C.c_void_p), ("z", C.c_void_p), ("d1", C.c_void_p), ("v1", C.c_void_p),
                ("sigma_g", C.c_float)]


def write_catalog(prefix, ipop, src, fmt=OUT_FITS, lensing=False, skewers=None):
    """<prefix>_srcs_s<ipop+1>_0.fits or .txt from Src records (n x 9 floats).
    lensing adds the E1 E2 KAPPA DRA DDEC columns; skewers (FITS only) is a
    dict with dens, vel (n x nr), r, z, d1, v1 (nr), sigma_g and gauss."""
    src = np.ascontiguousarray(src, np.float32).reshape(-1, 9)
    keep, ps = [], None
    if skewers is not None:
        arr = {k: np.ascontiguousarray(skewers[k], np.float32) for k in ("dens", "vel", "r", "z", "d1", "v1")}
        keep.append(arr)
        nr = arr["r"].size
        ps = SkewerSet(nr, int(bool(skewers.get("gauss", False))), arr["dens"].ctypes.data, arr["vel"].ctypes.data,
                       arr["r"].ctypes.data, arr["z"].ctypes.data, arr["d1"].ctypes.data, arr["v1"].ctypes.data,
                       float(skewers["sigma_g"]))
    if lib().cg_write_catalog(os.fsencode(prefix), ipop, fmt, src.ctypes.data, len(src), int(bool(lensing)),
                              C.byref(ps) if ps is not None else None):
        raise CGError("cannot write the catalogue of population %d under %s" % (ipop, prefix))


def write_density_grid(prefix, tag, grid, l_box):
    """<prefix>_dens_<tag>_0.dat from a padded [N][N][2(N/2+1)] float grid."""
    g = np.ascontiguousarray(grid, np.float32)
    if lib().cg_write_density_grid(os.fsencode(prefix), os.fsencode(tag), g.ctypes.data, g.shape[0], l_box):
        raise CGError("cannot write the density grid under %s" % prefix)


class Params:
    """Parsed run parameters and FP64 tables (cg_params, C-owned)."""

    def __init__(self, fname):
        L = lib()
        self._p = C.c_void_p()
        err = C.create_string_buffer(1024)
        rc = L.cg_read_run_params(os.fsencode(fname), C.byref(self._p), err, 1024)
        if rc:
            raise CGError("read_run_params(%s): %s" % (fname, err.value.decode()))
        self.config = Config()
        L.cg_params_to_config(self._p, C.byref(self.config))
        # the config's table pointers live in this object: keep it alive as
        # long as the config is referenced
        self.config._owner = self

    def __del__(self):
        if getattr(self, "_p", None) and _lib is not None:
            _lib.cg_params_free(self._p)
            self._p = None


def grid_shape(n):
    """Padded real grid shape [z][y][2(N/2+1)] of the in-place layout."""
    return (n, n, 2 * (n // 2 + 1))


class Mock:
    """One GPU context running CoLoRe's stages (cg_* C ABI)."""

    def __init__(self, params, device=0, _handle=None):
        self.params = params
        self.cfg = params.config
        L = lib()
        self._owned = _handle is None
        if _handle is not None:  # a context owned by a Batch
            self._c = C.c_void_p(_handle)
            return
        self._c = C.c_void_p()
        rc = L.cg_create(C.byref(self._c), C.byref(self.cfg), device)
        if rc:
            raise CGError("cg_create failed (%s)" % ERRORS.get(rc, rc))

    @classmethod
    def from_param_file(cls, fname, device=0):
        return cls(Params(fname), device)

    def close(self):
        if getattr(self, "_c", None):
            if self._owned:
                lib().cg_destroy(self._c)
            self._c = None

    def graph_capture(self):
        """Capture fields, density, normalisation and sources into a CUDA graph."""
        self._chk(lib().cg_graph_capture(self._c), "cg_graph_capture")

    def graph_launch(self, stream_handle=None):
        self._chk(lib().cg_graph_launch(self._c, C.c_void_p(stream_handle) if stream_handle else None),
                  "cg_graph_launch")

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc, what):
        if rc:
            msg = lib().cg_last_error(self._c)
            raise CGError("%s: %s (%s)" % (what, ERRORS.get(rc, rc), msg.decode() if msg else ""))

    @property
    def n(self):
        return self.cfg.n_grid

    def set_stream(self, stream_handle):
        self._chk(lib().cg_set_stream(self._c, C.c_void_p(stream_handle)), "cg_set_stream")

    def sync(self):
        self._chk(lib().cg_sync(self._c), "cg_sync")

    def upload_tables(self):
        self._chk(lib().cg_upload_tables(self._c, C.byref(self.cfg)), "cg_upload_tables")

    # stages (src/main.c:66-125)
    def create_cartesian_fields(self):
        self._chk(lib().cg_create_cartesian_fields(self._c), "create_cartesian_fields")

    def sigma2(self):
        s, m = C.c_double(), C.c_double()
        self._chk(lib().cg_get_sigma2(self._c, C.byref(s), C.byref(m)), "get_sigma2")
        return s.value, m.value

    def compute_physical_density_field(self):
        self._chk(lib().cg_compute_physical_density_field(self._c), "compute_physical_density_field")

    def compute_density_normalization(self):
        self._chk(lib().cg_compute_density_normalization(self._c), "compute_density_normalization")

    def srcs_set_cartesian(self):
        n = (C.c_longlong * NPOP_MAX)()
        self._chk(lib().cg_srcs_set_cartesian(self._c, n), "srcs_set_cartesian")
        return [n[i] for i in range(self.cfg.n_srcs)]

    def imap_set_cartesian(self):
        self._chk(lib().cg_imap_set_cartesian(self._c), "imap_set_cartesian")

    def set_imap_list_cap(self, cap):
        """Bound the intensity-map cell list (0: by free device memory);
        cells past it are painted by the listing kernel."""
        self._chk(lib().cg_set_imap_list_cap(self._c, int(cap)), "set_imap_list_cap")

    def set_host_outputs(self, catalogs=None, imaps=None, kappa=None):
        """Register page-locked host arrays that run() fills as each output
        is final, overlapping the later stages (valid after sync()):
        catalogs {ipop: (src float32 (cap, 9), n int64 (1,))}, imaps
        {ipop: float32 (nr, npix)}, kappa float32 (n_kappa, npix).  Passing
        None for a group leaves it as it is; an entry of None stops it."""
        L = lib()
        hold = self.__dict__.setdefault("_host_out", {})
        for ip, v in (catalogs or {}).items():
            if v is None:
                self._chk(L.cg_set_host_catalog(self._c, ip, None, 0, None), "set_host_catalog")
                hold.pop(("cat", ip), None)
                continue
            src, n = v
            if src.dtype != np.float32 or src.ndim != 2 or src.shape[1] != 9 or not src.flags.c_contiguous:
                raise ValueError("catalogue buffers are C-contiguous float32 arrays of shape (cap, 9)")
            if n.dtype != np.int64 or n.size < 1:
                raise ValueError("the count slot is an int64 array")
            self._chk(L.cg_set_host_catalog(self._c, ip, src.ctypes.data, src.shape[0], n.ctypes.data),
                      "set_host_catalog")
            hold[("cat", ip)] = v
        for ip, a in (imaps or {}).items():
            if a is not None:
                ns, nr = self.cfg.nside_imap[ip], self.cfg.imap_nr[ip]
                if a.dtype != np.float32 or a.size != nr * 12 * ns * ns or not a.flags.c_contiguous:
                    raise ValueError("map buffers are C-contiguous float32 arrays of nr x 12 nside^2")
            self._chk(L.cg_set_host_imap(self._c, ip, a.ctypes.data if a is not None else None), "set_host_imap")
            hold[("imap", ip)] = a
        if kappa is not None:
            ns = self.cfg.nside_kappa
            if kappa.dtype != np.float32 or kappa.size != self.cfg.n_kappa * 12 * ns * ns or \
                    not kappa.flags.c_contiguous:
                raise ValueError("the kappa buffer is a C-contiguous float32 array of n_kappa x 12 nside^2")
            self._chk(L.cg_set_host_kappa(self._c, kappa.ctypes.data), "set_host_kappa")
            hold["kappa"] = kappa

    def imap_samples(self, ipop):
        """Sub-samples painted for intensity species ipop by the last run."""
        n = C.c_ulonglong()
        self._chk(lib().cg_imap_samples(self._c, ipop, C.byref(n)), "imap_samples")
        return n.value

    def get_beam_properties(self):
        self._chk(lib().cg_get_beam_properties(self._c), "get_beam_properties")

    def run(self):
        self._chk(lib().cg_run_mock(self._c), "run_mock")

    def launches(self):
        return lib().cg_kernel_launches(self._c)

    def set_profiling(self, on=True):
        self._chk(lib().cg_set_profiling(self._c, 1 if on else 0), "set_profiling")

    def kernel_times(self):
        """[(group name, ms)] of the launch groups since the last call."""
        names = C.create_string_buffer(1 << 16)
        ms = (C.c_float * 4096)()
        n = C.c_int()
        self._chk(lib().cg_kernel_times(self._c, names, 1 << 16, ms, 4096, C.byref(n)), "kernel_times")
        nm = [s for s in names.value.decode().split(";") if s]
        return list(zip(nm, [ms[i] for i in range(min(n.value, 4096))]))

    # host mirrors
    def grid(self, which=0, out=None):
        """Padded grid `which` (cg_download_grid) into a new host array, or
        into `out`: a host array or a CUDA torch tensor of the padded shape."""
        a = out if out is not None else np.empty(grid_shape(self.n), np.float32)
        ptr = a.data_ptr() if hasattr(a, "data_ptr") else a.ctypes.data
        self._chk(lib().cg_download_grid(self._c, which, ptr), "download_grid")
        return a

    def num_sources(self, ipop):
        return lib().cg_num_sources(self._c, ipop)

    def catalog(self, ipop, pos=True, ipix=True, src=True, out=None):
        n = self.num_sources(ipop)
        d = out or {}
        if pos and "pos" not in d:
            d["pos"] = np.empty((n, 4), np.float32)
        if ipix and "ipix" not in d:
            d["ipix"] = np.empty(n, np.int32)
        if src and "src" not in d:
            d["src"] = np.empty((n, 9), np.float32)
        ptr = lambda k: d[k].ctypes.data if (k in d and d[k] is not None and n > 0) else None
        self._chk(lib().cg_download_catalog(self._c, ipop, ptr("pos"), ptr("ipix"), ptr("src")), "download_catalog")
        return d

    def count_map(self, ipop, out=None):
        ns = self.cfg.nside_count[ipop]
        a = out if out is not None else np.empty(12 * ns * ns, np.int32)
        self._chk(lib().cg_download_count_map(self._c, ipop, a.ctypes.data), "download_count_map")
        return a

    def imap(self, ipop, with_nadd=False, out=None):
        ns, nr = self.cfg.nside_imap[ipop], self.cfg.imap_nr[ipop]
        m = out if out is not None else np.empty((nr, 12 * ns * ns), np.float32)
        na = np.empty((nr, 12 * ns * ns), np.int32) if with_nadd else None
        self._chk(lib().cg_download_imap(self._c, ipop, m.ctypes.data, na.ctypes.data if with_nadd else None),
                  "download_imap")
        return (m, na) if with_nadd else m

    def isw(self, out=None):
        """ISW maps, n_isw x 12 nside_isw^2, RING order."""
        ns = self.cfg.nside_isw
        m = out if out is not None else np.empty((self.cfg.n_isw, 12 * ns * ns), np.float32)
        self._chk(lib().cg_download_isw(self._c, m.ctypes.data), "download_isw")
        return m

    def skewers(self, ipop):
        """(dens, vel) skewers of population ipop, n_sources x n_grid/2 each."""
        n = self.num_sources(ipop)
        nr = self.cfg.n_grid // 2
        d = np.empty((n, nr), np.float32)
        v = np.empty((n, nr), np.float32)
        self._chk(lib().cg_download_skewers(self._c, ipop, d.ctypes.data, v.ctypes.data), "download_skewers")
        return d, v

    def custom(self, ipop, out=None):
        """Custom map ipop, 12 nside_cstm^2 values in NEST order (the order the
        reference's custom-map writer stores)."""
        ns = self.cfg.nside_cstm[ipop]
        m = out if out is not None else np.empty(12 * ns * ns, np.float32)
        self._chk(lib().cg_download_custom(self._c, ipop, m.ctypes.data), "download_custom")
        return m

    def kappa(self, out=None):
        ns = self.cfg.nside_kappa
        m = out if out is not None else np.empty((self.cfg.n_kappa, 12 * ns * ns), np.float32)
        self._chk(lib().cg_download_kappa(self._c, m.ctypes.data), "download_kappa")
        return m

    def norm_table(self, kind, ipop):
        """Current FP32 normalisation table (kind 0: sources, 1: intensity maps)
        and its (below, above) edge values, as used by the kernels."""
        t = np.empty(NA, np.float32)
        e = np.empty(2, np.float32)
        self._chk(lib().cg_download_norm(self._c, kind, ipop, t.ctypes.data, e.ctypes.data), "download_norm")
        return t, e

    def norm_table64(self, kind, ipop):
        """The same table in double, as the double decisions read it."""
        t = np.empty(NA, np.float64)
        e = np.empty(2, np.float64)
        self._chk(lib().cg_download_norm64(self._c, kind, ipop, t.ctypes.data, e.ctypes.data), "download_norm64")
        return t, e

    # passes of the transform whose tile width the autotuner picks
    PASSES = {"fill2": 0, "fill3": 1, "y": 2, "x": 3}

    def set_field_variant(self, pass_name, v):
        """Force tile variant v (0 the plan's, 1 half, 2 twice; -1 the tuner's
        choice) for one pass of the transforms."""
        self._chk(lib().cg_set_field_variant(self._c, self.PASSES[pass_name], v), "set_field_variant")

    def field_plan(self):
        """The transform passes' tile widths in use at this grid size and the
        autotuner's timings per candidate (ms), as a dict."""
        import json
        buf = C.create_string_buffer(4096)
        self._chk(lib().cg_field_plan(self._c, buf, len(buf)), "field_plan")
        return json.loads(buf.value.decode())

    def set_decisions_in_double(self, on=True):
        """Take every integer decision (counts, pixels, hits) in double."""
        self._chk(lib().cg_set_decisions_in_double(self._c, 1 if on else 0), "set_decisions_in_double")

    def exact_stats(self, reset=False):
        """Decisions taken in double since the last reset: dict of counts."""
        a = np.zeros(4, np.uint64)
        self._chk(lib().cg_exact_stats(self._c, a.ctypes.data, 1 if reset else 0), "exact_stats")
        return dict(count_cells=int(a[0]), src_pixels=int(a[1]), imap_cells=int(a[2]), imap_samples=int(a[3]))


class Batch:
    """Independent realisations run as graph replays over several streams
    (cg_batch_* C ABI).  nstreams = 0 autotunes the stream count."""

    def __init__(self, params_list, device=0, nstreams=0):
        self.params = list(params_list)
        n = len(self.params)
        self._cfgs = (Config * n)(*[p.config for p in self.params])
        self._b = C.c_void_p()
        L = lib()
        rc = L.cg_batch_create(C.byref(self._b), n, C.cast(self._cfgs, C.c_void_p), device, nstreams)
        if rc:
            msg = L.cg_batch_last_error(self._b) if self._b else b""
            self.close()
            raise CGError("cg_batch_create: %s (%s)" % (ERRORS.get(rc, rc), msg.decode() if msg else ""))
        self.mocks = [Mock(self.params[i], _handle=L.cg_batch_context(self._b, i)) for i in range(n)]
        self._hold = {}  # host catalogue buffers the runs write to

    def run(self):
        """Every realisation once; returns the device time of the pass in ms."""
        ms = C.c_float()
        rc = lib().cg_batch_run(self._b, C.byref(ms))
        if rc:
            raise CGError("cg_batch_run: %s (%s)" % (ERRORS.get(rc, rc), lib().cg_batch_last_error(self._b).decode()))
        return ms.value

    def set_host_catalog(self, i, ipop, src, n_out):
        """Copy realisation i's Src array of population ipop into src (a
        page-locked float32 array of shape (cap, 9)) and its source count
        into n_out[0] (a page-locked int64 array) during every run(); None
        stops the copies."""
        if src is None:
            rc = lib().cg_batch_set_host_catalog(self._b, i, ipop, None, 0, None)
            self._hold.pop(i, None)
        else:
            if src.dtype != np.float32 or src.ndim != 2 or src.shape[1] != 9 or not src.flags.c_contiguous:
                raise ValueError("src must be a C-contiguous float32 array of shape (cap, 9)")
            if n_out.dtype != np.int64 or n_out.size < 1:
                raise ValueError("n_out must be an int64 array")
            rc = lib().cg_batch_set_host_catalog(self._b, i, ipop, src.ctypes.data, src.shape[0], n_out.ctypes.data)
            if not rc:
                self._hold[i] = (src, n_out)
        if rc:
            raise CGError("cg_batch_set_host_catalog: %s (%s)" % (ERRORS.get(rc, rc),
                                                                  lib().cg_batch_last_error(self._b).decode()))

    @property
    def streams(self):
        return lib().cg_batch_streams(self._b)

    def tuning(self):
        buf = (C.c_float * 16)()
        k = lib().cg_batch_tuning(self._b, buf, 16)
        return list(buf[:k])

    def close(self):
        if getattr(self, "mocks", None):
            for m in self.mocks:
                m.close()
        if getattr(self, "_b", None):
            lib().cg_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Mock64:
    """The plain FP64 path of the same sequence on the same GPU (cg64_* C ABI):
    the baseline the FP32 path is measured against."""

    def __init__(self, params, device=0):
        self.params = params
        self.cfg = params.config
        self._c = C.c_void_p()
        rc = lib().cg64_create(C.byref(self._c), C.byref(self.cfg), device)
        if rc:
            raise CGError("cg64_create failed (%s)" % ERRORS.get(rc, rc))

    def close(self):
        if getattr(self, "_c", None):
            lib().cg64_destroy(self._c)
            self._c = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc, what):
        if rc:
            msg = lib().cg64_last_error(self._c)
            raise CGError("%s: %s (%s)" % (what, ERRORS.get(rc, rc), msg.decode() if msg else ""))

    def run(self):
        """Run the whole sequence; returns its device time in ms."""
        ms = C.c_float()
        self._chk(lib().cg64_run_mock(self._c, C.byref(ms)), "cg64_run_mock")
        return ms.value

    def create_cartesian_fields(self):
        """Only the Gaussian field and potential (then density(0) is delta_G)."""
        self._chk(lib().cg64_create_cartesian_fields(self._c), "cg64_create_cartesian_fields")

    def num_sources(self, ipop):
        return lib().cg64_num_sources(self._c, ipop)

    def density(self, which=0, out=None):
        """Unpadded N^3 doubles of the density (0) or potential (1), into a new
        host array or into `out` (a host array or a CUDA torch tensor)."""
        n = self.cfg.n_grid
        a = out if out is not None else np.empty((n, n, n), np.float64)
        ptr = a.data_ptr() if hasattr(a, "data_ptr") else a.ctypes.data
        self._chk(lib().cg64_download(self._c, which, 0, ptr), "cg64_download")
        return a

    def imap(self, ipop):
        """(summed temperatures, hit counts), nr x npix in RING order."""
        ns, nr = self.cfg.nside_imap[ipop], self.cfg.imap_nr[ipop]
        d = np.empty((nr, 12 * ns * ns), np.float64)
        k = np.empty((nr, 12 * ns * ns), np.int32)
        self._chk(lib().cg64_download(self._c, 2, ipop, d.ctypes.data), "cg64_download")
        self._chk(lib().cg64_download(self._c, 3, ipop, k.ctypes.data), "cg64_download")
        return d, k

    def kappa(self):
        ns = self.cfg.nside_kappa
        m = np.empty((self.cfg.n_kappa, 12 * ns * ns), np.float64)
        self._chk(lib().cg64_download(self._c, 4, 0, m.ctypes.data), "cg64_download")
        return m

    def count_map(self, ipop):
        """Sources of population ipop per RING pixel at nside_count[ipop]."""
        ns = self.cfg.nside_count[ipop]
        m = np.empty(12 * ns * ns, np.int32)
        self._chk(lib().cg64_download(self._c, 6, ipop, m.ctypes.data), "cg64_download")
        return m

    def norm_table(self, tracer):
        t = np.empty(NA, np.float64)
        self._chk(lib().cg64_download(self._c, 5, tracer, t.ctypes.data), "cg64_download")
        return t
