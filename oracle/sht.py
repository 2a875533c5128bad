"""ORACLE angular power spectra of HEALPix RING maps (test infrastructure only).

An FP64 restatement of the reference's map -> C_ell path, for nside up to a
few hundred:

  he_anafast      (healpix_extra.c:467-514)  a_lm of each map up to lmax, then
  he_alm2cl       (healpix_extra.c:437-465)  C_l = [a_l0 b_l0 + 2 sum_{m>0}
                                             Re(a_lm b_lm*)] / (2l + 1)
  sht_wrapper     (healpix_extra.c:399-411)  libsharp's map2alm on the HEALPix
                                             geometry with unit ring weights:
                                             a_lm = (4 pi / Npix) sum_p map_p
                                             Y*_lm(theta_p, phi_p)

libsharp is not available here, so the transform is written from its
definition: per ring an FFT of the pixel values gives
F_m = exp(-i m phi_0) sum_j map_j exp(-2 pi i m j / n_ring) (periodic in m,
so m >= n_ring folds back), and per m the normalised associated Legendre
functions lambda_lm(z) (Condon-Shortley phase) come from the standard
three-term recursion in l, started from lambda_mm evaluated in logarithms so
that the polar rings underflow to zero instead of overflowing.  map2alm runs
the Legendre sums in C (or_sht.c, OpenMP over m, north and south rings
paired through lambda_lm(-z) = (-1)^(l+m) lambda_lm(z)); map2alm_py is the
same transform in numpy, kept as an independent check.  The ring geometry is
that of he_ang2pix (healpix_extra.c:141-172): the tests check that every
pixel centre produced here maps back to its own index, and both transforms
against scipy's spherical harmonics on small maps.
"""
import numpy as np


def ring_geometry(nside):
    """Per ring: cos(theta), phi of its first pixel, pixel count, first index."""
    ns = int(nside)
    npix = 12 * ns * ns
    z, phi0, nr, first = [], [], [], []
    for i in range(1, 4 * ns):
        if i < ns:                      # north polar cap
            z.append(1.0 - i * i / (3.0 * ns * ns))
            nr.append(4 * i)
            phi0.append(np.pi / (4.0 * i))
            first.append(2 * i * (i - 1))
        elif i <= 3 * ns:               # equatorial belt
            z.append(4.0 / 3.0 - 2.0 * i / (3.0 * ns))
            nr.append(4 * ns)
            phi0.append(np.pi / (4.0 * ns) if (i - ns) % 2 == 0 else 0.0)
            first.append(2 * ns * (ns - 1) + (i - ns) * 4 * ns)
        else:                           # south polar cap
            k = 4 * ns - i
            z.append(-(1.0 - k * k / (3.0 * ns * ns)))
            nr.append(4 * k)
            phi0.append(np.pi / (4.0 * k))
            first.append(npix - 2 * k * (k + 1))
    return np.array(z), np.array(phi0), np.array(nr, np.int64), np.array(first, np.int64)


def pixel_centres(nside):
    """(cos theta, phi) of every RING pixel centre, in index order."""
    z, phi0, nr, first = ring_geometry(nside)
    cth = np.empty(12 * nside * nside)
    phi = np.empty(12 * nside * nside)
    for zr, p0, n, f in zip(z, phi0, nr, first):
        cth[f:f + n] = zr
        phi[f:f + n] = p0 + 2.0 * np.pi * np.arange(n) / n
    return cth, phi


def _ring_fourier(maps, nside, lmax):
    """F[m, ring, map] for m = 0..lmax."""
    z, phi0, nr, first = ring_geometry(nside)
    K = maps.shape[0]
    m = np.arange(lmax + 1)
    F = np.empty((lmax + 1, len(z), K), np.complex128)
    for r, (p0, n, f) in enumerate(zip(phi0, nr, first)):
        c = np.fft.fft(maps[:, f:f + n], axis=1)          # sum_j x_j exp(-2 pi i k j / n)
        F[:, r, :] = (c[:, m % n] * np.exp(-1j * m * p0)[None, :]).T
    return F, z


def map2alm(maps, nside, lmax=None):
    """a_lm of one map or a stack of maps (RING order), as alm[k][l, m]
    (m <= l, zero above the diagonal), with pixel-area quadrature."""
    import ctypes as C
    import oracle as orc
    maps = np.atleast_2d(np.asarray(maps, np.float64))
    ns = int(nside)
    lmax = 3 * ns - 1 if lmax is None else int(lmax)
    z, phi0, nr, first = ring_geometry(ns)
    K = maps.shape[0]
    m = np.arange(lmax + 1)
    nn = 2 * ns  # northern rings, the equator included
    S = np.zeros((lmax + 1, nn, K), np.complex128)
    A = np.zeros((lmax + 1, nn, K), np.complex128)
    for r in range(len(z)):
        n, f = nr[r], first[r]
        c = np.fft.fft(maps[:, f:f + n], axis=1)
        Fr = (c[:, m % n] * np.exp(-1j * m * phi0[r])[None, :]).T
        if r < nn:
            S[:, r, :] += Fr
            A[:, r, :] += Fr
        else:
            q = 4 * ns - 2 - r  # the northern mirror
            S[:, q, :] += Fr
            A[:, q, :] -= Fr
    alm = np.zeros((K, lmax + 1, lmax + 1), np.complex128)
    zn = np.ascontiguousarray(z[:nn])
    rc = orc.lib().or_sht_legendre(lmax, nn, K, zn.ctypes.data, S.ctypes.data, A.ctypes.data,
                                   C.c_double(4.0 * np.pi / (12.0 * ns * ns)), alm.ctypes.data)
    if rc:
        raise MemoryError("or_sht_legendre")
    return alm


def map2alm_py(maps, nside, lmax=None):
    """map2alm in numpy (per m, the recursion over every ring and a matrix
    product with the ring Fourier sums)."""
    maps = np.atleast_2d(np.asarray(maps, np.float64))
    lmax = 3 * nside - 1 if lmax is None else int(lmax)
    F, z = _ring_fourier(maps, nside, lmax)
    K = maps.shape[0]
    omega = 4.0 * np.pi / (12.0 * nside * nside)
    s2 = np.maximum(1.0 - z * z, 0.0)
    logs = 0.5 * np.log(np.where(s2 > 0, s2, 1e-300))
    alm = np.zeros((K, lmax + 1, lmax + 1), np.complex128)
    logc = 0.0  # log of prod_{k<=m} (2k-1)/(2k)
    for m in range(lmax + 1):
        if m > 0:
            logc += np.log((2.0 * m - 1.0) / (2.0 * m))
        lam_mm = np.exp(0.5 * (np.log((2.0 * m + 1.0) / (4.0 * np.pi)) + logc) + m * logs)
        if m % 2:
            lam_mm = -lam_mm
        L = np.empty((lmax - m + 1, len(z)))
        L[0] = lam_mm
        if m < lmax:
            L[1] = np.sqrt(2.0 * m + 3.0) * z * lam_mm
        a_prev = np.sqrt(2.0 * m + 3.0)
        for l in range(m + 2, lmax + 1):
            a_l = np.sqrt((4.0 * l * l - 1.0) / (l * l - m * m))
            L[l - m] = a_l * (z * L[l - m - 1] - L[l - m - 2] / a_prev)
            a_prev = a_l
        Fm = F[m]
        alm[:, m:, m] = ((L @ np.ascontiguousarray(Fm.real)) + 1j * (L @ np.ascontiguousarray(Fm.imag))).T * omega
    return alm


def alm2cl(alm1, alm2=None):
    """C_l of he_alm2cl for each pair of maps of the two stacks (auto when
    alm2 is None): shape [K1][K2][lmax+1], or [K][lmax+1] for auto spectra."""
    lmax = alm1.shape[1] - 1
    l = np.arange(lmax + 1)
    w = np.full(lmax + 1, 2.0)
    w[0] = 1.0
    if alm2 is None:
        p = alm1.real ** 2 + alm1.imag ** 2
        return (p * w[None, None, :]).sum(axis=2) / (2.0 * l + 1.0)
    p = np.einsum("alm,blm->ablm", alm1.real, alm2.real) + np.einsum("alm,blm->ablm", alm1.imag, alm2.imag)
    return (p * w).sum(axis=3) / (2.0 * l + 1.0)


def anafast(maps, nside, lmax=None):
    """Auto spectra of a stack of RING maps (he_anafast with maps_1 == maps_2)."""
    return alm2cl(map2alm(maps, nside, lmax))
