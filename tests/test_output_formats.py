"""Output writers (no GPU): HEALPix maps and catalogues as FITS binary tables
and ASCII, density grids in the native binary layout, read back with a small
FITS reader written here (2880-byte blocks, 80-character cards, big-endian
data) and checked against the keywords and columns of the reference's
writers (healpix_extra.c:4-57, io.c:565-595, io.c:1069-1236)."""
import os
import struct

import numpy as np


def read_fits(fname):
    """[(header dict, raw data bytes)] for every HDU of a FITS file."""
    raw = open(fname, "rb").read()
    assert len(raw) % 2880 == 0
    hdus, pos = [], 0
    while pos < len(raw):
        hdr, order = {}, []
        while True:
            card = raw[pos:pos + 80].decode("ascii")
            pos += 80
            key = card[:8].strip()
            if key == "END":
                break
            if card[8:10] == "= ":
                v = card[10:].split("/")[0].strip() if not card[10:].strip().startswith("'") else \
                    card[10:].strip()[1:].split("'")[0].rstrip()
                if v in ("T", "F"):
                    v = v == "T"
                else:
                    try:
                        v = int(v)
                    except ValueError:
                        pass
                hdr[key] = v
                order.append(key)
        pos = (pos + 2879) // 2880 * 2880
        nbytes = 0
        if hdr.get("NAXIS", 0) > 0:
            nbytes = abs(hdr["BITPIX"]) // 8 * hdr["NAXIS1"] * hdr["NAXIS2"]
        hdr["_order"] = order
        hdus.append((hdr, raw[pos:pos + nbytes]))
        pos += (nbytes + 2879) // 2880 * 2880
    return hdus


def test_healpix_map_fits(built, tmp_path):
    import colore_gb300 as cg
    nside = 8
    m = np.random.default_rng(1).standard_normal(12 * nside * nside).astype(np.float32)
    f = str(tmp_path / "map.fits")
    cg.write_healpix_map(f, m, nside)
    (h0, d0), (h1, d1) = read_fits(f)
    assert h0["SIMPLE"] is True and h0["NAXIS"] == 0 and h0["EXTEND"] is True and d0 == b""
    assert h1["XTENSION"] == "BINTABLE" and h1["NAXIS1"] == 4 and h1["NAXIS2"] == m.size
    assert (h1["TFIELDS"], h1["TTYPE1"], h1["TFORM1"], h1["TUNIT1"]) == (1, "map 1", "1E", "uK")
    assert (h1["PIXTYPE"], h1["ORDERING"], h1["NSIDE"], h1["COORDSYS"]) == ("HEALPIX", "RING", nside, "G")
    assert np.array_equal(np.frombuffer(d1, ">f4"), m)


def _src(n, seed):
    rng = np.random.default_rng(seed)
    s = np.zeros((n, 9), np.float32)
    s[:, 0] = rng.uniform(0, 360, n)
    s[:, 1] = rng.uniform(-90, 90, n)
    s[:, 2] = rng.uniform(0, 1.5, n)
    s[:, 3] = rng.normal(0, 1e-3, n)
    s[:, 4:6] = -1
    return s


def test_catalog_fits(built, tmp_path):
    import colore_gb300 as cg
    s = _src(1234, 2)
    prefix = str(tmp_path / "out")
    cg.write_catalog(prefix, 1, s, cg.OUT_FITS)
    (h0, _), (h1, d1) = read_fits(prefix + "_srcs_s2_0.fits")
    assert h1["TFIELDS"] == 5 and h1["NAXIS1"] == 20 and h1["NAXIS2"] == len(s)
    assert [h1["TTYPE%d" % i] for i in range(1, 6)] == ["TYPE", "RA", "DEC", "Z_COSMO", "DZ_RSD"]
    assert [h1["TFORM%d" % i] for i in range(1, 6)] == ["1J", "1E", "1E", "1E", "1E"]
    assert [h1["TUNIT%d" % i] for i in range(1, 6)] == ["NA", "DEG", "DEG", "NA", "NA"]
    assert h1["CONTENTS"] == "Source catalog"
    rows = np.frombuffer(d1, np.dtype([("t", ">i4"), ("c", ">f4", (4,))]))
    assert np.all(rows["t"] == 1)
    assert np.array_equal(rows["c"], s[:, :4])


def test_catalog_ascii(built, tmp_path):
    import colore_gb300 as cg
    s = _src(300, 3)
    prefix = str(tmp_path / "out")
    cg.write_catalog(prefix, 0, s, cg.OUT_ASCII)
    lines = open(prefix + "_srcs_s1_0.txt").read().splitlines()
    assert lines[0] == "#[1]type [2]RA, [3]dec, [4]z0, [5]dz_RSD "
    a = np.array([[float(x) for x in ln.split()] for ln in lines[1:]])
    assert a.shape == (300, 5) and np.all(a[:, 0] == 0)
    np.testing.assert_allclose(a[:, 1:], s[:, :4], rtol=1e-6, atol=1e-12)
    assert lines[1].endswith(" ") and "E" in lines[1]


def test_empty_catalog(built, tmp_path):
    import colore_gb300 as cg
    prefix = str(tmp_path / "e")
    cg.write_catalog(prefix, 0, np.zeros((0, 9), np.float32), cg.OUT_FITS)
    (_, _), (h1, d1) = read_fits(prefix + "_srcs_s1_0.fits")
    assert h1["NAXIS2"] == 0 and d1 == b""


def test_density_grid_binary(built, tmp_path):
    import colore_gb300 as cg
    n = 16
    g = np.random.default_rng(4).standard_normal((n, n, 2 * (n // 2 + 1))).astype(np.float32)
    prefix = str(tmp_path / "d")
    cg.write_density_grid(prefix, "lightcone", g, 123.5)
    raw = open(prefix + "_dens_lightcone_0.dat", "rb").read()
    nn, sz, lb, ng, nz, iz0 = struct.unpack("=iidiii", raw[:28])
    assert (nn, sz, lb, ng, nz, iz0) == (1, 4, 123.5, n, n, 0)
    body = np.frombuffer(raw[28:], np.float32).reshape(n, n, n)
    assert np.array_equal(body, g[:, :, :n])
    assert len(raw) == 28 + 4 * n ** 3
    assert os.path.getsize(prefix + "_dens_lightcone_0.dat") == len(raw)
