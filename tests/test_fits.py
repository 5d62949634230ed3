"""FITS I/O of MW / MWSS maps (host code, no GPU): the s2let_fits entry points
(include/s2let/s2let_fits.h:18-106) written from the FITS standard instead of
cfitsio.  Round trips are bit-exact; files are checked by an independent
parse here (80-character cards, 2880-byte blocks, big-endian data); the
reference's own data file data/earth_tomo_mw_128.fits (4-byte float column)
is read when the reference tree is present."""
import ctypes as C
import os

import numpy as np
import pytest

from s2let_gb300.capi import FITS_SIGNATURES, GPU_SIGNATURES, SIGNATURES, bind, ptr


@pytest.fixture(scope="module")
def lib():
    import s2let_gb300

    path = s2let_gb300.LIB_PATH
    if not os.path.exists(path):
        pytest.skip("library not built")
    lib = C.CDLL(path)
    for table in (SIGNATURES, GPU_SIGNATURES, FITS_SIGNATURES):
        bind(lib, table, required=False)
    return lib


def parse_fits(path, strict=True):
    """Minimal independent reader of the first two HDUs: (raw bytes, [(header
    dict, data offset)]).  strict: the file is padded to whole 2880-byte blocks
    (ours are; the reference's data file ends mid-block)."""
    raw = open(path, "rb").read()
    if strict:
        assert len(raw) % 2880 == 0
    hdus, pos = [], 0
    while len(hdus) < 2 and pos < len(raw):
        h = {}
        while True:
            block = raw[pos:pos + 2880]
            pos += 2880
            cards = [block[i:i + 80].decode("ascii") for i in range(0, 2880, 80)]
            done = False
            for c in cards:
                if c.startswith("END"):
                    done = True
                    break
                if c[8:10] == "= ":
                    v = c[10:].split("/")[0].strip() if not c[10:].strip().startswith("'") else \
                        c[10:].strip()[1:].split("'")[0].strip()
                    h[c[:8].strip()] = v
            if done:
                break
        hdus.append((h, pos))
        n = 0
        if int(h.get("NAXIS", 0)) > 0:
            n = abs(int(h["BITPIX"])) // 8
            for i in range(1, int(h["NAXIS"]) + 1):
                n *= int(h[f"NAXIS{i}"])
        pos += (n + 2879) // 2880 * 2880
    return raw, hdus


def column(raw, h, off, col):
    nrows, width = int(h["NAXIS2"]), int(h["NAXIS1"])
    forms = [h[f"TFORM{c}"] for c in range(1, int(h["TFIELDS"]) + 1)]
    size = {"D": 8, "E": 4}
    start = sum(size[f[-1]] * (int(f[:-1]) if f[:-1] else 1) for f in forms[:col - 1])
    f = forms[col - 1]
    rep = int(f[:-1]) if f[:-1] else 1
    dt = ">f8" if f[-1] == "D" else ">f4"
    rows = np.frombuffer(raw[off:off + nrows * width], dtype=np.uint8).reshape(nrows, width)
    return rows[:, start:start + size[f[-1]] * rep].copy().view(dt).ravel().astype(np.float64)


@pytest.mark.parametrize("L,mwss", [(8, False), (13, True), (32, False)])
def test_map_round_trip_and_layout(lib, tmp_path, L, mwss):
    npx = (L + 1) * 2 * L if mwss else L * (2 * L - 1)
    f = np.random.default_rng(L).normal(size=npx)
    name = str(tmp_path / "m.fits").encode()
    (lib.s2let_fits_mwss_write_map if mwss else lib.s2let_fits_mw_write_map)(name, ptr(f), L)
    assert lib.s2let_gpu_last_error() == 0
    g = np.zeros(npx)
    (lib.s2let_fits_mwss_read_map if mwss else lib.s2let_fits_mw_read_map)(ptr(g), name, L)
    assert lib.s2let_gpu_last_error() == 0
    np.testing.assert_array_equal(g, f)
    assert lib.s2let_fits_mw_read_bandlimit(name) == L
    assert lib.s2let_fits_hpx_read_nside(name) == -1
    raw, hdus = parse_fits(name.decode())
    (p, _), (h, off) = hdus
    assert p["SIMPLE"] == "T" and p["NAXIS"] == "0" and p["EXTEND"] == "T"
    assert h["XTENSION"] == "BINTABLE" and h["EXTNAME"] == "BINTABLE" and h["TTYPE1"] == "SIGNAL"
    assert h["TFORM1"] == "1D" and int(h["NAXIS2"]) == npx and int(h["L"]) == L
    assert (h.get("MWSS") == "1") == mwss
    np.testing.assert_array_equal(column(raw, h, off, 1), f)


@pytest.mark.parametrize("mwss", [False, True])
def test_spin_maps_round_trip(lib, tmp_path, capfd, mwss):
    L = 9
    npx = (L + 1) * 2 * L if mwss else L * (2 * L - 1)
    rng = np.random.default_rng(3)
    q, u = rng.normal(size=npx), rng.normal(size=npx)
    name = str(tmp_path / "s.fits").encode()
    (lib.s2let_fits_mwss_write_spin_maps if mwss else lib.s2let_fits_mw_write_spin_maps)(name, ptr(q), ptr(u), L)
    q2, u2 = np.zeros(npx), np.zeros(npx)
    (lib.s2let_fits_mwss_read_spin_maps if mwss else lib.s2let_fits_mw_read_spin_maps)(ptr(q2), ptr(u2), name, L)
    assert lib.s2let_gpu_last_error() == 0
    np.testing.assert_array_equal(q2, q)
    np.testing.assert_array_equal(u2, u)
    out = capfd.readouterr().out  # the reference prints the table shape (src/c/s2let_fits.c:430-431)
    assert "naxis[0] = 16" in out and f"naxis[1] = {npx}" in out
    raw, hdus = parse_fits(name.decode())
    h, off = hdus[1]
    assert h["TTYPE1"] == "Q_POLARISATION" and h["TTYPE2"] == "U_POLARISATION"
    np.testing.assert_array_equal(column(raw, h, off, 2), u)


def test_existing_file_needs_bang_and_wrong_L_warns(lib, tmp_path, capfd):
    L = 6
    f = np.arange(L * (2 * L - 1), dtype=np.float64)
    path = tmp_path / "w.fits"
    lib.s2let_fits_mw_write_map(str(path).encode(), ptr(f), L)
    before = path.read_bytes()
    lib.s2let_fits_mw_write_map(str(path).encode(), ptr(f * 2), L)  # cfitsio: file exists
    assert lib.s2let_gpu_last_error() != 0
    assert path.read_bytes() == before
    lib.s2let_fits_mw_write_map(("!" + str(path)).encode(), ptr(f * 2), L)
    assert lib.s2let_gpu_last_error() == 0
    g = np.zeros_like(f)
    capfd.readouterr()
    lib.s2let_fits_mw_read_map(ptr(g), str(path).encode(), L)
    np.testing.assert_array_equal(g, f * 2)
    # a file with more samples than asked for: the first ones are read, with the reference's warning
    h = np.zeros(5 * 9)
    lib.s2let_fits_mw_read_map(ptr(h), str(path).encode(), 5)
    assert "Attention : read L = 6 but you specified L = 5" in capfd.readouterr().out
    np.testing.assert_array_equal(h, f[:45] * 2)
    lib.s2let_fits_mw_read_map(ptr(g), str(tmp_path / "missing.fits").encode(), L)
    assert lib.s2let_gpu_last_error() != 0


def _reference_data_dir():
    from __graft_entry__ import REFERENCE_CHECKOUT

    return os.path.join(REFERENCE_CHECKOUT, "data")


def test_reads_the_reference_data_file(lib):
    path = os.path.join(_reference_data_dir(), "earth_tomo_mw_128.fits")
    if not os.path.exists(path):
        pytest.skip("reference data not present")
    L = lib.s2let_fits_mw_read_bandlimit(path.encode())
    assert L == 128
    f = np.zeros(L * (2 * L - 1))
    lib.s2let_fits_mw_read_map(ptr(f), path.encode(), L)
    assert lib.s2let_gpu_last_error() == 0
    raw, hdus = parse_fits(path, strict=False)
    h, off = hdus[1]
    assert h["TFORM1"] == "1E"
    np.testing.assert_array_equal(f, column(raw, h, off, 1))
    assert np.abs(f).max() > 0


def test_header_readers_on_the_reference_data_files(lib):
    """NSIDE of the reference's HEALPix files and L of its MW files; a missing
    keyword reads as -1 (src/c/s2let_fits.c:17-85)."""
    data = _reference_data_dir()
    files = {"somecmbsimu_hpx_128.fits": (128, -1), "wmap_mcmc_base_k_synch_stk_q_9yr_v5.fits": (64, -1),
             "earth_tomo_mw_128.fits": (-1, 128), "earth_tomo_mw_128_rot.fits": (-1, 128)}
    present = [f for f in files if os.path.exists(os.path.join(data, f))]
    if not present:
        pytest.skip("reference data not present")
    for f in present:
        path = os.path.join(data, f).encode()
        assert (lib.s2let_fits_hpx_read_nside(path), lib.s2let_fits_mw_read_bandlimit(path)) == files[f], f
        assert lib.s2let_gpu_last_error() == 0


def _set_card(raw, key, value):
    """raw bytes with the first header card `key` given the integer `value`"""
    k = raw.index(key.ljust(8).encode() + b"= ")
    card = (key.ljust(8) + "= " + str(value).rjust(20)).ljust(80).encode()
    return raw[:k] + card + raw[k + 80:]


@pytest.mark.parametrize("key,value", [("NAXIS1", 4), ("NAXIS1", 0), ("NAXIS2", -3)])
def test_malformed_table_header_is_rejected(lib, tmp_path, key, value):
    """A binary table whose column does not fit in its row (a header that
    claims narrower rows than its TFORMs), or with nonsensical row counts, is
    refused with a status; the output buffer is left as it was."""
    L = 6
    f = np.arange(L * (2 * L - 1), dtype=np.float64)
    good = tmp_path / "good.fits"
    lib.s2let_fits_mw_write_map(str(good).encode(), ptr(f), L)
    raw = good.read_bytes()
    ext = raw.index(b"XTENSION")
    bad = tmp_path / "bad.fits"
    bad.write_bytes(raw[:ext] + _set_card(raw[ext:], key, value))
    g = np.full_like(f, -7.0)
    lib.s2let_fits_mw_read_map(ptr(g), str(bad).encode(), L)
    assert lib.s2let_gpu_last_error() == 1
    assert (g == -7.0).all()
