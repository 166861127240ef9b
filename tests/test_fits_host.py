"""The FITS primary-array reader of the fits_to_hpc drop-in
(acumen_gb300/drivers/fits.h), on the host: every BITPIX the FITS standard
allows for a primary array, BZERO/BSCALE scaling, headers longer than one
2880-byte block, comments after values, a degenerate third axis, and the
errors for files it cannot read.  The reference reads these files with
cfitsio's ftgpve (tomography/fits_to_hpc.F90:160-210), which returns
BZERO + BSCALE * stored value in single precision.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
DRIVERS = os.path.join(HERE, "..", "acumen_gb300", "drivers")

HARNESS = r"""
#include <cstdio>
#include "fits.h"
int main(int argc, char** argv)
{
    try {
        const hpc::FitsImage im = hpc::read_fits(argv[1]);
        FILE* f = std::fopen(argv[2], "wb");
        const long long dims[2] = {im.naxis1, im.naxis2};
        std::fwrite(dims, sizeof dims[0], 2, f);
        std::fwrite(im.data.data(), sizeof(float), im.data.size(), f);
        std::fclose(f);
        return 0;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
}
"""


@pytest.fixture(scope="module")
def reader(tmp_path_factory):
    cxx = os.environ.get("CXX", "g++")
    if shutil.which(cxx) is None:
        pytest.skip("no C++ compiler")
    d = tmp_path_factory.mktemp("fits")
    src, exe = d / "read.cpp", d / "read"
    src.write_text(HARNESS)
    r = subprocess.run([cxx, "-O1", "-std=c++17", "-Wall", "-I" + DRIVERS, str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr

    def read(path):
        out = path.with_suffix(".out")
        p = subprocess.run([str(exe), str(path), str(out)], capture_output=True, text=True, timeout=60)
        if p.returncode != 0:
            return None, p.stderr
        raw = out.read_bytes()
        n1, n2 = np.frombuffer(raw[:16], np.int64)
        return np.frombuffer(raw[16:], np.float32).reshape(int(n2), int(n1)), ""

    return read


def card(key, value, comment=None):
    s = f"{key:<8}= {value:>20}"
    if comment is not None:
        s += f" / {comment}"
    return s.ljust(80)[:80]


def fits_bytes(cards, data_bytes):
    head = "".join(cards) + "END".ljust(80)
    head = head.ljust((len(head) + 2879) // 2880 * 2880)
    pad = b"\0" * ((-len(data_bytes)) % 2880)
    return head.encode("ascii") + data_bytes + pad


STORED = {8: ">u1", 16: ">i2", 32: ">i4", 64: ">i8", -32: ">f4", -64: ">f8"}


def sample(bitpix, shape, rng):
    t = np.dtype(STORED[bitpix])
    if t.kind == "f":
        return (rng.standard_normal(shape) * 1e3).astype(t)
    info = np.iinfo(t)
    lo, hi = max(info.min, -(1 << 40)), min(info.max, 1 << 40)
    v = rng.integers(lo, hi, size=shape, endpoint=True)
    v.flat[0], v.flat[-1] = lo, hi    # the extremes of the stored type
    return v.astype(t)


@pytest.mark.parametrize("bitpix", [8, 16, 32, 64, -32, -64])
@pytest.mark.parametrize("scaled", [False, True])
def test_every_bitpix(reader, tmp_path, bitpix, scaled):
    rng = np.random.default_rng(abs(bitpix) * 2 + scaled)
    h, w = 7, 13
    v = sample(bitpix, (h, w), rng)
    bzero, bscale = (32768.0, 0.5) if scaled else (0.0, 1.0)
    cards = [card("SIMPLE", "T"), card("BITPIX", str(bitpix)), card("NAXIS", "2"),
             card("NAXIS1", str(w)), card("NAXIS2", str(h))]
    if scaled:
        cards += [card("BZERO", "32768", "offset"), card("BSCALE", "0.5")]
    p = tmp_path / "a.fits"
    p.write_bytes(fits_bytes(cards, v.tobytes()))
    got, err = reader(p)
    assert got is not None, err
    want = (bzero + bscale * v.astype(np.float64)).astype(np.float32)
    np.testing.assert_array_equal(got, want)


def test_unsigned_16_bit_detector_counts(reader, tmp_path):
    """The usual detector file: unsigned 16-bit counts stored as BITPIX 16
    with BZERO 32768; every count from 0 to 65535 is read back exactly."""
    counts = np.arange(65536, dtype=np.int64).reshape(256, 256)
    cards = [card("SIMPLE", "T"), card("BITPIX", "16"), card("NAXIS", "2"), card("NAXIS1", "256"),
             card("NAXIS2", "256"), card("BZERO", "32768"), card("BSCALE", "1")]
    p = tmp_path / "u16.fits"
    p.write_bytes(fits_bytes(cards, (counts - 32768).astype(">i2").tobytes()))
    got, err = reader(p)
    assert got is not None, err
    np.testing.assert_array_equal(got, counts.astype(np.float32))


def test_long_header_comments_and_third_axis(reader, tmp_path):
    """A header of two blocks (keywords the reader does not use, COMMENT and
    HISTORY cards, a string value holding a slash) and NAXIS = 3 with
    NAXIS3 = 1 read as the 2-D image."""
    h, w = 5, 4
    v = np.arange(h * w, dtype=">i4").reshape(h, w)
    cards = [card("SIMPLE", "T", "conforms"), card("BITPIX", "32", "bits"), card("NAXIS", "3"),
             card("NAXIS1", str(w), "fastest"), card("NAXIS2", str(h)), card("NAXIS3", "1")]
    cards += [card(f"KEY{k}", str(k), "filler") for k in range(40)]
    cards += [("COMMENT   a / slash in a comment card").ljust(80), ("HISTORY   written by a test").ljust(80),
              card("OBJECT", "'a/b     '"), card("BZERO", "-1.5E+01", "exponent form")]
    p = tmp_path / "long.fits"
    p.write_bytes(fits_bytes(cards, v.tobytes()))
    assert len(p.read_bytes()) > 2 * 2880
    got, err = reader(p)
    assert got is not None, err
    np.testing.assert_array_equal(got, (v.astype(np.float64) - 15.0).astype(np.float32))


@pytest.mark.parametrize("case, message", [
    ("not_fits", "SIMPLE"),
    ("bitpix", "BITPIX"),
    ("cube", "2-D"),
    ("short_data", "truncated FITS data"),
    ("short_header", "truncated FITS header"),
    ("missing", "cannot open"),
])
def test_errors(reader, tmp_path, case, message):
    h, w = 3, 3
    v = np.zeros((h, w), ">i2")
    base = [card("SIMPLE", "T"), card("BITPIX", "16"), card("NAXIS", "2"), card("NAXIS1", str(w)),
            card("NAXIS2", str(h))]
    p = tmp_path / f"{case}.fits"
    if case == "not_fits":
        p.write_bytes(fits_bytes([card("SIMPLE", "F")] + base[1:], v.tobytes()))
    elif case == "bitpix":
        p.write_bytes(fits_bytes([base[0], card("BITPIX", "12")] + base[2:], v.tobytes()))
    elif case == "cube":
        cards = [base[0], base[1], card("NAXIS", "3"), base[3], base[4], card("NAXIS3", "2")]
        p.write_bytes(fits_bytes(cards, np.zeros((2, h, w), ">i2").tobytes()))
    elif case == "short_data":
        p.write_bytes(fits_bytes(base, v.tobytes())[:2880 + 10])
    elif case == "short_header":
        p.write_bytes(fits_bytes(base, v.tobytes())[:1000])
    got, err = reader(p)
    assert got is None and message in err, err
