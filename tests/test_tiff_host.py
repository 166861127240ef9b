"""The result-image tool (acumen_gb300/bin/to_tiff, in place of the
reference's tomography/convert_to_tiff.m and projections_sino_tiff.m), on the
CPU: a small reconstruction directory in the reference's file layout (slices
split over several files) is written by the test, and every TIFF the tool
writes is parsed back and compared with the pixels MATLAB's imwrite gives a
double matrix (round(255 v) clipped to [0, 1], the file's fastest index along
the image's rows), or with the floats themselves (ACUMEN_TIFF=float)."""
import os
import struct
import subprocess

import numpy as np
import pytest

from acumen_gb300 import build as B

NFILES, NIMG, NSINO, NREC = 5, 6, 2, 3          # nimage even: grid 7


def read_tiff(path):
    b = open(path, "rb").read()
    assert b[:4] == b"II*\x00"
    ifd = struct.unpack_from("<I", b, 4)[0]
    n = struct.unpack_from("<H", b, ifd)[0]
    tags = {}
    for i in range(n):
        tid, typ, cnt = struct.unpack_from("<HHI", b, ifd + 2 + 12 * i)
        val = struct.unpack_from("<H" if typ == 3 else "<I", b, ifd + 2 + 12 * i + 8)[0]
        tags[tid] = val
    w, h, bps = tags[256], tags[257], tags[258]
    off, nb = tags[273], tags[279]
    assert tags[259] == 1 and tags[262] == 1 and tags[277] == 1 and tags[278] == h
    dt = np.float32 if bps == 32 else np.uint8
    if bps == 32:
        assert tags[339] == 3
    a = np.frombuffer(b[off:off + nb], dtype=dt).reshape(h, w)
    return a


def locate(k, count, nf):
    r = np.float32(count) / np.float32(nf)
    j = int(np.ceil(np.float32(k) / r))
    item = k - int(np.floor(np.float32(j - 1) * r)) - 1
    return j, item


def write_split(rec, base, items, nf):
    files = {}
    for k, it in enumerate(items, start=1):
        j, pos = locate(k, len(items), nf)
        files.setdefault(j, {})[pos] = it
    for j, d in files.items():
        arr = np.concatenate([d[p].ravel() for p in sorted(d)]).astype(np.float32)
        arr.tofile(rec / f"{base}{j}.dat")


def matlab_u8(a):
    return np.round(255.0 * np.clip(np.nan_to_num(a.astype(np.float64), nan=0.0), 0, 1)).astype(np.uint8)


@pytest.fixture(scope="module")
def dataset(tmp_path_factory):
    B.build_drivers()
    root = tmp_path_factory.mktemp("tiff")
    rec = root / "exp" / "reconstruction"
    rec.mkdir(parents=True)
    np.array([NFILES, NIMG, NSINO, NREC], np.float32).tofile(rec / "fileinfo_projections.dat")
    rng = np.random.default_rng(0)
    N = NIMG + 1
    fbp = [rng.uniform(-0.3, 1.3, (N, N)) for _ in range(NIMG)]          # [y][x]
    tv = [rng.uniform(-0.3, 1.3, (N, N)) for _ in range(NIMG)]
    proj = [rng.uniform(-0.3, 1.3, (NIMG, NIMG)) for _ in range(NFILES)]  # [row][det]
    sino = [rng.uniform(-0.3, 1.3, (NFILES, N)) for _ in range(NIMG)]    # [angle][det]
    fbp[2][3, 4] = np.nan
    write_split(rec, "fbp", fbp, NREC)
    write_split(rec, "fbp_tv", tv, NREC)
    write_split(rec, "projections", proj, NSINO)
    write_split(rec, "sinograms", sino, NSINO)
    env = dict(os.environ, ROOT_CT_DIR=str(root), EXP_CT_NAME="exp")
    return dict(root=root, env=env, fbp=fbp, tv=tv, proj=proj, sino=sino)


def run(env, *args):
    r = subprocess.run([os.path.join(B.BIN, "to_tiff"), *args], env=env, capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_reconstruction_images(dataset):
    out = run(dataset["env"], "fbp")
    assert f"{2 * NIMG} images" in out
    for j in range(1, NIMG + 1):
        for base, ref in (("fbp", dataset["fbp"]), ("fbp_tv", dataset["tv"])):
            img = read_tiff(dataset["root"] / "exp" / f"{base}_images" / f"{base}{j}.tiff")
            # image row = x (the file's fastest index), column = y
            np.testing.assert_array_equal(img, matlab_u8(ref[j - 1].astype(np.float32).T))


def test_sub_sampled_images(dataset, tmp_path):
    """Sub-sampled results (tv_hpc with Sub_Sample_Radial = 2): side
    floor((nimage + add - 1) / 2) + 1 = 4 for nimage = 6."""
    rec = tmp_path / "s" / "reconstruction"
    rec.mkdir(parents=True)
    np.array([NFILES, NIMG, NSINO, NREC], np.float32).tofile(rec / "fileinfo_projections.dat")
    rng = np.random.default_rng(1)
    side = (NIMG + 1 - 1) // 2 + 1
    sub = [rng.uniform(-0.3, 1.3, (side, side)) for _ in range(NIMG)]
    subtv = [rng.uniform(-0.3, 1.3, (side, side)) for _ in range(NIMG)]
    write_split(rec, "fbp_sub", sub, NREC)
    write_split(rec, "fbp_sub_tv", subtv, NREC)
    env = dict(os.environ, ROOT_CT_DIR=str(tmp_path), EXP_CT_NAME="s", Sub_Sample_Radial="2")
    assert f"{2 * NIMG} images" in run(env, "sub")
    for j in range(1, NIMG + 1):
        for base, ref in (("fbp_sub", sub), ("fbp_sub_tv", subtv)):
            img = read_tiff(tmp_path / "s" / f"{base}_images" / f"{base}{j}.tiff")
            np.testing.assert_array_equal(img, matlab_u8(ref[j - 1].astype(np.float32).T))


def test_projection_and_sinogram_images_as_floats(dataset):
    env = dict(dataset["env"], ACUMEN_TIFF="float")
    run(env, "sino")
    for j in range(1, NFILES + 1):
        img = read_tiff(dataset["root"] / "exp" / "projections_images" / f"projections{j}.tiff")
        np.testing.assert_array_equal(img, dataset["proj"][j - 1].astype(np.float32).T)
    for j in range(1, NIMG + 1):
        img = read_tiff(dataset["root"] / "exp" / "sinogram_images" / f"sinogram{j}.tiff")
        assert img.shape == (NIMG + 1, NFILES)
        np.testing.assert_array_equal(img, dataset["sino"][j - 1].astype(np.float32).T)


def test_missing_files_fail_cleanly(dataset, tmp_path):
    rec = tmp_path / "e" / "reconstruction"
    rec.mkdir(parents=True)
    np.array([NFILES, NIMG, NSINO, NREC], np.float32).tofile(rec / "fileinfo_projections.dat")
    env = dict(os.environ, ROOT_CT_DIR=str(tmp_path), EXP_CT_NAME="e")
    assert "skipped" in run(env, "fbp")
    r = subprocess.run([os.path.join(B.BIN, "to_tiff"), "sino"], env=env, capture_output=True, text=True,
                       timeout=120)
    assert r.returncode != 0 and "projection" in r.stderr
    r = subprocess.run([os.path.join(B.BIN, "to_tiff"), "bogus"], env=env, capture_output=True, text=True,
                       timeout=120)
    assert r.returncode != 0 and "usage" in r.stderr
