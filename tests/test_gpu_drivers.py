"""The C++ drop-ins for the reference's driver programs, run end to end on a
small synthetic dataset laid out as the reference's files
($ROOT_CT_DIR/$EXP_CT_NAME/reconstruction/...), checked against the oracle:
raw_to_hpc (fits_to_hpc.F90's normalisation), projections_to_sinogram_hpc,
fbp_hpc, tv_hpc (with and without sub-sampling) and tv_hpc_slice.  The file
split is forced to several files (ACUMEN_FILE_BYTES) so that the chunked
reads and writes are exercised.
"""
import os
import subprocess

import numpy as np
import pytest
import torch

from acumen_gb300 import build as B
from acumen_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

NIMG, NPROJ, WPU = 48, 73, 4


def rel(a, b, m=None):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    if m is not None:
        a, b = a[..., m], b[..., m]
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def dataset(tmp_path_factory, built_lib):
    B.build_drivers()
    root = tmp_path_factory.mktemp("ct")
    exp = "synthetic_exp"
    raw = root / exp / "raw"
    raw.mkdir(parents=True)
    th, proj, flats, darks = syn.projection_stack(NPROJ, NIMG, NIMG, axis_offset=2.0, seed=21, I0=3e4)
    u16 = lambda t: t.to(torch.int32).numpy().astype(np.uint16)
    proj, flats, darks = u16(proj), u16(flats), u16(darks)
    proj.tofile(raw / "projections.u16")
    flats.tofile(raw / "OB.u16")
    darks.tofile(raw / "DF.u16")
    np.savetxt(raw / "theta.txt", th)
    (raw / "info.txt").write_text(f"{NPROJ} {NIMG} {flats.shape[0]} {darks.shape[0]}\n")
    env = dict(os.environ, ROOT_CT_DIR=str(root), EXP_CT_NAME=exp, ACUMEN_FILE_BYTES="400000",
               ACUMEN_NORM_MODE="1")
    return dict(root=root, exp=exp, rec=root / exp / "reconstruction", env=env, th=th, proj=proj,
                flats=flats, darks=darks)


def run(name, env):
    r = subprocess.run([os.path.join(B.BIN, name)], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def read_split(rec, base, nfiles_field, per_item, count):
    """Concatenate {base}{k}.dat in file order (each holds whole items)."""
    out = []
    for k in range(1, nfiles_field + 1):
        out.append(np.fromfile(rec / f"{base}{k}.dat", np.float32))
    a = np.concatenate(out)
    assert a.size >= per_item * count
    return a[: per_item * count]


def test_pipeline_through_drivers(dataset, oracle):
    env, rec = dataset["env"], dataset["rec"]
    run("raw_to_hpc", env)
    info = np.fromfile(rec / "fileinfo_projections.dat", np.float32)
    nfiles, nimage, nfs, nfr = (int(v) for v in info)
    assert (nfiles, nimage) == (NPROJ, NIMG) and nfs > 1 and nfr > 1
    np.testing.assert_array_equal(np.fromfile(rec / "theta.dat", np.float32), dataset["th"])
    # normalisation vs the oracle (C library logf vs CUDA logf: ulp-level)
    ob = oracle.frame_average(dataset["flats"].astype(np.float32))
    df = oracle.frame_average(dataset["darks"].astype(np.float32))
    ref_proj = np.stack([oracle.normalize(p.astype(np.float32), ob, df, 1) for p in dataset["proj"]])
    got_proj = read_split(rec, "projections", nfs, NIMG * NIMG, NPROJ).reshape(NPROJ, NIMG, NIMG)
    np.testing.assert_allclose(got_proj, ref_proj, rtol=1e-6, atol=1e-6)

    out = run("projections_to_sinogram_hpc", env)
    line = [l for l in out.splitlines() if "Best theta" in l][0].split()
    theta_b, shift_b = float(line[2]), float(line[5])
    add = 1
    sino = read_split(rec, "sinograms", nfs, NPROJ * (NIMG + add), NIMG).reshape(NIMG, NPROJ, NIMG + add)
    ref_sino = oracle.proj_to_sino(got_proj, theta_b, shift_b)
    np.testing.assert_allclose(sino, ref_sino, rtol=1e-5, atol=1e-6)
    # the recovered axis: the synthetic axis offset is +2 pixels
    axis_true = (NIMG + add + 1) // 2 + 2.0
    assert abs((NIMG + add + 1) / 2 - shift_b * NIMG - axis_true) < 0.75

    # FBP of every slice (fbp_hpc)
    (dataset["root"] / dataset["exp"] / "input_parm.txt").write_text("1\n1\n1\n3\n3\n0.05\n1.0\n4\n")
    run("fbp_hpc", env)
    N = NIMG + add
    th = dataset["th"]
    jts = oracle.minloc_abs(th, 0.0)
    jte = oracle.minloc_abs(th, 180.0)
    tw = th[jts - 1:jte]
    f = sino[:, jts - 1:jte, :]
    fbp = read_split(rec, "fbp", nfr, N * N, NIMG).reshape(NIMG, N, N)
    ref_fbp64 = oracle.iradon(f.astype(np.float64), tw, 4, 64)
    assert rel(fbp, ref_fbp64) < 1e-5
    # several batches through the read / reconstruct / write pipeline, and in sequence
    for pipe in ("1", "0"):
        run("fbp_hpc", dict(env, ACUMEN_BATCH="10", ACUMEN_PIPELINE=pipe))
        np.testing.assert_array_equal(read_split(rec, "fbp", nfr, N * N, NIMG).reshape(NIMG, N, N), fbp)
    # exact sample positions are the default (ACUMEN_POSITIONS=exact gives the same files);
    # ACUMEN_POSITIONS=reference selects the reference's single-precision arithmetic; a bad value fails
    run("fbp_hpc", dict(env, ACUMEN_POSITIONS="exact"))
    np.testing.assert_array_equal(read_split(rec, "fbp", nfr, N * N, NIMG).reshape(NIMG, N, N), fbp)
    run("fbp_hpc", dict(env, ACUMEN_POSITIONS="reference"))
    fbpr = read_split(rec, "fbp", nfr, N * N, NIMG).reshape(NIMG, N, N)
    assert rel(fbpr, oracle.iradon(f.astype(np.float32), tw, 4, 32)) < 1e-5 and not np.array_equal(fbpr, fbp)
    r = subprocess.run([os.path.join(B.BIN, "fbp_hpc")], env=dict(env, ACUMEN_POSITIONS="bogus"),
                       capture_output=True, text=True, timeout=600)
    assert r.returncode != 0 and "ACUMEN_POSITIONS" in (r.stdout + r.stderr)

    # TV of every slice (tv_hpc), full resolution
    tenv = dict(env, Sub_Sample_Radial="1", Sub_Sample_Theta="1", Ninner_Loops="1", Nouter_Loops="3",
                Opt_ncg="3", Opt_lambda="0.05", Opt_mu="1.0", Radon_wpu="4", ACUMEN_BATCH="20")
    run("tv_hpc", tenv)
    tv = read_split(rec, "fbp_tv", nfr, N * N, NIMG).reshape(NIMG, N, N)
    mask = oracle.cmask(N, len(tw), 4, 64) > 0
    for s in (5, 24, 40):
        ref, _ = oracle.tvopt(f[s].astype(np.float64), tw, 4, 1, 3, 3, 0.05, 1.0, prec=64)
        assert rel(tv[s], ref, mask) < 1e-4, s

    # sub-sampled TV (nsub = nsub_t = 2): fbp_sub / fbp_sub_tv outputs
    senv = dict(tenv, Sub_Sample_Radial="2", Sub_Sample_Theta="2")
    run("tv_hpc", senv)
    ns = (N - 1) // 2 + 1
    nt = (jte - jts + 1) // 2
    tws = th[jts - 1:jts - 1 + 2 * nt:2]
    tvs = read_split(rec, "fbp_sub_tv", nfr, ns * ns, NIMG).reshape(NIMG, ns, ns)
    fs = sino[:, jts - 1:jts - 1 + 2 * nt:2, 0:N:2]
    ref, _ = oracle.tvopt(fs[12].astype(np.float64), tws, 4, 1, 3, 3, 0.05, 1.0, prec=64)
    assert rel(tvs[12], ref, oracle.cmask(ns, nt, 4, 64) > 0) < 1e-4


def test_tv_hpc_slice_driver(dataset, oracle):
    rec = dataset["rec"]
    if not (rec / "sinograms1.dat").exists():
        pytest.skip("needs the pipeline test's sinograms")
    # the single-slice program reads one sinogram file: concatenate the split ones
    nfs = int(np.fromfile(rec / "fileinfo_projections.dat", np.float32)[2])
    allsino = read_split(rec, "sinograms", nfs, NPROJ * (NIMG + 1), NIMG)
    single = dataset["root"] / "single" / "reconstruction"
    single.mkdir(parents=True)
    allsino.tofile(single / "sinograms1.dat")
    info = np.fromfile(rec / "fileinfo_projections.dat", np.float32).copy()
    info[2] = 1
    info.tofile(single / "fileinfo_projections.dat")
    np.fromfile(rec / "theta.dat", np.float32).tofile(single / "theta.dat")
    (dataset["root"] / "single" / "input_parm.txt").write_text("1\n1\n1\n10\n2\n0.05\n1.0\n4\n")
    env = dict(dataset["env"], EXP_CT_NAME="single")
    out = run("tv_hpc_slice", env)
    assert out.count("Slice:") == 1 and "Loop:" in out
    N = NIMG + 1
    th = dataset["th"]
    jts, jte = oracle.minloc_abs(th, 0.0), oracle.minloc_abs(th, 180.0)
    sino = allsino.reshape(NIMG, NPROJ, N)
    job = N // 2
    f = sino[job - 1, jts - 1:jte, :]
    ref_tv, ref_fbp = oracle.tvopt(f.astype(np.float64), th[jts - 1:jte], 4, 1, 10, 2, 0.05, 1.0, prec=64)
    tv = np.fromfile(single / "fbp_tv_slice.dat", np.float32).reshape(N, N)
    fbp = np.fromfile(single / "fbp_sub_slice.dat", np.float32).reshape(N, N)
    assert rel(fbp, ref_fbp) < 1e-5
    assert rel(tv, ref_tv, oracle.cmask(N, jte - jts + 1, 4, 64) > 0) < 1e-4


def write_fits_u16(path, img):
    """A FITS primary array of unsigned 16-bit pixels (BITPIX 16, BZERO 32768),
    as detector software writes them."""
    h, w = img.shape
    cards = [("SIMPLE", "T"), ("BITPIX", "16"), ("NAXIS", "2"), ("NAXIS1", str(w)), ("NAXIS2", str(h)),
             ("BZERO", "32768"), ("BSCALE", "1")]
    head = "".join(f"{k:<8}= {v:>20}".ljust(80) for k, v in cards) + "END".ljust(80)
    head = head.ljust((len(head) + 2879) // 2880 * 2880)
    data = (img.astype(np.int32) - 32768).astype(">i2").tobytes()
    data += b"\0" * ((-len(data)) % 2880)
    path.write_bytes(head.encode("ascii") + data)


def test_fits_to_hpc_reads_the_reference_layout(dataset):
    """fits_to_hpc on FITS images in projections/, OB/, DF/ named as the
    reference expects (angle digits after EXP_CT_NAME): the same projections
    as raw_to_hpc on the same counts, and theta.dat as the reference's
    single-precision digit sum of the names (fits_to_hpc.F90:75-96)."""
    root, exp = dataset["root"], "fits_exp"
    base = root / exp
    for d in ("projections", "OB", "DF", "raw"):
        (base / d).mkdir(parents=True)
    f32 = np.float32
    names, th_expected = [], []
    for j, t in enumerate(dataset["th"]):
        m = int(round(float(t) * 1000))
        deg, frac = m // 1000, m % 1000
        names.append(f"{exp}_{'p' * 9}{deg:03d}_{frac:03d}_{j:04d}.fits")
        digits = [int(c) for c in f"{deg:03d}{frac:03d}"]
        acc = f32(0)
        for sc, dgt in zip((100.0, 10.0, 1.0, 0.1, 0.01, 0.001), digits):
            acc = f32(acc + f32(f32(sc) * f32(dgt)))
        th_expected.append(acc)
    for n, img in zip(names, dataset["proj"]):
        write_fits_u16(base / "projections" / n, img)
    for k, img in enumerate(dataset["flats"]):
        write_fits_u16(base / "OB" / f"ob_{k:03d}.fits", img)
    for k, img in enumerate(dataset["darks"]):
        write_fits_u16(base / "DF" / f"df_{k:03d}.fits", img)
    # the same counts through raw_to_hpc
    raw = base / "raw"
    dataset["proj"].tofile(raw / "projections.u16")
    dataset["flats"].tofile(raw / "OB.u16")
    dataset["darks"].tofile(raw / "DF.u16")
    np.savetxt(raw / "theta.txt", np.array(th_expected, np.float32))
    (raw / "info.txt").write_text(f"{NPROJ} {NIMG} {len(dataset['flats'])} {len(dataset['darks'])}\n")
    env = dict(dataset["env"], EXP_CT_NAME=exp)
    rec = base / "reconstruction"
    for mode in ("0", "1"):
        envm = dict(env, ACUMEN_NORM_MODE=mode)
        run("raw_to_hpc", envm)
        info = np.fromfile(rec / "fileinfo_projections.dat", np.float32)
        nfs = int(info[2])
        ref = read_split(rec, "projections", nfs, NIMG * NIMG, NPROJ)
        out = run("fits_to_hpc", envm)
        assert "Number of raw projections" in out and "Determining Average Background" in out
        np.testing.assert_array_equal(np.fromfile(rec / "fileinfo_projections.dat", np.float32), info)
        got = read_split(rec, "projections", nfs, NIMG * NIMG, NPROJ)
        np.testing.assert_allclose(got, ref, rtol=1e-6, atol=1e-6)
        np.testing.assert_array_equal(np.fromfile(rec / "theta.dat", np.float32), np.array(th_expected, np.float32))
    # no open-beam images: a clear error
    for f in (base / "OB").iterdir():
        f.unlink()
    r = subprocess.run([os.path.join(B.BIN, "fits_to_hpc")], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode != 0 and "open-beam" in r.stderr
