"""The drivers' file and parameter conventions (acumen_gb300/drivers/hpc_io.h)
on the host, through a small C++ harness: the split of a sequence over files
(`locate`, the reference's single-precision ceiling rule of
tomography/fits_to_hpc.F90:217-252 and tv_hpc.F90:461-626), Fortran MINLOC of
|theta - target|, the 8-value input_parm.txt, the 4-float
fileinfo_projections.dat, positioned float I/O, and the read/compute/write
pipeline of fbp_hpc (same results as in sequence, slots alternate, worker
errors reach the caller)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
DRIVERS = os.path.join(HERE, "..", "acumen_gb300", "drivers")

HARNESS = r"""
#include <atomic>
#include <cstdio>
#include <cstring>
#include <mutex>
#include "hpc_io.h"
using namespace hpc;

int main(int argc, char** argv)
{
    const std::string mode = argv[1];
    try {
        if (mode == "locate") {
            const int count = std::atoi(argv[2]), nf = std::atoi(argv[3]);
            for (int k = 1; k <= count; ++k) {
                const Where w = locate(k, count, nf);
                std::printf("%d %lld\n", w.file, w.item);
            }
        } else if (mode == "minloc") {
            std::vector<float> th;
            for (int i = 3; i < argc; ++i) th.push_back((float)std::atof(argv[i]));
            std::printf("%d\n", minloc_abs(th, (float)std::atof(argv[2])));
        } else if (mode == "parm") {
            const Params p = read_input_parm(argv[2]);
            std::printf("%d %d %d %d %d %.9g %.9g %d\n", p.nsub, p.nsub_t, p.ninner, p.nouter, p.ncg, p.lambda, p.mu,
                        p.wpu);
        } else if (mode == "fileinfo") {
            const std::string dir = argv[2];
            write_fileinfo(dir, FileInfo{std::atoi(argv[3]), std::atoi(argv[4]), std::atoi(argv[5]),
                                         std::atoi(argv[6])});
            const FileInfo f = read_fileinfo(dir);
            std::printf("%d %d %d %d\n", f.nfiles, f.nimage, f.n_files_sino, f.n_files_rec);
        } else if (mode == "file") {
            File f(argv[2], true);
            std::vector<float> a(1000);
            for (int i = 0; i < 1000; ++i) a[i] = (float)i;
            f.write(5000, a.data(), a.size());   // float offset 5000
            f.write(0, a.data() + 10, 3);
            std::vector<float> b(1000);
            f.read(5000, b.data(), b.size());
            std::printf("%d\n", (int)(b == a));
        } else if (mode == "pipe") {
            // batch k reads k, computes k*k + 1 into the output slot, writes it at position k;
            // with fail_at >= 0 the reader throws at that batch
            const int nb = std::atoi(argv[2]), fail_at = std::atoi(argv[3]);
            long in[2] = {-1, -1}, out[2] = {-1, -1};
            std::vector<long> result(nb, -1);
            std::vector<int> rslot(nb, -1), wslot(nb, -1);
            std::mutex m;
            pipelined(
                nb,
                [&](int k, int slot) {
                    if (k == fail_at) throw Fail("reader failed at batch " + std::to_string(k));
                    in[slot] = k;
                    std::lock_guard<std::mutex> g(m);
                    rslot[k] = slot;
                },
                [&](int k, int slot) {
                    if (in[slot] != k) throw Fail("compute saw the wrong input");
                    out[slot] = (long)k * k + 1;
                },
                [&](int k, int slot) {
                    std::lock_guard<std::mutex> g(m);
                    result[k] = out[slot];
                    wslot[k] = slot;
                });
            for (int k = 0; k < nb; ++k) std::printf("%ld %d %d\n", result[k], rslot[k], wslot[k]);
        }
        return 0;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
}
"""


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    cxx = os.environ.get("CXX", "g++")
    if shutil.which(cxx) is None:
        pytest.skip("no C++ compiler")
    d = tmp_path_factory.mktemp("hpcio")
    src, exe = d / "h.cpp", d / "h"
    src.write_text(HARNESS)
    r = subprocess.run([cxx, "-O1", "-std=c++17", "-Wall", "-pthread", "-I" + DRIVERS, str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr

    def run(*args, env=None):
        e = dict(os.environ, **(env or {}))
        return subprocess.run([str(exe), *map(str, args)], capture_output=True, text=True, timeout=60, env=e)

    return run


@pytest.mark.parametrize("count, nf", [(1200, 1), (1200, 7), (2049, 3), (25, 25), (1001, 13), (7, 3)])
def test_locate_splits_a_sequence_over_files(harness, count, nf):
    r = harness("locate", count, nf)
    assert r.returncode == 0, r.stderr
    got = np.array([[int(v) for v in l.split()] for l in r.stdout.split("\n") if l])
    # restatement: r = real(count)/real(nf); file = ceiling(k / r); item = k - floor((file-1) r) - 1,
    # in single precision
    f32 = np.float32
    rr = f32(count) / f32(nf)
    k = np.arange(1, count + 1)
    j = np.ceil((k.astype(f32) / rr).astype(f32)).astype(int)
    item = k - np.floor((f32(1) * (j - 1).astype(f32) * rr).astype(f32)).astype(int) - 1
    np.testing.assert_array_equal(got[:, 0], j)
    np.testing.assert_array_equal(got[:, 1], item)
    # every file is used, and holds items 0, 1, ... in sequence order
    assert set(got[:, 0]) == set(range(1, nf + 1))
    for f in range(1, nf + 1):
        items = got[got[:, 0] == f, 1]
        np.testing.assert_array_equal(items, np.arange(len(items)))


def test_minloc_takes_the_first_minimum(harness):
    assert harness("minloc", 90.0, 0.0, 45.0, 89.5, 90.5, 135.0).stdout.strip() == "3"
    assert harness("minloc", 0.0, 0.5, 0.1, -0.1, 0.1).stdout.strip() == "2"
    assert harness("minloc", 180.0, 0.0, 90.0, 179.99).stdout.strip() == "3"


def test_input_parm(harness, tmp_path):
    p = tmp_path / "input_parm.txt"
    p.write_text("2\n 1\n1 40\n10\n5.0E-2\n1.0\n   100\n")
    r = harness("parm", p)
    assert r.returncode == 0, r.stderr
    v = r.stdout.split()
    assert v[:5] == ["2", "1", "1", "40", "10"] and float(v[5]) == np.float32(0.05) and float(v[6]) == 1.0
    assert v[7] == "100"
    p.write_text("2 1 1 40\n")
    r = harness("parm", p)
    assert r.returncode != 0 and "malformed" in r.stderr
    r = harness("parm", tmp_path / "missing.txt")
    assert r.returncode != 0 and "cannot open" in r.stderr


def test_fileinfo_round_trip_and_layout(harness, tmp_path):
    d = str(tmp_path) + "/"
    r = harness("fileinfo", d, 1200, 2049, 2, 3)
    assert r.returncode == 0 and r.stdout.split() == ["1200", "2049", "2", "3"]
    raw = np.fromfile(tmp_path / "fileinfo_projections.dat", np.float32)
    np.testing.assert_array_equal(raw, np.array([1200, 2049, 2, 3], np.float32))


def test_positioned_float_io(harness, tmp_path):
    f = tmp_path / "x.dat"
    r = harness("file", f)
    assert r.returncode == 0 and r.stdout.strip() == "1"
    raw = np.fromfile(f, np.float32)
    assert raw.size == 6000
    np.testing.assert_array_equal(raw[:3], [10, 11, 12])
    np.testing.assert_array_equal(raw[5000:], np.arange(1000, dtype=np.float32))


@pytest.mark.parametrize("pipeline", ["1", "0"])
@pytest.mark.parametrize("nb", [0, 1, 2, 7])
def test_pipeline_results_and_slots(harness, nb, pipeline):
    r = harness("pipe", nb, -1, env={"ACUMEN_PIPELINE": pipeline})
    assert r.returncode == 0, r.stderr
    rows = [[int(v) for v in l.split()] for l in r.stdout.split("\n") if l]
    assert len(rows) == nb
    for k, (res, rs, ws) in enumerate(rows):
        assert res == k * k + 1
        want = k % 2 if pipeline == "1" else 0
        assert rs == want and ws == want


def test_pipeline_reader_error_reaches_the_caller(harness):
    r = harness("pipe", 6, 3)
    assert r.returncode == 1 and "reader failed at batch 3" in r.stderr
