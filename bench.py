"""Benchmark of the batched split-Bregman TV reconstruction (tomography/tv_hpc.F90
tvopt) on GB300, following the repository's bench contract.

Workload (one GPU): S = 256 slices of the 2049^2 grid (2048-pixel detector made
odd, tv_hpc.F90:552-555) at T = 1200 angles over [0, 180] degrees, Bregman
parameters ninner = 1, ncg = 10, lambda = 0.05, mu = 1.0, wpu = 100, nouter = 50.
Inputs are seeded synthetic sinograms (random-ellipse phantoms, analytic
projections, Poisson counts at I0 = 5e3): the reference's neutron-CT datasets
are not available.

A "step" is one Bregman outer iteration of the whole batch (10 CG steps: 10
projections (11 every fifth iteration, which recomputes radon(uk)) and 11
filtered backprojections plus the fused element-wise kernels, replayed as one
CUDA graph).  value = S / (t_warm + nouter * t_step):
slices per second of the full 50-iteration reconstruction with the inputs
resident in HBM (t_warm = the FBP warm start, timed once).  e2e = the same
through the host-buffer C ABI call acu_tvopt (pinned host input and outputs,
copies inside the timed region) for one outer iteration, plus the remaining
nouter - 1 device-timed steps.

--impl reference times the reference's algorithm on the host cores instead
(the CPU oracle's single-precision restatement, every host thread), on a
bounded sample of the same workload scaled to the same metric.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "TV slices/sec 2048²@1200 angles batched vs plain GPU at relL2≤1e-4; FBP GUPS"
N_GRID, T_ANG, S_BATCH = 2049, 1200, 256
NINNER, NCG, NOUTER, LAM, MU, WPU = 1, 10, 50, 0.05, 1.0, 100
POSITIONS = {"reference": 0, "exact": 1}   # ACU_OPT_POSITIONS values
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one projection
# by the pixel-line projector (k_lines_from_lanes, the 17 band launches of
# k_radon_lines, k_lines_finish) per 32-slice line group at 2049^2 x 1200
# angles, from one ncu capture of a 32-slice projection (scaled by line groups
# below): 5.19 GB read + 3.25 GB written, mostly the ray sums' round trips
# between the 17 band launches
RADON_TRAFFIC_PER_LINE_GROUP = 5189434368 + 3248563968


def projector_variant(option, S):
    """The 4-slice projector variant the library runs for S slices
    (ACU_OPT_PROJECTOR; 7 = automatic, as csrc/api.cu projector_variant)."""
    G = (S + 3) // 4
    if option != 7:
        return option
    return 6 if 8 * ((G + 7) // 8) <= G + G // 8 else 5


def radon_launches(variant, N):
    """Kernels of one batched projection: line conversion, one launch per
    band of rows and the finish for the pixel-line projector (csrc/kernels_lines.cu
    lines_band_rows); transpose and projector for the others."""
    if variant != 6:
        return 2
    H = max(16, (32 << 20) // (N * 128) - 1)
    return 2 + max(1, (N - 2 + H - 1) // H)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)   # one period of the radon(uk) refresh
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--slices", type=int, default=S_BATCH)
    ap.add_argument("--size", type=int, default=N_GRID)
    ap.add_argument("--angles", type=int, default=T_ANG)
    ap.add_argument("--op", default=None,
                    choices=[None, "radon", "iradon", "backproject", "filter", "tvstep", "accuracy", "prep"],
                    help="time one operator on the workload's batch (used for ncu captures); 'accuracy' prints the "
                         "full FP64 comparison of both position modes")
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--positions", default="exact", choices=["exact", "reference"],
                    help="single-precision sample positions (ACU_OPT_POSITIONS): exact (split FP64 angle tables, "
                         "the mode that meets relL2 <= 1e-4 against FP64 at the TV configurations) or the "
                         "reference's single-precision arithmetic")
    ap.add_argument("--option", action="append", default=[], metavar="ID=VALUE",
                    help="set a context option (acu_set_option) before running, e.g. 8=1")
    ap.add_argument("--no-extras", action="store_true", help="skip e2e / plain / FBP / CPU legs")
    return ap.parse_args()


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": len(self.rows)}
        try:
            sm = [float(r[0]) for r in self.rows if r[0] not in ("", "[N/A]")]
            mx = [float(r[1]) for r in self.rows if r[1] not in ("", "[N/A]")]
            if sm:
                out["sm_mhz"] = statistics.median(sm)
            if mx:
                out["sm_max_mhz"] = max(mx)
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            for i, n in enumerate(names):
                if any(len(r) > 4 + i and r[4 + i].lower().startswith("active") for r in self.rows):
                    out["reasons"].append(n)
        except Exception:
            pass
        return out


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------
def make_batch(S, N, T, device):
    """S seeded synthetic sinograms (distinct phantoms for the first 16 slices,
    repeated with a per-slice gain beyond that)."""
    import torch
    from acumen_gb300 import synthetic as syn
    th = syn.angles(T, closed=True)
    base = []
    nbase = min(S, 16)
    for s in range(nbase):
        base.append(syn.normalised_sinogram(syn.random_ellipses(1000 + s, 0.35 * N), N, th, I0=5e3, seed=1000 + s,
                                            device=device))
    f = torch.empty(S, T, N, device=device, dtype=torch.float32)
    for s in range(S):
        f[s] = base[s % nbase] * (1.0 + 0.01 * (s // nbase))
    return th, f


def cuda_time(fn, reps, stream=None):
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1000.0 / reps


# ---------------------------------------------------------------------------
def max_over_ranks(values, world, device):
    """Timing of the slowest rank (the ranks share no data: each solves its own
    batch, so the only collective is this reduction of step times)."""
    if world <= 1:
        return list(values)
    import torch
    import torch.distributed as dist
    tt = torch.tensor(list(values), device=device, dtype=torch.float64)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return tt.tolist()


def job_value(world, slices_per_rank, t_warm, t_step):
    """Whole-job slices/s of the full nouter-iteration reconstruction, all ranks."""
    return world * slices_per_rank / (t_warm + NOUTER * t_step)


# ---------------------------------------------------------------------------
def _cpu_slice(N, T, seed=1000):
    """One seeded synthetic sinogram of the workload (the first slice of the batch)."""
    import numpy as np
    from acumen_gb300 import synthetic as syn
    th = syn.angles(T, closed=True)
    f = syn.normalised_sinogram(syn.random_ellipses(seed, 0.35 * N), N, th, I0=5e3, seed=seed).numpy()
    return th, np.ascontiguousarray(f, np.float32)


def cpu_outer_iteration(N, T):
    """The reference's algorithm on the host cores, measured: the oracle's
    single-precision restatement of tomography/tv_hpc.F90:162-363 (source
    operation order, single-precision reductions, direct filter) on one
    full-size slice, OpenMP over every host core inside each operator.  Times
    the FBP warm start (one iradon) and one complete Bregman outer iteration
    (orc_tvopt with nouter = 1 minus its warm start: the right-hand side, the
    initial residual, ncg CG steps, the shrinkage and the Bregman update).
    slices/s = 1 / (t_warm + nouter * t_outer): only the iteration count is
    scaled."""
    from oracle import oracle as O
    ncores = os.cpu_count() or 1
    th, f = _cpu_slice(N, T)
    O.lib()
    t0 = time.perf_counter()
    O.iradon(f, th, WPU, 32)
    t_warm = time.perf_counter() - t0
    t0 = time.perf_counter()
    O.tvopt(f, th, WPU, NINNER, 1, NCG, LAM, MU, prec=32, red_mode=0)
    t_one = time.perf_counter() - t0
    t_outer = max(t_one - t_warm, 1e-9)
    desc = (f"oracle single-precision tvopt (tv_hpc.F90:162-363) of one {N}^2 slice at {T} angles with nouter=1 "
            f"(ninner={NINNER}, ncg={NCG}): warm start {t_warm:.2f} s + one outer iteration {t_outer:.2f} s, "
            f"OpenMP over {ncores} threads inside each operator; slices/s = 1/(t_warm + {NOUTER} t_outer)")
    return 1.0 / (t_warm + NOUTER * t_outer), ncores, desc, t_warm, t_outer


# ---------------------------------------------------------------------------
# ---------------------------------------------------------------------------
def measure_l1_peak():
    """The measured L1 load bandwidth: acumen_gb300/bin/l1_peak (csrc/l1_peak.cu),
    128-bit loads over an L1-resident buffer on every SM.  None if the probe
    cannot run."""
    from acumen_gb300 import build as _build
    try:
        exe = _build.build_probe()
        r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
        d = json.loads(r.stdout.strip().splitlines()[-1])
        return d if "l1_gbps" in d else None
    except Exception:
        return None


def l1_level(achieved_gbps, clocks, probe=None, **extra):
    """The gather kernels run from L2 and L1, so their bound is the L1 data path.
    Peak: the probe's measured L1 load bandwidth, scaled from the probe's own SM
    clock to the median SM clock of the timed region; without the probe, the
    nominal 128 bytes per clock per SM."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
    if probe:
        scale = mhz / probe["sm_mhz_from_cycles"] if probe.get("sm_mhz_from_cycles") else 1.0
        peak = probe["l1_gbps"] * scale
        kind = (f"measured: {probe['l1_gbps']:.0f} GB/s = {probe['bytes_per_clk_per_sm']:.1f} B/clk/SM at "
                f"{probe['sm_mhz_from_cycles']:.0f} MHz (bin/l1_peak), scaled to {mhz:.0f} MHz")
    else:
        peak = 128.0 * sms * mhz * 1e6 / 1e9
        kind = f"nominal: 128 B/clk/SM x {sms} SMs x {mhz:.0f} MHz"
    out = {"achieved_GBps": achieved_gbps, "peak_GBps": peak, "frac": achieved_gbps / peak, "peak_kind": kind}
    out.update(extra)
    return out


GOLDEN_TV = {k: os.path.join(ROOT, "tests", "golden", f"tv_1449sq_900ang_{k}.npz") for k in ("input", "fp64", "fp32")}


def tv_golden():
    """TV at 1449^2 x 900 angles, 50 x 10 (lambda 0.05, mu 1), against the
    committed golden results of the CPU oracle in FP64 and in the reference's
    single precision (tests/golden/make_golden.py), both position modes, the
    batched and the plain per-slice path; relative L2 inside the
    reconstruction disc and over the full image."""
    import numpy as np
    import torch
    from acumen_gb300.tomography import Tomography
    if not os.path.exists(GOLDEN_TV["input"]) or not os.path.exists(GOLDEN_TV["fp64"]):
        return {"missing": [p for p in GOLDEN_TV.values() if not os.path.exists(p)]}
    z = np.load(GOLDEN_TV["input"])
    N, T = int(z["params"][0]), int(z["params"][1])
    I0 = float(z["params"][2])
    f = torch.from_numpy((-np.log(z["counts"].astype(np.float64) / max(I0, 1.0))).astype(np.float32))[None].cuda()
    ref = {k: torch.from_numpy(np.load(GOLDEN_TV[k])["tv"]).cuda() for k in ("fp64", "fp32")
           if os.path.exists(GOLDEN_TV[k])}
    t = Tomography(N, z["theta"], WPU)
    mask = (t.backproject(torch.ones(1, T, N, device="cuda")) != 0)[0]
    rel = lambda a, b, m=None: float(torch.linalg.norm((a.double() - b.double())[..., m] if m is not None else
                                                       a.double() - b.double()) /
                                     torch.linalg.norm(b.double()[..., m] if m is not None else b.double()))
    out = {"grid": N, "angles": T, "iterations": f"{NOUTER} x {NCG}", "reference": "oracle FP64 and FP32 (golden)"}
    t0 = time.perf_counter()
    for name, pos in POSITIONS.items():
        t.set_option(8, pos)
        for path, plain in (("batched", False), ("plain", True)):
            tv, _ = t.tvopt(f, NINNER, NOUTER, NCG, LAM, MU, plain=plain)
            tv = tv[0]
            r = {"rel_l2_disc_vs_fp64": rel(tv, ref["fp64"], mask), "rel_l2_full_vs_fp64": rel(tv, ref["fp64"])}
            if "fp32" in ref:
                r.update({"rel_l2_disc_vs_fp32_oracle": rel(tv, ref["fp32"], mask),
                          "rel_l2_full_vs_fp32_oracle": rel(tv, ref["fp32"])})
            out[f"{name}_positions_{path}"] = r
    if "fp32" in ref:
        out["fp32_oracle_rel_l2_disc_vs_fp64"] = rel(ref["fp32"], ref["fp64"], mask)
    out["seconds"] = time.perf_counter() - t0
    t.close()
    return out


def accuracy(full=False):
    """Errors at the configurations' full sizes for both single-precision
    position modes (ACU_OPT_POSITIONS): TV against the committed golden
    results of the CPU oracle (tv_golden), FBP against the library's
    double-precision path (itself checked against the FP64 CPU oracle to 1e-11
    at test sizes, tests/test_gpu_ops.py).  full=True (bench.py --op accuracy)
    adds a second 1449^2 phantom and one slice of the 2049^2 x 1200 workload
    against the library's FP64 solver; the FP64 solves take minutes there."""
    import torch
    from acumen_gb300 import synthetic as syn
    from acumen_gb300.tomography import Tomography

    def rel(a, b, m=None):
        a, b = a.double(), b.double()
        if m is not None:
            a, b = a[..., m], b[..., m]
        return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))

    def tv_case(N, T, seed, plain):
        th = syn.angles(T)
        f = syn.normalised_sinogram(syn.random_ellipses(seed, 0.35 * N), N, th, I0=5e3, seed=seed, device="cuda")[None]
        t = Tomography(N, th, WPU)
        tv64, fbp64 = t.tvopt(f.double(), NINNER, NOUTER, NCG, LAM, MU)
        mask = (t.backproject(torch.ones(1, T, N, device="cuda")) != 0)[0]   # cmask support
        t0 = time.perf_counter()
        res = {"grid": N, "angles": T, "iterations": f"{NOUTER} x {NCG}"}
        for name, pos in POSITIONS.items():
            t.set_option(8, pos)
            tv32, fbp32 = t.tvopt(f.float(), NINNER, NOUTER, NCG, LAM, MU)
            r = {"rel_l2_disc_vs_fp64": rel(tv32, tv64, mask), "rel_l2_full_vs_fp64": rel(tv32, tv64),
                 "fbp_rel_l2_vs_fp64": rel(fbp32, fbp64)}
            if plain:
                tvp, _ = t.tvopt(f.float(), NINNER, NOUTER, NCG, LAM, MU, plain=True)
                r["plain_rel_l2_disc_vs_fp64"] = rel(tvp, tv64, mask)
            res[name + "_positions"] = r
        t.close()
        res["seconds"] = time.perf_counter() - t0
        return res

    out = {"tv_1449sq_900ang_golden": tv_golden()}
    if full:
        out["tv_1449sq_900ang"] = tv_case(1449, 900, 2, True)      # single slice, 1448 bins made odd
        out["tv_2049sq_1200ang_one_slice"] = tv_case(N_GRID, T_ANG, 3, False)
    # FBP of one 725^2 slice at 720 angles from Poisson counts
    N, T = 725, 720
    th, ell, counts, flat, dark = syn.counts_sinogram_725(seed=1, device="cuda")
    p = (-torch.log(torch.clamp(counts - dark, min=1e-16) / max(flat - dark, 1.0))).float()[None]
    t = Tomography(N, th, WPU)
    fbp64 = t.iradon(p.double())
    res = {"grid": N, "angles": T}
    for name, pos in POSITIONS.items():
        t.set_option(8, pos)
        res[name + "_positions_rel_l2_vs_fp64"] = rel(t.iradon(p), fbp64)
    out["fbp_725sq_720ang"] = res
    t.close()
    return out


def pipeline(nproj=1200, ndet=2048, nrows=256, seed=3):
    """Preprocessing of 1200 projections of 2048 x 256: raw uint16 projections with flat/dark stacks and
    a random rotation-axis offset in [-8, 8] px -> averages, normalisation,
    0/180 picks, registration, median, resample, transpose to 256 sinograms,
    through the host-buffer C ABI (acu_proj_to_sino_u16)."""
    import numpy as np
    import torch
    from acumen_gb300 import synthetic as syn
    from acumen_gb300.preprocess import Preprocessor
    rng = np.random.default_rng(seed)
    offset = float(rng.uniform(-8, 8))
    th, raw, flats, darks = syn.projection_stack(nproj, ndet, nrows, offset, seed, device="cuda")
    u16 = lambda x: x.to(torch.int32).cpu().numpy().astype(np.uint16)
    raw, flats, darks = u16(raw), u16(flats), u16(darks)
    pp = Preprocessor()
    out = {}
    for reg in (0, 1):
        pp.proj_to_sino_u16(raw[:8], th[:8], flats, darks, norm_mode=1, reg_method=reg)   # warm
        t0 = time.perf_counter()
        sino, theta_b, shift_b = pp.proj_to_sino_u16(raw, th, flats, darks, norm_mode=1, reg_method=reg)
        dt = time.perf_counter() - t0
        add = 1 if ndet % 2 == 0 else 0
        axis_true = (ndet + add + 1) // 2 + offset
        axis_found = (ndet + add + 1) / 2 - shift_b * ndet
        out["pattern_search" if reg == 0 else "xcorr"] = {
            "seconds": dt, "projections_per_s": nproj / dt, "theta_rad": theta_b,
            "axis_error_px": axis_found - axis_true}
    pp.close()
    out.update({"offset_px": offset, "shape": [nproj, nrows, ndet], "input": "uint16 + 10 flat + 10 dark",
                "how": "host buffers in and out (1.26 GB in, 2.5 GB of sinograms out)"})
    return out


def pipeline_device(nproj=1200, ndet=2048, nrows=256, seed=3, acc_outer=3, tv=True):
    """Config 3 end to end in HBM: 1200 uint16 projections of 2048 x 256 with
    10 flat and 10 dark frames and a random rotation-axis offset in [-8, 8] px
    -> frame averages -> normalisation (mode 1) -> 0/180-degree picks ->
    cross-correlation registration -> median, resample and transpose to 256
    sinograms of 1200 x 2049 -> batched TV on those sinograms.  Each stage is
    timed on the device (CUDA events, inputs resident); the HBM fraction of
    the streaming stages is their compulsory bytes over their time against the
    measured copy bandwidth.  slices/s = S / (t_prep + t_warm + nouter t_step)
    with the TV warm start and steps timed on the pipeline's own sinograms;
    accuracy: slice nrows/2 after acc_outer outer iterations against the
    library's double-precision solver on that slice."""
    import numpy as np
    import torch
    from acumen_gb300 import synthetic as syn
    from acumen_gb300.preprocess import Preprocessor
    from acumen_gb300.tomography import Tomography
    hbm, kind = measured_peaks()
    rng = np.random.default_rng(seed)
    offset = float(rng.uniform(-8, 8))
    th, raw, flats, darks = syn.projection_stack(nproj, ndet, nrows, offset, seed, device="cuda")
    bits = lambda x: x.to(torch.int32).to(torch.int16).contiguous()   # the uint16 counts' bit pattern
    raw, flats, darks = bits(raw), bits(flats), bits(darks)
    pp = Preprocessor()
    npix = ndet * nrows
    add = 1 if ndet % 2 == 0 else 0
    res = {"shape": [nproj, nrows, ndet], "offset_px": offset, "input": "uint16 + 10 flat + 10 dark, in HBM"}

    def timed(fn, reps=3):
        fn()
        return cuda_time(fn, reps)

    t_avg = timed(lambda: (pp.frame_average(flats), pp.frame_average(darks)))
    ob, df = pp.frame_average(flats), pp.frame_average(darks)
    t_norm = timed(lambda: pp.normalize(raw, ob, df, 1))
    proj = pp.normalize(raw, ob, df, 1)
    t_pick = timed(lambda: (pp.pick_angle(th, proj, 0.0), pp.pick_angle(th, proj, 180.0)))
    p0, p180 = pp.pick_angle(th, proj, 0.0), pp.pick_angle(th, proj, 180.0)
    kmax = max(1, min(ndet // 4, 512))
    t_reg = timed(lambda: pp.xcorr_register(p0, p180, kmax, want_corr=False))
    kb, ks, _ = pp.xcorr_register(p0, p180, kmax, want_corr=False)
    shift = (add - ks) / (2.0 * ndet)
    t_mrt = timed(lambda: pp.proj_to_sino(proj, 0.0, shift), 2)
    sino = pp.proj_to_sino(proj, 0.0, shift)
    del proj
    nx = ndet + add
    stages = {
        "frame_average": {"ms": 1e3 * t_avg, "bytes": 2 * 20 * npix + 2 * 4 * npix},
        "normalize": {"ms": 1e3 * t_norm, "bytes": nproj * npix * (2 + 4) + 2 * 4 * npix},
        "pick_0_180": {"ms": 1e3 * t_pick, "bytes": 2 * (2 * 4 * npix + 4 * npix)},
        "xcorr_register": {"ms": 1e3 * t_reg, "bytes": 2 * 4 * npix, "kmax": kmax},
        "median_resample_transpose": {"ms": 1e3 * t_mrt, "bytes": nproj * npix * 4 + nproj * nrows * nx * 4},
    }
    for v in stages.values():
        v["GBps"] = v["bytes"] / (v["ms"] * 1e-3) / 1e9
        v["hbm_frac"] = v["GBps"] / hbm
    res["stages"] = stages
    t_prep = (t_avg + t_norm + t_pick + t_reg + t_mrt)
    res["prep_device_s"] = t_prep
    add_axis = (nx + 1) / 2 - shift * ndet
    res["axis_error_px"] = add_axis - ((nx + 1) // 2 + offset)
    del raw
    torch.cuda.empty_cache()
    if not tv:
        pp.close()
        return res
    # batched TV on the pipeline's sinograms: f[slice][angle][bin]
    t = Tomography(nx, th, WPU)
    t_warm = cuda_time(lambda: t.tv_begin(sino, NINNER, NCG, LAM, MU), 1)
    t.tv_iterate(1)
    t_step = cuda_time(lambda: t.tv_iterate(1), 2)
    S = nrows
    res.update({"tv_warm_s": t_warm, "tv_step_s": t_step,
                "value": S / (t_prep + t_warm + NOUTER * t_step), "unit": "slices/s",
                "how": "S / (device preprocessing + TV warm start + 50 x TV step), TV batched in exact positions"})
    # accuracy of one slice of the chain's output against FP64 at acc_outer outer iterations
    k = S // 2
    f1 = sino[k:k + 1].contiguous()
    tv32, _ = t.tvopt(f1, NINNER, acc_outer, NCG, LAM, MU)
    tv64, _ = t.tvopt(f1.double(), NINNER, acc_outer, NCG, LAM, MU)
    mask = (t.backproject(torch.ones(1, nproj, nx, device="cuda")) != 0)[0]
    a, b = tv32[0].double()[mask], tv64[0][mask]
    res["rel_l2_disc_vs_fp64"] = float(torch.linalg.norm(a - b) / torch.linalg.norm(b))
    res["accuracy_how"] = f"slice {k}, {acc_outer} outer x {NCG} CG iterations, FP32 batched vs the FP64 solver"
    t.close()
    pp.close()
    del sino
    torch.cuda.empty_cache()
    return res


def uneven_batch(nprob=64, seed=7, positions=1, acc_outer=1):
    """Config 4: 64 independent problems with sides drawn from {256, 512, 1024,
    1536, 2048} (grid = ceil(sqrt(2) side), made odd) and 180-1500 angles, one
    ragged batch (acu_batch_tvopt).  Throughput from t(nouter=1) and
    t(nouter=6); accuracy: every problem's single-precision batched result
    after acc_outer outer iterations (x ncg CG steps) against the library's
    double-precision solver on that problem alone, relative L2 inside the
    reconstruction disc."""
    import numpy as np
    import torch
    from acumen_gb300 import synthetic as syn
    from acumen_gb300.batch import RaggedBatch
    from acumen_gb300.tomography import Tomography
    rng = np.random.default_rng(seed)
    sides = rng.choice([256, 512, 1024, 1536, 2048], nprob)
    Ns = [int(np.ceil(np.sqrt(2) * sd)) | 1 for sd in sides]
    Ts = [int(rng.integers(180, 1501)) for _ in range(nprob)]
    ths = [syn.angles(T) for T in Ts]
    sinos = [syn.analytic_sinogram(syn.random_ellipses(500 + i, 0.5 * sd), N, th, device="cuda")
             .float().cpu().numpy() for i, (sd, N, th) in enumerate(zip(sides, Ns, ths))]
    b = RaggedBatch(Ns, ths, WPU)
    b.set_option(8, positions)
    b.tvopt(sinos, NINNER, 1, NCG, LAM, MU)             # tuning, graph capture
    t0 = time.perf_counter()
    tv1, _ = b.tvopt(sinos, NINNER, 1, NCG, LAM, MU)
    t1 = time.perf_counter() - t0
    t0 = time.perf_counter()
    b.tvopt(sinos, NINNER, 6, NCG, LAM, MU)          # outer iterations 2..6: one radon(uk) refresh period
    t6 = time.perf_counter() - t0
    t_outer = max((t6 - t1) / 5, 1e-9)
    t_job = t1 + (NOUTER - 1) * t_outer
    w, r = b.tuning()
    b.close()
    tv_acc = tv1 if acc_outer == 1 else None
    if tv_acc is None:
        b = RaggedBatch(Ns, ths, WPU)
        b.set_option(8, positions)
        tv_acc, _ = b.tvopt(sinos, NINNER, acc_outer, NCG, LAM, MU)
        b.close()
    t0 = time.perf_counter()
    errs = []
    for N, th, f, tvb in zip(Ns, ths, sinos, tv_acc):
        t = Tomography(N, th, WPU)
        mask = (t.backproject(torch.ones(1, len(th), N, device="cuda")) != 0)[0]
        tv64, _ = t.tvopt(torch.from_numpy(f[None]).double().cuda(), NINNER, acc_outer, NCG, LAM, MU)
        a, ref = torch.from_numpy(tvb).cuda().double()[mask], tv64[0][mask]
        errs.append(float(torch.linalg.norm(a - ref) / torch.linalg.norm(ref)))
        t.close()
    return {"value": nprob / t_job, "unit": "problems/s", "problems": nprob, "outer_s": t_outer,
            "grid_sides": sorted(set(Ns)), "angles": [min(Ts), max(Ts)],
            "samples_per_outer": float(sum((NCG + 1) * T * N * N for N, T in zip(Ns, Ts))),
            "tuned": {"radon_warps": w, "bp_rows": r},
            "how": "host-buffer acu_batch_tvopt; t(nouter=1) + 49 x [t(nouter=6) - t(nouter=1)] / 5",
            "rel_l2_max": max(errs), "rel_l2_median": statistics.median(errs),
            "rel_l2_per_problem": errs,
            "accuracy_how": f"single-precision ragged batch after {acc_outer} outer x {NCG} CG iterations against "
                            f"the library's FP64 solver on each problem alone, inside the disc "
                            f"({time.perf_counter() - t0:.0f} s of FP64 solves)"}


def gradient_config5(S=32, N=N_GRID, T=1500, seed=11):
    """Config 5: the registration-aware TV objective
    1/2 |A_s u - y|^2 + lambda TV_eps(u) and its gradient with respect to the
    image and to per-angle detector offsets s ~ N(0, 2 px), for 32 slices of
    2049^2 at 1500 angles (acu_tv_loss_grad_dev).  Reports the time of one
    loss + gradient of the batch, the device memory the call holds, the
    single-precision gradient of slice 0 against the double-precision kernels,
    and central finite differences (h = 1e-3) of the double-precision loss
    against its analytic gradient at a few image coordinates and offsets."""
    import numpy as np
    import torch
    from acumen_gb300 import synthetic as syn
    from acumen_gb300.tomography import Tomography
    LAMG, EPS = 0.05, 0.05
    th = syn.angles(T)
    rng = np.random.default_rng(seed)
    u = torch.empty(S, N, N, device="cuda")
    y = torch.empty(S, T, N, device="cuda")
    for s in range(S):
        ell = syn.random_ellipses(seed + s, 0.35 * N)
        u[s] = syn.rasterize(ell, N, device="cuda").float()
        y[s] = syn.analytic_sinogram(ell, N, th, device="cuda").float()
    u += 0.01 * torch.randn(S, N, N, device="cuda", generator=torch.Generator("cuda").manual_seed(seed))
    off = torch.from_numpy(rng.normal(0.0, 2.0, (S, T))).float().cuda()
    t = Tomography(N, th, WPU)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    loss, gu, go = t.tv_loss_grad(u, off, y, LAMG, EPS)           # allocates the work buffers
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    sec = cuda_time(lambda: t.tv_loss_grad(u, off, y, LAMG, EPS), 2)
    # slice 0 in double precision: gradient and finite differences
    u0, off0, y0 = u[:1].double(), off[:1].double(), y[:1].double()
    l64, gu64, go64 = t.tv_loss_grad(u0, off0, y0, LAMG, EPS)
    rel = lambda a, b: float(torch.linalg.norm(a.double() - b) / torch.linalg.norm(b))
    out = {"slices": S, "grid": N, "angles": T, "seconds_loss_and_grad": sec,
           "slices_per_s": S / sec,
           "device_bytes_held_by_call": int(free0 - free1),
           "inputs_bytes": int(4 * (2 * S * N * N + S * T * N + S * T)),
           "grad_u_f32_rel_l2_vs_f64": rel(gu[:1], gu64), "grad_off_f32_rel_l2_vs_f64": rel(go[:1], go64),
           "loss_f32_rel_vs_f64": abs(float(np.ravel(loss)[0]) - float(np.ravel(l64)[0])) / abs(float(np.ravel(l64)[0]))}
    h = 1e-3

    def f64loss(uu, oo):
        return float(np.ravel(t.tv_loss_grad(uu, oo, y0, LAMG, EPS, want_grad=False)[0])[0])

    fd_u, fd_o = [], []
    for _ in range(3):
        i, j = (int(v) for v in rng.integers(N // 4, 3 * N // 4, 2))
        up, um = u0.clone(), u0.clone()
        up[0, i, j] += h
        um[0, i, j] -= h
        fd = (f64loss(up, off0) - f64loss(um, off0)) / (2 * h)
        g = float(gu64[0, i, j])
        fd_u.append(abs(fd - g) / max(1.0, abs(g)))
    gscale = float(torch.sqrt(torch.mean(go64 ** 2)))
    for k in rng.choice(T, 3, replace=False):
        op, om = off0.clone(), off0.clone()
        op[0, k] += h
        om[0, k] -= h
        fd = (f64loss(u0, op) - f64loss(u0, om)) / (2 * h)
        fd_o.append(abs(fd - float(go64[0, k])) / gscale)
    out.update({"fd_u_max_err": max(fd_u), "fd_off_max_err_over_rms": max(fd_o),
                "fd_how": "central differences h=1e-3 of the FP64 loss of slice 0: image error relative to "
                          "max(1, |g|); offset error relative to the offset gradient's RMS (the bilinear "
                          "projector is piecewise smooth in the offsets)"})
    t.close()
    return out


def run_reference(args, rank, world):
    """The reference arm: the reference's algorithm on the host cores (the
    oracle's single-precision restatement; the reference is Fortran and has no
    compiler here).  A step is one CG step of the inner solve
    (tomography/tv_hpc.F90:253-300: radon(p), iradon, the operator's Laplacian
    term, the inner products and the vector updates) on one full-size slice,
    OpenMP over every host core.  An outer iteration of the reference holds
    ncg + 2 such radon + iradon pairs (tv_hpc.F90:227-229 right-hand side and
    initial residual, :253-254 the CG steps, :339-340 the Bregman update), so
    slices/s = 1 / (nouter * (ncg + 2) * t_step)."""
    if rank != 0:
        return
    import numpy as np
    from oracle import oracle as O
    from acumen_gb300 import synthetic as syn
    N, T = args.size, args.angles
    ncores = os.cpu_count() or 1
    th = syn.angles(T, closed=True)
    cg = O.CGState(N, th, WPU, LAM, MU, prec=32, red_mode=0)
    for _ in range(args.warmup):
        cg.step()
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        cg.step()
        ts.append(time.perf_counter() - t0)
    t_step = statistics.mean(ts)
    v = 1.0 / (NOUTER * (NCG + 2) * t_step)
    desc = (f"oracle single-precision CG step (tv_hpc.F90:253-300: radon, iradon with the direct filter, "
            f"Laplacian, inner products, updates) of one {N}^2 slice at {T} angles, OpenMP over {ncores} threads; "
            f"slices/s = 1/({NOUTER} outer x {NCG + 2} radon+iradon pairs x t_step)")
    line = {"metric": METRIC, "value": v, "unit": "slices/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * t_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": f"split-Bregman TV, {args.slices} slices of {N}^2, {T} angles, "
                                   f"ninner={NINNER} ncg={NCG} nouter={NOUTER} lambda={LAM} mu={MU} wpu={WPU}; "
                                   f"step = one CG step of one slice",
                       "global_batch": args.slices, "parallelism": "host threads"},
            "cpu_baseline": {"value": v, "unit": "slices/s", "cores": ncores, "kind": "port", "sample": desc},
            "e2e": {"value": v, "unit": "slices/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_op(args, t, f, S):
    """One operator on the batch, for ncu captures and kernel timings."""
    import torch
    N = args.size
    if args.op == "accuracy":
        print(json.dumps(accuracy(full=True)), flush=True)
        return
    if args.op == "prep":
        # the preprocessing chain on --angles projections of 2048 x 256 (uint16, in HBM)
        print(json.dumps(pipeline_device(nproj=args.angles, tv=False)), flush=True)
        return
    if args.op == "radon":
        img = torch.rand(S, N, N, device="cuda")
        fn = lambda: t.radon(img)
    elif args.op == "iradon":
        fn = lambda: t.iradon(f)
    elif args.op == "backproject":
        fn = lambda: t.backproject(f)
    elif args.op == "filter":
        fn = lambda: t.filter(f)
    else:
        t.tv_begin(f, NINNER, NCG, LAM, MU)
        fn = lambda: t.tv_iterate(1)
    for _ in range(args.warmup):
        fn()
    sec = cuda_time(fn, args.reps)
    print(json.dumps({"op": args.op, "slices": S, "N": N, "T": args.angles, "ms": 1000 * sec}), flush=True)


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import numpy as np
    import torch
    import torch.distributed as dist
    from acumen_gb300 import build as _build
    from acumen_gb300.tomography import Tomography

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    _build.build()
    N, T, S = args.size, args.angles, args.slices
    th, f = make_batch(S, N, T, "cuda")
    t = Tomography(N, th, WPU)
    t.set_option(8, POSITIONS[args.positions])
    for o in args.option:
        k, v = o.split("=")
        t.set_option(int(k), int(v))
    if args.op:
        return run_op(args, t, f, S)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    # warm start (FBP + initialisation), timed once
    barrier()
    t_warm = cuda_time(lambda: t.tv_begin(f, NINNER, NCG, LAM, MU), 1)
    for _ in range(args.warmup):
        t.tv_iterate(1)
    barrier()
    sampler = ClockSampler(local)
    sampler.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        t.tv_iterate(1)
    e1.record()
    torch.cuda.synchronize()
    clocks = sampler.stop()
    t_step = e0.elapsed_time(e1) / 1000.0 / args.steps
    t_step, t_warm = max_over_ranks([t_step, t_warm], world, "cuda")
    value = job_value(world, S, t_warm, t_step)
    # kernels of one outer iteration (the captured graph): the projector's
    # launches per radon, filter + backprojection per iradon, and the
    # element-wise / finaliser kernels.  ACU_OPT_RESIDUAL: 0 the reference's
    # two backprojections for the initial residual, 1 one, 2 none (carried,
    # refreshed with radon(uk): two backprojections and two differences then,
    # one image sum otherwise)
    residual = t.get_option(9)
    refresh = t.get_option(11)        # radon(uk) recomputed every refresh-th outer iteration
    carried = refresh != 1
    carried_res = residual == 2 and carried
    n_full = args.steps if not carried else (0 if refresh == 0 else sum(
        1 for k in range(args.warmup + 1, args.warmup + args.steps + 1) if k % refresh == 0))
    n_radon = NINNER * NCG + (0 if carried else NINNER - 1)
    res_iradon = 0 if carried_res else (1 if residual == 1 else 2)
    n_iradon = NINNER * (res_iradon + NCG)
    n_ew = NINNER * ((5 if residual == 1 and not carried_res else 4) + 5 * NCG) + 1
    n_ew += NINNER * NCG if carried else 0          # the sinogram updates ruk += alpha radon(p)
    n_ew += 1 if carried_res else 0                 # iradon(fk - f) += iradon(f - radon(uk))
    variant = projector_variant(t.get_option(7), S)
    per_radon = radon_launches(variant, N)
    kernel_launches = (per_radon * n_radon + 2 * n_iradon + n_ew) * args.steps + per_radon * n_full
    if carried_res:   # each refresh: two differences and two backprojections instead of the sum
        kernel_launches += n_full * (2 * 2 + 2 - 1)

    # solver state: 10 image-sized and 5 sinogram-sized FP32 arrays per slice
    state_gb = S * (10 * N * N + 5 * T * N) * 4 / 1e9
    line = {"metric": METRIC, "value": value, "unit": "slices/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * t_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded random-ellipse phantoms, Poisson I0=5e3)",
            "config": {"workload": f"split-Bregman TV, {S} slices of {N}^2, {T} angles over [0,180], "
                                   f"ninner={NINNER} ncg={NCG} nouter={NOUTER} lambda={LAM} mu={MU} wpu={WPU}; "
                                   f"step = one outer iteration of the batch",
                       "global_batch": S * world, "seq_len": T, "parallelism": f"slices sharded, {world} rank(s)",
                       "l2": (f"inputs larger than L2 (batch state {state_gb:.1f} GB)" if state_gb > 0.129
                              else f"L2-resident small case (batch state {state_gb:.3f} GB)"),
                       "positions": args.positions,
                       "t_warm_s": t_warm, "t_step_s": t_step},
            "clocks": clocks, "gpu_launches": kernel_launches}

    if rank == 0 and not args.no_extras:
        # the same solver in the reference's order of operations: the initial CG
        # residual from two backprojections (ACU_OPT_RESIDUAL = 0) and radon(uk)
        # recomputed after every outer iteration (ACU_OPT_RADON_REFRESH = 1):
        # (ncg + 2) projections and (ncg + 2) filtered backprojections per step,
        # the work of the plain per-slice path
        opt9, opt11 = t.get_option(9), t.get_option(11)
        t.set_option(9, 0)
        t.set_option(11, 1)
        t_warm_eq = cuda_time(lambda: t.tv_begin(f, NINNER, NCG, LAM, MU), 1)
        t.tv_iterate(1)
        t_step_eq = cuda_time(lambda: t.tv_iterate(1), 2)
        t.set_option(9, opt9)
        t.set_option(11, opt11)
        equal = {"value": S / (t_warm_eq + NOUTER * t_step_eq), "unit": "slices/s", "t_step_s": t_step_eq,
                 "t_warm_s": t_warm_eq,
                 "options": "ACU_OPT_RESIDUAL=0, ACU_OPT_RADON_REFRESH=1: the reference's order "
                            "(tv_hpc.F90:227-229, 253-254, 339-340), 12 projections + 12 filtered "
                            "backprojections per outer iteration"}
        probe = measure_l1_peak()
        line["l1_probe"] = probe
        # dominant kernel: the projector, timed alone on the same batch (lane layout, 64 slice groups)
        img = torch.rand(S, N, N, device="cuda")
        t_radon = cuda_time(lambda: t.radon(img), 2)
        del img
        hbm, kind = measured_peaks()
        alg_bytes = 4.0 * (N * N + N * T) * S
        achieved = alg_bytes / t_radon / 1e9
        line_groups = ((S + 3) // 4 + 7) // 8
        traffic = (RADON_TRAFFIC_PER_LINE_GROUP * line_groups
                   if (N, T) == (N_GRID, T_ANG) and variant == 6 and RADON_TRAFFIC_PER_LINE_GROUP else None)
        kname = ("k_radon_lines (pixel lines of 32 slices, %d band launches + conversions; projector, "
                 "tv_hpc.F90:137-156)" % (radon_launches(6, N) - 2) if variant == 6 else
                 "k_radon_stag_reuse<4, exact, f32x2> (projector, tv_hpc.F90:137-156)")
        line["roofline"] = {"bound": "hbm", "kernel": kname,
                            "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                            "peak_kind": kind, "traffic": traffic,
                            "algorithmic_bytes": alg_bytes, "launch_ms": 1000 * t_radon,
                            "note": "runs from L2 and L1, not from HBM (each band of rows stays in L2); traffic (from "
                                    "one 32-slice ncu capture, scaled by 32-slice line groups) is mostly the ray "
                                    "sums carried between the band launches, ~1.4 % of the HBM bandwidth",
                            "l1_level": l1_level(16.0 * N * N * T * S / t_radon / 1e9, clocks, probe,
                                                 bytes_per_sample_slice=16,
                                                 sample_slices_per_s=N * N * T * S / t_radon)}
        # end to end through the host-buffer C ABI: one outer iteration with copies
        fh = f.cpu().pin_memory()
        tvh = torch.empty(S, N, N, pin_memory=True)
        fbph = torch.empty(S, N, N, pin_memory=True)
        import ctypes
        from acumen_gb300._lib import call

        def e2e_call():
            call("acu_tvopt", t.handle, S, ctypes.c_void_p(fh.data_ptr()), NINNER, 1, NCG, LAM, MU,
                 ctypes.c_void_p(tvh.data_ptr()), ctypes.c_void_p(fbph.data_ptr()), ctx=t.handle)
        e2e_call()
        t0 = time.perf_counter()
        e2e_call()
        t_e2e1 = time.perf_counter() - t0
        e2e_val = S / (t_e2e1 + (NOUTER - 1) * t_step)
        line["e2e"] = {"value": e2e_val, "unit": "slices/s", "h2d_bytes_per_step": 4 * S * T * N,
                       "d2h_bytes_per_step": 2 * 4 * S * N * N,
                       "how": "acu_tvopt host call (pinned in, tv+fbp out, FBP + 1 outer iteration) "
                              f"= {t_e2e1:.3f} s, plus {NOUTER - 1} device-timed steps"}
        del fh, tvh, fbph
        # the plain per-slice GPU path (reference structure) on one slice
        f1 = f[:1].contiguous()
        tp1 = cuda_time(lambda: t.tvopt(f1, NINNER, 1, NCG, LAM, MU, plain=True), 1)
        tp2 = cuda_time(lambda: t.tvopt(f1, NINNER, 2, NCG, LAM, MU, plain=True), 1)
        t_plain_outer = max(tp2 - tp1, 1e-9)
        plain_val = 1.0 / (tp1 - t_plain_outer + NOUTER * t_plain_outer)
        equal["batched_over_plain"] = equal["value"] / plain_val
        line["plain_gpu"] = {"value": plain_val, "unit": "slices/s", "outer_s_per_slice": t_plain_outer,
                             "batched_over_plain": value / plain_val,
                             "batched_over_plain_equal_work": equal["batched_over_plain"]}
        line["equal_work"] = equal
        # FBP GUPS: one 725^2 slice at 720 angles, and the batch
        from acumen_gb300 import synthetic as syn
        t1c = Tomography(725, syn.angles(720), WPU)
        t1c.set_option(8, POSITIONS[args.positions])
        s1 = torch.rand(1, 720, 725, device="cuda")
        t1c.iradon(s1)                     # first call builds the context's tables (host)
        g1 = 725 * 725 * 720 / cuda_time(lambda: t1c.iradon(s1), 10) / 1e9
        t.iradon(f[:4])
        gb = N * N * T * S / cuda_time(lambda: t.iradon(f), 2) / 1e9
        line["fbp_gups"] = {"single_slice_725sq_720ang": g1, "batch_2049sq_1200_x256": gb}
        # the other hot kernel: the backprojection (8 bytes per update at L1 level)
        t_bp = cuda_time(lambda: t.backproject(f), 2)
        line["roofline_backprojection"] = {
            "kernel": "k_backproject_exact_ct<4, 1> (tv_hpc.F90:107-123)", "launch_ms": 1000 * t_bp,
            "updates_per_s": N * N * T * S / t_bp,
            "l1_level": l1_level(8.0 * N * N * T * S / t_bp / 1e9, clocks, probe, bytes_per_update=8),
            "note": "neighbouring pixels' taps often fall in the same bins and are broadcast within a "
                    "quarter-warp, so bytes delivered to registers can exceed the data path's 128 B/clk; "
                    "ncu: 84 % of L1 data-pipe wavefronts, 73 % issue; launch includes the lane-layout "
                    "conversions"}
        # ragged batch: 64 problems, grids {363,725,1449,2173,2897},
        # 180-1500 angles; one outer iteration timed as [tvopt(6) - tvopt(1)] / 5
        del f
        torch.cuda.empty_cache()
        line["uneven_batch"] = uneven_batch(positions=POSITIONS[args.positions])
        line["gradient"] = gradient_config5()
        line["pipeline"] = pipeline()
        line["pipeline_device"] = pipeline_device()
        line["accuracy"] = accuracy()
        # CPU baseline (one measured outer iteration of one slice, all host cores)
        v, ncores, desc, _, _ = cpu_outer_iteration(N, T)
        line["cpu_baseline"] = {"value": v, "unit": "slices/s", "cores": ncores, "kind": "port", "sample": desc}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
