"""Benchmark of the raw SFB decomposition (points*modes/s).

Default workload: the split-precision raw SFB -- 10M points uniform in a ball of
rmax=1000 (r = rmax u^(1/3), cos(theta) ~ U[-1,1], phi ~ U[0,2pi)), weights
U[0.5,1.5] (float64), lmax=256, nmax=128, seed 2.  A "step" is one full
decomposition of that catalog (f_lmn and C_ln for every l < lmax, n < nmax).
modes = nmax * sum_{l<lmax} (l+1); the unit counts points * modes per second.

value   device-resident inputs (points 240 MB + weights 80 MB, larger than L2),
        device outputs, CUDA events on the launching stream, max over ranks.
e2e     the same through the host-buffer C ABI (catana_gpu_sfb_raw): pinned host
        input, host->device copy, compute, device->host copy of k_ln and C_ln.
roofline  the dominant kernel (the tcgen05 contraction, k_split_l) timed with CUDA
        events inside the timed region; algorithmic work = 4 flops per point-mode;
        peak = measured dense bf16/fp16 burst peak / 3 (three hi/lo products per MAC).
cpu_baseline  the oracle's OpenMP restatement of the reference's raw path, all host
        cores, same lmax/nmax: timed on samples of 300 and 1500 points, fitted as
        fixed (the per-l j_l tables) + per-point cost, extrapolated to the catalog.

--impl reference times only that CPU path (rank 0), a bounded sample per step.
Multi-GPU (torchrun): every rank decomposes its own 10M-point shard of one catalog
(weak scaling); the unnormalised f_lmn are summed with one NCCL all-reduce.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "raw SFB points·modes/s, split-precision vs FP64 plain, C_l err≤1e-6"
UNIT = "point*modes/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--form", default="split", choices=["split", "plain"])
    p.add_argument("--points", type=int, default=10_000_000)
    p.add_argument("--lmax", type=int, default=256)
    p.add_argument("--nmax", type=int, default=128)
    p.add_argument("--rmax", type=float, default=1000.0)
    p.add_argument("--seed", type=int, default=2)
    p.add_argument("--plain-sample", type=int, default=20_000, help="points for the FP64 plain GPU comparison")
    p.add_argument("--side", type=int, default=1, help="also time the FP64 (100k, 32, 32) and HEALPix cases")
    p.add_argument("--no-extras", action="store_true", help="skip e2e/cpu/plain/accuracy legs")
    p.add_argument("--no-accuracy", action="store_true",
                   help="skip the full-catalog FP64 comparison (about four minutes of FP64 GPU work)")
    p.add_argument("--stream-chunks", type=int, default=2,
                   help="8M-point chunks of the streamed lmax 512 / nmax 256 survey leg (0 skips it)")
    p.add_argument("--stream-points", type=int, default=8_000_000,
                   help="points per chunk of the streamed survey leg (the survey's chunks hold 8M; smaller "
                        "chunks make a case small enough for a kernel profile)")
    p.add_argument("--only", default=None, choices=["side", "batched", "streamed", "next"],
                   help="time one secondary workload alone (side: FP64 100k and HEALPix nside 256) and print "
                        "its JSON")
    return p.parse_args()


def catalog(n, rmax, seed, shard=0):
    rng = np.random.default_rng([seed, shard])
    r = rmax * rng.random(n) ** (1.0 / 3.0)
    th = np.arccos(rng.uniform(-1.0, 1.0, n))
    ph = rng.uniform(0.0, 2.0 * np.pi, n)
    w = rng.uniform(0.5, 1.5, n)
    return np.ascontiguousarray(np.stack([r, th, ph], axis=1)), w


def modes(lmax, nmax):
    return nmax * lmax * (lmax + 1) // 2


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        self.f.seek(0)
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = max(smax, float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.f.name)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    """(bf16 burst TF/s, bf16 sustained TF/s, HBM GB/s, source)."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return (float(d["bf16_tflops"]), float(d.get("bf16_tflops_sustained", d["bf16_tflops"])),
                float(d["hbm_gbs"]), "measured")
    except (OSError, KeyError, ValueError):
        return 1900.0, 1700.0, 6800.0, "fallback"


def cpu_time(pts, w, lmax, nmax, rmax):
    """Seconds of the oracle's OpenMP restatement of sfb_raw.cpp (per l: the lerp table,
    then OpenMP over the points) on one point sample, all host cores."""
    from oracle import oracle as O
    O.build()
    t = time.perf_counter()
    O.sfb_raw(pts, lmax, nmax, rmax, interpolated=True, weights=w, store_flmn=False)
    return time.perf_counter() - t


def cpu_fit(a, n_small=300, n_large=1500):
    """The CPU cost of the full catalog as fixed + per-point: each l rebuilds a
    1000 nmax-node j_l table whatever the sample size (sfb_raw.cpp:45-49), so two
    sample sizes separate that fixed cost from the per-point work, which is exactly
    linear in N.  Returns (seconds for the full catalog, fixed s, s per point, note)."""
    pts, w = catalog(n_large, a.rmax, a.seed)
    cpu_time(pts[:50], w[:50], a.lmax, a.nmax, a.rmax)  # page in the library and OpenMP pool
    ts = cpu_time(pts[:n_small], w[:n_small], a.lmax, a.nmax, a.rmax)
    tl = cpu_time(pts, w, a.lmax, a.nmax, a.rmax)
    slope = max(tl - ts, 1e-9) / (n_large - n_small)
    fixed = max(0.0, tl - slope * n_large)
    note = ("samples of %d and %d points of the same catalog (same lmax/nmax/rmax/weights, interpolated j_l as the "
            "reference uses for N > 1000): %.2f s and %.2f s -> %.2f s fixed (per-l j_l tables) + %.3g s per point, "
            "extrapolated to %d points" % (n_small, n_large, ts, tl, fixed, slope, a.points))
    return fixed + slope * a.points, fixed, slope, note


def run_reference(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    n_large = 1500
    t_full, fixed, slope, note = cpu_fit(a, n_large=n_large)
    pts, w = catalog(n_large, a.rmax, a.seed)
    for _ in range(a.warmup):
        cpu_time(pts, w, a.lmax, a.nmax, a.rmax)
    t = time.perf_counter()
    for _ in range(a.steps):
        cpu_time(pts, w, a.lmax, a.nmax, a.rmax)
    dt = (time.perf_counter() - t) / a.steps
    # each step: the 1500-point sample; its per-point share after the fixed cost,
    # extrapolated to the whole catalog
    per_point = max(dt - fixed, 1e-9) / n_large
    v = a.points * modes(a.lmax, a.nmax) / (fixed + per_point * a.points)
    cores = os.cpu_count()
    sample = "each step %d of the %d points; fixed %.2f s from a calibration (%s)" % (n_large, a.points, fixed, note)
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(a),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def side_workloads(torch, _lib, catana, sp, fp64_peak=None):
    """Two secondary workloads, timed through the public API after the main line:
    the plain FP64 raw SFB of 100k points uniform in a ball (rmax 1000, lmax = nmax =
    32, seed 0) on device-resident data, and the HEALPix SFB of 1M points (90% uniform
    in the ball, 10% in 1000 Gaussian clumps of sigma 5; nside 256, lmax 128, nmax 64,
    seed 1) including its binning."""
    res = {}
    pts, _ = catalog(100000, 1000.0, 0)
    d_pts = torch.from_numpy(pts).cuda()
    L, M = 32, 32
    fc = int(_lib.lib.catana_gpu_flmn_size(L, M))
    d_k = torch.zeros(L * M, dtype=torch.float64, device="cuda")
    d_c = torch.zeros_like(d_k)
    d_f = torch.zeros(2 * fc, dtype=torch.float64, device="cuda")

    def run(jl=_lib.JL_AUTO):
        _lib.check(_lib.lib.catana_gpu_sfb_raw_dev(ctypes.c_void_p(d_pts.data_ptr()), None, 100000, L, M, 1000.0,
                                                   _lib.FORM_PLAIN | jl, ctypes.c_void_p(d_k.data_ptr()),
                                                   ctypes.c_void_p(d_c.data_ptr()), ctypes.c_void_p(d_f.data_ptr()),
                                                   None, sp), "fp64")
    for _ in range(3):
        run()
    torch.cuda.synchronize()
    _lib.lib.catana_gpu_profile_enable(1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(5):
        run()
    e1.record()
    torch.cuda.synchronize()
    _lib.lib.catana_gpu_profile_enable(0)
    kms, kn, kfl = ctypes.c_double(), ctypes.c_uint64(), ctypes.c_double()
    _lib.check(_lib.lib.catana_gpu_profile_report(ctypes.byref(kms), ctypes.byref(kn), ctypes.byref(kfl)))
    ms = e0.elapsed_time(e1) / 5
    ktf = kfl.value / (kms.value / 1e3) / 1e12
    pk = fp64_peak["tflops"] if fp64_peak else None
    res["plain_fp64_100k_l32_n32"] = {"value": 100000 * modes(L, M) / (ms / 1e3), "unit": UNIT, "ms_per_step": ms,
                                     "roofline": {"bound": "fp64", "kernel": "k_fp64_raw_l", "achieved": ktf,
                                                  "peak": pk, "unit": "TFLOP/s",
                                                  "frac": (ktf / pk) if pk else None,
                                                  "peak_source": "measured in this run (catana_gpu_fp64_peak)"}}
    # the same case with exact j_l per (point, l, n) (the reference's branch for N <= 1000)
    run(_lib.JL_EXACT)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(3):
        run(_lib.JL_EXACT)
    e1.record()
    torch.cuda.synchronize()
    ms_x = e0.elapsed_time(e1) / 3
    res["plain_fp64_100k_l32_n32"]["exact_jl"] = {"value": 100000 * modes(L, M) / (ms_x / 1e3), "unit": UNIT,
                                                  "ms_per_step": ms_x}
    # HEALPix
    R = HP_RADIUS
    pc = catana.PointContainer(healpix_catalog(), "cartesian")
    catana.PixelizedPointContainer(256, pc)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ppc = catana.PixelizedPointContainer(256, pc)
    tb = time.perf_counter() - t0
    catana.sfb_decomposition(ppc, 128, 64, R, False, False)
    torch.cuda.synchronize()
    _lib.lib.catana_gpu_profile_enable(1)
    t0 = time.perf_counter()
    catana.sfb_decomposition(ppc, 128, 64, R, False, False)
    ts = time.perf_counter() - t0
    _lib.lib.catana_gpu_profile_enable(0)
    _lib.check(_lib.lib.catana_gpu_profile_report(ctypes.byref(kms), ctypes.byref(kn), ctypes.byref(kfl)))
    res["healpix_nside256_1M_l128_n64"] = {"binning_s": tb, "sfb_s": ts, "ring_transform_s": kms.value / 1e3,
                                           "note": "host API incl. copies; FP64; ring transform: batched FFT "
                                                   "for the power-of-two rings (the 513 equatorial rings of "
                                                   "1024 pixels and 16 polar ones), direct sums over quarter-orbits for the rest"}
    return res


HP_RADIUS = 1000.0


def healpix_catalog(n=1_000_000, seed=1):
    """Cartesian positions: 90% uniform in a ball of radius 1000, 10% in 1000 Gaussian
    clumps of sigma 5 (centres uniform in the ball), clipped to the ball."""
    rng = np.random.default_rng(seed)
    nu = int(0.9 * n)
    nc = n - nu

    def ball(k):
        r = HP_RADIUS * rng.random(k) ** (1 / 3)
        ct = rng.uniform(-1, 1, k)
        ph = rng.uniform(0, 2 * np.pi, k)
        st = np.sqrt(1 - ct ** 2)
        return np.stack([r * st * np.cos(ph), r * st * np.sin(ph), r * ct], 1)
    xyz = [ball(nu)]
    cen = ball(1000)
    got = 0
    while got < nc:
        p = cen[rng.integers(0, 1000, nc)] + rng.normal(0, 5.0, (nc, 3))
        p = p[np.sum(p ** 2, 1) < HP_RADIUS ** 2][:nc - got]
        xyz.append(p)
        got += p.shape[0]
    return np.concatenate(xyz)


def cpu_healpix_baseline(lsample=8):
    """The HEALPix decomposition's CPU restatement with one r2c FFT per ring, as the
    reference computes it (oracle.sfb_healpix_fft: pixel maps in C over all host
    threads, numpy's rfft), on the same catalog binned at nside 256 with nmax 64 and the
    first `lsample` multipoles.  Its work per multipole (the maps over every point and
    radial order, the transforms of every ring) does not grow with l, so the lmax 128
    figure is the sample's time x 128 / lsample."""
    from oracle import oracle as O
    pts = O.cartesian_to_spherical(healpix_catalog())
    offs, rs = O.bin_points(256, pts)
    t0 = time.perf_counter()
    O.sfb_healpix_fft(256, offs, rs, lsample, 64, HP_RADIUS, interpolated=True)
    dt = time.perf_counter() - t0
    return {"value": dt * 128 / lsample, "unit": "s (lmax 128, scaled)", "cores": os.cpu_count(), "kind": "port",
            "sample": "lmax %d of 128 on the same 1M points, nside 256, nmax 64: %.1f s" % (lsample, dt)}


def batched_workload(torch, _lib, catana, sp, ncat=64, seed=3, kmax=0.2, nmax=128):
    """Batched raw SFB: 64 catalogs with point counts log-uniform in [10k, 2M], each
    uniform in a ball with rmax ~ U[500, 1500], lmax ~ U{64..200}, weights U[0.5, 1.5],
    nmax 128 cut at kmax = 0.2; split form, one call per step on device-resident data
    (level loop as one CUDA graph, autotuned schedule).  The FP64 plain form and the
    C_l error are measured on a 0.5% subsample of every catalog (same shapes and cut)."""
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(np.log(1e4), np.log(2e6), ncat)).astype(np.int64)
    rmaxs = rng.uniform(500.0, 1500.0, ncat)
    lmaxs = rng.integers(64, 201, ncat)
    host = []
    for i in range(ncat):
        p, w = catalog(int(ns[i]), float(rmaxs[i]), seed * 1000 + i)
        host.append((p, w))
    pm = 0.0
    for i in range(ncat):
        k = catana.compute_kln(int(lmaxs[i]), nmax, float(rmaxs[i]))
        pm += ns[i] * sum((l + 1) * int((k[l] <= kmax).sum()) for l in range(int(lmaxs[i])))

    def records(frac, dev):
        recs = (_lib.Catalog * ncat)()
        keep = []
        for i in range(ncat):
            n = int(ns[i]) if frac >= 1 else max(1000, int(ns[i] * frac))
            p, w = host[i][0][:n], host[i][1][:n]
            L = int(lmaxs[i])
            fc = int(_lib.lib.catana_gpu_flmn_size(L, nmax))
            if dev:
                dp, dw = torch.from_numpy(np.ascontiguousarray(p)).cuda(), torch.from_numpy(w).cuda()
                k = torch.zeros(L * nmax, dtype=torch.float64, device="cuda")
                c, f = torch.zeros_like(k), torch.zeros(2 * fc, dtype=torch.float64, device="cuda")
                ptr = lambda t: t.data_ptr()
            else:
                dp, dw = np.ascontiguousarray(p), np.ascontiguousarray(w)
                k, c, f = np.zeros(L * nmax), np.zeros(L * nmax), np.zeros(2 * fc)
                ptr = lambda t: t.ctypes.data
            r = recs[i]
            r.points, r.weights, r.npoints = ptr(dp), ptr(dw), n
            r.rmax, r.kmax, r.lmax, r.nmax = float(rmaxs[i]), kmax, L, nmax
            r.k_ln, r.c_ln, r.f_lmn = ptr(k), ptr(c), ptr(f)
            keep.append((dp, dw, k, c, f))
        return recs, keep

    recs, keep = records(1.0, True)
    flags = _lib.FORM_SPLIT

    def run():
        _lib.check(_lib.lib.catana_gpu_sfb_raw_batched_dev(ctypes.cast(recs, ctypes.c_void_p), ncat, flags, 0.0,
                                                           None, sp), "batched")
    run()  # autotunes (cached per catalog set)
    run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(3):
        run()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / 3
    res = {"value": pm / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "catalogs": ncat,
           "points": int(ns.sum()), "point_modes": pm, "waves_autotuned": _lib.lib.catana_gpu_batch_waves(),
           "mblock_autotuned": int(_lib.lib.catana_gpu_batch_mblk()),
           "graph": True}
    # subsample (0.5%, at least 1000 points a catalog): split vs FP64 plain with the
    # reference's j_l rule (interpolated for N > 1000) for the throughput ratio, and
    # vs FP64 plain with exact j_l on the first 8 catalogs for the C_l error
    srecs, skeep = records(0.005, False)
    spm = 0.0
    for i in range(ncat):
        k = catana.compute_kln(int(lmaxs[i]), nmax, float(rmaxs[i]))
        spm += srecs[i].npoints * sum((l + 1) * int((k[l] <= kmax).sum()) for l in range(int(lmaxs[i])))

    def timed(recs_, n_, fl):
        t0 = time.perf_counter()
        _lib.check(_lib.lib.catana_gpu_sfb_raw_batched(ctypes.cast(recs_, ctypes.c_void_p), n_, fl, 0.0, None))
        return time.perf_counter() - t0
    timed(srecs, ncat, flags)
    ts = timed(srecs, ncat, flags)
    tp = timed(srecs, ncat, _lib.FORM_PLAIN | _lib.JL_AUTO)
    ne = 8
    timed(srecs, ne, flags)
    c_split = [x[3].copy() for x in skeep[:ne]]
    timed(srecs, ne, _lib.FORM_PLAIN | _lib.JL_EXACT)
    rel = []
    for cs_, x in zip(c_split, skeep[:ne]):
        m = x[3] != 0
        rel.append(np.abs(cs_[m] - x[3][m]) / np.abs(x[3][m]))
    rel = np.concatenate(rel)
    res["subsample_0.5pct"] = {"points": int(sum(r.npoints for r in srecs)), "split_s": ts, "plain_fp64_s": tp,
                               "split_over_plain": tp / ts, "split_value": spm / ts, "plain_value": spm / tp,
                               "c_ln_rel_err_median": float(np.median(rel)),
                               "c_ln_rel_err_p99": float(np.percentile(rel, 99)),
                               "note": "host API incl. copies; plain uses interpolated j_l (N > 1000 rule); "
                                       "C_l error vs plain with exact j_l on the first %d catalogs" % ne}
    del keep
    return res


def survey_chunk(rng, n, rmax=1500.0, a=300.0):
    """n float32 (r, theta, phi) records: radial pdf ~ r^2 exp(-(r/a)^2) truncated at
    rmax (r = a/sqrt(2) chi_3), |theta - pi/2| < 20 deg masked out, phi uniform."""
    out = np.empty((n, 3), dtype=np.float32)
    got = 0
    smin = np.sin(np.deg2rad(20.0))
    while got < n:
        k = n - got
        r = a / np.sqrt(2.0) * np.sqrt((rng.standard_normal((k, 3)) ** 2).sum(1))
        r = r[r < rmax]
        m = r.shape[0]
        ct = rng.uniform(smin, 1.0, m) * np.where(rng.random(m) < 0.5, -1.0, 1.0)
        out[got:got + m, 0] = r
        out[got:got + m, 1] = np.arccos(ct)
        out[got:got + m, 2] = rng.uniform(0.0, 2.0 * np.pi, m)
        got += m
    return out


def streamed_workload(torch, _lib, catana, chunks=2, chunk=8_000_000, L=512, M=256, seed=4, form="split"):
    """Large masked survey through the chunked accumulator: float32 (r, theta, phi)
    records in pinned host memory, 8M-point chunks, lmax 512, nmax 256, split form (above
    lmax 256 always with the Reinsch-modified Legendre rows: a mode that the data reach
    only in j_l's evanescent zone is carried by the outermost few points, so their rows'
    accuracy enters its C_ln undiluted, and three-term rows lose a few 1e-6 for such a
    point near a pole).  The full survey has 100M points = 13 such chunks; the rate per point is
    the same for every chunk, so a bounded number of chunks is timed by default.  The
    timed region is create + every add (host-to-device copy overlapped with the previous
    chunk's decomposition) + finish (normalisation, C_ln, copies back)."""
    rng = np.random.default_rng(seed)
    host = []
    total = min(chunks * chunk, 100_000_000)  # the survey: 100M points, the last chunk shorter
    for c in range(chunks):
        n_c = min(chunk, total - c * chunk)
        t = torch.empty((n_c, 3), dtype=torch.float32, pin_memory=True)
        t.numpy()[:] = survey_chunk(rng, n_c)
        host.append(t)
    warm = survey_chunk(rng, 50000)
    with catana.SFBAccumulator(L, M, 1500.0, precision=form) as acc:  # builds the j_l tables once
        acc.add(warm)
        acc.finish()
    torch.cuda.synchronize()
    _lib.lib.catana_gpu_profile_enable(1)
    t0 = time.perf_counter()
    with catana.SFBAccumulator(L, M, 1500.0, precision=form) as acc:
        for t in host:
            acc.add(t.numpy())
        res = acc.finish()
    dt = time.perf_counter() - t0
    _lib.lib.catana_gpu_profile_enable(0)
    kms, kn, kfl = ctypes.c_double(), ctypes.c_uint64(), ctypes.c_double()
    _lib.check(_lib.lib.catana_gpu_profile_report(ctypes.byref(kms), ctypes.byref(kn), ctypes.byref(kfl)))
    pm = float(total) * modes(L, M)
    out = {"value": pm / dt, "unit": UNIT, "seconds": dt, "points": total, "chunks": chunks, "chunk": chunk, "lmax": L,
           "nmax": M, "precision": form, "input": "float32 (r, theta, phi), pinned host memory",
           "contraction_kernel_s": kms.value / 1e3, "contraction_tflops_algorithmic": kfl.value / (kms.value / 1e3) / 1e12,
           "c_ln_finite": bool(np.isfinite(res.c_ln).all())}
    # FP64 plain form on a 20k-point subsample (interpolated j_l, the reference's rule)
    sub = host[0].numpy()[:20000].astype(np.float64)
    pc = catana.PointContainer(sub)
    catana.sfb_decomposition(pc, L, M, 1500.0, False, False)
    t0 = time.perf_counter()
    catana.sfb_decomposition(pc, L, M, 1500.0, False, False)
    tp = time.perf_counter() - t0
    out["plain_fp64_20k_value"] = 20000 * modes(L, M) / tp
    out["split_over_plain"] = out["value"] / out["plain_fp64_20k_value"]
    # C_l and f error of the split form against the FP64 plain path (j_l from the FP64
    # polynomials, as accurate as the exact branch) on the first 100k points of chunk 0
    ns = 100_000
    e = host[0].numpy()[:ns].astype(np.float64)
    pe = catana.PointContainer(e)
    rp = catana.sfb_decomposition(pe, L, M, 1500.0, True, False, interpolation="poly")
    keep = rp.c_ln >= 1e-40 * rp.c_ln.max()  # below: j_l(k r) < ~1e-20 of its envelope at every point
    acc = {"sample_points": ns, "modes_below_1e-40_cmax": float(1.0 - keep.mean()),
           "reference": "FP64 plain path, j_l from the FP64 polynomials (CATANA_JL_POLY)",
           "note": "C_ln below 1e-40 of the largest C (j_l(k r) < ~1e-20 of its envelope at every point) leave "
                   "the FP32 operand range and come out 0; the statistics cover the modes above.  The sample's "
                   "outermost point lies 0.15 rad from a pole and alone carries the evanescent-zone modes"}
    rs = catana.sfb_decomposition(pe, L, M, 1500.0, True, False, precision=form)
    rel = np.abs(rs.c_ln - rp.c_ln) / np.abs(rp.c_ln)
    rms_l = [float(np.sqrt(np.mean(np.abs(x - y) ** 2) / np.mean(np.abs(y) ** 2)))
             for x, y in zip(rs.f_lmn, rp.f_lmn)]
    acc.update({"c_ln_rel_err_median": float(np.median(rel[keep])),
                "c_ln_rel_err_p99": float(np.percentile(rel[keep], 99)),
                "c_ln_rel_err_max": float(rel[keep].max()),
                "c_ln_modes_above_1e-6": int((rel[keep] > 1e-6).sum()),
                "f_lmn_rms_err_over_rms_f_by_l": {"l=0": rms_l[0], "l=%d" % (L // 2): rms_l[L // 2],
                                                  "l=%d" % (L - 1): rms_l[-1], "max": max(rms_l)}})
    out["accuracy_100k_pts"] = acc
    del host
    return out


def next_rows_workload(torch, _lib, catana):
    """The survey's "next" rows, one timing each:
    * _sfb_reverse on the HEALPix workload (nside 256, 1M points, lmax 128, nmax 64);
    * device ingest of 8M float32 Cartesian records (tophat + Gaussian window + angular
      mask): records/s and the kernels' HBM bytes per record;
    * shot-noise integrals: all (n1, n2) pairs for l < 32, nmax 32 (32k integrals) with
      a 10001-node window table, against the oracle's CPU quadrature on 64 of them."""
    res = {}
    rng = np.random.default_rng(1)
    pts, _ = catalog(1_000_000, 1000.0, 1)
    ppc = catana.PixelizedPointContainer(256, catana.PointContainer(pts))
    catana.sfb_reverse(ppc, 128, 64, 1000.0, False, False)
    t0 = time.perf_counter()
    catana.sfb_reverse(ppc, 128, 64, 1000.0, False, False)
    res["sfb_reverse_nside256_1M_l128_n64_s"] = time.perf_counter() - t0
    # ingest
    n = 8_000_000
    xyz = (rng.normal(size=(n, 3)) * 500.0).astype(np.float32)
    mask = (rng.random(12 * 64 * 64) < 0.7).astype(np.float32)
    kw = dict(coordinate_type="cartesian", tophat_r0=1500.0, gauss_r0=1000.0, mask=mask, seed=3)
    catana.ingest(xyz[:100000], **kw)
    t0 = time.perf_counter()
    kept = catana.ingest(xyz, **kw)
    dt = time.perf_counter() - t0
    res["ingest_8M_float32_cartesian"] = {"records_per_s": n / dt, "seconds": dt, "kept": len(kept),
                                          "note": "host API incl. 96 MB H2D and the kept points D2H",
                                          "device_bytes_per_record": 12 + 24 + 1 + 24 + 1}
    # integrals
    rmax = 1000.0
    fi = catana.FunctionInterpolator(lambda r: np.exp(-(r / 400.0) ** 2) * r ** 2, 10001, 0.0, rmax)
    L, M = 32, 32
    kk = catana.compute_kln(L, M, rmax)
    total = 0
    catana.besseltools.double_sbessel_integrator(fi, 1, rmax, kk[1][:2], kk[1][:2])
    t0 = time.perf_counter()
    for l in range(L):
        k1, k2 = np.meshgrid(kk[l], kk[l])
        catana.besseltools.double_sbessel_integrator(fi, l, rmax, k1, k2)
        total += k1.size
    dt = time.perf_counter() - t0
    res["shot_noise_integrals_l32_n32"] = {"integrals": total, "seconds": dt, "integrals_per_s": total / dt,
                                           "note": "one warp per pair, 32/8-point Gauss-Legendre between the zeros "
                                                   "and the window's nodes; host API incl. copies"}
    return res


def cpu_integrals_baseline():
    """The oracle's quadrature of the same integrals (adaptive Gauss-Legendre, one core)
    on 64 of them: the CPU side of the shot-noise-integral leg."""
    from oracle import oracle as O
    rmax = 1000.0
    x = np.linspace(0.0, rmax, 10001)
    w = np.exp(-(x / 400.0) ** 2) * x ** 2
    import catana_gb300 as catana
    kk = catana.compute_kln(32, 32, rmax)
    t0 = time.perf_counter()
    for i in range(8):
        for j in range(8):
            O.dsb_integral(w, (0.0, rmax), 16, rmax, kk[16][i], kk[16][j])
    return {"value": 64 / (time.perf_counter() - t0), "unit": "integrals/s", "cores": 1, "kind": "port",
            "sample": "64 (n1, n2) pairs at l = 16 of the same window and k_ln"}


def measure_fp64_peak(_lib):
    """FP64 FMA throughput of this GPU as the clocks stand (the library's own
    dependent-chain kernel, CUDA events), with the SM clock sampled meanwhile."""
    clk = Clocks(torch_device_index())
    clk.start()
    tf = ctypes.c_double(0.0)
    st = _lib.lib.catana_gpu_fp64_peak(ctypes.c_int(1500), ctypes.byref(tf))
    c = clk.stop()
    return {"tflops": tf.value if st == 0 else None, "clocks": c,
            "how": "catana_gpu_fp64_peak: 8 independent FMA chains per thread, 8 CTAs x 256 threads per SM, "
                   "about 1.5 s, best of 3 launches"}


def torch_device_index():
    import torch
    return torch.cuda.current_device()


def split_error_stats(f_s, c_s, f_p, c_p, L, M):
    """Error of a split result (f_s, c_s) against an FP64 one (f_p, c_p), every mode."""
    fs = f_s[0::2] + 1j * f_s[1::2]
    fp = f_p[0::2] + 1j * f_p[1::2]
    rel = np.abs(c_s - c_p) / np.abs(c_p)
    typ = np.abs(c_s - c_p) / np.maximum(np.abs(c_p), np.median(c_p, axis=1, keepdims=True))
    rms_l = np.zeros(L)
    off = 0
    for l in range(L):
        sl = slice(off, off + (l + 1) * M)
        rms_l[l] = np.sqrt(np.mean(np.abs(fs[sl] - fp[sl]) ** 2) / np.mean(np.abs(fp[sl]) ** 2))
        off += (l + 1) * M
    over = rel > 1e-6
    # modes above the 1e-6 bar, by number: how small their C_ln is against the median
    # C of their l (a chi-square draw far below the median inflates the relative error)
    ratio = (c_p / np.median(c_p, axis=1, keepdims=True))[over]
    ls_over = np.nonzero(over)[0]
    worst = np.argsort(rel, axis=None)[::-1][:8]
    med_l = np.median(c_p, axis=1)
    return {
        "c_ln_rel_err_median": float(np.median(rel)), "c_ln_rel_err_p99": float(np.percentile(rel, 99)),
        "c_ln_rel_err_p999": float(np.percentile(rel, 99.9)), "c_ln_rel_err_max": float(rel.max()),
        "c_ln_modes": int(rel.size), "c_ln_modes_above_1e-6": int(over.sum()),
        "c_ln_above_1e-6_c_over_median_c_l_max": float(ratio.max()) if ratio.size else None,
        "c_ln_above_1e-6_c_over_median_c_l_median": float(np.median(ratio)) if ratio.size else None,
        "c_ln_above_1e-6_l_min_median_max": ([int(ls_over.min()), float(np.median(ls_over)), int(ls_over.max())]
                                             if ls_over.size else None),
        "c_ln_worst_modes": [{"l": int(i // M), "n": int(i % M), "rel_err": float(rel.flat[i]),
                              "c_over_median_c_l": float(c_p.flat[i] / med_l[i // M]),
                              "abs_err_over_median_c_l": float(abs(c_s.flat[i] - c_p.flat[i]) / med_l[i // M])}
                             for i in worst],
        "c_ln_abs_err_over_max_c_or_median_c_l_max": float(typ.max()),
        "f_lmn_max_abs_err_over_max_f": float(np.max(np.abs(fs - fp)) / np.max(np.abs(fp))),
        "f_lmn_rms_err_over_rms_f_by_l": {"l=0": float(rms_l[0]), "l=%d" % (L // 2): float(rms_l[L // 2]),
                                          "l=%d" % (L - 1): float(rms_l[-1]), "max": float(rms_l.max()),
                                          "argmax_l": int(rms_l.argmax())},
    }


def accuracy_full(torch, _lib, a, d_pts, d_w, d_k, d_c, d_f, sp):
    """The split form's error on the whole catalog: d_f / d_c hold the split result of
    the last timed step; the same catalog runs once more through the FP64 plain path
    with j_l from the piecewise FP64 polynomials (CATANA_JL_POLY, pinned to the
    oracle's exact j_l at 1e-10 of max|f| in tests/test_raw_fp64_gpu.py), and every
    f_lmn and C_ln is compared.  The FP64 run is timed (events on its stream), and the
    CATANA_SPLIT_ACCURATE variant of the split form is run, timed and compared too."""
    L, M = a.lmax, a.nmax
    f_s = d_f.cpu().numpy()
    c_s = d_c.cpu().numpy().reshape(L, M)
    d_f2 = torch.zeros_like(d_f)
    d_c2 = torch.zeros_like(d_c)
    d_k2 = torch.zeros_like(d_k)

    def run(flags, reps=1):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            _lib.check(_lib.lib.catana_gpu_sfb_raw_dev(
                ctypes.c_void_p(d_pts.data_ptr()), ctypes.c_void_p(d_w.data_ptr()), a.points, L, M, a.rmax, flags,
                ctypes.c_void_p(d_k2.data_ptr()), ctypes.c_void_p(d_c2.data_ptr()), ctypes.c_void_p(d_f2.data_ptr()),
                None, sp), "sfb_raw_dev")
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3 / reps, d_f2.cpu().numpy(), d_c2.cpu().numpy().reshape(L, M)

    t_ref, f_p, c_p = run(_lib.FORM_PLAIN | _lib.JL_POLY)
    out = {"sample_points": a.points, "lmax": L, "nmax": M,
           "reference": "FP64 plain GPU path, j_l from piecewise FP64 polynomials (CATANA_JL_POLY), same catalog",
           "reference_seconds": t_ref, "reference_value": a.points * modes(L, M) / t_ref}
    out.update(split_error_stats(f_s, c_s, f_p, c_p, L, M))
    run(_lib.FORM_SPLIT | _lib.SPLIT_ACCURATE)  # tables and workspace for this variant
    t_acc, f_a, c_a = run(_lib.FORM_SPLIT | _lib.SPLIT_ACCURATE, reps=2)
    acc = {"value": a.points * modes(L, M) / t_acc, "unit": UNIT, "ms_per_step": t_acc * 1e3,
           "note": "CATANA_SPLIT_ACCURATE: Reinsch-modified Legendre rows for m < 128 (rows P_l and D_l at "
                   "|cos theta|); same catalog, same FP64 reference"}
    acc.update(split_error_stats(f_a, c_a, f_p, c_p, L, M))
    out["split_accurate"] = acc
    del d_f2, d_c2, d_k2
    return out


def workload_config(a):
    return {"workload": "raw SFB %s form: %d points uniform in a ball rmax=%g, weights U[0.5,1.5], lmax=%d, "
                        "nmax=%d, seed %d" % (a.form, a.points, a.rmax, a.lmax, a.nmax, a.seed),
            "points_per_gpu": a.points, "lmax": a.lmax, "nmax": a.nmax, "rmax": a.rmax,
            "form": a.form, "modes": modes(a.lmax, a.nmax),
            "l2": "inputs (%.0f MB) larger than L2 (129 MB); no flush" % (a.points * 32 / 1e6)}


def main():
    a = parse()
    if a.impl == "reference":
        return run_reference(a)
    import torch
    import catana_gb300 as catana  # noqa: F401
    from catana_gb300 import _lib

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if a.only is not None:
        sp0 = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        run_one = {"side": lambda: side_workloads(torch, _lib, catana, sp0),
                   "batched": lambda: batched_workload(torch, _lib, catana, sp0),
                   "streamed": lambda: streamed_workload(torch, _lib, catana, chunks=max(1, a.stream_chunks),
                                                         chunk=a.stream_points),
                   "next": lambda: next_rows_workload(torch, _lib, catana)}[a.only]
        print(json.dumps({"only": a.only, "result": run_one()}, default=float))
        return
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    flags = _lib.FORM_SPLIT if a.form == "split" else (_lib.FORM_PLAIN | _lib.JL_AUTO)
    L, M = a.lmax, a.nmax
    nmodes = modes(L, M)
    pts, w = catalog(a.points, a.rmax, a.seed, shard=rank)
    w_local = float(w.sum())
    from catana_gb300 import shards
    h_pts = torch.from_numpy(pts).pin_memory()
    h_w = torch.from_numpy(w).pin_memory()
    d_pts = h_pts.cuda()
    d_w = h_w.cuda()
    fsz = int(_lib.lib.catana_gpu_flmn_size(L, M))
    d_k = torch.zeros(L * M, dtype=torch.float64, device="cuda")
    d_c = torch.zeros_like(d_k)
    d_f = torch.zeros(2 * fsz, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)

    def step():
        st = _lib.lib.catana_gpu_sfb_raw_dev(ctypes.c_void_p(d_pts.data_ptr()), ctypes.c_void_p(d_w.data_ptr()),
                                             a.points, L, M, a.rmax, flags, ctypes.c_void_p(d_k.data_ptr()),
                                             ctypes.c_void_p(d_c.data_ptr()), ctypes.c_void_p(d_f.data_ptr()),
                                             None, sp)
        _lib.check(st, "sfb_raw_dev")
        if dist is not None:
            # one catalog sharded over ranks: each shard's f carries V / W_r, so the
            # union is f = sum_r (W_r / W) f_r (W_r = the shard's weight sum)
            shards.combine_flmn(d_f, w_local, dist.all_reduce)
            d_c.copy_(shards.cln_from_flmn(d_f, L, M).reshape(-1))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(a.warmup):
        step()
    barrier()
    clocks = Clocks(local)
    clocks.start()
    launches0 = int(_lib.lib.catana_gpu_launch_count())
    _lib.lib.catana_gpu_profile_enable(1)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    barrier()
    ev0.record(stream)
    for _ in range(a.steps):
        step()
    ev1.record(stream)
    barrier()
    _lib.lib.catana_gpu_profile_enable(0)
    ms_total = ev0.elapsed_time(ev1)
    launches = int(_lib.lib.catana_gpu_launch_count()) - launches0
    kms = ctypes.c_double(0.0)
    kn = ctypes.c_uint64(0)
    kfl = ctypes.c_double(0.0)
    _lib.check(_lib.lib.catana_gpu_profile_report(ctypes.byref(kms), ctypes.byref(kn), ctypes.byref(kfl)))
    clk = clocks.stop()
    if dist is not None:
        t = torch.tensor([ms_total], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_total = float(t.item())
    ms_step = ms_total / a.steps
    value = world * a.points * nmodes / (ms_step / 1e3)

    bf16, bf16_sus, hbm, src = peaks()
    fp64_peak = measure_fp64_peak(_lib)
    if a.form == "split":
        # each launch runs inside a seconds-long step: the sustained figure applies
        peak = bf16_sus / 3.0
        peak_note = ("bf16_tflops_sustained / 3 (three FP16 hi/lo products per MAC; the launches run inside a "
                     "%.1f s step), of %s" % (0.0, src))
        bound = "tensor"
        kernel = "k_split_l (tcgen05 kind::f16 contraction + operand generation)"
    else:
        peak = fp64_peak["tflops"]
        peak_note = "FP64 FMA throughput measured by catana_gpu_fp64_peak in this run"
        bound = "fp64"
        kernel = "k_fp64_raw_l"
    achieved = (kfl.value / (kms.value / 1e3)) / 1e12 if kms.value > 0 else None
    # DRAM bytes of an average k_split_l launch: the ncu capture of l = 200 on 300k points
    # (profiles/k_split_l_l200_300k_full.md) read+wrote 756.0 MB = 1.024 x the algorithmic
    # 12 B per (point, m) of Legendre rows + 48 B per point (738 MB); the traffic grows in
    # proportion to points x (l + 1), so that ratio is applied here to this run's catalog
    # pieces and averaged over the launches.
    traffic = None
    if a.form == "split":
        chunk = min(a.points, int(16e9 / (12.0 * L)))
        avg = sum((12.0 * (l + 1) + 48.0) * chunk for l in range(L)) / L
        traffic = 1.024 * avg
    if a.form == "split":
        peak_note = peak_note.replace("0.0 s step", "%.1f s step" % (ms_step / 1e3))
    roof = {"bound": bound, "kernel": kernel, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": (achieved / peak) if achieved else None, "traffic": traffic,
            "frac_of_burst_peak": (achieved / (bf16 / 3.0)) if (achieved and a.form == "split") else None,
            "traffic_unit": "bytes per launch (average over l): one ncu capture (l = 200, 300k points) scaled "
                            "by points x (l + 1)",
            "peak_source": peak_note,
            "kernel_ms_per_step": kms.value / a.steps, "kernel_launches_per_step": int(kn.value) // max(1, a.steps),
            "kernel_share_of_step": (kms.value / ms_total) if ms_total > 0 else None,
            "algo_flops_per_point_mode": 4}

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
           "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f16 hi+lo x3 / f32 accumulate / f64 reduce" if a.form == "split" else "f64",
           "data": "synthetic", "config": workload_config(a), "gpu_launches": launches, "roofline": roof,
           "clocks": clk, "fp64_peak": fp64_peak}

    if not a.no_extras and rank == 0:
        # ---- e2e through the host-buffer C ABI (pinned input, H2D + compute + D2H) ----
        kh = np.zeros(L * M)
        ch = np.zeros(L * M)
        times = []
        for _ in range(max(1, min(a.steps, 3))):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            st = _lib.lib.catana_gpu_sfb_raw(ctypes.c_void_p(h_pts.data_ptr()), ctypes.c_void_p(h_w.data_ptr()),
                                             a.points, L, M, a.rmax, flags, _lib.ptr(kh), _lib.ptr(ch), None, sp)
            _lib.check(st, "sfb_raw")
            times.append(time.perf_counter() - t0)
        e2e_t = float(np.median(times))
        out["e2e"] = {"value": a.points * nmodes / e2e_t, "unit": UNIT, "ms_per_step": e2e_t * 1e3,
                      "h2d_bytes_per_step": a.points * 32, "d2h_bytes_per_step": 2 * L * M * 8,
                      "api": "catana_gpu_sfb_raw (host buffers, pinned)"}
        # ---- FP64 plain GPU path (the drop-in, the reference's default j_l rule) on a subsample ----
        ns = min(a.plain_sample, a.points)
        sub = np.ascontiguousarray(pts[:ns])
        wsub = np.ascontiguousarray(w[:ns])
        fc = int(_lib.lib.catana_gpu_flmn_size(L, M))

        def host_call(fl, store):
            k2 = np.zeros(L * M)
            c2 = np.zeros(L * M)
            f2 = np.zeros(2 * fc) if store else None
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            _lib.check(_lib.lib.catana_gpu_sfb_raw(_lib.ptr(sub), _lib.ptr(wsub), ns, L, M, a.rmax, fl, _lib.ptr(k2),
                                                   _lib.ptr(c2), _lib.ptr(f2), sp), "sfb_raw")
            return time.perf_counter() - t0, c2, f2

        host_call(_lib.FORM_PLAIN | _lib.JL_AUTO, False)  # builds the cached tables
        tp = host_call(_lib.FORM_PLAIN | _lib.JL_AUTO, False)[0]
        out["plain_fp64"] = {"value": ns * nmodes / tp, "unit": UNIT, "sample_points": ns,
                             "note": "FP64 CUDA-core path, interpolated j_l (the reference's rule for N > 1000), "
                                     "host-buffer call incl. copies, same lmax/nmax/weights"}
        if a.form == "split":
            out["split_vs_plain_speedup"] = value / out["plain_fp64"]["value"]
            if not a.no_accuracy:
                out["accuracy_vs_fp64"] = accuracy_full(torch, _lib, a, d_pts, d_w, d_k, d_c, d_f, sp)
        # ---- side workloads: FP64 plain at 100k points / lmax = nmax = 32, HEALPix nside 256 ----
        if a.side:
            out["side"] = side_workloads(torch, _lib, catana, sp, fp64_peak)
            out["side"]["batched_64_catalogs_kmax0.2_split"] = batched_workload(torch, _lib, catana, sp)
            out["side"]["next_rows"] = next_rows_workload(torch, _lib, catana)
            if a.stream_chunks > 0:
                out["side"]["streamed_survey_l512_n256_split"] = streamed_workload(torch, _lib, catana,
                                                                                  chunks=a.stream_chunks,
                                                                                  chunk=a.stream_points)
        # ---- CPU baseline: the oracle's OpenMP restatement, fixed + per-point fit ----
        t_full, _, _, note = cpu_fit(a)
        v = a.points * nmodes / t_full
        if a.side:
            out["side"]["next_rows"]["shot_noise_integrals_l32_n32"]["cpu_baseline"] = cpu_integrals_baseline()
            try:  # the FP64 drop-in case in full: 100k points, lmax = nmax = 32, unit weights, seed 0
                p1, _ = catalog(100000, 1000.0, 0)
                t1 = cpu_time(p1, None, 32, 32, 1000.0)
                v1 = 100000 * modes(32, 32) / t1
                out["side"]["plain_fp64_100k_l32_n32"]["cpu_baseline"] = {
                    "value": v1, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                    "sample": "the whole workload (100k points), interpolated j_l as the reference uses for "
                              "N > 1000; %.2f s" % t1}
            except Exception as ex:  # a side measurement: never costs the main line
                out["side"]["plain_fp64_100k_l32_n32"]["cpu_baseline"] = {"error": repr(ex)}
            try:
                out["side"]["healpix_nside256_1M_l128_n64"]["cpu_baseline"] = cpu_healpix_baseline()
            except Exception as ex:  # a side measurement: never costs the main line
                out["side"]["healpix_nside256_1M_l128_n64"]["cpu_baseline"] = {"error": repr(ex)}
        out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": os.cpu_count(), "kind": "port", "sample": note}
    if rank == 0:
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
