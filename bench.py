"""Benchmark: batched fwd+adj slices/s of the log-polar Radon transform at N=2048.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one forward (Radon) transform plus one adjoint with the
shepp-logan FBP filter over a batch of 128 slices of 2048x2048 images and
3000x2048 sinograms (random-ellipse phantoms, 30 ellipses, seed 3, with
Gaussian noise of 1% of the sinogram maximum on the adjoint's input),
all resident in HBM.  `value` is slices/s over all ranks (replicas, weak
scaling).  `e2e` repeats the step through the public lpTransform API from
pinned host buffers with the host<->device copies inside the timed region.

`--impl reference` times the CPU float64 restatement of the reference
algorithm (the oracle; the reference itself has no CPU path and its CUDA code
does not build with CUDA 13) on the host cores, one slice per process.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "fwd+adj slices/s (N=2048, Nproj=3000, batched)"
UNIT = "slices/s"
WORKLOAD = dict(N=2048, Nproj=3000, S=128, filter="shepp-logan", interp="cubic", ellipses=30, seed=3, noise=0.01)
# algorithmic HBM bytes per slice of one fwd+adj step (N=2048, Nproj=3000, batch 128)
ALGO_BYTES_PER_SLICE = 1.541e9
# DRAM bytes (read + write) per slice and launch measured by ncu on an 8-slice step of the
# same geometry (launch averages / 8); the traffic of a 128-slice launch is taken as 128
# times these (every term but the per-launch tables grows with the slice count)
NCU_DRAM_BYTES_PER_SLICE = {
    "fwd_ingest": (134.2e6 + 85.5e6) / 8, "col_prefilter": (165.4e6 + 117.9e6) / 8,
    "fwd_c2lp": (129.7e6 + 121.7e6) / 8, "theta_conv": (168.2e6 + 79.9e6) / 8,
    "fwd_lp2polar": (143.8e6 + 44.2e6) / 8, "adj_ingest": (196.7e6 + 150.5e6) / 8,
    "adj_polar2lp": (83.2e6 + 87.9e6) / 8, "adj_lpcols": (135.6e6 + 92.3e6) / 8,
    "adj_lp2cart": (354.1e6 + 117.2e6) / 8,
}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, dev):
        self.dev = dev
        self.proc = None
        self.path = None
        self._summary = None

    def _lines(self):
        try:
            with open(self.path) as fh:
                return sum(1 for _ in fh)
        except OSError:
            return 0

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        # the sampler's first line before the timed region starts (nvidia-smi takes a
        # moment to come up; a short region would otherwise end before any sample)
        t_end = time.time() + 5.0
        while self.proc is not None and self._lines() == 0 and time.time() < t_end and self.proc.poll() is None:
            time.sleep(0.02)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        """Median SM clock, maximum clock and active throttle reasons of the samples
        (computed once; later calls return the same record)."""
        if self._summary is not None:
            return self._summary
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        if not self.path or not os.path.exists(self.path):
            return out
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if sm:
            out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                   "samples": len(sm)}
        self._summary = out
        return out


def phantoms_gpu(torch, N, S, n_ell, seed, dev):
    """Random-ellipse phantoms (the oracle's generator, vectorised on the GPU)."""
    rng = np.random.default_rng(seed)
    lin = torch.linspace(-1, 1, N, dtype=torch.float64, device=dev)
    x2, x1 = torch.meshgrid(-lin, lin, indexing="ij")
    out = torch.zeros((S, N, N), dtype=torch.float32, device=dev)
    for s in range(S):
        img = torch.zeros((N, N), dtype=torch.float64, device=dev)
        for _ in range(n_ell):
            r = 0.7 * np.sqrt(rng.uniform())
            phi = 2 * np.pi * rng.uniform()
            cx, cy = r * np.cos(phi), r * np.sin(phi)
            a, b = rng.uniform(0.05, 0.35, size=2)
            rot = rng.uniform(0, np.pi)
            val = rng.uniform(-0.2, 1.0)
            u = (x1 - cx) * np.cos(rot) + (x2 - cy) * np.sin(rot)
            v = -(x1 - cx) * np.sin(rot) + (x2 - cy) * np.cos(rot)
            img += val * (((u / a) ** 2 + (v / b) ** 2) <= 1)
        out[s] = img.float()
    return out


# ---------------------------------------------------------------------------
# CPU baseline: the oracle (float64 NumPy restatement of the reference
# algorithm).  One slice's fwd+adj per step; the three angular spans of each
# direction are independent in the reference's loop (lpRgpu.cu:257, :302), so
# they run in six worker processes while the parent does the prefilters, the
# FBP filter and the sums.
# ---------------------------------------------------------------------------
_W = {}


def _cpu_init(path):
    sys.path.insert(0, ROOT)
    from oracle import lprec_oracle as O
    z = np.load(path)
    _W["O"] = O
    _W["tr"] = O.Transform.from_packed(z["glpars"], z["fwdparsi"], z["fwdparamsf"], z["adjparsi"], z["adjparamsf"])


def _cpu_span(args):
    kind, k, arr = args
    O, tr = _W["O"], _W["tr"]
    if kind == "fwd":
        return O.fwd_span(tr.G, tr.Tf, arr, tr.erho, k)
    return O.adj_span(tr.G, tr.Ta, arr, k)


def _cpu_prep(args):
    """Per-slice preparation: centre and prefilter an image (fwd), or pad, FBP-filter and
    prefilter a sinogram (adj)."""
    kind, arr = args
    O, tr = _W["O"], _W["tr"]
    G = tr.G
    if kind == "fwd":
        o = G.N // 2 - G.N0 // 2
        d = np.zeros((1, G.N, G.N))
        d[:, o:o + G.N0, o:o + G.N0] = arr
    else:
        d = O.pad_sinogram(G, arr)
        if tr.Ta.get("filter") is not None:
            d = O.apply_filter(G, d, tr.Ta["filter"])
    return O.prefilter2d(d) if G.cubic else d


class CpuBaseline:
    """fwd+adj of B slices per step with the oracle in one process pool: the slices'
    preparation jobs, then the 3 spans of each direction and slice as parallel jobs
    (6 B jobs, so B = cores // 6 keeps every core busy)."""

    def __init__(self, packed, nproc, slices=1):
        import multiprocessing as mp
        sys.path.insert(0, ROOT)
        from oracle import lprec_oracle as O
        self.O = O
        fd, self.path = tempfile.mkstemp(suffix=".npz")
        os.close(fd)
        np.savez(self.path, glpars=packed[0], fwdparsi=packed[1], fwdparamsf=packed[2], adjparsi=packed[3],
                 adjparamsf=packed[4])
        self.tr = O.Transform.from_packed(*packed)
        self.pool = mp.get_context("spawn").Pool(nproc, initializer=_cpu_init, initargs=(self.path,))
        self.nproc = nproc
        self.B = max(1, int(slices))
        rng = np.random.default_rng(WORKLOAD["seed"])
        self.f = [O.ellipse_phantom(self.tr.G.N0, WORKLOAD["ellipses"], rng)[None] for _ in range(self.B)]
        self.R = None

    def step(self):
        tr, B = self.tr, self.B
        G = tr.G
        t0 = time.perf_counter()
        adj = self.R is not None
        prep = [("fwd", f) for f in self.f] + ([("adj", R) for R in self.R] if adj else [])
        pre = self.pool.map(_cpu_prep, prep)
        jobs = [("fwd", k, pre[b]) for b in range(B) for k in range(3)]
        if adj:
            jobs += [("adj", k, pre[B + b]) for b in range(B) for k in range(3)]
        res = self.pool.map(_cpu_span, jobs)
        Rs = []
        for b in range(B):
            R = np.zeros((1, G.Nproj * G.N))
            for k in range(3):
                R[:, tr.Tf["pids"][k]] += res[3 * b + k]
            Rs.append(R.reshape(1, G.Nproj, G.N)[:, ::G.osangles, G.N // 2 - G.cor:G.N // 2 - G.cor + G.N0])
        if adj:
            for b in range(B):
                f = np.zeros((1, G.N * G.N))
                for k in range(3):
                    f[:, tr.Ta["cids"]] += res[3 * B + 3 * b + k]
        self.R = Rs
        return time.perf_counter() - t0, adj

    def close(self):
        self.pool.close()
        self.pool.join()
        os.unlink(self.path)


def _fp64_init(N, Nproj, filt):
    sys.path.insert(0, ROOT)
    from oracle import lprec_oracle as O
    _W["O"] = O
    _W["tr"] = O.Transform(N, Nproj, 1, filt, N / 2, "cubic", mode="fp64", rounded=False)


def fp64_oracle_outputs(f, noise, seed, nproc):
    """The float64 oracle with unrounded float64 tables on one slice of the headline
    geometry: R = fwd(f), Rn = R + Gaussian noise (noise * max|R|), FBP(Rn) with the
    workload's filter and the unfiltered adj(Rn).  The spans run as jobs in a spawn
    pool whose workers build the tables themselves."""
    import multiprocessing as mp
    from oracle import lprec_oracle as O
    W = WORKLOAD
    N, Nproj = W["N"], W["Nproj"]
    t0 = time.perf_counter()
    pool = mp.get_context("spawn").Pool(min(nproc, 6), initializer=_fp64_init, initargs=(N, Nproj, W["filter"]))
    try:
        tr = O.Transform(N, Nproj, 1, W["filter"], N / 2, "cubic", mode="fp64", rounded=False)
        G = tr.G
        o = G.N // 2 - G.N0 // 2
        d = np.zeros((1, G.N, G.N))
        d[:, o:o + G.N0, o:o + G.N0] = f
        fp = O.prefilter2d(d)
        res = pool.map(_cpu_span, [("fwd", k, fp) for k in range(3)])
        Rfull = np.zeros((1, G.Nproj * G.N))
        for k in range(3):
            Rfull[:, tr.Tf["pids"][k]] += res[k]
        c0 = G.N // 2 - G.cor
        R = Rfull.reshape(1, G.Nproj, G.N)[:, ::G.osangles, c0:c0 + G.N0][:, :G.Nproj0]
        rng = np.random.default_rng(seed)
        Rn = np.float32(R + noise * np.abs(R).max() * rng.standard_normal(R.shape)).astype(np.float64)
        dR = O.pad_sinogram(G, Rn)
        pf = O.prefilter2d(O.apply_filter(G, dR, tr.Ta["filter"]))
        pn = O.prefilter2d(dR)
        res = pool.map(_cpu_span, [("adj", k, pf) for k in range(3)] + [("adj", k, pn) for k in range(3)])
        outs = []
        for j in range(2):
            full = np.zeros((1, G.N * G.N))
            for k in range(3):
                full[:, tr.Ta["cids"]] += res[3 * j + k]
            outs.append(full.reshape(1, G.N, G.N)[:, o:o + G.N0, o:o + G.N0])
    finally:
        pool.close()
        pool.join()
    return R, Rn, outs[0], outs[1], time.perf_counter() - t0


def rel_l2_vs_fp64(torch, dev, nproc):
    """Relative L2 of the GPU's fwd, unfiltered adj and FBP on one slice of the headline
    geometry against the float64 oracle with unrounded float64 tables, for both table
    precisions of lpTransform."""
    from oracle import lprec_oracle as O
    from lprec_gb300.lpTransform import lpTransform
    W = WORKLOAD
    N, Nproj = W["N"], W["Nproj"]
    f = O.ellipse_phantom(N, W["ellipses"], np.random.default_rng(W["seed"]))[None]
    R64, Rn, fbp64, adj64, secs = fp64_oracle_outputs(f, W["noise"], W["seed"], nproc)
    out = {"slice": "one N=%d slice, %d-ellipse phantom (seed %d), %g%% noise on the adjoint input"
                    % (N, W["ellipses"], W["seed"], 100 * W["noise"]), "oracle_seconds": round(secs, 1)}
    fd = torch.as_tensor(np.float32(f)).to(dev)
    Rd = torch.as_tensor(np.float32(Rn)).to(dev)
    for prec in ("fp64", "reference"):
        e = {}
        for filt in ("none", W["filter"]):
            lp = lpTransform(N, Nproj, 1, filt, N / 2, "cubic", precision=prec)
            lp.precompute(1)
            lp.initcmem(1, dev)
            Ro = torch.empty((1, Nproj, N), device=dev)
            fo = torch.empty((1, N, N), device=dev)
            if filt == "none":
                lp.fwdp(Ro, fd, dev)
                e["fwd"] = O.rel_l2(Ro.cpu().double().numpy(), R64)
            lp.adjp(fo, Rd, dev)
            if filt == "none":
                e["adj"] = O.rel_l2(fo.cpu().double().numpy(), adj64)
            else:
                e["fbp"] = O.rel_l2(fo.cpu().double().numpy(), fbp64)
            lp.close()
        out["tables_" + prec] = e
    return out


def e2e_timeline(tf, ta):
    """Summary of the per-chunk events of one e2e step (fwd call then adj call)."""
    def ms(a, b):
        return a.elapsed_time(b)
    calls = {}
    for name, tr in (("fwd", tf), ("adj", ta)):
        comp = sum(ms(c["c0"], c["c1"]) for c in tr)
        gaps = sum(max(0.0, ms(tr[i]["c1"], tr[i + 1]["c0"])) for i in range(len(tr) - 1))
        calls[name] = {"chunks": [c["slices"] for c in tr], "compute_ms": round(comp, 2),
                       "compute_gaps_ms": round(gaps, 2),
                       "head_exposed_ms": round(ms(tr[0]["in0"], tr[0]["c0"]), 2),
                       "tail_exposed_ms": round(ms(tr[-1]["c1"], tr[-1]["o1"]), 2),
                       "h2d_ms": round(sum(ms(c["in0"], c["in1"]) for c in tr), 2),
                       "d2h_ms": round(sum(ms(c["o0"], c["o1"]) for c in tr), 2)}
    calls["step_ms"] = round(ms(tf[0]["in0"], ta[-1]["o1"]), 2)
    calls["between_calls_ms"] = round(ms(tf[-1]["c1"], ta[0]["c0"]), 2)
    return calls


def cpu_plan():
    """(processes, slices per step) that keep the host's cores busy: 6 jobs per slice."""
    cores = len(os.sched_getaffinity(0))
    slices = max(1, cores // 6)
    return max(1, min(cores, 6 * slices)), slices


def cpu_baseline(packed, nproc, steps, slices=1):
    """slices/s of fwd+adj (`slices` per step) after one warm-up step that produces the sinograms."""
    cb = CpuBaseline(packed, nproc, slices)
    try:
        cb.step()
        times = [cb.step()[0] for _ in range(steps)]
    finally:
        cb.close()
    return slices / statistics.median(times), sum(times)


def cpu_side_configs():
    """Oracle fwd+adj of one slice at the two smaller workloads (single process)."""
    sys.path.insert(0, ROOT)
    from oracle import lprec_oracle as O
    out = {}
    for N, Nproj, filt, n_ell in ((256, 384, "ramp", 10), (1024, 1536, "shepp-logan", 20)):
        tr = O.Transform(N, Nproj, 1, filt, N / 2, "cubic", mode="fp64")
        f = O.ellipse_phantom(N, n_ell, np.random.default_rng(0))[None]
        R = tr.fwd(f)
        t0 = time.perf_counter()
        R = tr.fwd(f)
        tr.adj(R)
        out["n%d_slices_per_s" % N] = 1.0 / (time.perf_counter() - t0)
    return out


def run_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return
    from oracle import lprec_oracle as O
    W = WORKLOAD
    # the oracle's restatement of the reference's own float32 precompute (initsgl.py,
    # initsfwd.py, initsadj.py): nothing of this library is loaded in this arm
    packed = O.Transform(W["N"], W["Nproj"], 1, W["filter"], W["N"] / 2, W["interp"], mode="ref").packed()
    nproc, B = cpu_plan()
    cb = CpuBaseline(packed, nproc, B)
    try:
        cb.step()  # produces the adjoint's input sinograms
        for _ in range(args.warmup):
            cb.step()
        times = [cb.step()[0] for _ in range(args.steps)]
    finally:
        cb.close()
    value = B / statistics.median(times)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * statistics.median(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic random-ellipse phantom (30 ellipses, seed 3)",
            "config": {"workload": "fwd+adj batch: %d slices N=%d Nproj=%d cubic %s" % (W["S"], W["N"], W["Nproj"],
                                                                                      W["filter"]),
                       "slices": W["S"], "N": W["N"], "Nproj": W["Nproj"], "parallelism": "host processes",
                       "sample_slices_per_step": B},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nproc, "kind": "port",
                             "sample": "%d slice(s) fwd+adj per step; float64 NumPy restatement of the reference "
                                       "algorithm (its CUDA code does not build with CUDA 13) on tables from the "
                                       "restatement of the reference's float32 precompute; per-slice "
                                       "preparation and the 3 spans of fwd and adj of each slice as jobs in %d "
                                       "processes" % (B, nproc)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# GPU benchmark
# ---------------------------------------------------------------------------
def per_kernel_bytes(h, S, prof):
    """Algorithmic HBM bytes per kernel kind for the launches recorded in `prof`."""
    N, N0, Nk, Nth, Nrho = h.N, h.N0, h.Nrho // 2 + 1, h.Ntheta, h.Nrho
    P, P0 = h.Nproj_int, h.Nproj
    half = Nth // 2 + 8
    b = {
        "fwd_ingest": S * (N0 * N0 + N * N) * 4,
        "col_prefilter": S * (2 * N * N + 2 * P * N) * 4 / 2,      # mean of the fwd and adj launches
        # image read once, spectrum columns holding disk points written once, coordinate table
        "fwd_c2lp": S * (N * N * 4 + Nk * half * 8) + Nth * Nrho * 8 / 2,
        # columns in use read and written once, fZ once per launch
        "theta_conv": S * (Nk * half * 8 + Nk * half * 8) + Nk * Nth * 8,
        "fwd_lp2polar": S * (Nk * half * 8 + P0 // 3 * N0 * 4),
        "adj_ingest": S * (P0 * N0 + P * N) * 4,
        "adj_polar2lp": S * (P // 3 * N * 4 + Nk * half * 8),
        "adj_lpcols": S * (Nk * half * 8 + half * Nrho * 4),
        "adj_lp2cart": S * (3 * half * Nrho * 4 + N0 * N0 * 4) + 3 * N0 * N0 * 8,
    }
    return b


def uneven_requests(seed=1, n=48):
    """48 requests: N in {256,512,1024,2048} w.p. {.4,.3,.2,.1}, Nproj = 1.5 N, 1..32 slices."""
    rng = np.random.default_rng(seed)
    Ns = rng.choice([256, 512, 1024, 2048], size=n, p=[0.4, 0.3, 0.2, 0.1])
    Ss = rng.integers(1, 33, size=n)
    return [(int(N), int(3 * N // 2), int(S)) for N, S in zip(Ns, Ss)]


def run_uneven(torch, dev, reps):
    """One CUDA-graph launch running fwd+adj of all 48 requests; throughput and latencies."""
    from lprec_gb300.batch import UnevenBatch
    reqs = uneven_requests()
    t0 = time.perf_counter()
    b = UnevenBatch(reqs, "shepp-logan", "cubic", dev)
    t_setup = time.perf_counter() - t0
    seed = 1
    for i, (N, Nproj, S) in enumerate(reqs):
        b.input_f(i).copy_(phantoms_gpu(torch, N, S, 20, seed + i, dev))
    b.run_eager()
    for i in range(len(reqs)):
        b.input_R(i).copy_(b.output_R(i))
    b.capture()
    stream = torch.cuda.current_stream(dev)
    b.run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        b.run()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    lat = b.latencies_ms()
    e0.record(stream)
    for _ in range(reps):
        b.run_eager()
    e1.record(stream)
    torch.cuda.synchronize()
    ms_eager = e0.elapsed_time(e1) / reps
    out = {"requests": len(reqs), "slices": b.slices, "geometries": len(b.groups), "ms_per_launch": ms,
           "slices_per_s": b.slices / (ms / 1000.0), "ms_eager": ms_eager, "setup_s": round(t_setup, 2)}
    if lat is not None:
        out["latency_ms_p50"] = float(np.percentile(lat, 50))
        out["latency_ms_p99"] = float(np.percentile(lat, 99))
    return out


def run_side_configs(torch, dev, reps=5):
    """The two smaller workloads of the benchmark spec, reported beside the headline:
    64 slices at N=1024 (one batched call vs 64 one-slice calls) and one slice at
    N=256 (call latency, dot tests)."""
    from lprec_gb300.lpTransform import lpTransform
    out = {}
    stream = torch.cuda.current_stream(dev)

    def timed(fn, n):
        fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(n):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / n

    N, Nproj, S = 1024, 1536, 64
    lp = lpTransform(N, Nproj, S, "shepp-logan", N / 2, "cubic")
    lp.precompute(1)
    lp.initcmem(1, dev)
    sched = lp.autotune(dev)
    f = phantoms_gpu(torch, N, S, 20, 1, dev)
    R = torch.empty((S, Nproj, N), device=dev)
    fo = torch.empty_like(f)

    def batched():
        lp.fwdp(R, f, dev)
        lp.adjp(fo, R, dev)

    def plain():
        for s in range(S):
            lp.fwdp(R[s:s + 1], f[s:s + 1], dev)
            lp.adjp(fo[s:s + 1], R[s:s + 1], dev)
    tb, tp = timed(batched, reps), timed(plain, max(1, reps // 2))
    algo = 4.0e8  # algorithmic HBM bytes per slice of fwd+adj at N=1024, Nproj=1536, batch 64
    out["batched_n1024_s64"] = {"slices_per_s": S / tb * 1e3, "plain_slices_per_s": S / tp * 1e3,
                                "batched_over_plain": tp / tb, "ms_batched": tb, "ms_plain": tp,
                                "hbm_gbs_algorithmic": algo * S / tb * 1e-6, "schedule": sched}
    lp.close()
    del f, R, fo

    N, Nproj = 256, 384
    lp = lpTransform(N, Nproj, 1, "ramp", N / 2, "cubic")
    lp.precompute(1)
    lp.initcmem(1, dev)
    f = phantoms_gpu(torch, N, 1, 10, 0, dev)
    R = torch.empty((1, Nproj, N), device=dev)
    fo = torch.empty_like(f)
    tf = timed(lambda: lp.fwdp(R, f, dev), 20)
    ta = timed(lambda: lp.adjp(fo, R, dev), 20)
    rng = np.random.default_rng(0)
    fr = torch.as_tensor(rng.random((1, N, N), dtype=np.float32)).to(dev)
    gr = torch.as_tensor(rng.random((1, Nproj, N), dtype=np.float32)).to(dev)
    lp0 = lpTransform(N, Nproj, 1, "none", N / 2, "cubic")
    lp0.precompute(1)
    lp0.initcmem(1, dev)
    Rf = torch.empty_like(R)
    lp0.fwdp(Rf, fr, dev)
    Ag = torch.empty_like(fr)
    lp0.adjp(Ag, gr, dev)
    Tg = torch.empty_like(fr)
    lp0.fwdp_T(Tg, gr, dev)
    lhs = float((Rf.double() * gr.double()).sum())
    out["single_n256"] = {"fwd_ms": tf, "fbp_ms": ta,
                          "dot_test_adj": abs(lhs - float((fr.double() * Ag.double()).sum())) / abs(lhs),
                          "dot_test_exact_transpose": abs(lhs - float((fr.double() * Tg.double()).sum())) / abs(lhs)}
    lp.close()
    lp0.close()

    # padded sizes that are not powers of two (an off-centre axis pads N0 to
    # ceil((N0 + 2|N0/2 - cor|)/16)*16; the reference's foam data has N = 2016, 299
    # angles; 2560 is a common detector width): fwd+adj throughput per image sample
    # against the power-of-two size of the same (or the nearest) detector width
    geos = [("n512", 512, 768, 256, 64), ("n528_cor253", 512, 768, 253, 64),
            ("n2048", 2048, 3000, 1024, 16), ("n2064_cor1021", 2048, 3000, 1021, 16),
            ("n2080_cor1012", 2048, 3000, 1012, 16), ("n2560", 2560, 3750, 1280, 16),
            ("n2016_foam", 2016, 299, 1008, 16)]
    res = {}
    for name, N0, Np, cor, S in geos:
        lp = lpTransform(N0, Np, S, "shepp-logan", cor, "cubic")
        lp.precompute(1)
        lp.initcmem(1, dev)
        lp.autotune(dev)  # as for the headline: the schedule of this geometry
        h = lp.clphandle[dev]
        f = phantoms_gpu(torch, N0, S, 10, 4, dev)
        R = torch.empty((S, Np, N0), device=dev)
        fo = torch.empty_like(f)

        def step():
            lp.fwdp(R, f, dev)
            lp.adjp(fo, R, dev)
        t = timed(step, reps)
        res[name] = {"N": h.N, "Nrho": h.Nrho, "osangles": h.osangles, "slices": S, "ms": t, "schedule": h.schedule(),
                     "slices_per_s": S / t * 1e3, "ns_per_padded_pixel": t * 1e6 / (S * h.N * h.N)}
        lp.close()
        del f, R, fo
    for name, ref in (("n528_cor253", "n512"), ("n2064_cor1021", "n2048"), ("n2080_cor1012", "n2048"),
                      ("n2016_foam", "n2048"), ("n2560", "n2048")):
        res[name]["per_pixel_vs_pow2"] = res[name]["ns_per_padded_pixel"] / res[ref]["ns_per_padded_pixel"]
    out["padded_sizes"] = res

    # exact transpose (autograd backward) against the forward: 16 slices N=512, Nproj=768
    N, Nproj, S = 512, 768, 16
    lp = lpTransform(N, Nproj, S, "none", N / 2, "cubic")
    lp.precompute(1)
    lp.initcmem(1, dev)
    f = phantoms_gpu(torch, N, S, 10, 2, dev)
    R = torch.empty((S, Nproj, N), device=dev)
    g = torch.empty_like(f)
    lp.fwdp(R, f, dev)
    tf = timed(lambda: lp.fwdp(R, f, dev), 20)
    tt = timed(lambda: lp.fwdp_T(g, R, dev), 20)
    g2 = torch.empty_like(f)
    lp.fwdp_T(g2, R, dev)
    torch.cuda.synchronize()
    out["transpose_n512_s16"] = {"fwd_ms": tf, "transpose_ms": tt, "transpose_over_fwd": tt / tf,
                                 "bit_identical_repeat": bool(torch.equal(g, g2))}
    lp.close()
    return out


def run_ours(args):
    import torch
    from lprec_gb300 import _lib
    from lprec_gb300.lpTransform import lpTransform
    from lprec_gb300.replicas import max_over_ranks
    ws, rank, local = dist_env()
    dist = ws > 1
    if dist:
        import torch.distributed as tdist
        tdist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    dev = local
    torch.cuda.set_device(dev)
    W = WORKLOAD
    N, Nproj, S = W["N"], W["Nproj"], W["S"]
    if args.slices:
        S = args.slices
    if args.small:
        N, Nproj, S = 256, 384, 8
    lp = lpTransform(N, Nproj, S, W["filter"], N / 2, W["interp"], precision="fp64")
    t0 = time.perf_counter()
    lp.precompute(1)
    t_pre = time.perf_counter() - t0
    lp.initcmem(1, dev)
    h = lp.clphandle[dev]
    f = phantoms_gpu(torch, N, S, W["ellipses"], W["seed"] + rank, dev)
    R = torch.empty((S, Nproj, N), device=dev)
    lp.fwdp(R, f, dev)
    torch.cuda.synchronize()
    gen = torch.Generator(device=dev).manual_seed(W["seed"])
    Rn = R + W["noise"] * float(R.abs().max()) * torch.randn(R.shape, device=dev, generator=gen)
    Rout = torch.empty_like(R)
    fout = torch.empty_like(f)
    stream = torch.cuda.current_stream(dev)

    def step():
        lp.fwdp(Rout, f, dev)
        lp.adjp(fout, Rn, dev)

    # batch schedule (slice chunks, one or two streams) picked by the autotuner
    t0 = time.perf_counter()
    sched = lp.autotune(dev) if not args.no_tune else h.schedule()
    t_tune = time.perf_counter() - t0
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        tdist.barrier()
    n0 = _lib.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(dev) as clk:
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    launches = _lib.launch_count() - n0
    ms = e0.elapsed_time(e1)
    # per-kernel times: the same steps with the whole batch in one chunk on one
    # stream (launches do not overlap), CUDA events around every launch
    h.set_schedule(fwd_theta_block=sched["fwd_theta_block"], adj_theta_block=sched["adj_theta_block"])
    step()
    torch.cuda.synchronize()
    h.set_profiling(True)
    h.profile()  # clear
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    prof = h.profile()
    h.set_profiling(False)
    h.set_schedule(**sched)
    ms = max_over_ranks(ms, device=dev)
    ms_step = ms / args.steps
    value = ws * S / (ms_step / 1000.0)

    # plain drop-in: one slice per call
    nplain = min(S, 16)
    torch.cuda.synchronize()
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    for s in range(nplain):
        lp.fwdp(Rout[s:s + 1], f[s:s + 1], dev)
        lp.adjp(fout[s:s + 1], Rn[s:s + 1], dev)
    p1.record(stream)
    torch.cuda.synchronize()
    plain = nplain / (p0.elapsed_time(p1) / 1000.0)

    # e2e through the public API from pinned host buffers: lpTransform.fwd/adj on
    # host tensors, which pipeline host<->device copies against the transforms
    fh = f.cpu().pin_memory()
    Rh = Rn.cpu().pin_memory()
    Rh_out = torch.empty(R.shape, dtype=torch.float32).pin_memory()
    fh_out = torch.empty(f.shape, dtype=torch.float32).pin_memory()

    def e2e_step():
        lp.fwd(fh, dev, out=Rh_out)
        lp.adj(Rh, dev, out=fh_out)

    # the host link's copy bandwidth right now (the host is shared with other jobs, so it
    # varies from run to run and bounds e2e when it drops below ~200 GB/s both ways)
    def link_gbs():
        n = min(fh.numel(), Rh_out.numel())
        a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f.view(-1)[:n].copy_(fh.view(-1)[:n], non_blocking=True)
        torch.cuda.synchronize()
        a_.record(stream)
        f.view(-1)[:n].copy_(fh.view(-1)[:n], non_blocking=True)
        b_.record(stream)
        torch.cuda.synchronize()
        h2d_ = n * 4 / (a_.elapsed_time(b_) / 1e3) / 1e9
        a_.record(stream)
        Rh_out.view(-1)[:n].copy_(R.view(-1)[:n], non_blocking=True)
        b_.record(stream)
        torch.cuda.synchronize()
        return {"h2d": round(h2d_, 1), "d2h": round(n * 4 / (a_.elapsed_time(b_) / 1e3) / 1e9, 1)}
    link = link_gbs()

    for _ in range(max(2, args.warmup // 2)):
        e2e_step()
    torch.cuda.synchronize()
    # five timed windows, each preceded by a measurement of the host link (shared with
    # other jobs on the host: its device->host rate has been seen to drop from ~190 to
    # ~23 GB/s between windows); e2e is the median window
    q0, q1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ke = max(3, args.steps)
    windows = []
    for w in range(5):
        lb = link if w == 0 else link_gbs()
        traces = []
        q0.record(stream)
        for _ in range(ke):
            tf_, ta_ = [], []
            lp.fwd(fh, dev, out=Rh_out, trace=tf_)
            lp.adj(Rh, dev, out=fh_out, trace=ta_)
            traces.append((tf_, ta_))
        q1.record(stream)
        torch.cuda.synchronize()
        # per window: the transforms' busy time, the gaps in which they waited (on copies
        # or on the host), and the copies' effective rates
        tl = [e2e_timeline(a_, b_) for a_, b_ in traces]
        busy = sum(t["fwd"]["compute_ms"] + t["adj"]["compute_ms"] for t in tl) / ke
        h2d_ms = sum(t["fwd"]["h2d_ms"] + t["adj"]["h2d_ms"] for t in tl) / ke
        d2h_ms = sum(t["fwd"]["d2h_ms"] + t["adj"]["d2h_ms"] for t in tl) / ke
        nb = (f.numel() + R.numel()) * 4
        windows.append({"ms_per_step": round(q0.elapsed_time(q1) / ke, 2), "link_gbs_before": lb,
                        "transform_ms_per_step": round(busy, 2),
                        "h2d_gbs": round(nb / (h2d_ms / 1e3) / 1e9, 1), "d2h_gbs": round(nb / (d2h_ms / 1e3) / 1e9, 1)})
    e2e_ms = statistics.median(wd["ms_per_step"] for wd in windows)
    link_after = link_gbs()
    # one more step with events around every chunk's copies and transform
    tf_, ta_ = [], []
    lp.fwd(fh, dev, out=Rh_out, trace=tf_)
    lp.adj(Rh, dev, out=fh_out, trace=ta_)
    torch.cuda.synchronize()
    timeline = e2e_timeline(tf_, ta_)
    e2e_ms = max_over_ranks(e2e_ms, device=dev)
    e2e = ws * S / (e2e_ms / 1000.0)
    h2d = (f.numel() + R.numel()) * 4
    d2h = h2d
    e2e_ok = bool(torch.equal(Rh_out, Rout.cpu()))

    # roofline of the dominant kernel
    peak, peak_kind = peaks()
    kb = per_kernel_bytes(h, S, prof)
    top = max(prof.items(), key=lambda kv: kv[1][0])
    name, (tms, nl) = top
    per_launch_ms = tms / max(nl, 1)
    per_launch_bytes = kb[name]
    achieved = per_launch_bytes / (per_launch_ms / 1000.0) / 1e9
    # the theta convolution is transform-bound, not byte-bound: its FP32 rate by the usual
    # FFT count (5 L log2 L per transform, two per rho frequency, and the complex product)
    # against the FP32 FMA peak at the sampled maximum SM clock (152 SMs x 128 lanes x 2)
    fft = None
    if name == "theta_conv":
        Lt = h.Ntheta
        gflop = S * (h.Nrho // 2 + 1) * (2 * 5 * Lt * math.log2(Lt) + 6 * Lt) / 1e9
        clk_max = clk.summary().get("sm_max_mhz") or 2070.0
        peak_tf = 152 * 128 * 2 * clk_max * 1e6 / 1e12
        fft = {"gflop_per_launch": round(gflop, 2), "tflops": round(gflop / per_launch_ms, 2),
               "fp32_peak_tflops": round(peak_tf, 1), "frac": round(gflop / per_launch_ms / peak_tf, 3)}
    kernels = {k: {"ms_total": round(v[0], 3), "launches": v[1],
                   "share": round(v[0] / max(sum(x[0] for x in prof.values()), 1e-9), 4)}
               for k, v in prof.items() if v[1]}
    step_gbs = ALGO_BYTES_PER_SLICE * S / (ms_step / 1000.0) / 1e9

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic random-ellipse phantoms (30 ellipses, seed 3), 1% Gaussian noise on the adjoint input",
            "config": {"workload": "fwd+adj batch: %d slices N=%d Nproj=%d cubic %s" % (S, N, Nproj, W["filter"]),
                       "slices": S, "N": N, "Nproj": Nproj, "parallelism": "replicas" if ws > 1 else "single",
                       "l2": "inputs larger than L2 (%.1f GB per step)" % (S * (N * N + Nproj * N) * 4 / 1e9),
                       "precompute_s": round(t_pre, 2), "schedule": sched, "autotune_s": round(t_tune, 2)},
            "plain_value": plain, "batched_over_plain": value / plain / ws,
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "matches_device_result": e2e_ok, "windows": windows, "link_gbs_after": link_after,
                    "timeline": timeline},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind,
                         "traffic": (NCU_DRAM_BYTES_PER_SLICE[name] * S
                                     if (N, Nproj) == (2048, 3000) and name in NCU_DRAM_BYTES_PER_SLICE else None),
                         "traffic_source": "ncu dram__bytes_read+write, 8-slice capture scaled to the launch's slices",
                         "algorithmic_bytes_per_launch": per_launch_bytes, "ms_per_launch": per_launch_ms,
                         "fp32": fft},
            "step_roofline": {"algorithmic_bytes_per_slice": ALGO_BYTES_PER_SLICE, "achieved": step_gbs,
                              "peak": peak, "frac": step_gbs / peak},
            "kernels": kernels,
            "clocks": clk.summary()}
    if rank == 0 and not args.no_uneven and not args.small:
        line["uneven_batch"] = run_uneven(torch, dev, max(2, args.steps // 2))
    if rank == 0 and not args.no_side and not args.small:
        line.update(run_side_configs(torch, dev))
    if rank == 0 and not args.no_cpu and not args.small:
        line["rel_l2_vs_fp64"] = rel_l2_vs_fp64(torch, dev, cpu_plan()[0])
    if rank == 0 and not args.no_cpu:
        nproc, B = cpu_plan()
        packed = lp.tables()
        v, busy = cpu_baseline(packed, nproc, 3, B)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": nproc, "kind": "port",
                                "sample": "3 steps of %d slice(s) fwd+adj N=%d (%.1f s), float64 oracle, slice "
                                          "preparation and spans as jobs in %d processes" % (B, N, busy, nproc)}
        if not args.small:
            line["cpu_baseline"]["single_process"] = cpu_side_configs()
    if dist:
        tdist.barrier()
        tdist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line))


def run_report(args):
    """Precision and differentiation report (float64 oracle comparisons)."""
    import torch
    sys.path.insert(0, ROOT)
    from oracle import lprec_oracle as O
    from lprec_gb300.lpTransform import lpTransform
    from lprec_gb300 import lpmethods
    from lprec_gb300.autograd import radon
    rep = {}

    def rel(a, b):
        return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))

    # (1) N=2048, Nproj=3000: fwd, adj, FBP against the float64 oracle (float64 tables, unrounded)
    N, Nproj = 2048, 3000
    rng = np.random.default_rng(3)
    f = O.ellipse_phantom(N, 30, rng)[None]
    t0 = time.perf_counter()
    tr64 = O.Transform(N, Nproj, 1, "shepp-logan", N / 2, "cubic", mode="fp64", rounded=False)
    R64 = tr64.fwd(f)
    Rn = R64 + 0.01 * np.abs(R64).max() * rng.standard_normal(R64.shape)
    fbp64 = tr64.adj(Rn)
    tr64n = O.Transform(N, Nproj, 1, "none", N / 2, "cubic", mode="fp64", rounded=False)
    adj64 = tr64n.adj(Rn)
    t_oracle = time.perf_counter() - t0
    for prec in ("fp64", "reference"):
        out = {}
        for filt, ref in (("shepp-logan", fbp64), ("none", adj64)):
            lp = lpTransform(N, Nproj, 1, filt, N / 2, "cubic", precision=prec)
            lp.precompute(1)
            lp.initcmem(1, 0)
            if filt == "none":
                out["fwd"] = rel(lp.fwd(np.float32(f)), R64)
                out["adj"] = rel(lp.adj(np.float32(Rn)), ref)
            else:
                out["fbp"] = rel(lp.adj(np.float32(Rn)), ref)
            lp.close()
        rep["n2048_vs_fp64_oracle_tables_" + prec] = out
    rep["n2048_oracle_seconds"] = round(t_oracle, 1)

    # (2) N=512: CG x30 and EM x30 against float64 oracle solvers
    N, Nproj = 512, 768
    rng = np.random.default_rng(3)
    f = O.ellipse_phantom(N, 30, rng)[None]
    tr = O.Transform(N, Nproj, 1, "none", N / 2, "cubic", mode="fp64", rounded=False)
    R = tr.fwd(f)
    Rn = R + 0.01 * np.abs(R).max() * rng.standard_normal(R.shape)
    lp = lpTransform(N, Nproj, 1, "none", N / 2, "cubic")
    lp.precompute(1)
    lp.initcmem(1, 0)
    z = np.zeros((1, N, N), np.float32)
    rep["n512_cg30_vs_fp64_oracle"] = rel(lpmethods.cg(lp, z, np.float32(Rn), 30, 0, 0),
                                          O.solve_cg(tr, z.astype(np.float64), Rn, 30))
    Rp = np.abs(Rn)
    rep["n512_em30_vs_fp64_oracle"] = rel(lpmethods.em(lp, z + 1e-3, np.float32(Rp), 30, 0.01, 0),
                                          O.solve_em(tr, z.astype(np.float64) + 1e-3, Rp, 30, 0.01))

    # (3) differentiation, N=512, Nproj=768, 16 slices, Poisson data at 1e4 photons/ray
    S = 16
    rng = np.random.default_rng(2)
    ph = np.stack([O.ellipse_phantom(N, 10, rng) for _ in range(S)]).astype(np.float32)
    lp16 = lpTransform(N, Nproj, S, "none", N / 2, "cubic")
    lp16.precompute(1)
    lp16.initcmem(1, 0)
    Rt = torch.zeros((S, Nproj, N), device="cuda")
    lp16.fwdp(Rt, torch.as_tensor(ph).cuda(), 0)
    P = Rt.cpu().double().numpy()
    scale = 3.0 / P.max()          # attenuation scaled so that the largest line integral is 3
    P = P * scale
    counts = rng.poisson(1e4 * np.exp(-P))
    data = np.float32(-np.log(np.maximum(counts, 1) / 1e4))
    x0 = torch.zeros((S, N, N), device="cuda", requires_grad=True)
    y = torch.as_tensor(data).cuda()
    loss = 0.5 * ((radon(x0 + torch.as_tensor(ph).cuda() * 0.5, lp16, 0) - y) ** 2).sum()
    loss.backward()
    grad = x0.grad.cpu().double().numpy()
    # finite differences with the float64 oracle on 2 slices (same float32 tables)
    tr2 = O.Transform.from_packed(*lp16.tables())
    xx = ph[:2].astype(np.float64) * 0.5

    def L(v):
        return 0.5 * np.sum((tr2.fwd(v) - data[:2]) ** 2)
    errs = []
    drng = np.random.default_rng(7)
    for i in range(8):
        d = drng.standard_normal(xx.shape)
        fd = (L(xx + 1e-3 * d) - L(xx - 1e-3 * d)) / 2e-3
        errs.append(abs(fd - np.sum(grad[:2] * d)) / np.linalg.norm(grad[:2]))
    rep["grad_fd_max_err_over_norm"] = float(max(errs))
    # the reference's adjoint as a gradient: R_adj(R f - y) vs the exact transpose
    resid = torch.zeros((S, Nproj, N), device="cuda")
    lp16.fwdp(resid, torch.as_tensor(ph * 0.5).cuda(), 0)
    resid -= y
    gadj = torch.zeros((S, N, N), device="cuda")
    lp16.adjp(gadj, resid, 0)
    rep["grad_vs_reference_adj_rel_l2"] = rel(gadj.cpu().numpy(), grad)
    # dot test
    fr = np.random.default_rng(0).random((S, N, N), dtype=np.float32)
    gr = np.random.default_rng(1).random((S, Nproj, N), dtype=np.float32)
    Rf = torch.zeros((S, Nproj, N), device="cuda")
    lp16.fwdp(Rf, torch.as_tensor(fr).cuda(), 0)
    fT = torch.zeros((S, N, N), device="cuda")
    lp16.fwdp_T(fT, torch.as_tensor(gr).cuda(), 0)
    lhs = float(np.sum(Rf.cpu().double().numpy() * gr))
    rhs = float(np.sum(fr.astype(np.float64) * fT.cpu().double().numpy()))
    rep["dot_test_exact_transpose"] = abs(lhs - rhs) / abs(lhs)
    Ra = torch.zeros((S, N, N), device="cuda")
    lp16.adjp(Ra, torch.as_tensor(gr).cuda(), 0)
    rhs2 = float(np.sum(fr.astype(np.float64) * Ra.cpu().double().numpy()))
    rep["dot_test_reference_adj"] = abs(lhs - rhs2) / abs(lhs)
    # CG x50 (exact normal equations) and TV gradient descent x100 (lambda 1e-3)
    z = np.zeros((S, N, N), np.float32)

    def resid_norm(x):
        Rx = torch.zeros((S, Nproj, N), device="cuda")
        lp16.fwdp(Rx, torch.as_tensor(x).cuda(), 0)
        return float(torch.linalg.vector_norm((Rx - y).double()) / torch.linalg.vector_norm(y.double()))
    # one untimed call of each first: torch's own kernels load on first use
    lpmethods.cg_exact(lp16, z, data, 1, 0, 0)
    lpmethods.tv_gd(lp16, z, data, 1, 1e-3, 0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    xc = lpmethods.cg_exact(lp16, z, data, 50, 0, 0)
    t_cg = time.perf_counter() - t0
    t0 = time.perf_counter()
    xt = lpmethods.tv_gd(lp16, z, data, 100, 1e-3, 0)
    t_tv = time.perf_counter() - t0
    rep["cg50_exact"] = {"relative_residual": resid_norm(xc), "seconds": round(t_cg, 2),
                         "rel_l2_to_phantom": rel(xc, ph * scale)}
    rep["tv_gd100"] = {"relative_residual": resid_norm(xt), "seconds": round(t_tv, 2),
                       "rel_l2_to_phantom": rel(xt, ph * scale)}
    rep["solve_n2048_s128"] = run_large_solve(torch, 0)
    print(json.dumps(rep))


def run_large_solve(torch, dev):
    """128 slices, N=2048, Nproj=3000, 30-ellipse phantoms (seed 3), 1 % Gaussian noise:
    FBP (shepp-logan), then 30 CG and 30 EM iterations (unfiltered adjoint) on the GPU,
    timed with CUDA events; the results come back to the host inside the timing.  Also
    30 TV iterations, timed separately."""
    from lprec_gb300.lpTransform import lpTransform
    from lprec_gb300 import lpmethods
    N, Nproj, S = 2048, 3000, 128
    lpf = lpTransform(N, Nproj, S, "shepp-logan", N / 2, "cubic")
    lpf.precompute(1)
    lpf.initcmem(1, dev)
    lpn = lpTransform(N, Nproj, S, "none", N / 2, "cubic")
    lpn.precompute(1)
    lpn.initcmem(1, dev)
    lpf.autotune(dev)
    lpn.autotune(dev)
    f = phantoms_gpu(torch, N, S, 30, 3, dev)
    R = torch.empty((S, Nproj, N), device=dev)
    lpn.fwdp(R, f, dev)
    gen = torch.Generator(device=dev).manual_seed(3)
    R += 0.01 * float(R.abs().max()) * torch.randn(R.shape, device=dev, generator=gen)
    x0 = torch.zeros_like(f)

    def timed(fn):
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        out = fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b), out
    lpmethods.cg(lpn, x0, R, 1, 0, dev)      # warm-up
    t_fbp, _ = timed(lambda: lpmethods.fbp(lpf, x0, R, 0, 0, dev))
    t_cg, xc = timed(lambda: lpmethods.cg(lpn, x0, R, 30, 0, dev))
    Rp = R.abs()
    t_em, xe = timed(lambda: lpmethods.em(lpn, x0 + 1e-3, Rp, 30, 0.01, dev))
    total = t_fbp + t_cg + t_em
    # not part of the FBP+CG+EM sequence: 30 TV iterations (lambda 1e-3) on the same data
    t_tv, xt = timed(lambda: lpmethods.tv(lpn, x0, R, 30, 1e-3, dev))
    return {"fbp_ms": t_fbp, "cg30_ms": t_cg, "em30_ms": t_em, "total_ms": total,
            "slices_per_s": S / (total / 1000.0),
            "cg_ms_per_iteration": t_cg / 30, "em_ms_per_iteration": t_em / 30,
            "tv30_ms": t_tv, "tv_ms_per_iteration": t_tv / 30,
            "finite": bool(np.isfinite(xc).all() and np.isfinite(xe).all() and np.isfinite(xt).all())}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--small", action="store_true", help="N=256 smoke-size workload")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--slices", type=int, default=0, help="batch size (default 128); for profiling runs")
    ap.add_argument("--no-uneven", action="store_true", help="skip the uneven-geometry graph batch")
    ap.add_argument("--report", action="store_true", help="precision / differentiation report instead of timing")
    ap.add_argument("--no-tune", action="store_true", help="keep the default schedule (no autotuner)")
    ap.add_argument("--no-side", action="store_true", help="skip the N=1024 batch and N=256 single-slice lines")
    args = ap.parse_args()
    if args.report:
        run_report(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
