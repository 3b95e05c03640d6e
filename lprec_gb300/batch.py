"""Requests of uneven geometry in one CUDA-graph launch.

    b = UnevenBatch([(N, Nproj, slices), ...], filter_type, interp_type, gpu)
    b.input_f(i)[:] = ...; b.input_R(i)[:] = ...     # device views per request
    b.capture()                                      # fwd + adj of every request in one graph
    b.run()                                          # one graph launch
    b.output_R(i), b.output_f(i)

Requests with the same (N, Nproj) share one native handle whose batch
schedules the autotuner picks for the geometry and each of its wave sizes
(lp_autotune: slice chunks, streams, theta-convolution block), and are
concatenated into one batch,
fewest slices first.  The groups run one after another inside the graph,
smallest geometry first (shortest work first: running them on parallel graph
branches was measured slower, the large groups already fill the GPU and the
branches only compete for L2).  A group runs as one batch, except that the last
group's largest request runs alone after the others (last_alone), so every other
request completes before the launch does; wave_slices bounds a group's batches to
about that many slices' worth of N=2048 work, so requests complete with their wave
rather than with their whole group (lower latency for large requests, at some
throughput).  The graph records an event after each wave, which gives per-request
latencies measured from the start of the launch.
"""
import time

import torch

from .lpTransform import lpTransform


def wait_event(ev, timeout_s, poll_s=0.001, clock=time.monotonic, sleep=time.sleep):
    """Host-side watchdog: poll `ev.query()` until it reports completion or `timeout_s`
    seconds pass; raise TimeoutError in the second case (the GPU work is not cancelled,
    the caller learns of the stall without blocking in a synchronize)."""
    deadline = clock() + timeout_s
    while not ev.query():
        if clock() >= deadline:
            raise TimeoutError("graph launch not finished after %.3f s" % timeout_s)
        sleep(poll_s)


def group_requests(requests):
    """Requests (N, Nproj, slices) grouped by geometry, smallest N first, each group's
    requests fewest slices first.  Returns the groups as (N, Nproj, total slices,
    request indices in batch order) and, per request, its (group, slice offset in the
    group, slices)."""
    requests = [tuple(int(v) for v in r) for r in requests]
    for N, Nproj, S in requests:
        if N < 1 or Nproj < 1 or S < 1:
            raise ValueError("requests need N, Nproj and slices >= 1, got %s" % ((N, Nproj, S),))
    byg = {}
    for i, (N, Nproj, S) in enumerate(requests):
        byg.setdefault((N, Nproj), []).append(i)
    groups, where = [], {}
    for (N, Nproj), idx in sorted(byg.items(), key=lambda kv: kv[0]):
        idx = sorted(idx, key=lambda i: (requests[i][2], i))  # fewest slices first
        off = 0
        for i in idx:
            where[i] = (len(groups), off, requests[i][2])
            off += requests[i][2]
        groups.append((N, Nproj, off, idx))
    return groups, where


def plan_waves(requests, idx, N, wave_slices=None, last_alone=False):
    """Consecutive runs of a group's requests (in batch order) whose slices add up to
    at most wave_slices * (2048 / N)^2 (one request at least; None: no bound):
    [(first slice, end slice, request indices)].  With last_alone, the group's last
    request gets a wave of its own (the others then complete before it)."""
    cap = float("inf") if wave_slices is None else max(1, int(wave_slices * (2048.0 / N) ** 2))
    waves, cur, a, b = [], [], 0, 0
    for i in idx:
        S = requests[i][2]
        if cur and b - a + S > cap:
            waves.append((a, b, cur))
            cur, a = [], b
        cur.append(i)
        b += S
    if cur:
        waves.append((a, b, cur))
    if last_alone and len(waves[-1][2]) > 1:
        a, b, reqs = waves.pop()
        S = requests[reqs[-1]][2]
        waves += [(a, b - S, reqs[:-1]), (b - S, b, reqs[-1:])]
    return waves


class UnevenBatch:
    def __init__(self, requests, filter_type="ramp", interp_type="cubic", gpu=0, precision="reference",
                 wave_slices=None, autotune=True, last_alone=True):
        self.gpu = gpu
        self.dev = torch.device("cuda", gpu)
        self.requests = [tuple(int(v) for v in r) for r in requests]
        plan, self.where = group_requests(self.requests)
        self.groups = []
        for gi, (N, Nproj, total, idx) in enumerate(plan):
            lp = lpTransform(N, Nproj, total, filter_type, N / 2, interp_type, precision)
            lp.precompute(1)
            lp.initcmem(1, gpu)
            waves = plan_waves(self.requests, idx, N, wave_slices, last_alone and gi == len(plan) - 1)
            # one autotuned schedule per wave size of the group, set before each wave's
            # launches (the graph records the launches of the schedule in force)
            scheds = {}
            if autotune:
                for size in sorted({b - a for a, b, _ in waves}):
                    lp.autotune(gpu, size)
                    scheds[size] = lp.clphandle[gpu].schedule()
            g = dict(lp=lp, N=N, Nproj=Nproj, S=total, idx=idx, waves=waves, scheds=scheds,
                     f=torch.zeros((total, N, N), device=self.dev),
                     R=torch.zeros((total, Nproj, N), device=self.dev),
                     Rout=torch.zeros((total, Nproj, N), device=self.dev),
                     fout=torch.zeros((total, N, N), device=self.dev))
            self.groups.append(g)
        self.graph = None

    def _view(self, i, key):
        gi, off, S = self.where[i]
        return self.groups[gi][key][off:off + S]

    def input_f(self, i):
        return self._view(i, "f")

    def input_R(self, i):
        return self._view(i, "R")

    def output_R(self, i):
        return self._view(i, "Rout")

    def output_f(self, i):
        return self._view(i, "fout")

    def _work(self, g, a, b):
        if b - a in g["scheds"]:
            g["lp"].set_schedule(self.gpu, **g["scheds"][b - a])
        g["lp"].fwdp(g["Rout"][a:b], g["f"][a:b], self.gpu)
        g["lp"].adjp(g["fout"][a:b], g["R"][a:b], self.gpu)

    def run_eager(self):
        """The same work without the graph (one wave after the other)."""
        for g in self.groups:
            for a, b, _ in g["waves"]:
                self._work(g, a, b)

    def capture(self):
        main = torch.cuda.Stream(self.dev)
        with torch.cuda.stream(main):
            self.run_eager()  # warm-up outside capture
        torch.cuda.synchronize(self.dev)
        waves = [(g, a, b, reqs) for g in self.groups for a, b, reqs in g["waves"]]
        try:
            self.t_start = torch.cuda.Event(enable_timing=True, external=True)
            self.t_done = [torch.cuda.Event(enable_timing=True, external=True) for _ in waves]
        except TypeError:  # torch without event-record graph nodes: no per-request latencies
            self.t_start = None
            self.t_done = [None for _ in waves]
        self._wave_of = {}
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, stream=main):
            if self.t_start is not None:
                self.t_start.record(main)
            for w, ((g, a, b, reqs), ev) in enumerate(zip(waves, self.t_done)):
                self._work(g, a, b)
                if ev is not None:
                    ev.record(main)
                for i in reqs:
                    self._wave_of[i] = w
        self._main = main

    def run(self, timeout_s=None):
        """One graph launch; with timeout_s, wait for it (host-side watchdog, see wait())."""
        if self.graph is None:
            self.capture()
        self.graph.replay()
        if timeout_s is not None:
            self.wait(timeout_s)

    def wait(self, timeout_s):
        """Wait for the last launch without blocking in cudaDeviceSynchronize; raises
        TimeoutError when it has not finished within timeout_s seconds."""
        ev = torch.cuda.Event()
        ev.record(self._main)
        wait_event(ev, timeout_s)

    def latencies_ms(self):
        """Per-request latency of the last run: start of the launch to its wave's end."""
        torch.cuda.synchronize(self.dev)
        if self.t_start is None:
            return None
        per_wave = [self.t_start.elapsed_time(ev) for ev in self.t_done]
        return [per_wave[self._wave_of[i]] for i in range(len(self.requests))]

    @property
    def slices(self):
        return sum(r[2] for r in self.requests)
