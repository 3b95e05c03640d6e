"""Drop-in for lprec's operator facade (src/lprec/lpTransform.py:9-50).

    lp = lpTransform(N, Nproj, Nslices, filter_type, cor, interp_type)
    lp.precompute(flg)        # packed parameter arrays, as create_gl/create_fwd/create_adj
    lp.initcmem(flg, gpu)     # one native handle per GPU id (up to 16)
    lp.fwdp(R, f, gpu)        # device tensors: R[S0,Nproj,N] <- Radon(f[S0,N,N])
    lp.adjp(f, R, gpu)        # f[S0,N,N] <- back-projection of (filtered) R

Device arrays are CUDA tensors (torch) or anything exposing
``__cuda_array_interface__``; they must be C-contiguous float32 on device
``gpu``.  Outputs are written in place.  ``fwd``/``adj`` are host-array
(NumPy in, NumPy out) conveniences that do not exist in the reference.

``precision`` selects how the tables are evaluated.  'reference' (the default)
repeats lprec's own float32 precompute steps (initsgl.py, initsfwd.py,
initsadj.py), so a caller switching from lprec gets lprec's discretisation at
lprec's precision: the same index sets, and outputs within a few 1e-6 of those
computed from lprec's own tables.  'fp64' evaluates every table value in
float64 and keeps it (the precision form): the outputs then sit about 1e-7 from
a float64 evaluation of the same discretisation, while lprec's float32 tables
sit about 3e-4 from it at N=2048.

Differences from the reference, by design: errors raise ``LprecError`` instead
of printing and resetting the device (src/cuda/callerr.cu:3-8); work is
enqueued on the current torch stream of the device; ``filter_type`` None or
'None' means no filter (the reference raises for 'None', initsadj.py:107).
"""
import numpy as np

from . import _lib

FILTERS = ("none", "ramp", "shepp-logan", "cosine", "cosine2", "hamming", "hann", "parzen")


def _norm_filter(filter_type):
    if filter_type is None or str(filter_type).lower() == "none":
        return "none"
    if filter_type not in FILTERS:
        raise ValueError("unknown filter_type %r (one of %s)" % (filter_type, ", ".join(FILTERS)))
    return filter_type


def _dev_ptr(a):
    """(pointer, shape, device, stream) of a CUDA array-like; float32 C-contiguous required.

    For torch tensors the stream is None (work is enqueued on torch's current
    stream, which orders it after the tensor's producers).  For arrays exposing
    ``__cuda_array_interface__`` the device is the one the pointer's memory
    belongs to, and the stream is the interface's ``stream`` entry (None when
    the producer asks for no ordering; 1 and 2 are the legacy and per-thread
    default streams)."""
    try:
        import torch
        if isinstance(a, torch.Tensor):
            if not a.is_cuda:
                raise ValueError("expected a CUDA tensor")
            if a.dtype != torch.float32:
                raise ValueError("expected float32, got %s" % a.dtype)
            if not a.is_contiguous():
                raise ValueError("expected a C-contiguous tensor")
            return a.data_ptr(), tuple(a.shape), a.device.index, None
    except ImportError:
        pass
    iface = getattr(a, "__cuda_array_interface__", None)
    if iface is None:
        raise TypeError("expected a CUDA array (torch tensor or __cuda_array_interface__)")
    if np.dtype(iface["typestr"]) != np.float32:
        raise ValueError("expected float32")
    shape = tuple(iface["shape"])
    if iface.get("strides") is not None:
        want = tuple(int(np.prod(shape[i + 1:])) * 4 for i in range(len(shape)))
        if tuple(iface["strides"]) != want:
            raise ValueError("expected a C-contiguous array")
    ptr = int(iface["data"][0])
    dev = _lib.pointer_device(ptr) if ptr else None
    return ptr, shape, dev, iface.get("stream")


def _check_arrays(name, gpu, *arrs):
    """Raise unless every array lives on device `gpu`; order the launch stream after the
    streams that __cuda_array_interface__ producers named."""
    for _, _, d, _ in arrs:
        if d is not None and d != gpu:
            raise ValueError("%s: arrays live on cuda:%d, handle on cuda:%d" % (name, d, gpu))
    cur = None
    for _, _, _, st in arrs:
        if st is not None:
            if cur is None:
                cur = _stream(gpu)
            if int(st) != int(cur or 0):
                _lib.stream_wait(gpu, cur, int(st))


def _stream(gpu):
    import torch
    return torch.cuda.current_stream(gpu).cuda_stream


def pipeline_chunks(S, c):
    """Slice counts of the host pipeline's chunks for S slices and chunk size c.

    The first host->device copy and the last device->host copy of a call are not
    overlapped with any transform, and a chunk's device->host copy must finish
    within the next chunk's transform (the forward's output is about 1.5x its
    input).  So the chunks grow from c/16 by doubling, stay at c, and shrink by
    0.7 per chunk at the end: short exposed copies at both ends, no copy backlog
    in the tail.  Each chunk costs about 0.1 ms of launch tails at N=2048, which
    bounds how fine the ramps are."""
    if S < 1 or c < 1:
        raise ValueError("need S >= 1 and c >= 1")
    budget = S
    head = []
    u = max(1, c // 16)
    while u < c and 2 * u <= budget:
        head.append(u)
        budget -= u
        u *= 2
    tail = []
    t = int(c * 0.7)
    while t >= 1:
        if t <= budget:
            tail.append(t)
            budget -= t
        t = int(t * 0.7)
    mid = [c] * (budget // c) + ([budget % c] if budget % c else [])
    return head + sorted(mid + tail, reverse=True)


class lpTransform:
    def __init__(self, N, Nproj, Nslices, filter_type, cor, interp_type, precision="reference"):
        if precision not in ("reference", "fp64"):
            raise ValueError("precision must be 'reference' or 'fp64', got %r" % (precision,))
        self.N = int(N)
        self.Nslices = int(Nslices)
        self.filter_type = _norm_filter(filter_type)
        self.cor = cor
        self.Nproj = int(Nproj)
        self.interp_type = interp_type
        self.precision = precision
        self.clphandle = [None] * 16
        self.fwdparsi = self.fwdparamsf = None

    # ---- precompute / init (lpTransform.py:19-40) -------------------------
    def precompute(self, flg):
        """Parameters for the lp method (fwd ones too when flg), as packed arrays.

        With precision 'fp64' the float arrays are computed and kept in float64
        (the handle then stores interpolation coordinates with ~60x less rounding
        than the float32 format); `fwdparamsf`/`adjparamsf` hold their float32
        rounding, the reference's packed format."""
        wide = self.precision == "fp64"
        (self.glpars, self.fwdparsi, ff, self.adjparsi, af) = _lib.precompute(
            self.N, self.Nproj, self.Nslices, self.cor, self.interp_type, self.filter_type, self.precision,
            with_fwd=bool(flg), wide=wide)
        self._wide = (ff, af) if wide else None
        self.fwdparamsf = None if ff is None else ff.astype(np.float32)
        self.adjparamsf = af.astype(np.float32)

    def load_packed(self, glpars, fwdparsi, fwdparamsf, adjparsi, adjparamsf):
        """Use packed arrays made elsewhere (e.g. by the reference's own precompute);
        float64 float arrays are kept as the handle's tables."""
        self.glpars = np.asarray(glpars, np.float32)
        self.fwdparsi = None if fwdparsi is None else np.asarray(fwdparsi, np.int32)
        self.adjparsi = np.asarray(adjparsi, np.int32)
        wide = np.asarray(adjparamsf).dtype == np.float64
        self._wide = (None if fwdparamsf is None else np.asarray(fwdparamsf, np.float64),
                      np.asarray(adjparamsf, np.float64)) if wide else None
        self.fwdparamsf = None if fwdparamsf is None else np.asarray(fwdparamsf, np.float32)
        self.adjparamsf = np.asarray(adjparamsf, np.float32)

    def tables(self):
        """(glpars, fwdparsi, fwdparamsf, adjparsi, adjparamsf) as the handle receives them
        (float64 float arrays with precision 'fp64')."""
        ff, af = self._wide if getattr(self, "_wide", None) is not None else (self.fwdparamsf, self.adjparamsf)
        return self.glpars, self.fwdparsi, ff, self.adjparsi, af

    def initcmem(self, flg, gpu):
        """Create the native handle for device `gpu` and upload the tables."""
        h = _lib.Handle(self.glpars, gpu)
        _, fi, ff, ai, af = self.tables()
        if flg:
            if fi is None:
                raise RuntimeError("precompute(1) is needed before initcmem(1, gpu)")
            h.init_fwd(fi, ff)
        h.init_adj(ai, af)
        old = self.clphandle[gpu]
        self.clphandle[gpu] = h
        if old is not None:
            old.close()

    def _handle(self, gpu):
        h = self.clphandle[gpu]
        if h is None:
            raise RuntimeError("initcmem(flg, %d) has not been called" % gpu)
        return h

    # ---- transforms on device arrays (lpTransform.py:42-50) ---------------
    def fwdp(self, R, f, gpu):
        h = self._handle(gpu)
        fa, Ra = _dev_ptr(f), _dev_ptr(R)
        fs, Rs = fa[1], Ra[1]
        S0 = fs[0]
        if fs[1:] != (h.N0, h.N0) or Rs != (S0, h.Nproj, h.N0):
            raise ValueError("fwdp: f must be [S0,%d,%d] and R [S0,%d,%d]; got %s, %s"
                             % (h.N0, h.N0, h.Nproj, h.N0, fs, Rs))
        _check_arrays("fwdp", gpu, fa, Ra)
        h.fwd(Ra[0], fa[0], S0, _stream(gpu))

    def adjp(self, f, R, gpu):
        h = self._handle(gpu)
        fa, Ra = _dev_ptr(f), _dev_ptr(R)
        fs, Rs = fa[1], Ra[1]
        S0 = Rs[0]
        if Rs[1:] != (h.Nproj, h.N0) or fs != (S0, h.N0, h.N0):
            raise ValueError("adjp: R must be [S0,%d,%d] and f [S0,%d,%d]; got %s, %s"
                             % (h.Nproj, h.N0, h.N0, h.N0, Rs, fs))
        _check_arrays("adjp", gpu, fa, Ra)
        h.adj(fa[0], Ra[0], S0, _stream(gpu))

    def fwdp_T(self, f, R, gpu):
        """Exact transpose of fwdp: f[S0,N0,N0] <- Radon^T(R[S0,Nproj,N0]) (autograd backward)."""
        h = self._handle(gpu)
        fa, Ra = _dev_ptr(f), _dev_ptr(R)
        fs, Rs = fa[1], Ra[1]
        S0 = Rs[0]
        if Rs[1:] != (h.Nproj, h.N0) or fs != (S0, h.N0, h.N0):
            raise ValueError("fwdp_T: R must be [S0,%d,%d] and f [S0,%d,%d]; got %s, %s"
                             % (h.Nproj, h.N0, h.N0, h.N0, Rs, fs))
        _check_arrays("fwdp_T", gpu, fa, Ra)
        h.fwd_transpose(fa[0], Ra[0], S0, _stream(gpu))

    # ---- batch schedule (not in the reference) ------------------------------
    def autotune(self, gpu, S0=None):
        """Time the candidate batch schedules (slice chunks, one or two streams) of
        fwdp and adjp on S0 slices (default Nslices) of scratch tensors and keep the
        fastest for this handle; returns the chosen schedule."""
        import torch
        h = self._handle(gpu)
        S0 = int(S0 or self.Nslices)
        dev = torch.device("cuda", gpu)
        with torch.cuda.device(gpu):
            f = torch.rand((S0, h.N0, h.N0), device=dev)
            R = torch.rand((S0, h.Nproj, h.N0), device=dev)
            h.autotune(R.data_ptr(), f.data_ptr(), S0, _stream(gpu))
        del f, R
        return h.schedule()

    def set_schedule(self, gpu, **sched):
        """Batch schedule by keyword (fwd_chunk, fwd_streams, fwd_theta_block, adj_chunk,
        adj_streams, adj_theta_block); unnamed entries take their defaults."""
        self._handle(gpu).set_schedule(**sched)

    # ---- host arrays, pipelined ---------------------------------------------
    def _host_op(self, op, x, out, gpu, chunk, trace=None):
        """Run fwdp/adjp over host arrays in slice chunks (pipeline_chunks), overlapping
        the host->device copies of the next chunks and the device->host copies of the
        previous ones with the transform of the current chunk: three streams, three
        device buffers per side, events between them.  The buffers' last-use events
        persist across calls, so calls may be issued back to back.

        `trace`: a list to which one dict of timing events per chunk is appended
        (keys in0/in1 around its host->device copy, c0/c1 around its transform,
        o0/o1 around its device->host copy, and `slices`), for timelines."""
        import torch
        NB = 3  # device buffers per side
        h = self._handle(gpu)
        dev = torch.device("cuda", gpu)
        as_numpy = not isinstance(x, torch.Tensor)
        xt = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32)) if as_numpy else x
        if xt.dtype != torch.float32 or xt.device.type != "cpu":
            raise ValueError("expected a float32 host array")
        xt = xt.contiguous()
        ishape = (h.N0, h.N0) if op == "fwd" else (h.Nproj, h.N0)
        if xt.dim() != 3 or tuple(xt.shape[1:]) != ishape:
            raise ValueError("%s: input must be [S0,%d,%d], got %s" % (op, ishape[0], ishape[1], tuple(xt.shape)))
        S = xt.shape[0]
        oshape = (S, h.Nproj, h.N0) if op == "fwd" else (S, h.N0, h.N0)
        if out is None:
            out = torch.empty(oshape, dtype=torch.float32, pin_memory=torch.cuda.is_available())
        elif not isinstance(out, torch.Tensor):
            raise TypeError("out must be a torch CPU tensor")
        if tuple(out.shape) != oshape:
            raise ValueError("out has shape %s, expected %s" % (tuple(out.shape), oshape))
        c = max(1, min(int(chunk or 32), h.Nslices, S))
        key = (op, gpu, c) + tuple(xt.shape[1:])
        bufs = self._pipe_bufs.get(key) if hasattr(self, "_pipe_bufs") else None
        if bufs is None:
            if not hasattr(self, "_pipe_bufs"):
                self._pipe_bufs = {}
            # device buffers, copy streams, and per buffer the events of its last use
            # (compute done, copy-out done); the events outlive the call, so the next
            # call on the same buffers waits for this one's work in flight
            bufs = ([torch.empty((c,) + tuple(xt.shape[1:]), dtype=torch.float32, device=dev) for _ in range(NB)],
                    [torch.empty((c,) + oshape[1:], dtype=torch.float32, device=dev) for _ in range(NB)],
                    torch.cuda.Stream(dev), torch.cuda.Stream(dev), [None] * NB, [None] * NB, [0])
            self._pipe_bufs[key] = bufs
        ins, outs, s_in, s_out, done_comp, done_out, nxt = bufs
        comp = torch.cuda.current_stream(dev)
        # the copies in read host memory that work already on the caller's stream
        # may write (e.g. the previous call's output)
        s_in.wait_stream(comp)
        sizes = pipeline_chunks(S, c)
        n = len(sizes)
        b = 0
        for i in range(n):
            a, b = b, b + sizes[i]
            k = nxt[0]
            nxt[0] = (k + 1) % NB
            tr = None
            if trace is not None:
                tr = {key: torch.cuda.Event(enable_timing=True) for key in ("in0", "in1", "c0", "c1", "o0", "o1")}
                tr["slices"] = b - a
                trace.append(tr)
            with torch.cuda.stream(s_in):
                if done_comp[k] is not None:
                    s_in.wait_event(done_comp[k])       # buffer's previous chunk consumed
                if tr:
                    tr["in0"].record(s_in)
                ins[k][:b - a].copy_(xt[a:b], non_blocking=True)
                ev_in = tr["in1"] if tr else torch.cuda.Event()
                ev_in.record(s_in)
            comp.wait_event(ev_in)
            if done_out[k] is not None:
                comp.wait_event(done_out[k])            # output buffer drained
            if tr:
                tr["c0"].record(comp)
            if op == "fwd":
                self.fwdp(outs[k][:b - a], ins[k][:b - a], gpu)
            else:
                self.adjp(outs[k][:b - a], ins[k][:b - a], gpu)
            ev_c = tr["c1"] if tr else torch.cuda.Event()
            ev_c.record(comp)
            done_comp[k] = ev_c
            with torch.cuda.stream(s_out):
                s_out.wait_event(ev_c)
                if tr:
                    tr["o0"].record(s_out)
                out[a:b].copy_(outs[k][:b - a], non_blocking=True)
                ev_o = tr["o1"] if tr else torch.cuda.Event()
                ev_o.record(s_out)
            done_out[k] = ev_o
        comp.wait_event(done_out[(nxt[0] - 1) % NB])   # the copies out run in order
        if as_numpy:
            torch.cuda.current_stream(dev).synchronize()
            return out.numpy()
        return out

    def fwd(self, f, gpu=0, out=None, chunk=None, trace=None):
        """Forward transform of host images f[S,N0,N0] -> host sinograms.  With torch
        CPU tensors the result is enqueued on the current stream (synchronise before
        reading it); NumPy input returns a NumPy array after synchronising."""
        return self._host_op("fwd", f, out, gpu, chunk, trace)

    def adj(self, R, gpu=0, out=None, chunk=None, trace=None):
        """Adjoint / FBP of host sinograms R[S,Nproj,N0] -> host images (see fwd)."""
        return self._host_op("adj", R, out, gpu, chunk, trace)

    def close(self):
        for i, h in enumerate(self.clphandle):
            if h is not None:
                h.close()
                self.clphandle[i] = None
