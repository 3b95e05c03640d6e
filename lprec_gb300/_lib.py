"""ctypes binding of liblprec_gb300.so (the C ABI declared in include/lprec_gb300.h).

The library is built in-tree by ``lprec_gb300.build``; importing this module
loads it and raises if it is missing -- there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblprec_gb300.so")

LP_OK = 0
LP_ERR_ARG = 1
LP_ERR_CUDA = 2
LP_ERR_OOM = 3
LP_ERR_STATE = 4
LP_ERR_UNSUPPORTED = 5
PRECISION = {"reference": 0, "fp64": 1}

# every symbol include/lprec_gb300.h declares
EXPORTS = ("lp_last_error", "lp_version", "lp_precompute_sizes", "lp_precompute", "lp_create", "lp_init_fwd",
           "lp_init_adj", "lp_destroy", "lp_fwd", "lp_adj", "lp_get_geometry", "lp_device_bytes",
           "lp_launch_count", "lp_kernel_count", "lp_kernel_name", "lp_set_profiling", "lp_profile_collect",
           "lp_fwd_noalloc", "lp_noalloc_scratch_bytes", "lp_fwd_transpose", "lp_debug_fill_scratch",
           "lp_set_schedule", "lp_get_schedule", "lp_autotune",
           "lp_precompute_f64", "lp_init_fwd_f64", "lp_init_adj_f64",
           "lp_vec_work_doubles", "lp_vec_dot", "lp_cg_step", "lp_cg_dir", "lp_em_ratio", "lp_em_step",
           "lp_tv_prox0", "lp_tv_prox1", "lp_tv_recon", "lp_debug_fill_noalloc_scratch", "lp_pointer_device",
           "lp_stream_wait")


class LprecError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("lprec_gb300 error %d: %s" % (code, msg))
        self.code = code


_lib = None

c_int, c_int64, c_double, c_void_p, c_char_p = ctypes.c_int, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p, ctypes.c_char_p
P_i32 = ctypes.POINTER(ctypes.c_int32)
P_f32 = ctypes.POINTER(ctypes.c_float)
P_i64 = ctypes.POINTER(ctypes.c_int64)
P_f64 = ctypes.POINTER(ctypes.c_double)


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("liblprec_gb300.so is not built (run `python -m lprec_gb300.build`): %s" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    sig = {
        "lp_last_error": (c_char_p, []),
        "lp_version": (c_int, []),
        "lp_precompute_sizes": (c_int, [c_int, c_int, c_int, c_double, c_int, c_char_p, P_i64]),
        "lp_precompute": (c_int, [c_int, c_int, c_int, c_double, c_int, c_char_p, c_int, c_int, c_int,
                                  P_f32, P_i32, P_f32, P_i32, P_f32]),
        "lp_precompute_f64": (c_int, [c_int, c_int, c_int, c_double, c_int, c_char_p, c_int, c_int, c_int,
                                      P_f32, P_i32, P_f64, P_i32, P_f64]),
        "lp_init_fwd_f64": (c_int, [c_void_p, P_i32, c_int64, P_f64, c_int64]),
        "lp_init_adj_f64": (c_int, [c_void_p, P_i32, c_int64, P_f64, c_int64]),
        "lp_vec_work_doubles": (c_int64, [c_int]),
        "lp_vec_dot": (c_int, [c_void_p, c_void_p, c_int64, c_int, c_void_p, c_void_p, c_void_p]),
        "lp_cg_step": (c_int, [c_void_p] * 4 + [c_int64] + [c_void_p] * 5),
        "lp_cg_dir": (c_int, [c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p]),
        "lp_em_ratio": (c_int, [c_void_p, c_void_p, ctypes.c_float, c_int64, c_void_p]),
        "lp_em_step": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p]),
        "lp_tv_prox0": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_double, c_double, c_void_p]),
        "lp_tv_prox1": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_double, c_int, c_void_p]),
        "lp_tv_recon": (c_int, [c_void_p] * 5 + [c_int, c_int, c_int, c_double, c_void_p]),
        "lp_create": (c_int, [P_f32, c_int64, c_int, ctypes.POINTER(c_void_p)]),
        "lp_init_fwd": (c_int, [c_void_p, P_i32, c_int64, P_f32, c_int64]),
        "lp_init_adj": (c_int, [c_void_p, P_i32, c_int64, P_f32, c_int64]),
        "lp_destroy": (c_int, [c_void_p]),
        "lp_fwd": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
        "lp_adj": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
        "lp_get_geometry": (c_int, [c_void_p, P_i32]),
        "lp_device_bytes": (c_int, [c_void_p, P_i64]),
        "lp_fwd_noalloc": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
        "lp_fwd_transpose": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
        "lp_noalloc_scratch_bytes": (c_int, [c_void_p, c_int, P_i64]),
        "lp_launch_count": (ctypes.c_longlong, []),
        "lp_kernel_count": (c_int, []),
        "lp_kernel_name": (c_char_p, [c_int]),
        "lp_set_profiling": (c_int, [c_void_p, c_int]),
        "lp_profile_collect": (c_int, [c_void_p, ctypes.POINTER(ctypes.c_double), P_i64]),
        "lp_debug_fill_scratch": (c_int, [c_void_p, ctypes.c_float, c_void_p]),
        "lp_set_schedule": (c_int, [c_void_p, P_i32, c_int]),
        "lp_get_schedule": (c_int, [c_void_p, P_i32, c_int]),
        "lp_autotune": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p, P_f32]),
        "lp_debug_fill_noalloc_scratch": (c_int, [c_int, ctypes.c_float, c_void_p]),
        "lp_pointer_device": (c_int, [c_void_p, ctypes.POINTER(c_int)]),
        "lp_stream_wait": (c_int, [c_int, c_void_p, c_void_p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(rc):
    if rc != LP_OK:
        raise LprecError(rc, lib().lp_last_error().decode(errors="replace"))


def _ptr(a, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def pointer_device(ptr):
    """Device id that the memory at device pointer `ptr` belongs to."""
    d = c_int(-1)
    check(lib().lp_pointer_device(c_void_p(ptr), ctypes.byref(d)))
    return d.value


def stream_wait(device, waiter, producer):
    """Make stream `waiter` wait for the work enqueued on stream `producer` so far."""
    check(lib().lp_stream_wait(int(device), c_void_p(waiter), c_void_p(producer)))


def debug_fill_noalloc_scratch(device, value, stream):
    """Test hook: fill the allocation-free scratch array of `device` with `value`."""
    check(lib().lp_debug_fill_noalloc_scratch(int(device), float(value), c_void_p(stream)))


def launch_count():
    return int(lib().lp_launch_count())


def precompute(N0, Nproj, Nslices, cor, interp_type, filter_type, precision="reference", with_fwd=True,
               nthreads=0, wide=False):
    """Host precompute; returns (glpars, fwdparsi, fwdparamsf, adjparsi, adjparamsf).  With
    wide=True the two float arrays are float64 (same layout; for Handle.init_fwd/init_adj)."""
    L = lib()
    cubic = 1 if interp_type == "cubic" else 0
    filt = (filter_type or "none").encode()
    sizes = np.zeros(5, dtype=np.int64)
    check(L.lp_precompute_sizes(int(N0), int(Nproj), int(Nslices), float(cor), cubic, filt, _ptr(sizes, ctypes.c_int64)))
    gl = np.empty(sizes[0], np.float32)
    fi = np.empty(sizes[1] if with_fwd else 1, np.int32)
    ai = np.empty(sizes[3], np.int32)
    if wide:
        ff = np.empty(sizes[2] if with_fwd else 1, np.float64)
        af = np.empty(sizes[4], np.float64)
        fn, ct = L.lp_precompute_f64, ctypes.c_double
    else:
        ff = np.empty(sizes[2] if with_fwd else 1, np.float32)
        af = np.empty(sizes[4], np.float32)
        fn, ct = L.lp_precompute, ctypes.c_float
    check(fn(int(N0), int(Nproj), int(Nslices), float(cor), cubic, filt, PRECISION[precision],
             1 if with_fwd else 0, int(nthreads), _ptr(gl, ctypes.c_float), _ptr(fi, ctypes.c_int32),
             _ptr(ff, ct), _ptr(ai, ctypes.c_int32), _ptr(af, ct)))
    if not with_fwd:
        fi = ff = None
    return gl, fi, ff, ai, af


class Handle:
    """Owner of one lp_handle (one geometry on one device)."""

    def __init__(self, glpars, device=0):
        self._h = None
        L = lib()
        gl = np.ascontiguousarray(glpars, dtype=np.float32)
        h = c_void_p()
        check(L.lp_create(_ptr(gl, ctypes.c_float), gl.size, int(device), ctypes.byref(h)))
        self._h = h
        self.device = int(device)
        g = np.zeros(10, np.int32)
        check(L.lp_get_geometry(h, _ptr(g, ctypes.c_int32)))
        (self.N, self.N0, self.Ntheta, self.Nrho, self.Nproj_int, self.Nproj, self.Nslices, self.cor,
         self.osangles, self.cubic) = [int(x) for x in g]
        self.has_fwd = False
        self.has_adj = False

    @staticmethod
    def _parsf(parsf):
        """float64 arrays go to the *_f64 entry points, anything else as float32."""
        if np.asarray(parsf).dtype == np.float64:
            return np.ascontiguousarray(parsf), ctypes.c_double, "_f64"
        return np.ascontiguousarray(parsf, dtype=np.float32), ctypes.c_float, ""

    def init_fwd(self, parsi, parsf):
        pi = np.ascontiguousarray(parsi, dtype=np.int32)
        pf, ct, sfx = self._parsf(parsf)
        fn = getattr(lib(), "lp_init_fwd" + sfx)
        check(fn(self._h, _ptr(pi, ctypes.c_int32), pi.size, _ptr(pf, ct), pf.size))
        self.has_fwd = True

    def init_adj(self, parsi, parsf):
        pi = np.ascontiguousarray(parsi, dtype=np.int32)
        pf, ct, sfx = self._parsf(parsf)
        fn = getattr(lib(), "lp_init_adj" + sfx)
        check(fn(self._h, _ptr(pi, ctypes.c_int32), pi.size, _ptr(pf, ct), pf.size))
        self.has_adj = True

    def fwd(self, R_ptr, f_ptr, S0, stream):
        check(lib().lp_fwd(self._h, c_void_p(R_ptr), c_void_p(f_ptr), int(S0), c_void_p(stream)))

    def adj(self, f_ptr, R_ptr, S0, stream):
        check(lib().lp_adj(self._h, c_void_p(f_ptr), c_void_p(R_ptr), int(S0), c_void_p(stream)))

    def fwd_transpose(self, f_ptr, R_ptr, S0, stream):
        check(lib().lp_fwd_transpose(self._h, c_void_p(f_ptr), c_void_p(R_ptr), int(S0), c_void_p(stream)))

    def fwd_noalloc(self, R_ptr, f_ptr, S0, stream):
        check(lib().lp_fwd_noalloc(self._h, c_void_p(R_ptr), c_void_p(f_ptr), int(S0), c_void_p(stream)))

    def noalloc_scratch_bytes(self, S0):
        b = np.zeros(1, np.int64)
        check(lib().lp_noalloc_scratch_bytes(self._h, int(S0), _ptr(b, ctypes.c_int64)))
        return int(b[0])

    def device_bytes(self):
        b = np.zeros(1, np.int64)
        check(lib().lp_device_bytes(self._h, _ptr(b, ctypes.c_int64)))
        return int(b[0])

    SCHEDULE_KEYS = ("fwd_chunk", "fwd_streams", "fwd_theta_block", "adj_chunk", "adj_streams", "adj_theta_block")

    def set_schedule(self, fwd_chunk=0, fwd_streams=1, fwd_theta_block=256, adj_chunk=0, adj_streams=1,
                     adj_theta_block=256):
        v = np.array([fwd_chunk, fwd_streams, fwd_theta_block, adj_chunk, adj_streams, adj_theta_block], np.int32)
        check(lib().lp_set_schedule(self._h, _ptr(v, ctypes.c_int32), len(v)))

    def schedule(self):
        out = np.zeros(len(self.SCHEDULE_KEYS), np.int32)
        check(lib().lp_get_schedule(self._h, _ptr(out, ctypes.c_int32), len(out)))
        return dict(zip(self.SCHEDULE_KEYS, (int(x) for x in out)))

    def autotune(self, R, f, S0, stream):
        """Pick the fastest batch schedule on S0 slices of the device buffers R, f (overwritten)."""
        ms = np.zeros(2, np.float32)
        check(lib().lp_autotune(self._h, R, f, int(S0), stream, _ptr(ms, ctypes.c_float)))
        return float(ms[0]), float(ms[1])

    def debug_fill_scratch(self, value, stream):
        """Fill the intermediate buffers with `value` (test hook: results must not change)."""
        check(lib().lp_debug_fill_scratch(self._h, float(value), stream))

    def set_profiling(self, on):
        check(lib().lp_set_profiling(self._h, 1 if on else 0))

    def profile(self):
        """{kernel name: (total ms, launches)} of the launches recorded since the last call."""
        L = lib()
        n = L.lp_kernel_count()
        ms = np.zeros(n, np.float64)
        cnt = np.zeros(n, np.int64)
        check(L.lp_profile_collect(self._h, _ptr(ms, ctypes.c_double), _ptr(cnt, ctypes.c_int64)))
        return {L.lp_kernel_name(i).decode(): (float(ms[i]), int(cnt[i])) for i in range(n)}

    def close(self):
        if self._h is not None and _lib is not None:
            _lib.lp_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- fused solver vector kernels (device pointers; see include/lprec_gb300.h) ----
def vec_work_doubles(S=1):
    return int(lib().lp_vec_work_doubles(int(S)))


def vec_dot(a, b, m, S, work, out, stream):
    check(lib().lp_vec_dot(c_void_p(a), c_void_p(b), int(m), int(S), c_void_p(work), c_void_p(out),
                           c_void_p(stream)))


def cg_step(x, r, p, q, n, num, den, work, rr, stream):
    check(lib().lp_cg_step(c_void_p(x), c_void_p(r), c_void_p(p), c_void_p(q), int(n), c_void_p(num),
                           c_void_p(den), c_void_p(work), c_void_p(rr), c_void_p(stream)))


def cg_dir(p, r, n, num, den, stream):
    check(lib().lp_cg_dir(c_void_p(p), c_void_p(r), int(n), c_void_p(num), c_void_p(den), c_void_p(stream)))


def em_ratio(g, tomo, eps, n, stream):
    check(lib().lp_em_ratio(c_void_p(g), c_void_p(tomo), float(eps), int(n), c_void_p(stream)))


def em_step(x, upd, xi, n, stream):
    check(lib().lp_em_step(c_void_p(x), c_void_p(upd), c_void_p(xi), int(n), c_void_p(stream)))


TV_MODES = {"tv": 0, "tve": 1, "tvl1": 2}  # LP_TV_L2, LP_TV_ENTROPY, LP_TV_L1


def tv_prox0(prox0x, prox0y, recon, S, ny, nx, c, lam, stream):
    check(lib().lp_tv_prox0(c_void_p(prox0x), c_void_p(prox0y), c_void_p(recon), int(S), int(ny), int(nx),
                            float(c), float(lam), c_void_p(stream)))


def tv_prox1(prox1, g, tomo, n, c, mode, stream):
    check(lib().lp_tv_prox1(c_void_p(prox1), c_void_p(g), c_void_p(tomo), int(n), float(c), TV_MODES[mode],
                            c_void_p(stream)))


def tv_recon(recon0, recon, p, prox0x, prox0y, S, ny, nx, c, stream):
    check(lib().lp_tv_recon(c_void_p(recon0), c_void_p(recon), c_void_p(p), c_void_p(prox0x), c_void_p(prox0y),
                            int(S), int(ny), int(nx), float(c), c_void_p(stream)))
