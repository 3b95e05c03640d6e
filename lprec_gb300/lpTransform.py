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
    """(pointer, shape, device) of a CUDA array-like; float32 C-contiguous required."""
    try:
        import torch
        if isinstance(a, torch.Tensor):
            if not a.is_cuda:
                raise ValueError("expected a CUDA tensor")
            if a.dtype != torch.float32:
                raise ValueError("expected float32, got %s" % a.dtype)
            if not a.is_contiguous():
                raise ValueError("expected a C-contiguous tensor")
            return a.data_ptr(), tuple(a.shape), a.device.index
    except ImportError:
        pass
    iface = getattr(a, "__cuda_array_interface__", None)
    if iface is None:
        raise TypeError("expected a CUDA array (torch tensor or __cuda_array_interface__)")
    if np.dtype(iface["typestr"]) != np.float32:
        raise ValueError("expected float32")
    if iface.get("strides") not in (None,):
        shape = iface["shape"]
        want = tuple(int(np.prod(shape[i + 1:])) * 4 for i in range(len(shape)))
        if tuple(iface["strides"]) != want:
            raise ValueError("expected a C-contiguous array")
    return iface["data"][0], tuple(iface["shape"]), None


def _stream(gpu):
    import torch
    return torch.cuda.current_stream(gpu).cuda_stream


class lpTransform:
    def __init__(self, N, Nproj, Nslices, filter_type, cor, interp_type, precision="fp64"):
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
        """Parameters for the lp method (fwd ones too when flg), as packed arrays."""
        (self.glpars, self.fwdparsi, self.fwdparamsf, self.adjparsi,
         self.adjparamsf) = _lib.precompute(self.N, self.Nproj, self.Nslices, self.cor, self.interp_type,
                                            self.filter_type, self.precision, with_fwd=bool(flg))

    def load_packed(self, glpars, fwdparsi, fwdparamsf, adjparsi, adjparamsf):
        """Use packed arrays made elsewhere (e.g. by the reference's own precompute)."""
        self.glpars = np.asarray(glpars, np.float32)
        self.fwdparsi = None if fwdparsi is None else np.asarray(fwdparsi, np.int32)
        self.fwdparamsf = None if fwdparamsf is None else np.asarray(fwdparamsf, np.float32)
        self.adjparsi = np.asarray(adjparsi, np.int32)
        self.adjparamsf = np.asarray(adjparamsf, np.float32)

    def initcmem(self, flg, gpu):
        """Create the native handle for device `gpu` and upload the tables."""
        h = _lib.Handle(self.glpars, gpu)
        if flg:
            if self.fwdparsi is None:
                raise RuntimeError("precompute(1) is needed before initcmem(1, gpu)")
            h.init_fwd(self.fwdparsi, self.fwdparamsf)
        h.init_adj(self.adjparsi, self.adjparamsf)
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
        fp, fs, fd = _dev_ptr(f)
        Rp, Rs, Rd = _dev_ptr(R)
        S0 = fs[0]
        if fs[1:] != (h.N0, h.N0) or Rs != (S0, h.Nproj, h.N0):
            raise ValueError("fwdp: f must be [S0,%d,%d] and R [S0,%d,%d]; got %s, %s"
                             % (h.N0, h.N0, h.Nproj, h.N0, fs, Rs))
        for d in (fd, Rd):
            if d is not None and d != gpu:
                raise ValueError("fwdp: arrays live on cuda:%d, handle on cuda:%d" % (d, gpu))
        h.fwd(Rp, fp, S0, _stream(gpu))

    def adjp(self, f, R, gpu):
        h = self._handle(gpu)
        fp, fs, fd = _dev_ptr(f)
        Rp, Rs, Rd = _dev_ptr(R)
        S0 = Rs[0]
        if Rs[1:] != (h.Nproj, h.N0) or fs != (S0, h.N0, h.N0):
            raise ValueError("adjp: R must be [S0,%d,%d] and f [S0,%d,%d]; got %s, %s"
                             % (h.Nproj, h.N0, h.N0, h.N0, Rs, fs))
        for d in (fd, Rd):
            if d is not None and d != gpu:
                raise ValueError("adjp: arrays live on cuda:%d, handle on cuda:%d" % (d, gpu))
        h.adj(fp, Rp, S0, _stream(gpu))

    # ---- host-array conveniences -------------------------------------------
    def fwd(self, f, gpu=0):
        import torch
        h = self._handle(gpu)
        ft = torch.as_tensor(np.ascontiguousarray(f, dtype=np.float32)).cuda(gpu)
        R = torch.empty((ft.shape[0], h.Nproj, h.N0), dtype=torch.float32, device=ft.device)
        self.fwdp(R, ft, gpu)
        return R.cpu().numpy()

    def adj(self, R, gpu=0):
        import torch
        h = self._handle(gpu)
        Rt = torch.as_tensor(np.ascontiguousarray(R, dtype=np.float32)).cuda(gpu)
        f = torch.empty((Rt.shape[0], h.N0, h.N0), dtype=torch.float32, device=Rt.device)
        self.adjp(f, Rt, gpu)
        return f.cpu().numpy()

    def close(self):
        for i, h in enumerate(self.clphandle):
            if h is not None:
                h.close()
                self.clphandle[i] = None
