"""Host-array reconstruction in the call form of tomopy's external backends.

lprec's main consumer is tomopy, which reaches it through a wrapper of the form
``lprec(tomo, center, recon, theta, **kwargs)`` (README.rst:32-35 of the
reference).  This module provides that entry on top of lpTransform and lpmethods:

    from lprec_gb300.recon import lprec
    recon = np.zeros((S, N, N), np.float32)
    lprec(tomo, center, recon, theta, lpmethod='cg', num_iter=30, gpu_list=[0])

tomo      [Nslices, Nproj, N] float32 sinograms (sinogram order)
center    rotation axis in detector pixels (N/2 = centred), one value or one per slice
recon     [Nslices, N, N] float32 array, read as the initial guess and overwritten
theta     [Nproj] angles in radians; the log-polar geometry is built for
          theta[k] = k*pi/Nproj (initsgl.py:36), anything else raises ValueError
kwargs    lpmethod   'fbp' (default), 'grad', 'cg', 'em', 'tv', 'tve', 'tvl1'
          filter_name  FBP filter (default 'ramp'); iterative methods use the
                       unfiltered adjoint
          interp_type  'cubic' (default) or 'linear'
          num_iter, reg_par  as in lpmethods (defaults 64 and 0.001)
          gpu_list   devices (default [0]): slices are split into chunks spread over
                     them, one host thread per device
          chunk      slices per transform call (default 32; bounds device memory)
          precision  table precision of lpTransform: 'reference' (default) or 'fp64'

Slices with different centers get separate geometries (one precompute per
distinct center and device).
"""
import threading

import numpy as np

from . import lpmethods
from .lpTransform import lpTransform

METHODS = ("fbp", "grad", "cg", "em", "tv", "tve", "tvl1")


def check_theta(theta, Nproj, tol=1e-4):
    """Raise unless theta[k] == k*pi/Nproj (within tol radians)."""
    theta = np.asarray(theta, np.float64).ravel()
    if theta.size != Nproj:
        raise ValueError("theta has %d angles, tomo has %d projections" % (theta.size, Nproj))
    want = np.arange(Nproj) * np.pi / Nproj
    err = float(np.max(np.abs(theta - want))) if Nproj else 0.0
    if err > tol:
        raise ValueError("the log-polar geometry needs theta[k] = k*pi/Nproj (uniform on [0, pi), no "
                         "endpoint); max deviation %.3g rad" % err)


def plan_chunks(centers, chunk, gpus):
    """Work per device: lists of (center, start, stop) slice ranges.  Runs of equal
    center are cut into chunks of at most `chunk` slices, dealt to the devices in turn."""
    centers = np.asarray(centers, np.float64).ravel()
    if chunk < 1 or not gpus:
        raise ValueError("need chunk >= 1 and at least one device")
    jobs = []
    start = 0
    for i in range(1, centers.size + 1):
        if i == centers.size or centers[i] != centers[start]:
            for a in range(start, i, chunk):
                jobs.append((float(centers[start]), a, min(i, a + chunk)))
            start = i
    plan = {g: [] for g in gpus}
    for j, job in enumerate(jobs):
        plan[gpus[j % len(gpus)]].append(job)
    return plan


def lprec(tomo, center, recon, theta, **kwargs):
    """Reconstruct every slice of tomo into recon (see the module docstring)."""
    lpmethod = kwargs.get("lpmethod", "fbp")
    if lpmethod not in METHODS:
        raise ValueError("lpmethod must be one of %s" % (METHODS,))
    tomo = np.asarray(tomo)
    if tomo.ndim != 3:
        raise ValueError("tomo must be [Nslices, Nproj, N]")
    S, Nproj, N = tomo.shape
    if not isinstance(recon, np.ndarray) or recon.shape != (S, N, N) or recon.dtype != np.float32:
        raise ValueError("recon must be a float32 array of shape %s" % ((S, N, N),))
    check_theta(theta, Nproj)
    centers = np.broadcast_to(np.asarray(center, np.float64), (S,))
    filt = kwargs.get("filter_name", "ramp") if lpmethod == "fbp" else "none"
    interp = kwargs.get("interp_type", "cubic")
    precision = kwargs.get("precision", "reference")
    num_iter = int(kwargs.get("num_iter", 64))
    reg_par = float(kwargs.get("reg_par", 0.001))
    gpus = [int(g) for g in kwargs.get("gpu_list", [0])]
    chunk = max(1, min(int(kwargs.get("chunk", 32)), S))
    plan = plan_chunks(centers, chunk, list(dict.fromkeys(gpus)))
    method = getattr(lpmethods, lpmethod)
    flg = 0 if lpmethod == "fbp" else 1
    errors = []

    def work(gpu, jobs):
        ops = {}
        try:
            for cor, a, b in jobs:
                lp = ops.get(cor)
                if lp is None:
                    lp = lpTransform(N, Nproj, chunk, filt, cor, interp, precision)
                    ops[cor] = lp
                    lp.precompute(flg)
                    lp.initcmem(flg, gpu)
                recon[a:b] = method(lp, np.ascontiguousarray(recon[a:b]), np.ascontiguousarray(tomo[a:b],
                                    dtype=np.float32), num_iter, reg_par, gpu)
        except BaseException as e:  # re-raised in the caller's thread
            errors.append(e)
        finally:
            # the handles' device buffers are released whether or not a job failed
            for lp in ops.values():
                lp.close()

    threads = [threading.Thread(target=work, args=(g, jobs)) for g, jobs in plan.items() if jobs]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    if errors:
        raise errors[0]
    return recon
