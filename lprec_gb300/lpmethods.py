"""Reconstruction methods built on fwdp/adjp (drop-in for src/lprec/lpmethods.py).

Every method has the reference's signature

    method(lp, init_recon, tomo0, num_iter, reg_par, gpu) -> numpy.ndarray

with `init_recon` [S, N, N] and `tomo0` [S, Nproj, N] host arrays (or CUDA
tensors).  Vectors stay float32 on the GPU, as in the reference; inner
products and norms are accumulated in float64 (the reference sums float32).
Work is enqueued on the current torch stream of device `gpu`.

cg, cg_exact and em run their vector updates with the library's fused kernels
(one pass per update, the inner product it needs in the same pass, float64
scalars kept on the device, deterministic reductions); tv, tve and tvl1 with
the fused TV kernels (three passes per iteration besides fwdp/adjp); grad uses
torch elementwise updates and the fused per-slice inner products.
"""
import numpy as np

from . import _lib

C_TV = 0.35  # step of the primal-dual TV iterations (lpmethods.py:202)


def _torch():
    import torch
    return torch


def _dev(a, gpu):
    torch = _torch()
    if isinstance(a, torch.Tensor):
        return a.to(device="cuda:%d" % gpu, dtype=torch.float32).contiguous().clone()
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float32)).to("cuda:%d" % gpu)


def _out(x):
    return x.cpu().numpy()


def _stream(x):
    import torch
    return torch.cuda.current_stream(x.device).cuda_stream


def _cg(lp, init_recon, tomo0, num_iter, gpu, normal_op):
    """CG on the normal equations A f = normal_op(tomo) with A = normal_op o fwdp; the
    vector updates, step lengths and residual norms on the device (fused kernels)."""
    torch = _torch()
    with torch.cuda.device(gpu):
        recon = _dev(init_recon, gpu)
        tomo = _dev(tomo0, gpu)
        n = recon.numel()
        st = _stream(recon)
        b = torch.zeros_like(recon)
        q = torch.zeros_like(recon)
        g = torch.zeros_like(tomo)
        work = torch.empty(_lib.vec_work_doubles(1), dtype=torch.float64, device=recon.device)
        sc = torch.zeros(3, dtype=torch.float64, device=recon.device)  # rs_old, <p, A p>, rs_new
        normal_op(b, tomo)
        lp.fwdp(g, recon, gpu)
        normal_op(q, g)
        r = b - q
        p = r.clone()
        ptr = [sc.data_ptr() + 8 * i for i in range(3)]
        _lib.vec_dot(r.data_ptr(), r.data_ptr(), n, 1, work.data_ptr(), ptr[0], st)
        for i in range(num_iter):
            lp.fwdp(g, p, gpu)
            normal_op(q, g)
            _lib.vec_dot(p.data_ptr(), q.data_ptr(), n, 1, work.data_ptr(), ptr[1], st)
            # alpha = rs_old / <p, A p>: recon += alpha p, r -= alpha A p, rs_new = <r, r>
            _lib.cg_step(recon.data_ptr(), r.data_ptr(), p.data_ptr(), q.data_ptr(), n, ptr[0], ptr[1],
                         work.data_ptr(), ptr[2], st)
            # p = r + (rs_new / rs_old) p
            _lib.cg_dir(p.data_ptr(), r.data_ptr(), n, ptr[2], ptr[0], st)
            sc[0:1].copy_(sc[2:3])
        return _out(recon)


def fbp(lp, init_recon, tomo0, num_iter=0, reg_par=0, gpu=0):
    """Filtered back-projection: one adjp (the filter is applied inside), lpmethods.py:7-19."""
    torch = _torch()
    with torch.cuda.device(gpu):
        recon = _dev(init_recon, gpu)
        tomo = _dev(tomo0, gpu)
        lp.adjp(recon, tomo, gpu)
        return _out(recon)


def grad(lp, init_recon, tomo0, num_iter, reg_par, gpu=0):
    """Gradient descent on 1/2||R f - g||^2; reg_par < 0 picks a Barzilai-Borwein step
    per slice (lpmethods.py:22-59)."""
    torch = _torch()
    with torch.cuda.device(gpu):
        recon = _dev(init_recon, gpu)
        tomo = _dev(tomo0, gpu)
        S = tomo.shape[0]
        m = recon[0].numel()
        st = _stream(recon)
        recon0 = recon.clone()
        grad0 = torch.zeros_like(recon)
        g = torch.zeros_like(tomo)
        gr = torch.zeros_like(recon)
        work = torch.empty(_lib.vec_work_doubles(S), dtype=torch.float64, device=recon.device)
        num = torch.empty(S, dtype=torch.float64, device=recon.device)
        den = torch.empty(S, dtype=torch.float64, device=recon.device)
        for i in range(num_iter):
            lp.fwdp(g, recon, gpu)
            g.sub_(tomo).mul_(2)
            lp.adjp(gr, g, gpu)
            if reg_par < 0:
                if i == 0:
                    lam = torch.full((S,), 1e-3, dtype=torch.float64, device=recon.device)
                else:
                    # Barzilai-Borwein step per slice: <dx, dg> / <dg, dg>, float64 sums of
                    # the float32 differences (fused kernel, no float64 copies of the arrays)
                    dg = gr - grad0
                    dx = recon - recon0
                    _lib.vec_dot(dx.data_ptr(), dg.data_ptr(), m, S, work.data_ptr(), num.data_ptr(), st)
                    _lib.vec_dot(dg.data_ptr(), dg.data_ptr(), m, S, work.data_ptr(), den.data_ptr(), st)
                    lam = num / den
            else:
                lam = torch.full((S,), float(reg_par), dtype=torch.float64, device=recon.device)
            recon0.copy_(recon)
            grad0.copy_(gr)
            recon.sub_(lam.float().view(S, 1, 1) * gr)
        return _out(recon)


def cg(lp, init_recon, tomo0, num_iter, reg_par=0, gpu=0):
    """Conjugate gradients on the normal equations R*R f = R*g (lpmethods.py:62-97)."""
    return _cg(lp, init_recon, tomo0, num_iter, gpu, lambda out, x: lp.adjp(out, x, gpu))


def em(lp, init_recon, tomo0, num_iter, reg_par, gpu=0):
    """Expectation maximisation; reg_par keeps the division away from 0 (lpmethods.py:100-128)."""
    torch = _torch()
    with torch.cuda.device(gpu):
        recon = _dev(init_recon, gpu)
        tomo = _dev(tomo0, gpu)
        xi = torch.zeros_like(recon)
        upd = torch.zeros_like(recon)
        g = torch.zeros_like(tomo)
        lp.adjp(xi, torch.ones_like(tomo), gpu)
        xi.add_(1e-5)
        eps = float(np.float32(reg_par))
        st = _stream(recon)
        for i in range(num_iter):
            lp.fwdp(g, recon, gpu)
            _lib.em_ratio(g.data_ptr(), tomo.data_ptr(), eps, g.numel(), st)   # g = tomo / (g + eps)
            lp.adjp(upd, g, gpu)
            _lib.em_step(recon.data_ptr(), upd.data_ptr(), xi.data_ptr(), recon.numel(), st)
        return _out(recon)


def _tv_family(lp, init_recon, tomo0, num_iter, reg_par, gpu, mode):
    """Chambolle-Pock iterations shared by tv, tve, tvl1 (lpmethods.py:131-288): per
    iteration the TV dual update, fwdp, the data-term dual update, adjp and the
    divergence + primal update, each update one fused pass (results equal the
    reference's float32 statement sequence bit for bit)."""
    torch = _torch()
    with torch.cuda.device(gpu):
        recon = _dev(init_recon, gpu)
        tomo = _dev(tomo0, gpu)
        S, ny, nx = recon.shape
        g = torch.zeros_like(tomo)
        p = torch.zeros_like(recon)
        recon0 = recon.clone()
        prox0x = torch.zeros_like(recon)
        prox0y = torch.zeros_like(recon)
        prox1 = torch.zeros_like(tomo)
        c = C_TV
        st = _stream(recon)
        for i in range(num_iter):
            _lib.tv_prox0(prox0x.data_ptr(), prox0y.data_ptr(), recon.data_ptr(), S, ny, nx, c, reg_par, st)
            lp.fwdp(g, recon, gpu)
            _lib.tv_prox1(prox1.data_ptr(), g.data_ptr(), tomo.data_ptr(), g.numel(), c, mode, st)
            lp.adjp(p, prox1, gpu)
            _lib.tv_recon(recon0.data_ptr(), recon.data_ptr(), p.data_ptr(), prox0x.data_ptr(), prox0y.data_ptr(),
                          S, ny, nx, c, st)
        return _out(recon)


def tv(lp, init_recon, tomo0, num_iter, reg_par, gpu=0):
    """1/2||R f - g||^2 + reg_par TV(f) (lpmethods.py:131-180)."""
    return _tv_family(lp, init_recon, tomo0, num_iter, reg_par, gpu, "tv")


def tve(lp, init_recon, tomo0, num_iter, reg_par, gpu=0):
    """sum(R f - g log R f) + reg_par TV(f) (lpmethods.py:182-230)."""
    return _tv_family(lp, init_recon, tomo0, num_iter, reg_par, gpu, "tve")


def tvl1(lp, init_recon, tomo0, num_iter, reg_par, gpu=0):
    """||R f - g||_1 + reg_par TV(f) (lpmethods.py:232-288)."""
    return _tv_family(lp, init_recon, tomo0, num_iter, reg_par, gpu, "tvl1")


# ---------------------------------------------------------------------------
# Methods on the exact transpose (not in the reference, whose adjp is only
# approximately the transpose of fwdp): least squares with the true normal
# equations R^T R f = R^T g, and gradient descent through autograd.
# ---------------------------------------------------------------------------
def cg_exact(lp, init_recon, tomo0, num_iter, reg_par=0, gpu=0):
    """CG on R^T R f = R^T g with R^T the exact transpose (lp.fwdp_T); float64 inner products."""
    return _cg(lp, init_recon, tomo0, num_iter, gpu, lambda out, x: lp.fwdp_T(out, x, gpu))


def tv_gd(lp, init_recon, tomo0, num_iter, reg_par, gpu=0, step=None, eps=1e-8):
    """Gradient descent on 1/2||R f - g||^2 + reg_par * TV_eps(f) with gradients from
    autograd (backward = exact transpose).  `step` defaults to 1/||R^T R|| estimated
    by a few power iterations."""
    torch = _torch()
    from .autograd import radon
    with torch.cuda.device(gpu):
        x = _dev(init_recon, gpu)
        tomo = _dev(tomo0, gpu)
        if step is None:
            v = torch.rand_like(x)
            for _ in range(8):
                w = torch.zeros_like(tomo)
                lp.fwdp(w, v, gpu)
                u = torch.zeros_like(x)
                lp.fwdp_T(u, w, gpu)
                nrm = torch.linalg.vector_norm(u.double())
                v = (u / nrm).float()
            step = 0.9 / float(nrm)
        for i in range(num_iter):
            x.requires_grad_(True)
            dx = x[:, :, 1:] - x[:, :, :-1]
            dy = x[:, 1:, :] - x[:, :-1, :]
            tv = torch.sqrt(dx[:, :-1, :] ** 2 + dy[:, :, :-1] ** 2 + eps).sum()
            loss = 0.5 * ((radon(x, lp, gpu) - tomo) ** 2).sum() + reg_par * tv
            (gx,) = torch.autograd.grad(loss, x)
            with torch.no_grad():
                x = x - step * gx
        return _out(x.detach())
