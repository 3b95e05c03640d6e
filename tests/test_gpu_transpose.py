"""Exact-transpose backward: against the oracle, dot-product test, FP64 finite differences."""
import os

import numpy as np
import pytest

from oracle import lprec_oracle as O

pytestmark = pytest.mark.gpu
NAMES = ['glpars', 'fwdparsi', 'fwdparamsf', 'adjparsi', 'adjparamsf']


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _lp(N0, Nproj, S, cor, interp, filt='none'):
    from lprec_gb300.lpTransform import lpTransform
    lp = lpTransform(N0, Nproj, S, filt, cor, interp)
    lp.precompute(1)
    lp.initcmem(1, 0)
    return lp


def _fwdT(torch, lp, g):
    gt = torch.as_tensor(np.float32(g)).cuda()
    f = torch.full((g.shape[0], lp.clphandle[0].N0, lp.clphandle[0].N0), float('nan'), device='cuda')
    lp.fwdp_T(f, gt, 0)
    torch.cuda.synchronize()
    return f.cpu().double().numpy()


@pytest.mark.parametrize("args", [(64, 96, 32, 'cubic'), (48, 72, 21, 'cubic'), (32, 24, 16, 'linear'),
                                  (256, 384, 128, 'cubic'), (512, 768, 256, 'cubic')])
def test_transpose_matches_oracle(torch_cuda, args):
    N0, Nproj, cor, interp = args
    lp = _lp(N0, Nproj, 2, cor, interp)
    tr = O.Transform.from_packed(*lp.tables())
    g = np.random.default_rng(5).standard_normal((2, Nproj, N0)).astype(np.float32).astype(np.float64)
    fg = _fwdT(torch_cuda, lp, g)
    fo = tr.fwd_T(g)
    assert np.all(np.isfinite(fg))
    assert O.rel_l2(fg, fo) < 1e-5, O.rel_l2(fg, fo)


@pytest.mark.parametrize("args", [(512, 768, 256, 'cubic', 2), (128, 192, 64, 'linear', 3)])
def test_dot_product(torch_cuda, args):
    """<R f, g> == <f, R^T g> to 1e-6 (config: N=512, Nproj=768)."""
    torch = torch_cuda
    N0, Nproj, cor, interp, S = args
    lp = _lp(N0, Nproj, S, cor, interp)
    rng = np.random.default_rng(0)
    f = rng.random((S, N0, N0), dtype=np.float32)
    g = rng.random((S, Nproj, N0), dtype=np.float32)
    R = torch.zeros((S, Nproj, N0), device='cuda')
    lp.fwdp(R, torch.as_tensor(f).cuda(), 0)
    Rf = R.cpu().double().numpy()
    fT = _fwdT(torch, lp, g)
    lhs = np.sum(Rf * g)
    rhs = np.sum(f.astype(np.float64) * fT)
    assert abs(lhs - rhs) / abs(lhs) < 1e-6, abs(lhs - rhs) / abs(lhs)


def test_autograd_finite_differences(torch_cuda):
    """Gradient of 1/2||R f - y||^2 vs float64 central differences (eps=1e-3), 8 directions."""
    torch = torch_cuda
    from lprec_gb300.autograd import radon
    N0, Nproj, S = 128, 192, 2
    lp = _lp(N0, Nproj, S, 64, 'cubic')
    tr = O.Transform.from_packed(*lp.tables())
    rng = np.random.default_rng(2)
    f0 = np.stack([O.ellipse_phantom(N0, 10, rng) for _ in range(S)]).astype(np.float32)
    y = (tr.fwd(f0) * 1.1).astype(np.float32)
    x = torch.as_tensor(f0 * 0.9).cuda().requires_grad_(True)
    loss = 0.5 * ((radon(x, lp, 0) - torch.as_tensor(y).cuda()) ** 2).sum()
    loss.backward()
    grad = x.grad.cpu().double().numpy()
    f64 = f0.astype(np.float64) * 0.9

    def L(v):
        return 0.5 * np.sum((tr.fwd(v) - y) ** 2)
    eps = 1e-3
    # <grad, d> for d ~ N(0, 1) has magnitude ~ ||grad||; a float32 gradient with
    # relative L2 error e changes it by ~ e ||grad||, so that is the scale of the bound
    scale = np.linalg.norm(grad)
    for i in range(8):
        d = rng.standard_normal(f64.shape)
        fd = (L(f64 + eps * d) - L(f64 - eps * d)) / (2 * eps)
        an = np.sum(grad * d)
        assert abs(fd - an) <= 1e-5 * scale, (i, fd, an, scale)


def _cg_exact_oracle(tr, init, tomo, num_iter):
    """CG on R^T R f = R^T g with the oracle's exact transpose (float64)."""
    recon = np.array(init, dtype=np.float64)
    r = tr.fwd_T(tomo) - tr.fwd_T(tr.fwd(recon))
    p = r.copy()
    rsold = np.sum(r * r)
    for _ in range(num_iter):
        q = tr.fwd_T(tr.fwd(p))
        alpha = rsold / np.sum(p * q)
        recon = recon + alpha * p
        r = r - alpha * q
        rsnew = np.sum(r * r)
        p = r + (rsnew / rsold) * p
        rsold = rsnew
    return recon


def test_cg_exact_matches_oracle(torch_cuda):
    from lprec_gb300 import lpmethods
    N0, Nproj = 64, 96
    lp = _lp(N0, Nproj, 2, 32, 'cubic')
    tr = O.Transform.from_packed(*lp.tables())
    rng = np.random.default_rng(4)
    ph = np.stack([O.ellipse_phantom(N0, 5, rng) for _ in range(2)])
    tomo = np.float32(tr.fwd(ph)).astype(np.float64)
    z = np.zeros((2, N0, N0), np.float32)
    got = lpmethods.cg_exact(lp, z, np.float32(tomo), 10, 0, 0)
    ref = _cg_exact_oracle(tr, z, tomo, 10)
    # R^T R is ill-conditioned: ten CG steps amplify the float32 rounding of the
    # operator (~1e-7) to ~1e-3 against the float64 iteration
    assert O.rel_l2(got, ref) < 5e-3, O.rel_l2(got, ref)
    # the data residual falls below the one of the starting point
    assert np.linalg.norm(tr.fwd(got) - tomo) < 0.2 * np.linalg.norm(tomo)


def test_tv_gd_decreases_objective(torch_cuda):
    """Gradient descent with autograd gradients (exact transpose) decreases its objective."""
    torch = torch_cuda
    from lprec_gb300 import lpmethods
    N0, Nproj = 64, 96
    lp = _lp(N0, Nproj, 2, 32, 'cubic')
    tr = O.Transform.from_packed(*lp.tables())
    rng = np.random.default_rng(6)
    ph = np.stack([O.ellipse_phantom(N0, 5, rng) for _ in range(2)])
    tomo = tr.fwd(ph)

    def objective(x, lam=1e-3, eps=1e-8):
        dx = x[:, :, 1:] - x[:, :, :-1]
        dy = x[:, 1:, :] - x[:, :-1, :]
        tv = np.sqrt(dx[:, :-1, :] ** 2 + dy[:, :, :-1] ** 2 + eps).sum()
        return 0.5 * np.sum((tr.fwd(x) - tomo) ** 2) + lam * tv
    z = np.zeros((2, N0, N0), np.float32)
    o0 = objective(z.astype(np.float64))
    x5 = lpmethods.tv_gd(lp, z, np.float32(tomo), 5, 1e-3, 0)
    x20 = lpmethods.tv_gd(lp, z, np.float32(tomo), 20, 1e-3, 0)
    o5, o20 = objective(x5.astype(np.float64)), objective(x20.astype(np.float64))
    assert o20 < o5 < o0, (o0, o5, o20)


def test_n4096_dot_product(torch_cuda):
    """N=4096: 8192-point register FFTs in 512-thread blocks.  Forward and exact transpose
    pass the dot test, the drop-in adjoint passes the reference's looser one (1e-2)."""
    torch = torch_cuda
    N0, Nproj, S = 4096, 6144, 1
    lp = _lp(N0, Nproj, S, N0 // 2, 'cubic')
    rng = np.random.default_rng(0)
    f = rng.random((S, N0, N0), dtype=np.float32)
    g = rng.random((S, Nproj, N0), dtype=np.float32)
    R = torch.zeros((S, Nproj, N0), device='cuda')
    lp.fwdp(R, torch.as_tensor(f).cuda(), 0)
    fT = _fwdT(torch, lp, g)
    fa = torch.zeros((S, N0, N0), device='cuda')
    lp.adjp(fa, torch.as_tensor(g).cuda(), 0)
    torch.cuda.synchronize()
    Rn = R.cpu().double().numpy()
    assert np.all(np.isfinite(Rn)) and np.all(np.isfinite(fT))
    lhs = float(np.sum(Rn * g))
    assert abs(lhs - float(np.sum(f.astype(np.float64) * fT))) / abs(lhs) < 1e-6
    assert abs(lhs - float(np.sum(f.astype(np.float64) * fa.cpu().double().numpy()))) / abs(lhs) < 1e-2


@pytest.mark.parametrize("args", [(512, 768, 256, 'cubic', 16), (96, 144, 45, 'cubic', 3), (128, 192, 64, 'linear', 2),
                                  (64, 40, 32.5, 'cubic', 2), (512, 768, 253, 'cubic', 9), (512, 768, 243, 'cubic', 5),
                                  (2048, 512, 1021, 'cubic', 2)])
def test_transpose_bit_reproducible(torch_cuda, args):
    """The backward has no atomics: two calls on the same input give the same bits, also
    after the scratch buffers were poisoned in between (odd padded sizes, a non-integer
    axis, a slice count that is not a multiple of the gather's slice group, and the
    register FFT's prime-17 and prime-43 stages at N = 544 and 2064 included)."""
    torch = torch_cuda
    N0, Nproj, cor, interp, S = args
    lp = _lp(N0, Nproj, S, cor, interp)
    g = torch.as_tensor(np.random.default_rng(9).standard_normal((S, Nproj, N0)).astype(np.float32)).cuda()
    f1 = torch.empty((S, N0, N0), device='cuda')
    f2 = torch.empty((S, N0, N0), device='cuda')
    lp.fwdp_T(f1, g, 0)
    lp.clphandle[0].debug_fill_scratch(float('nan'), torch.cuda.current_stream().cuda_stream)
    lp.fwdp_T(f2, g, 0)
    torch.cuda.synchronize()
    assert torch.isfinite(f1).all()
    assert torch.equal(f1, f2)
    tr = O.Transform.from_packed(*lp.tables())
    gs = g[:2].cpu().double().numpy()
    assert O.rel_l2(f1[:2].cpu().double().numpy(), tr.fwd_T(gs)) < 1e-5
