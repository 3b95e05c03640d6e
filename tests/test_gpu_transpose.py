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
    tr = O.Transform.from_packed(lp.glpars, lp.fwdparsi, lp.fwdparamsf, lp.adjparsi, lp.adjparamsf)
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
    tr = O.Transform.from_packed(lp.glpars, lp.fwdparsi, lp.fwdparamsf, lp.adjparsi, lp.adjparamsf)
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
