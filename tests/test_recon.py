"""The tomopy-form host wrapper (lprec_gb300.recon): angle check, work plan and
argument errors on the CPU; results against direct lpmethods calls on the GPU."""
import numpy as np
import pytest

from lprec_gb300.recon import check_theta, lprec, plan_chunks


def test_check_theta():
    n = 12
    check_theta(np.arange(n) * np.pi / n, n)
    with pytest.raises(ValueError, match="k\\*pi/Nproj"):
        check_theta(np.linspace(0, np.pi, n), n)          # endpoint included: another grid
    with pytest.raises(ValueError, match="angles"):
        check_theta(np.arange(n - 1) * np.pi / n, n)


def test_plan_chunks():
    plan = plan_chunks([10, 10, 10, 12, 12, 10], 2, [0, 1])
    assert plan == {0: [(10.0, 0, 2), (12.0, 3, 5)], 1: [(10.0, 2, 3), (10.0, 5, 6)]}
    plan = plan_chunks([5.0] * 7, 3, [2])
    assert plan == {2: [(5.0, 0, 3), (5.0, 3, 6), (5.0, 6, 7)]}
    covered = sorted((a, b) for jobs in plan_chunks(np.r_[np.zeros(9), np.ones(4)], 4, [0, 1, 2]).values()
                     for _, a, b in jobs)
    assert covered == [(0, 4), (4, 8), (8, 9), (9, 13)]
    with pytest.raises(ValueError):
        plan_chunks([1.0], 0, [0])


def test_lprec_rejects_bad_arguments():
    tomo = np.zeros((2, 12, 16), np.float32)
    theta = np.arange(12) * np.pi / 12
    with pytest.raises(ValueError, match="lpmethod"):
        lprec(tomo, 8, np.zeros((2, 16, 16), np.float32), theta, lpmethod="art")
    with pytest.raises(ValueError, match="recon"):
        lprec(tomo, 8, np.zeros((2, 16, 16), np.float64), theta)
    with pytest.raises(ValueError, match="recon"):
        lprec(tomo, 8, np.zeros((2, 15, 16), np.float32), theta)
    with pytest.raises(ValueError, match="theta"):
        lprec(tomo, 8, np.zeros((2, 16, 16), np.float32), np.linspace(0, np.pi, 12))


@pytest.mark.gpu
@pytest.mark.parametrize("method,kw", [("fbp", {}), ("cg", {"num_iter": 4}), ("tv", {"num_iter": 3})])
def test_lprec_matches_lpmethods(method, kw):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import lprec_oracle as O
    from lprec_gb300 import lpmethods
    from lprec_gb300.lpTransform import lpTransform
    S, Nproj, N, chunk = 5, 96, 64, 2
    rng = np.random.default_rng(6)
    f = np.stack([O.ellipse_phantom(N, 8, rng) for _ in range(S)]).astype(np.float32)
    centers = np.array([32, 32, 32, 30, 30], np.float64)
    tomo = np.empty((S, Nproj, N), np.float32)
    for c in (32, 30):
        lp = lpTransform(N, Nproj, S, 'none', c, 'cubic')
        lp.precompute(1)
        lp.initcmem(1, 0)
        R = torch.empty((S, Nproj, N), device='cuda')
        lp.fwdp(R, torch.as_tensor(f).cuda(), 0)
        tomo[centers == c] = R.cpu().numpy()[centers == c]
        lp.close()
    theta = np.arange(Nproj) * np.pi / Nproj
    got = lprec(tomo, centers, np.zeros((S, N, N), np.float32), theta, lpmethod=method, chunk=chunk,
                gpu_list=[0], filter_name='shepp-logan', reg_par=1e-3, **kw)
    filt = 'shepp-logan' if method == 'fbp' else 'none'
    want = np.empty_like(got)
    for c, a, b in [(32, 0, 2), (32, 2, 3), (30, 3, 5)]:
        lp = lpTransform(N, Nproj, chunk, filt, c, 'cubic')
        lp.precompute(0 if method == 'fbp' else 1)
        lp.initcmem(0 if method == 'fbp' else 1, 0)
        want[a:b] = getattr(lpmethods, method)(lp, np.zeros((b - a, N, N), np.float32), tomo[a:b],
                                               kw.get("num_iter", 0), 1e-3, 0)
        lp.close()
    assert np.array_equal(got, want)
    assert np.all(np.isfinite(got)) and np.linalg.norm(got) > 0
