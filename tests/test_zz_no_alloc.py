"""lp_fwd_noalloc: the forward transform for callers that may not allocate device memory.

Some callers run inside applications whose device memory belongs to another
allocator (a framework's caching allocator, or a fixed pool reserved at
start-up): they may not call cudaMalloc/cudaFree while processing.  The
allocation-free entry point takes its scratch from a fixed device array inside
the library.  This file is collected last so that a run stopping at the first
failure has already run every other test.
"""

import numpy as np
import pytest

from oracle import lprec_oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_noalloc_matches_lp_fwd_twice(torch_cuda):
    torch = torch_cuda
    from lprec_gb300 import _lib
    N, Nproj, S = 128, 192, 4
    packed = _lib.precompute(N, Nproj, S, N / 2, 'cubic', 'ramp', precision='fp64')
    h = _lib.Handle(packed[0], 0)
    h.init_fwd(packed[1], packed[2])
    h.init_adj(packed[3], packed[4])
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(11)
    for call in range(2):  # two calls in a row, different inputs
        f = torch.as_tensor(rng.random((S, N, N), dtype=np.float32)).cuda()
        R_ref = torch.full((S, Nproj, N), float('nan'), device='cuda')
        R_new = torch.full((S, Nproj, N), float('nan'), device='cuda')
        h.fwd(R_ref.data_ptr(), f.data_ptr(), S, stream)
        h.fwd_noalloc(R_new.data_ptr(), f.data_ptr(), S, stream)
        torch.cuda.synchronize()
        a, b = R_new.cpu().double().numpy(), R_ref.cpu().double().numpy()
        assert np.all(np.isfinite(a)), call
        assert _rel(a, b) <= TOL, (call, _rel(a, b))


def test_noalloc_rejects_oversize(torch_cuda):
    torch = torch_cuda
    from lprec_gb300 import _lib
    N, Nproj, S = 512, 768, 24
    packed = _lib.precompute(N, Nproj, S, N / 2, 'cubic', 'none', precision='fp64')
    h = _lib.Handle(packed[0], 0)
    h.init_fwd(packed[1], packed[2])
    limit = 64 * 1024 * 1024
    assert h.noalloc_scratch_bytes(S) > limit
    f = torch.zeros((S, N, N), device='cuda')
    R = torch.zeros((S, Nproj, N), device='cuda')
    with pytest.raises(_lib.LprecError) as ei:
        h.fwd_noalloc(R.data_ptr(), f.data_ptr(), S, torch.cuda.current_stream().cuda_stream)
    assert ei.value.code == _lib.LP_ERR_UNSUPPORTED
    assert "scratch" in str(ei.value)


@pytest.mark.parametrize("fill", [float('nan'), 1e30])
def test_noalloc_ignores_stale_scratch(torch_cuda, fill):
    """The shared array keeps whatever the last call (or anything else) left in it: filled
    with NaN or 1e30 before each call, the result still equals lp_fwd's."""
    torch = torch_cuda
    from lprec_gb300 import _lib
    N, Nproj, S = 128, 192, 3
    packed = _lib.precompute(N, Nproj, S, 61, 'cubic', 'none', precision='fp64')
    h = _lib.Handle(packed[0], 0)
    h.init_fwd(packed[1], packed[2])
    stream = torch.cuda.current_stream().cuda_stream
    f = torch.as_tensor(np.random.default_rng(12).random((S, N, N), dtype=np.float32)).cuda()
    R_ref = torch.empty((S, Nproj, N), device='cuda')
    h.fwd(R_ref.data_ptr(), f.data_ptr(), S, stream)
    for _ in range(2):
        _lib.debug_fill_noalloc_scratch(0, fill, stream)
        R_new = torch.full((S, Nproj, N), float('nan'), device='cuda')
        h.fwd_noalloc(R_new.data_ptr(), f.data_ptr(), S, stream)
        torch.cuda.synchronize()
        a, b = R_new.cpu().double().numpy(), R_ref.cpu().double().numpy()
        assert np.all(np.isfinite(a))
        assert _rel(a, b) <= TOL, _rel(a, b)


@pytest.mark.parametrize("args", [(2048, 3000, 'cubic', 1), (256, 384, 'linear', 4)])
def test_noalloc_against_oracle(torch_cuda, args):
    """One N=2048 slice (50 MB of the 64 MiB array) and linear interpolation: the
    allocation-free forward against the float64 oracle fed the same tables, and against
    lp_fwd."""
    torch = torch_cuda
    from lprec_gb300 import _lib
    N, Nproj, interp, S = args
    packed = _lib.precompute(N, Nproj, S, N / 2, interp, 'none', precision='fp64', wide=True)
    h = _lib.Handle(packed[0], 0)
    h.init_fwd(packed[1], packed[2])
    assert h.noalloc_scratch_bytes(S) <= 64 * 1024 * 1024
    stream = torch.cuda.current_stream().cuda_stream
    f = np.stack([O.ellipse_phantom(N, 10, np.random.default_rng(20 + s)) for s in range(S)])
    ft = torch.as_tensor(np.float32(f)).cuda()
    R_new = torch.full((S, Nproj, N), float('nan'), device='cuda')
    R_ref = torch.full((S, Nproj, N), float('nan'), device='cuda')
    h.fwd_noalloc(R_new.data_ptr(), ft.data_ptr(), S, stream)
    h.fwd(R_ref.data_ptr(), ft.data_ptr(), S, stream)
    torch.cuda.synchronize()
    a = R_new.cpu().double().numpy()
    tr = O.Transform.from_packed(*packed)
    assert _rel(a, tr.fwd(f)) <= TOL, _rel(a, tr.fwd(f))
    assert _rel(a, R_ref.cpu().double().numpy()) <= TOL


def test_noalloc_setup_call_and_argument_checks(torch_cuda):
    """S0 = 0 only resolves the array (the set-up call made before a caller reserves its
    pool or captures a stream); negative slice counts are refused by both entry points."""
    torch = torch_cuda
    from lprec_gb300 import _lib
    packed = _lib.precompute(64, 96, 2, 32, 'cubic', 'none')
    h = _lib.Handle(packed[0], 0)
    h.init_fwd(packed[1], packed[2])
    stream = torch.cuda.current_stream().cuda_stream
    h.fwd_noalloc(0, 0, 0, stream)
    with pytest.raises(_lib.LprecError) as ei:
        h.noalloc_scratch_bytes(-1)
    assert ei.value.code == _lib.LP_ERR_ARG
    with pytest.raises(_lib.LprecError) as ei:
        h.noalloc_scratch_bytes(3)
    assert ei.value.code == _lib.LP_ERR_ARG
    with pytest.raises(_lib.LprecError) as ei:
        h.fwd_noalloc(0, 0, -1, stream)
    assert ei.value.code == _lib.LP_ERR_ARG
