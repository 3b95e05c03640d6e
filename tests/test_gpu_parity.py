"""GPU path against the oracle on identical float32 tables (relative L2 <= 1e-5).

Tables come either from the reference's own precompute (fixtures made by
tests/golden/make_golden.py) or from this library's precompute; the oracle is
fed exactly the same packed arrays, so any difference is the kernels'.
"""
import os

import numpy as np
import pytest

from oracle import lprec_oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-5
NAMES = ['glpars', 'fwdparsi', 'fwdparamsf', 'adjparsi', 'adjparamsf']


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _handle(packed):
    from lprec_gb300 import _lib
    h = _lib.Handle(packed[0], 0)
    if packed[1] is not None:
        h.init_fwd(packed[1], packed[2])
    h.init_adj(packed[3], packed[4])
    return h


def _fwd(torch, h, f):
    ft = torch.as_tensor(np.float32(f)).cuda()
    R = torch.full((f.shape[0], h.Nproj, h.N0), float('nan'), device='cuda')
    h.fwd(R.data_ptr(), ft.data_ptr(), f.shape[0], torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return R.cpu().numpy().astype(np.float64)


def _adj(torch, h, R):
    Rt = torch.as_tensor(np.float32(R)).cuda()
    f = torch.full((R.shape[0], h.N0, h.N0), float('nan'), device='cuda')
    h.adj(f.data_ptr(), Rt.data_ptr(), R.shape[0], torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return f.cpu().numpy().astype(np.float64)


def _inputs(G, S, seed):
    rng = np.random.default_rng(seed)
    f = rng.random((S, G.N0, G.N0)).astype(np.float32).astype(np.float64)
    R = rng.random((S, G.Nproj0, G.N0)).astype(np.float32).astype(np.float64)
    return f, R


@pytest.mark.parametrize("case", ["n64_cubic_ramp", "n48_cor_shepp", "n32_os2_linear_hann", "n64_cubic_none"])
def test_reference_tables(torch_cuda, golden_dir, case):
    """Reference-made tables: GPU fwd/adj == oracle fwd/adj."""
    z = np.load(os.path.join(golden_dir, 'packed_%s.npz' % case))
    packed = [z[n] for n in NAMES]
    packed[0] = packed[0].copy()
    packed[0][6] = 3  # batch capacity (Nslices)
    tr = O.Transform.from_packed(*packed)
    h = _handle(packed)
    f, R = _inputs(tr.G, 3, 0)
    Rg = _fwd(torch_cuda, h, f)
    fg = _adj(torch_cuda, h, R)
    Ro = tr.fwd(f)
    fo = tr.adj(R)
    assert np.all(np.isfinite(Rg)) and np.all(np.isfinite(fg))
    assert O.rel_l2(Rg, Ro) < TOL, O.rel_l2(Rg, Ro)
    assert O.rel_l2(fg, fo) < TOL, O.rel_l2(fg, fo)


@pytest.mark.parametrize("args", [(256, 384, 'cubic', 'ramp', 128), (96, 150, 'cubic', 'hamming', 45),
                                  (128, 64, 'linear', 'none', 64), (80, 120, 'cubic', 'parzen', 40.5)])
def test_own_tables(torch_cuda, args):
    """This library's fp64 precompute, same float32 tables in the oracle, noise inputs."""
    from lprec_gb300 import _lib
    N0, Nproj, interp, filt, cor = args
    packed = _lib.precompute(N0, Nproj, 2, cor, interp, filt, precision='fp64')
    h = _handle(packed)
    tr = O.Transform.from_packed(*packed)
    f, R = _inputs(tr.G, 2, 1)
    assert O.rel_l2(_fwd(torch_cuda, h, f), tr.fwd(f)) < TOL
    assert O.rel_l2(_adj(torch_cuda, h, R), tr.adj(R)) < TOL


@pytest.mark.parametrize("args", [(256, 384, 'cubic', 'shepp-logan', 128), (96, 150, 'cubic', 'ramp', 45)])
def test_fp64_oracle_error_phantom(torch_cuda, args):
    """Error against the float64 oracle (unrounded float64 tables) on phantom data."""
    from lprec_gb300 import _lib
    N0, Nproj, interp, filt, cor = args
    packed = _lib.precompute(N0, Nproj, 2, cor, interp, filt, precision='fp64')
    h = _handle(packed)
    tr = O.Transform(N0, Nproj, 2, filt, cor, interp, mode='fp64', rounded=False)
    rng = np.random.default_rng(7)
    f = np.stack([O.ellipse_phantom(N0, 10, rng) for _ in range(2)])
    R = tr.fwd(f)
    assert O.rel_l2(_fwd(torch_cuda, h, f), R) < TOL
    assert O.rel_l2(_adj(torch_cuda, h, R), tr.adj(R)) < TOL


@pytest.mark.parametrize("args", [(256, 384, 'cubic', 'shepp-logan', 128), (512, 768, 'cubic', 'ramp', 256),
                                  (192, 288, 'linear', 'hann', 90), (2048, 3000, 'cubic', 'shepp-logan', 1024)])
def test_float64_tables(torch_cuda, args):
    """Handles fed float64 tables (fixed-point coordinates on the device): parity with the
    oracle fed the same float64 tables, and FBP within 1e-6 of the unrounded float64
    oracle (float32 tables leave 4.6e-6 at N=512 and 3.3e-5 at N=2048)."""
    from lprec_gb300 import _lib
    N0, Nproj, interp, filt, cor = args
    wide = _lib.precompute(N0, Nproj, 1, cor, interp, filt, precision='fp64', wide=True)
    assert wide[2].dtype == np.float64 and wide[4].dtype == np.float64
    h = _handle(wide)
    tr = O.Transform.from_packed(*wide)
    rng = np.random.default_rng(11)
    f = O.ellipse_phantom(N0, 10, rng)[None]
    R = tr.fwd(f)
    Rn = R + 0.01 * np.abs(R).max() * rng.standard_normal(R.shape)
    Rn = np.float32(Rn).astype(np.float64)
    assert O.rel_l2(_fwd(torch_cuda, h, f), R) < TOL
    fb = _adj(torch_cuda, h, Rn)
    assert O.rel_l2(fb, tr.adj(Rn)) < TOL
    if N0 <= 512:
        exact = O.Transform(N0, Nproj, 1, filt, cor, interp, mode='fp64', rounded=False)
        assert O.rel_l2(fb, exact.adj(Rn)) < 1e-6, O.rel_l2(fb, exact.adj(Rn))


def test_reference_pins_adj_many(torch_cuda, golden_dir):
    """tests/test_adj_many.py pins on the GPU: 8 slices scaled by (8-k)."""
    from lprec_gb300.lpTransform import lpTransform
    torch = torch_cuda
    d = np.load(os.path.join(golden_dir, 'testdata.npz'))
    S = 8
    fa = np.stack([d['f'] * (S - k) for k in range(S)]).astype(np.float32)
    Ra = np.stack([d['R'] * (S - k) for k in range(S)]).astype(np.float32)
    lp = lpTransform(512, 384, S, 'None', 256, 'cubic')
    lp.precompute(1)
    lp.initcmem(1, 0)
    fg, Rg = torch.as_tensor(fa).cuda(), torch.as_tensor(Ra).cuda()
    Rfg = torch.zeros((S, 384, 512), device='cuda')
    fRg = torch.zeros((S, 512, 512), device='cuda')
    RfRg = torch.zeros((S, 384, 512), device='cuda')
    lp.fwdp(Rfg, fg, 0)
    lp.adjp(fRg, Rg, 0)
    lp.fwdp(RfRg, fRg, 0)
    Rf, fR, RfR = [x.cpu().double().numpy() for x in (Rfg, fRg, RfRg)]
    s1 = np.sum(Rf * Ra)
    s2 = np.sum(fR * fa)
    err0 = abs(s1 - s2) / abs(s2)
    err1 = np.linalg.norm(fR - fa) / np.linalg.norm(fa)
    err2 = np.linalg.norm(RfR - Rf) / np.linalg.norm(Rf)
    assert err0 < 5e-3 and err1 < 7e-3 and err2 < 7e-4, (err0, err1, err2)


def test_batch_equals_single(torch_cuda):
    from lprec_gb300 import _lib
    packed = _lib.precompute(64, 96, 4, 32, 'cubic', 'shepp-logan')
    h = _handle(packed)
    G = O.create_geometry(64, 96, 4, 32, 'cubic')
    f, R = _inputs(G, 4, 5)
    Rb = _fwd(torch_cuda, h, f)
    fb = _adj(torch_cuda, h, R)
    for s in range(4):
        assert np.array_equal(_fwd(torch_cuda, h, f[s:s + 1])[0], Rb[s])
        assert np.array_equal(_adj(torch_cuda, h, R[s:s + 1])[0], fb[s])


def test_deterministic(torch_cuda):
    from lprec_gb300 import _lib
    packed = _lib.precompute(128, 192, 2, 64, 'cubic', 'ramp')
    h = _handle(packed)
    G = O.create_geometry(128, 192, 2, 64, 'cubic')
    f, R = _inputs(G, 2, 9)
    assert np.array_equal(_fwd(torch_cuda, h, f), _fwd(torch_cuda, h, f))
    assert np.array_equal(_adj(torch_cuda, h, R), _adj(torch_cuda, h, R))


@pytest.mark.parametrize("interp", ['cubic', 'linear'])
def test_schedules_bit_identical(torch_cuda, interp):
    """Chunked and two-stream batch schedules (and the autotuner's pick) give the
    same bits as one whole-batch launch sequence."""
    torch = torch_cuda
    from lprec_gb300 import _lib
    S = 7
    packed = _lib.precompute(128, 192, S, 64, interp, 'shepp-logan', precision='fp64')
    h = _handle(packed)
    G = O.create_geometry(128, 192, S, 64, interp)
    f, R = _inputs(G, S, 23)
    Rc, fc = _fwd(torch, h, f), _adj(torch, h, R)
    for sched in ((3, 2, 512, 2, 2, 256), (2, 1, 256, 3, 1, 512), (1, 2, 512, 1, 2, 512), (4, 2, 256, 0, 1, 256)):
        h.set_schedule(*sched)
        assert h.schedule() == dict(zip(h.SCHEDULE_KEYS, sched))
        assert np.array_equal(_fwd(torch, h, f), Rc), sched
        assert np.array_equal(_adj(torch, h, R), fc), sched
    Rt = torch.zeros((S, 192, 128), device='cuda')
    ft = torch.zeros((S, 128, 128), device='cuda')
    ms = h.autotune(Rt.data_ptr(), ft.data_ptr(), S, torch.cuda.current_stream().cuda_stream)
    assert ms[0] > 0 and ms[1] > 0
    sc = h.schedule()
    assert sc['fwd_streams'] in (1, 2) and sc['adj_streams'] in (1, 2)
    assert np.array_equal(_fwd(torch, h, f), Rc), sc
    assert np.array_equal(_adj(torch, h, R), fc), sc
    with pytest.raises(_lib.LprecError):
        h.set_schedule(1, 3)
    with pytest.raises(_lib.LprecError):
        h.set_schedule(fwd_theta_block=384)


@pytest.mark.parametrize("args", [(128, 192, 64, 'cubic', 'ramp'), (96, 144, 45, 'cubic', 'none'),
                                  (256, 384, 128, 'linear', 'hann'), (64, 96, 32, 'cubic', 'shepp-logan')])
def test_scratch_poison_invariant(torch_cuda, args):
    """Intermediate buffers filled with NaN or a large value before a call give the same
    result: no kernel reads an element that the call itself did not write first."""
    torch = torch_cuda
    from lprec_gb300 import _lib
    N0, Nproj, cor, interp, filt = args
    packed = _lib.precompute(N0, Nproj, 2, cor, interp, filt, precision='fp64')
    h = _handle(packed)
    G = O.create_geometry(N0, Nproj, 2, cor, interp)
    f, R = _inputs(G, 2, 17)
    st = torch.cuda.current_stream().cuda_stream
    Rc, fc = _fwd(torch, h, f), _adj(torch, h, R)
    for v in (float('nan'), 1e30):
        h.debug_fill_scratch(v, st)
        assert np.array_equal(_fwd(torch, h, f), Rc), v
        h.debug_fill_scratch(v, st)
        assert np.array_equal(_adj(torch, h, R), fc), v


@pytest.mark.parametrize("args", [(512, 768, 'cubic', 'shepp-logan', 256, 2), (1024, 1536, 'linear', 'hann', 512, 1),
                                  (2048, 3000, 'cubic', 'shepp-logan', 1024, 1)])
def test_large_sizes(torch_cuda, args):
    """Power-of-two sizes served by the register-FFT kernels, including N=2048."""
    from lprec_gb300 import _lib
    N0, Nproj, interp, filt, cor, S = args
    packed = _lib.precompute(N0, Nproj, S, cor, interp, filt, precision='fp64')
    h = _handle(packed)
    tr = O.Transform.from_packed(*packed)
    rng = np.random.default_rng(21)
    f = np.stack([O.ellipse_phantom(N0, 10, rng) for _ in range(S)])
    Rg = _fwd(torch_cuda, h, f)
    assert O.rel_l2(Rg, tr.fwd(f)) < TOL
    Rn = Rg + 0.01 * np.abs(Rg).max() * rng.standard_normal(Rg.shape)
    assert O.rel_l2(_adj(torch_cuda, h, Rn), tr.adj(Rn)) < TOL


def test_host_array_pipeline(torch_cuda):
    """lpTransform.fwd/adj on host arrays (chunked, overlapped copies) == fwdp/adjp."""
    torch = torch_cuda
    from lprec_gb300.lpTransform import lpTransform
    S, N, Nproj = 7, 128, 192
    lp = lpTransform(N, Nproj, 4, 'ramp', N / 2, 'cubic')
    lp.precompute(1)
    lp.initcmem(1, 0)
    rng = np.random.default_rng(3)
    f = rng.random((S, N, N), dtype=np.float32)
    R = rng.random((S, Nproj, N), dtype=np.float32)
    Rh = lp.fwd(f, 0, chunk=3)                      # numpy in, numpy out
    fh = lp.adj(torch.from_numpy(R).pin_memory(), 0, chunk=4)
    torch.cuda.synchronize()
    fh = fh.numpy()
    for s in range(S):
        Rd = torch.zeros((1, Nproj, N), device='cuda')
        fd = torch.zeros((1, N, N), device='cuda')
        lp.fwdp(Rd, torch.as_tensor(f[s:s + 1]).cuda(), 0)
        lp.adjp(fd, torch.as_tensor(R[s:s + 1]).cuda(), 0)
        assert np.array_equal(Rh[s], Rd.cpu().numpy()[0])
        assert np.array_equal(fh[s], fd.cpu().numpy()[0])


def test_host_calls_back_to_back(torch_cuda):
    """Host calls issued without a synchronisation in between share the pipeline's
    device buffers: each call waits for the previous call's compute and copy-out of a
    buffer before reusing it, so every call's result equals the device path's."""
    torch = torch_cuda
    from lprec_gb300.lpTransform import lpTransform
    S, N, Nproj, calls = 24, 256, 384, 4
    lp = lpTransform(N, Nproj, S, 'ramp', N / 2, 'cubic')
    lp.precompute(1)
    lp.initcmem(1, 0)
    rng = np.random.default_rng(5)
    fs = [torch.from_numpy(rng.random((S, N, N), dtype=np.float32)).pin_memory() for _ in range(calls)]
    Rs = [torch.from_numpy(rng.random((S, Nproj, N), dtype=np.float32)).pin_memory() for _ in range(calls)]
    Routs = [torch.empty((S, Nproj, N)).pin_memory() for _ in range(calls)]
    fouts = [torch.empty((S, N, N)).pin_memory() for _ in range(calls)]
    for i in range(calls):
        lp.fwd(fs[i], 0, out=Routs[i], chunk=4)
        lp.adj(Rs[i], 0, out=fouts[i], chunk=4)
    # chained: the adjoint's host input is the forward's host output, still being copied
    fc = lp.adj(lp.fwd(fs[0], 0, chunk=8), 0, chunk=8)
    torch.cuda.synchronize()
    Rd = torch.empty((S, Nproj, N), device='cuda')
    fd = torch.empty((S, N, N), device='cuda')
    lp.fwdp(Rd, fs[0].cuda(), 0)
    lp.adjp(fd, Rd, 0)
    assert torch.equal(fc, fd.cpu())
    for i in range(calls):
        Rd = torch.empty((S, Nproj, N), device='cuda')
        fd = torch.empty((S, N, N), device='cuda')
        lp.fwdp(Rd, fs[i].cuda(), 0)
        lp.adjp(fd, Rs[i].cuda(), 0)
        assert torch.equal(Routs[i], Rd.cpu()), i
        assert torch.equal(fouts[i], fd.cpu()), i


def test_uneven_batch_graph(torch_cuda):
    """Requests of different geometry in one CUDA graph == per-request calls."""
    torch = torch_cuda
    from lprec_gb300.batch import UnevenBatch
    from lprec_gb300.lpTransform import lpTransform
    reqs = [(64, 96, 2), (128, 192, 1), (64, 96, 3), (256, 384, 2)]
    b = UnevenBatch(reqs, 'ramp', 'cubic', 0)
    rng = np.random.default_rng(8)
    for i, (N, Nproj, S) in enumerate(reqs):
        b.input_f(i).copy_(torch.as_tensor(rng.random((S, N, N), dtype=np.float32)))
        b.input_R(i).copy_(torch.as_tensor(rng.random((S, Nproj, N), dtype=np.float32)))
    b.capture()
    b.run()
    torch.cuda.synchronize()
    lat = b.latencies_ms()
    assert lat is None or len(lat) == len(reqs)
    for i, (N, Nproj, S) in enumerate(reqs):
        lp = lpTransform(N, Nproj, S, 'ramp', N / 2, 'cubic')
        lp.precompute(1)
        lp.initcmem(1, 0)
        R = torch.zeros((S, Nproj, N), device='cuda')
        f = torch.zeros((S, N, N), device='cuda')
        lp.fwdp(R, b.input_f(i).contiguous(), 0)
        lp.adjp(f, b.input_R(i).contiguous(), 0)
        torch.cuda.synchronize()
        assert torch.equal(R, b.output_R(i)), i
        assert torch.equal(f, b.output_f(i)), i


@pytest.mark.parametrize("args", [(64, 70, 32, 'ramp'), (48, 36, 24, 'none'), (80, 100, 40, 'shepp-logan'),
                                  (64, 40, 32.5, 'hann')])
def test_prefilter_chunk_edges(torch_cuda, args):
    """Column lengths that end a few rows into a 64-row chunk's warm-up (H = 70, 72, 80)
    or fit one chunk (H = 40): the staged column prefilter's exact boundary
    initialisations against the oracle."""
    from lprec_gb300 import _lib
    N0, Nproj, cor, filt = args
    packed = _lib.precompute(N0, Nproj, 2, cor, 'cubic', filt, precision='fp64')
    h = _handle(packed)
    tr = O.Transform.from_packed(*packed)
    f, R = _inputs(tr.G, 2, 4)
    assert O.rel_l2(_fwd(torch_cuda, h, f), tr.fwd(f)) < TOL
    assert O.rel_l2(_adj(torch_cuda, h, R), tr.adj(R)) < TOL


@pytest.mark.parametrize("args", [(176, 264, 88, 'cubic', 'ramp'), (272, 408, 136, 'cubic', 'shepp-logan'),
                                  (208, 150, 104, 'linear', 'hann'), (368, 552, 184, 'cubic', 'parzen')])
def test_prime_radix_lengths(torch_cuda, args):
    """Padded sizes with a prime factor above 7 (176 = 16*11, 272 = 16*17, 208 = 16*13,
    368 = 16*23): the generic FFT's output-parallel odd-prime stage against the oracle."""
    from lprec_gb300 import _lib
    N0, Nproj, cor, interp, filt = args
    packed = _lib.precompute(N0, Nproj, 2, cor, interp, filt, precision='fp64')
    h = _handle(packed)
    tr = O.Transform.from_packed(*packed)
    f, R = _inputs(tr.G, 2, 6)
    assert O.rel_l2(_fwd(torch_cuda, h, f), tr.fwd(f)) < TOL
    assert O.rel_l2(_adj(torch_cuda, h, R), tr.adj(R)) < TOL


@pytest.mark.parametrize("args", [(512, 768, 'cubic', 'shepp-logan', 253), (1008, 1512, 'linear', 'hann', 504),
                                  (1536, 2304, 'cubic', 'ramp', 768), (2016, 3024, 'cubic', 'parzen', 1008),
                                  (2048, 1024, 'cubic', 'shepp-logan', 1021), (512, 768, 'cubic', 'ramp', 243),
                                  (1024, 1536, 'linear', 'shepp-logan', 509), (1024, 1536, 'cubic', 'hann', 500),
                                  (2048, 1024, 'cubic', 'shepp-logan', 1012), (1280, 1920, 'cubic', 'ramp', 640),
                                  (2560, 768, 'linear', 'shepp-logan', 1280)])
def test_mixed_radix_lengths(torch_cuda, args):
    """Padded sizes that are not powers of two, served by the mixed-radix register FFT:
    N = 528 = 16*3*11 (an off-centre axis at N0 = 512), 1008 = 16*63, 1536 = 16*96,
    2016 = 16*126, 2064 = 16*3*43 (an axis 3 pixels off centre at N0 = 2048: the prime
    43 takes the output-parallel stage), 544 = 16*2*17, 1040 = 16*5*13, 1056 (Nrho 2112)
    and 2080 = 16*2*5*13 (axes 3 to 16 pixels off centre), the detector widths 1280 and
    2560 = 16*32*5, Nrho = 2N; one slice each against the oracle."""
    from lprec_gb300 import _lib
    N0, Nproj, interp, filt, cor = args
    packed = _lib.precompute(N0, Nproj, 1, cor, interp, filt, precision='fp64')
    h = _handle(packed)
    tr = O.Transform.from_packed(*packed)
    rng = np.random.default_rng(31)
    f = O.ellipse_phantom(N0, 10, rng)[None]
    Rg = _fwd(torch_cuda, h, f)
    assert O.rel_l2(Rg, tr.fwd(f)) < TOL, O.rel_l2(Rg, tr.fwd(f))
    Rn = Rg + 0.01 * np.abs(Rg).max() * rng.standard_normal(Rg.shape)
    fa = _adj(torch_cuda, h, Rn)
    assert O.rel_l2(fa, tr.adj(Rn)) < TOL, O.rel_l2(fa, tr.adj(Rn))
