"""The oracle against the reference's own precompute and its test pins (CPU only)."""
import glob
import os

import numpy as np
import pytest

from oracle import lprec_oracle as O

NAMES = ['glpars', 'fwdparsi', 'fwdparamsf', 'adjparsi', 'adjparamsf']


def _cases(golden_dir):
    return sorted(glob.glob(os.path.join(golden_dir, 'packed_*.npz')))


def test_packed_tables_match_reference(golden_dir):
    """Oracle tables (mode 'ref') equal the reference precompute bit for bit."""
    files = _cases(golden_dir)
    assert len(files) >= 4
    for fn in files:
        z = np.load(fn)
        N0, Nproj, S, cor = z['args']
        tr = O.Transform(int(N0), int(Nproj), int(S), str(z['filter']), cor, str(z['interp']), mode='ref')
        for name, mine in zip(NAMES, tr.packed()):
            ref = z[name]
            assert mine.shape == ref.shape, (fn, name)
            assert np.array_equal(mine, ref), (fn, name, int(np.sum(mine != ref)))


def test_unpack_roundtrip(golden_dir):
    for fn in _cases(golden_dir):
        z = np.load(fn)
        arrs = [z[n] for n in NAMES]
        tr = O.Transform.from_packed(*arrs)
        for a, b in zip(tr.packed(), arrs):
            assert np.array_equal(a, b)


def test_fp64_mode_same_index_sets():
    a = O.Transform(64, 96, 1, 'ramp', 32, 'cubic', mode='ref')
    b = O.Transform(64, 96, 1, 'ramp', 32, 'cubic', mode='fp64')
    for key in ('cids', 'pids'):
        for x, y in zip(np.atleast_1d(a.Tf[key]) if key == 'cids' else a.Tf[key],
                        np.atleast_1d(b.Tf[key]) if key == 'cids' else b.Tf[key]):
            assert np.array_equal(x, y)
    for key in ('cids', 'lpids', 'wids'):
        assert np.array_equal(a.Ta[key], b.Ta[key])
    for key in ('lp2C1', 'p2lp2', 'C2lp1', 'lp2p2w'):
        T = a.Tf if key in a.Tf else a.Ta
        U = b.Tf if key in b.Tf else b.Ta
        for x, y in zip(T[key], U[key]):
            assert np.max(np.abs(x - y)) < 2e-3


def test_prefilter_interpolates():
    """Cubic B-spline coefficients reproduce the samples at the grid points (away from the edges)."""
    rng = np.random.default_rng(3)
    img = rng.random((1, 40, 48))
    c = O.prefilter2d(img)
    yy, xx = np.meshgrid(np.arange(40), np.arange(48), indexing='ij')
    v = O.interp2d(c, xx.ravel(), yy.ravel(), True).reshape(40, 48)
    inner = (slice(14, 26), slice(14, 34))
    assert np.max(np.abs(v[inner] - img[0][inner])) < 1e-9


def test_apply_filter_is_circular_convolution():
    """The shift/FFT sequence of applyFilter equals irfft(rfft(pad(x)) * filter[(k+2N) mod 4N])."""
    G = O.create_geometry(32, 48, 1, 16, 'cubic')
    filt = O.take_filter(G.N, 'shepp-logan')
    rng = np.random.default_rng(1)
    R = rng.random((2, G.Nproj, G.N))
    a = O.apply_filter(G, R, filt)
    M = 4 * G.N
    pad = np.zeros((2, G.Nproj, M))
    pad[..., :G.N] = R
    H = filt[(np.arange(M) + 2 * G.N) % M]
    b = np.fft.ifft(np.fft.fft(pad, axis=-1) * H, axis=-1).real[..., :G.N]
    assert np.max(np.abs(a - b)) < 1e-12 * np.max(np.abs(a))


@pytest.mark.slow
def test_reference_pins_adj_many(golden_dir):
    """tests/test_adj_many.py pins (run_test.py:18-20) on the reference's own data."""
    d = np.load(os.path.join(golden_dir, 'testdata.npz'))
    f = d['f'][None].astype(np.float64)
    R = d['R'][None].astype(np.float64)
    tr = O.Transform(512, 384, 1, 'none', 256, 'cubic')
    Rf = tr.fwd(f)
    fR = tr.adj(R)
    RfR = tr.fwd(fR)
    err0 = abs(np.sum(Rf * R) - np.sum(fR * f)) / abs(np.sum(fR * f))
    err1 = O.rel_l2(fR, f)
    err2 = O.rel_l2(RfR, Rf)
    assert err0 < 5e-3 and err1 < 7e-3 and err2 < 7e-4, (err0, err1, err2)


@pytest.mark.slow
def test_reference_pin_adj_ptr():
    """tests/test_adj_ptr.py pin (run_test.py:14-16): random dot test < 1e-2."""
    rng = np.random.default_rng(0)
    f = rng.random((1, 512, 512)).astype(np.float32).astype(np.float64)
    R = rng.random((1, 768, 512)).astype(np.float32).astype(np.float64)
    tr = O.Transform(512, 768, 1, 'none', 256, 'cubic')
    err = abs(np.sum(tr.fwd(f) * R) - np.sum(tr.adj(R) * f)) / abs(np.sum(tr.adj(R) * f))
    assert err < 1e-2


def test_prefilter_transpose_matches_matrix():
    for L in (5, 13, 40):
        M = O.prefilter_lines(np.eye(L), 0)          # column j = filter applied to e_j
        y = np.random.default_rng(L).standard_normal(L)
        assert np.allclose(O.prefilter_lines_T(y[:, None], 0)[:, 0], M.T @ y, atol=1e-12)


@pytest.mark.parametrize("args", [(48, 72, 'cubic', 21), (32, 24, 'linear', 16), (64, 96, 'cubic', 32)])
def test_fwd_transpose_dot(args):
    """<fwd f, g> == <f, fwd_T g> in float64 (exact discrete transpose)."""
    N0, Nproj, interp, cor = args
    tr = O.Transform(N0, Nproj, 1, 'none', cor, interp)
    rng = np.random.default_rng(2)
    f = rng.standard_normal((2, N0, N0))
    g = rng.standard_normal((2, Nproj, N0))
    lhs = np.sum(tr.fwd(f) * g)
    rhs = np.sum(f * tr.fwd_T(g))
    assert abs(lhs - rhs) <= 1e-10 * abs(lhs)
