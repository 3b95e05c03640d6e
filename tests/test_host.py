"""Host side of the library, no GPU: the C ABI exports, the C++ precompute
against the oracle and the reference's own tables, argument checking."""
import ctypes
import glob
import os
import re
import sys
import time

import numpy as np
import pytest

from oracle import lprec_oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NAMES = ['glpars', 'fwdparsi', 'fwdparamsf', 'adjparsi', 'adjparamsf']


@pytest.fixture(scope="module")
def lib():
    from lprec_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from lprec_gb300 import build
        build.build()
    return _lib


def _declared():
    names = []
    for hdr in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(hdr).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+char\s*\*|int|long long|int64_t|void)\s*\*?\s*(lp_\w+)\s*\(",
                            text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(lib):
    names = _declared()
    assert len(names) >= 20, names
    so = ctypes.CDLL(lib.LIB_PATH)
    missing = [n for n in names if not hasattr(so, n)]
    assert not missing, missing
    # the Python binding declares a signature for each of them
    assert set(names) <= set(lib.EXPORTS), sorted(set(names) - set(lib.EXPORTS))


def test_version_and_kernel_names(lib):
    L = lib.lib()
    assert L.lp_version() >= 100
    n = L.lp_kernel_count()
    names = [L.lp_kernel_name(i).decode() for i in range(n)]
    for k in ("fwd_c2lp", "theta_conv", "fwd_lp2polar", "adj_polar2lp", "adj_lp2cart"):
        assert k in names
    assert L.lp_kernel_name(n) == b""


@pytest.mark.parametrize("args", [(64, 96, 1, 32, 'cubic', 'ramp'), (48, 72, 2, 21, 'cubic', 'shepp-logan'),
                                  (32, 24, 1, 16, 'linear', 'hann'), (64, 96, 3, 32, 'cubic', 'none'),
                                  (80, 60, 1, 37, 'linear', 'parzen')])
def test_precompute_fp64_equals_oracle(lib, args):
    """C++ float64 precompute against the oracle's float64 tables rounded once: index
    arrays, geometry, e^rho and every interpolation coordinate bit for bit; the FFT-made
    kernels fZ to 1e-6 of their maximum (FFT round-off moves the last bit of small
    entries); the FBP filter to 1e-5 (its quadrature weights invert an ill-conditioned
    12x12 moment matrix, initsadj.py:128-144, by LAPACK in one and Gauss-Jordan in the
    other)."""
    N0, Nproj, S, cor, interp, filt = args
    mine = lib.precompute(N0, Nproj, S, cor, interp, filt, precision='fp64')
    tr = O.Transform(N0, Nproj, S, filt, cor, interp, mode='fp64', rounded=True)
    ref = tr.packed()
    for name, a, b in zip(NAMES, mine, ref):
        assert a.shape == b.shape, name
        if name.endswith('i') or name == 'glpars':
            assert np.array_equal(a, b), name
    _, Tf_a, Ta_a, _ = O.unpack_params(*mine)
    _, Tf_b, Ta_b, _ = O.unpack_params(*ref)
    for Ta, Tb in ((Tf_a, Tf_b), (Ta_a, Ta_b)):
        for key in Tb:
            x, y = Ta[key], Tb[key]
            if key == 'fZ':
                assert np.max(np.abs(x - y)) <= 1e-6 * np.max(np.abs(y)), key
            elif key == 'filter':
                assert (x is None) == (y is None)
                if y is not None:
                    assert np.linalg.norm(x - y) <= 1e-5 * np.linalg.norm(y), key
            else:
                for u, v in zip(np.atleast_1d(x) if not isinstance(x, list) else x,
                                np.atleast_1d(y) if not isinstance(y, list) else y):
                    assert np.array_equal(u, v), key


def test_precompute_reference_mode_against_reference_tables(lib, golden_dir):
    """C++ reference-precision precompute against the reference's own packed arrays:
    identical integer arrays (index sets, sizes); float arrays within a few ulp except
    fZ, whose float32 cos (NumPy's, not correctly rounded) leaves ~1e-5 relative."""
    files = sorted(glob.glob(os.path.join(golden_dir, 'packed_*.npz')))
    assert files
    for fn in files:
        z = np.load(fn)
        N0, Nproj, S, cor = z['args']
        mine = lib.precompute(int(N0), int(Nproj), int(S), float(cor), str(z['interp']), str(z['filter']),
                              precision='reference')
        for name, a in zip(NAMES, mine):
            ref = z[name]
            assert a.shape == ref.shape, (fn, name)
            if name.endswith('i'):
                assert np.array_equal(a, ref), (fn, name)
            else:
                err = np.linalg.norm(a.astype(np.float64) - ref) / np.linalg.norm(ref)
                assert err < 5e-5, (fn, name, err)


def test_precompute_rejects_bad_arguments(lib):
    with pytest.raises(lib.LprecError, match="filter"):
        lib.precompute(64, 96, 1, 32, 'cubic', 'no-such-filter')
    with pytest.raises(lib.LprecError):
        lib.precompute(0, 96, 1, 32, 'cubic', 'ramp')
    with pytest.raises(lib.LprecError):
        lib.precompute(64, 0, 1, 32, 'cubic', 'ramp')


def test_create_rejects_malformed_glpars(lib):
    """Validation happens before any device work, so it runs without a GPU."""
    gl = lib.precompute(64, 96, 1, 32, 'cubic', 'ramp')[0].copy()
    with pytest.raises(lib.LprecError):
        lib.Handle(gl[:5], 0)
    bad = gl.copy()
    bad[4] = 4  # Nspan other than 3
    with pytest.raises(lib.LprecError, match="Nspan"):
        lib.Handle(bad, 0)
    bad = gl.copy()
    bad[0] = 72  # N not a power of the layout rules / inconsistent Ntheta
    with pytest.raises(lib.LprecError):
        lib.Handle(bad, 0)


def test_null_handle_calls_return_errors(lib):
    L = lib.lib()
    assert L.lp_fwd(None, None, None, 1, None) == 1
    assert L.lp_adj(None, None, None, 1, None) == 1
    assert L.lp_set_schedule(None, None, 0) == 1
    assert b"null" in L.lp_last_error()
    assert L.lp_destroy(None) == 0


def test_graph_watchdog_times_out_on_host():
    """The uneven-batch watchdog on a fake event that never completes (no GPU involved)."""
    from lprec_gb300.batch import wait_event

    class Never:
        def query(self):
            return False

    class After:
        def __init__(self, n):
            self.n = n

        def query(self):
            self.n -= 1
            return self.n <= 0

    t = [0.0]

    def clock():
        return t[0]

    def sleep(dt):
        t[0] += dt
    with pytest.raises(TimeoutError):
        wait_event(Never(), 0.05, poll_s=0.01, clock=clock, sleep=sleep)
    assert 0.05 <= t[0] < 0.07
    t[0] = 0.0
    wait_event(After(3), 1.0, poll_s=0.01, clock=clock, sleep=sleep)
    assert t[0] < 0.05


@pytest.mark.parametrize("S,c", [(128, 32), (128, 16), (7, 3), (1, 32), (5, 1), (100, 32), (33, 32), (128, 64)])
def test_pipeline_chunks(S, c):
    """The host pipeline's chunk sizes cover the slices once, never above c, growing
    to their largest and shrinking after it (short first and last copies)."""
    from lprec_gb300.lpTransform import pipeline_chunks
    sizes = pipeline_chunks(S, c)
    assert sum(sizes) == S and max(sizes) <= c and min(sizes) >= 1
    top = sizes.index(max(sizes))
    assert sizes[:top + 1] == sorted(sizes[:top + 1])
    assert sizes[top:] == sorted(sizes[top:], reverse=True)
    if S >= 2 * c >= 16:
        assert sizes[0] <= c // 8 and sizes[-1] <= c // 8
    with pytest.raises(ValueError):
        pipeline_chunks(0, c)


def test_host_pipeline_rejects_bad_arrays():
    """lpTransform.fwd/adj on host arrays check dtype and shape against the handle
    before any device work (a stand-in handle carries the geometry)."""
    pytest.importorskip("torch")
    from lprec_gb300.lpTransform import lpTransform

    class Geometry:
        N0, Nproj, Nslices = 8, 12, 4
    lp = lpTransform(8, 12, 4, 'ramp', 4, 'cubic')
    lp.clphandle[0] = Geometry()
    with pytest.raises(ValueError, match="input must be"):
        lp.fwd(np.zeros((2, 8, 9), np.float32), 0)
    with pytest.raises(ValueError, match="input must be"):
        lp.adj(np.zeros((2, 8, 8), np.float32), 0)
    import torch
    with pytest.raises(ValueError, match="float32"):
        lp.fwd(torch.zeros((2, 8, 8), dtype=torch.float64), 0)
    with pytest.raises(ValueError, match="out has shape"):
        lp.fwd(torch.zeros((2, 8, 8)), 0, out=torch.zeros((2, 12, 9)))
    with pytest.raises(TypeError):
        lp.adj(torch.zeros((2, 12, 8)), 0, out=np.zeros((2, 8, 8), np.float32))
    lp.clphandle[0] = None


def test_uneven_request_grouping():
    """Requests of the same geometry share one handle and one graph segment, smallest
    geometry first, fewest slices first within a geometry; each request keeps its slice
    range in its group; waves pack consecutive requests up to the slice budget, and the
    last request can be split off into a wave of its own."""
    pytest.importorskip("torch")
    from lprec_gb300.batch import group_requests, plan_waves
    reqs = [(512, 768, 2), (256, 384, 3), (512, 768, 1), (256, 384, 4), (1024, 96, 1)]
    groups, where = group_requests(reqs)
    assert groups == [(256, 384, 7, [1, 3]), (512, 768, 3, [2, 0]), (1024, 96, 1, [4])]
    assert where == {1: (0, 0, 3), 3: (0, 3, 4), 2: (1, 0, 1), 0: (1, 1, 2), 4: (2, 0, 1)}
    with pytest.raises(ValueError):
        group_requests([(256, 384, 0)])
    big = [(2048, 3000, s) for s in (5, 20, 9, 40, 3)]
    (_, _, total, idx), = group_requests(big)[0]
    assert idx == [4, 0, 2, 1, 3] and total == 77
    waves = plan_waves(big, idx, 2048, 32)
    assert waves == [(0, 17, [4, 0, 2]), (17, 37, [1]), (37, 77, [3])]
    assert plan_waves(big, idx, 1024, 32) == [(0, 77, [4, 0, 2, 1, 3])]
    # no bound: one wave; the last request alone at the end on request
    assert plan_waves(big, idx, 2048) == [(0, 77, [4, 0, 2, 1, 3])]
    assert plan_waves(big, idx, 2048, None, True) == [(0, 37, [4, 0, 2, 1]), (37, 77, [3])]
    assert plan_waves(big, idx, 2048, 32, True) == waves  # its last wave is one request already
    assert plan_waves(big[:1], [0], 2048, None, True) == [(0, 5, [0])]


@pytest.mark.parametrize("precision", ["fp64", "reference"])
def test_precompute_thread_count_invariant(lib, precision):
    """The tables are built row-parallel and concatenated in row order: one thread and
    all threads give the same arrays, bit for bit."""
    args = (176, 264, 1, 88.5, 'cubic', 'cosine')
    one = lib.precompute(*args, precision=precision, nthreads=1, wide=precision == "fp64")
    many = lib.precompute(*args, precision=precision, nthreads=0, wide=precision == "fp64")
    for a, b in zip(one, many):
        assert a.dtype == b.dtype and np.array_equal(a, b, equal_nan=True)


def test_c_header_compiles_and_links(lib, tmp_path):
    """include/lprec_gb300.h is plain C (what a cgo/JNI/C caller includes): a C99 program
    includes it, links liblprec_gb300.so and calls host-only entry points."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "abi.c"
    src.write_text(r'''
#include <stdio.h>
#include "lprec_gb300.h"
int main(void) {
  int64_t sizes[5];
  if (lp_version() < 100) return 2;
  if (lp_precompute_sizes(64, 96, 1, 32.0, 1, "ramp", sizes) != LP_OK) return 3;
  if (lp_precompute_sizes(64, 96, 1, 32.0, 1, "no-such-filter", sizes) == LP_OK) return 4;
  if (lp_last_error()[0] == 0) return 5;
  printf("%lld %lld %lld %lld %lld\n", (long long)sizes[0], (long long)sizes[1], (long long)sizes[2],
         (long long)sizes[3], (long long)sizes[4]);
  return 0;
}
''')
    exe = tmp_path / "abi"
    libdir = os.path.dirname(lib.LIB_PATH)
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                    "-L", libdir, "-llprec_gb300", "-Wl,-rpath," + libdir], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, (out.returncode, out.stderr)
    got = [int(v) for v in out.stdout.split()]
    arrays = lib.precompute(64, 96, 1, 32.0, 'cubic', 'ramp')
    assert got == [a.size for a in arrays]


def test_bench_clock_sampler(tmp_path, monkeypatch):
    """The bench's clock record: samples of a stand-in nvidia-smi (one per 100 ms),
    the first one present before the timed region starts, median and maximum clock and
    the active throttle reasons; a second summary() returns the same record."""
    fake = tmp_path / "nvidia-smi"
    fake.write_text("#!/bin/sh\nwhile true; do echo '0, 1965, 2070, 900.5, 0x4, Not Active, Not Active, "
                    "Not Active, Active'; sleep 0.1; done\n")
    fake.chmod(0o755)
    monkeypatch.setenv("PATH", str(tmp_path) + os.pathsep + os.environ.get("PATH", ""))
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), ".."))
    import bench
    with bench.Clocks(0) as clk:
        assert clk._lines() >= 1
        time.sleep(0.35)
    first = clk.summary()
    assert first["sm_mhz"] == 1965 and first["sm_max_mhz"] == 2070 and first["samples"] >= 2
    assert first["reasons"] == ["sw_power_cap"]
    assert clk.summary() == first
