"""Generate the golden fixtures under tests/golden/ from the lprec reference.

Run where the lprec sources are available, naming their root directory
(the one holding src/lprec and tests/data) by argument or by LPREC_REFERENCE:

    python tests/golden/make_golden.py <lprec-root>

What it writes:

* ``packed_<case>.npz`` -- the reference's own packed parameter arrays
  (``glpars``, ``fwdparsi``, ``fwdparamsf``, ``adjparsi``, ``adjparamsf``) as
  returned by src/lprec/initsgl.py:create_gl, initsfwd.py:create_fwd and
  initsadj.py:create_adj.  CuPy is not installed, so the reference modules are
  imported with NumPy standing in for CuPy (``cupy`` -> ``numpy`` and
  ``.get()`` -> identity); nothing else in them is changed.
* ``testdata.npz`` -- the reference's test inputs tests/data/f (512x512) and
  tests/data/R (384x512) as float32, used by the test_adj_many pins
  (tests/test_adj_many.py:53-62, tests/run_test.py:18-20).
* ``rfoam.npz`` -- the reference's measured foam sinogram tests/data/Rfoam
  (299 angles x 2016 samples, float32, in the [angle][s] order that
  tests/test_foam.py:39-41 reads it into), used by the test_foam pins
  (tests/run_test.py:28-32).
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

# cases: name -> (N0, Nproj, Nslices, cor, interp_type, filter_type)
CASES = {
    'n64_cubic_ramp': (64, 96, 1, 32, 'cubic', 'ramp'),
    'n48_cor_shepp': (48, 72, 1, 21, 'cubic', 'shepp-logan'),
    'n32_os2_linear_hann': (32, 24, 1, 16, 'linear', 'hann'),
    'n64_cubic_none': (64, 64, 1, 32.0, 'cubic', 'none'),
    # the small benchmark configuration: one slice N=256, 384 angles, centred, ramp
    'n256_cubic_ramp': (256, 384, 1, 128, 'cubic', 'ramp'),
    'n48_cubic_cosine': (48, 80, 1, 24, 'cubic', 'cosine'),
    'n48_cubic_cosine2': (48, 64, 1, 25, 'cubic', 'cosine2'),
}


def reference_root():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get('LPREC_REFERENCE')
    if not ref or not os.path.isdir(os.path.join(ref, 'src', 'lprec')):
        sys.exit('usage: make_golden.py <lprec-root>  (or set LPREC_REFERENCE)')
    return ref


def load_reference(REF):
    cp = types.ModuleType('cupy')
    for k in dir(np):
        try:
            setattr(cp, k, getattr(np, k))
        except Exception:
            pass
    sys.modules['cupy'] = cp
    sys.path.insert(0, os.path.join(REF, 'src'))
    from lprec import initsgl, initsfwd, initsadj
    for mod in (initsgl, initsfwd, initsadj):
        src = open(mod.__file__).read().replace('.get()', '')
        exec(compile(src, mod.__file__, 'exec'), mod.__dict__)
    return initsgl, initsfwd, initsadj


def main():
    REF = reference_root()
    initsgl, initsfwd, initsadj = load_reference(REF)
    for name, (N0, Nproj, S, cor, interp, filt) in CASES.items():
        P, glpars = initsgl.create_gl(N0, Nproj, S, cor, interp)
        _, fi, ff = initsfwd.create_fwd(P)
        _, ai, af = initsadj.create_adj(P, filt)
        np.savez_compressed(os.path.join(HERE, 'packed_%s.npz' % name),
                            glpars=np.asarray(glpars, np.float32), fwdparsi=fi, fwdparamsf=ff,
                            adjparsi=ai, adjparamsf=af,
                            args=np.array([N0, Nproj, S, cor], dtype=np.float64),
                            interp=np.array(interp), filter=np.array(filt))
        print(name, 'N=%d os=%d' % (P.N, P.osangles), fi.shape, ff.shape, ai.shape, af.shape)
    f = np.fromfile(os.path.join(REF, 'tests/data/f'), dtype='<f4').reshape(512, 512)
    R = np.fromfile(os.path.join(REF, 'tests/data/R'), dtype='<f4').reshape(384, 512)
    np.savez_compressed(os.path.join(HERE, 'testdata.npz'), f=f, R=R)
    # tests/test_foam.py:39-41: Nproj*N floats read as [Ns, N, Nproj], then swapaxes(1, 2)
    Rfoam = np.fromfile(os.path.join(REF, 'tests/data/Rfoam'), dtype='<f4')[:299 * 2016]
    Rfoam = Rfoam.reshape(2016, 299).T.copy()
    np.savez_compressed(os.path.join(HERE, 'rfoam.npz'), R=Rfoam)


if __name__ == '__main__':
    main()
