"""lprec_gb300: GB300-native log-polar Radon transform and back-projection.

Drop-in for lprec's ``lpTransform`` (precompute / initcmem / fwdp / adjp) and
the ``lpmethods`` solvers, backed by hand-written sm_103a CUDA kernels behind a
C ABI (include/lprec_gb300.h).  PyTorch supplies device tensors and streams.
"""
from . import lpTransform  # noqa: F401  (module, as in lprec: lpTransform.lpTransform(...))
from . import lpmethods  # noqa: F401
from . import autograd  # noqa: F401
from . import batch  # noqa: F401

__version__ = "0.1.0"
