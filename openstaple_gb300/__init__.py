"""GB300 (sm_103a) implementation of the OpenStaPLE rooted-staggered RHMC
fermion hot path: even/odd staggered Dirac operator, CG and multi-shift CG on
M^+M, mixed-precision and batched solvers, stout smearing and the rational
fermion force, behind the reference's C entry points (``include/ostaple_gb300.h``).

The compute path is the in-tree CUDA library ``libostaple_gb300.so``; this
package is its host-side Python mirror (ctypes), field generators and build.
"""
from . import fields  # noqa: F401

__all__ = ["fields", "api", "native", "build"]
