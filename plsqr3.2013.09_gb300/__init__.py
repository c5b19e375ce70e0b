"""GB300-native PLSQR3: the LSQR driver and aprod operator of PLSQR3 on one GPU.

The native library (csrc/, built into lib/libplsqr_gpu.so) does all the
work; this package binds its C ABI (_native), generates the synthetic
problems in the reference's formats (synth), converts ray kernels from their
ASCII exchange format (raykernels) and exposes the reference's
operator/driver interface (solver.Context).

The directory name is not a valid Python identifier; load it with
__graft_entry__.load_package(), which registers it as ``plsqr_gb300``.
"""
from . import _native, synth, solver, batch, multi, warm, raykernels  # noqa: F401
from .solver import Context  # noqa: F401
from .synth import CONFIGS, Problem, generate, read_files, write_files  # noqa: F401

__all__ = ["Context", "Problem", "generate", "read_files", "write_files", "CONFIGS"]
