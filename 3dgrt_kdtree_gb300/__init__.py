"""GB300-native (sm_103a) hybrid kd-tree Gaussian ray tracer.

A from-scratch implementation of the render hot path of
hydarlisk/3dgrt_kdtree: the host C++ library ``libkdgr.so`` (tree builder,
scene upload, serving loop) over hand-written CUDA kernels, behind the C ABI
declared in ``include/kdgr.h``.  The Python modules here are thin ctypes
bindings used by tests and benchmarks:

* :mod:`.capi`     -- ABI structs and strict library loading;
* :mod:`.kdtree`   -- kd-tree build / .kdt I/O;
* :mod:`.renderer` -- scenes, render calls, batches, autotuning;
* :mod:`.scenes`   -- seeded synthetic scenes and cameras.
"""
from . import capi, kdtree, renderer, scenes  # noqa: F401
