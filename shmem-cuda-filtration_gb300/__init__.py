"""GB300-native hot path of the two-phase water/DNAPL porous-media flow step.

Import name: ``shmem_cuda_filtration_gb300`` (the directory name carries
hyphens, so it is loaded by path; see __graft_entry__.load_package()).

Layers:
  csrc/    CUDA kernels for sm_103a, the extern "C" ABI (include/gbflow.h) and
           the reference's defines.h host function set (C++ linkage).
  abi.py   ctypes mirror of include/gbflow.h and the library loader.
  build.py nvcc recipe that builds _build/libgbflow.so in-tree.
"""
from . import abi  # noqa: F401
from .abi import load_library, reference_model  # noqa: F401
