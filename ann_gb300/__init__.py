"""GB300 Behler-Parrinello energy/force library (Python binding of libann_gpu.so).

The compute path is the CUDA library ``ann_gb300/libann_gpu.so`` behind the C ABI declared in
``include/ann_gpu.h``; this package only loads it with ctypes and moves numpy arrays across.
There is no CPU fallback: if the library is missing or no CUDA device is present, the calls
raise ``AnnError``.
"""
from .api import (AnnError, Context, FP64, MIXED, NEWTON_ALL_IMAGES, NEWTON_UNTRANSLATED, build_library,
                  library_path, load_library)

__all__ = ["AnnError", "Context", "FP64", "MIXED", "NEWTON_ALL_IMAGES", "NEWTON_UNTRANSLATED", "build_library",
           "library_path", "load_library"]
