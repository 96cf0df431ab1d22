"""xin26x_gb300 -- the xin26x VVC encoder pixel hot path on a GB300 GPU.

The product is the C-ABI CUDA library libxingpu{8,10}.so (include/xingpu.h):
per-call drop-ins for the reference's xin_func_struct / xin_me_func entries,
ME drivers on the reference's xin_me_struct, and the batched frame form.
This package builds it (build.py), binds it (_lib.py) and wraps the frame form
(frame.py).  It has no CPU fallback: load() raises when the library is missing.
"""
from ._lib import load, check  # noqa: F401
