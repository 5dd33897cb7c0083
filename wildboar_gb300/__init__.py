"""wildboar_gb300: wildboar's distance hot path on GB300 (sm_103a).

The public functions live in ``wildboar_gb300.distance`` with the reference's
signatures.  All arithmetic runs in libwbgpu.so (hand-written CUDA, C ABI in
include/wbgpu.h); the package raises if that library is unavailable.
"""

__version__ = "0.1.0"
