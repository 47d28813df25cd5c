"""GB300 (sm_103a) backend for the HyperPlonk prover hot path.

The product is libhp_cuda.so (C ABI, include/hp_cuda.h); this package holds
its CUDA sources (csrc/), the in-tree build (build.py) and the Python mirror
of the reference backend traits (backend.py, virtual_polynomial.py).
"""
from .errors import BackendError, InvalidParameters, InvalidState  # noqa: F401
from .virtual_polynomial import VirtualPolynomial, VPAuxInfo  # noqa: F401
