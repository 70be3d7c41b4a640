"""Oracle for the FFT-based 3D convolution — test infrastructure, not the product.

Importable only from the tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline / reference arm. See :mod:`oracle.fftconv`.
"""
from .fftconv import *  # noqa: F401,F403
from .fftconv import __all__  # noqa: F401
