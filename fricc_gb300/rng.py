"""Per-replica copies of the reference's random stream.

The reference draws one uniform per systematic compression as
``rand() / RAND_MAX`` from libc's process-global generator
(fri-cc src/fri_utils.cpp:47).  Independent replicas or requests need
independent streams that are still the reference's: glibc's reentrant
``initstate_r(seed, state, 128, buf)`` + ``random_r`` with a private
128-byte state produce exactly the sequence ``srand(seed); rand(), rand(), ...``
(both use the same additive-feedback generator of degree 31).  The draws stay
on the host; the GPU never generates randomness.
"""
from __future__ import annotations

import ctypes

RAND_MAX = 2147483647

_libc = ctypes.CDLL(None)
_libc.initstate_r.argtypes = [ctypes.c_uint, ctypes.c_char_p, ctypes.c_size_t, ctypes.c_void_p]
_libc.random_r.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32)]


class GlibcRand:
    """An independent glibc rand() stream seeded like srand(seed)."""

    def __init__(self, seed: int):
        self._state = ctypes.create_string_buffer(128)
        self._data = ctypes.create_string_buffer(128)  # struct random_data, zeroed
        if _libc.initstate_r(ctypes.c_uint(seed), self._state, 128, self._data) != 0:
            raise OSError("initstate_r failed")
        self._out = ctypes.c_int32()

    def rand(self) -> int:
        _libc.random_r(self._data, ctypes.byref(self._out))
        return int(self._out.value)

    def uniform(self) -> float:
        """rand() / RAND_MAX, the reference's draw."""
        return float(self.rand()) / float(RAND_MAX)

    __call__ = uniform
