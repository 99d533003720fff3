"""Per-replica copies of the reference's random stream.

The reference draws its uniforms as ``rand() / RAND_MAX`` from libc's
process-global generator: one per systematic compression
(fri-cc src/fri_utils.cpp:47), one per visited element in pivotal sampling
(:73).  Independent replicas or requests need independent streams that are
still the reference's.  ``GlibcRand(seed)`` is glibc's default generator
(the additive lagged-Fibonacci "TYPE_3" of ``random``) restated: seeded as
``srand(seed)`` does (31 words from the Park-Miller recurrence
16807 x mod (2^31 - 1), Schrage's factorisation, then 310 outputs discarded),
then r_k = r_{k-31} + r_{k-3} mod 2^32 and ``rand() = r_k >> 1``.  Its state is
the 31-word history, which the GPU can take (``history()``) to generate a
long run of draws itself and hand back (``set_history``); the tests check
the stream against libc's ``srand``/``rand`` word for word.
"""
from __future__ import annotations

import numpy as np

RAND_MAX = 2147483647
_DEG, _SEP = 31, 3


def _c_div(a: int, b: int):
    """C's truncating division and remainder."""
    q = abs(a) // abs(b)
    q = q if (a >= 0) == (b >= 0) else -q
    return q, a - q * b


class GlibcRand:
    """An independent glibc rand() stream seeded like srand(seed)."""

    def __init__(self, seed: int):
        seed = int(seed) & 0xFFFFFFFF
        if seed == 0:
            seed = 1
        word = seed - (1 << 32) if seed >= 1 << 31 else seed  # the int32 glibc stores
        state = [word]
        for _ in range(1, _DEG):
            hi, lo = _c_div(word, 127773)
            word = 16807 * lo - 2836 * hi
            if word < 0:
                word += 2147483647
            state.append(word)
        # front pointer at index 3, rear at 0: the history starts at the front
        self._h = [state[(_SEP + t) % _DEG] & 0xFFFFFFFF for t in range(_DEG)]
        self._i = 0  # index of the oldest word
        for _ in range(10 * _DEG):
            self.rand()

    def rand(self) -> int:
        i = self._i
        w = (self._h[i] + self._h[(i + _DEG - _SEP) % _DEG]) & 0xFFFFFFFF
        self._h[i] = w
        self._i = (i + 1) % _DEG
        return w >> 1

    def uniform(self) -> float:
        """rand() / RAND_MAX, the reference's draw."""
        return float(self.rand()) / float(RAND_MAX)

    __call__ = uniform

    def history(self) -> np.ndarray:
        """The 31 words r[k-31..k-1] before the next draw (oldest first)."""
        return np.array([self._h[(self._i + t) % _DEG] for t in range(_DEG)], dtype=np.uint32)

    def set_history(self, h) -> None:
        h = np.asarray(h, dtype=np.uint32)
        if h.shape != (_DEG,):
            raise ValueError("a glibc history has 31 words")
        self._h = [int(v) for v in h]
        self._i = 0
