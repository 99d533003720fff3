"""Per-replica random streams equal the reference's libc srand/rand stream."""
import ctypes

from fricc_gb300.rng import GlibcRand


def test_glibc_stream_matches_srand_rand():
    libc = ctypes.CDLL(None)
    for seed in (1, 7, 12345, 2**31 - 1):
        g = GlibcRand(seed)
        libc.srand(ctypes.c_uint(seed))
        for _ in range(1000):
            assert g.rand() == libc.rand()


def test_independent_streams_and_first_draw():
    a, b = GlibcRand(1), GlibcRand(1)
    x = [a.uniform() for _ in range(5)]
    assert x == [b.uniform() for _ in range(5)]
    assert x[0] == 0.8401877171547095  # the first draw after srand(1)
    c = GlibcRand(2)
    assert c.uniform() != x[0]
