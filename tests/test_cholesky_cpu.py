"""Host logic of the tensor-core path (no GPU): tile counts, the K-split
policy, the operand layouts' sizes."""
from fricc_gb300 import cholesky as C


def test_tiles_and_kp():
    assert C._tiles(128, 256) == 1 and C._tiles(129, 256) == 2 and C._tiles(128, 257) == 2
    assert C._tiles(1000, 30) == 8       # N <= 64: 128 x 64 tiles
    assert C._tiles(1000, 64) == 8 and C._tiles(1000, 65) == 8
    assert C._kp(150) == 456 and C._kp(8) == 24 and C._kp(1) == 8   # 3K rounded up to 8


def test_wave_efficiency():
    assert C._wave_eff(152) == 1.0 and C._wave_eff(304) == 1.0
    assert abs(C._wave_eff(160) - 160 / 304) < 1e-12


def test_ksplit_policy():
    # two rounds of tiles or more: no split
    assert C._ksplit(304, 3 * 22500) == 1 and C._ksplit(2041, 120000) == 1
    # a partial second round: split until the rounds are >= 90% busy
    ks = C._ksplit(160, 30000)
    assert ks > 1 and C._wave_eff(160 * ks) >= 0.9 and (C._kp(10000) // 64) // ks >= 8
    # one tile and a long K: spread over every SM
    assert C._ksplit(1, 3 * 675000) == 152
    # few tiles and a short K: the FP32-pair GEMM (0)
    assert C._ksplit(10, 3 * 100) == 0
    # each slice keeps >= 8 K blocks
    for tiles, kp in ((1, 64 * 40), (3, 64 * 100), (20, 64 * 300)):
        ks = C._ksplit(tiles, kp)
        assert ks >= 1 and (kp // 64) // ks >= 8


def test_ksplit_weighs_the_partials():
    # 128 tiles of a 2000 x 2000 output, K' = 6000: a split would fill the
    # idle SMs, but its FP32 partials (8 x 4M floats written and read back)
    # cost more than the round it saves
    assert C._ksplit(128, 6000) > 1
    assert C._ksplit(128, 6000, 2000 * 2000, 256) == 1
    # the O^2V^4 term at o20v100 (160 tiles, K' = 30000): still split, less
    ks = C._ksplit(160, 30000, 400 * 10000, 256)
    assert 1 < ks < C._ksplit(160, 30000)
    # a 20 x 20 output with a long K: every SM (its partials are tiny)
    assert C._ksplit(1, 600000, 400, 64) == 152


def test_dense_spmm_eligibility():
    # o10v40 terms: 2323 dense (long K), 0101 too small and short (falls back)
    dims = (10, 10, 40, 40)
    assert C.dense_spmm_ok(dims, 0, 1, 2, 3, 1600)
    assert not C.dense_spmm_ok(dims, 2, 3, 0, 1, 100)
