"""The oracle's restricted outer-pair loops (the CPU baseline's samples):
blocks of outer pairs, or every s-th pair from an offset, add up bit for bit
to the whole term, since every output element belongs to one outer pair."""
import numpy as np
import pytest

TERMS = ["0101", "2323", "1302", "1202", "1303", "1203", "1323", "0112", "0113", "0313", "0312"]


def _w_shape(term, o, v):
    return {"0101": (o, o, o, o), "2323": (v, v, v, v), "1323": (o, v, o, v)}.get(
        term, (v, o, o, v) if term in ("1302", "1303") else (o, v, o, v) if term[:2] in ("01", "03") else (v, o, v, o))


def _out_shape(term, o, v):
    return {"1323": (o, o, o, o), "0112": (v, o, o, v), "0113": (v, o, o, v), "0313": (v, o, o, v),
            "0312": (v, o, v, o)}.get(term, (o, o, v, v))


@pytest.mark.parametrize("term", TERMS)
def test_blocks_and_strides_add_up_to_the_term(oracle, term):
    o, v = 4, 6
    rng = np.random.default_rng(3)
    t2 = rng.standard_normal((o, o, v, v))
    T = oracle.SparseTensor4d(t2, t2.shape, 150, "fri", "systematic", rn=0.25)
    W = rng.standard_normal(_w_shape(term, o, v))
    full = np.zeros(_out_shape(term, o, v))
    oracle.contract_DTSpT(W, T, full, term)
    n = oracle.outer_size(term, T.dims, W.shape)
    for plan in ([(0, n // 3), (n // 3, n)], [(0, n, 3), (1, n, 3), (2, n, 3)]):
        out = np.zeros_like(full)
        for r in plan:
            oracle.contract_DTSpT(W, T, out, term, outer_range=r)
        assert np.array_equal(out, full)
