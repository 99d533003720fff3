"""The library's strided elementwise kernel (fricc_combine) and zero fill
against torch FP64 on the iteration's patterns: permuted copies, linear
combinations, broadcast products, accumulation, several outputs, diagonal
views.  Inputs of one layout are summed in the order given, so a
combination whose inputs share a layout matches torch's left-to-right
expression bit for bit; inputs of different layouts are summed group by
group, within a few roundings of it."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def _close(got, ref, *terms):
    """|got - ref| within 4 roundings of the sum of the terms' magnitudes."""
    bound = 4 * torch.finfo(torch.float64).eps * sum(t.abs() for t in terms)
    return bool(((got - ref).abs() <= bound).all())


def _r(*shape, seed=0):
    g = torch.Generator(device="cuda").manual_seed(seed)
    return torch.randn(*shape, dtype=torch.float64, device="cuda", generator=g)


def test_permuted_copy_and_linear_combination(gpulib):
    from fricc_gb300.rccsd_dense import combine
    o, v = 5, 7
    R = _r(o * v * v, o, seed=1).view(o, v, v, o)
    Y = _r(v, o, o, v, seed=2)
    Z = _r(o, v, v, o, seed=3)
    out = torch.empty(v, o, o, v, dtype=torch.float64, device="cuda")       # [a,i,k,c]
    combine([out], [R.permute(2, 3, 0, 1), Y, Z.permute(2, 3, 0, 1)], [[1.0, -1.0, 1.0]])
    ref = R.permute(2, 3, 0, 1) - Y + Z.permute(2, 3, 0, 1)
    assert _close(out, ref, R.permute(2, 3, 0, 1), Y, Z.permute(2, 3, 0, 1))
    same = torch.empty_like(out)
    combine([same], [R.permute(2, 3, 0, 1), Z.permute(2, 3, 0, 1)], [[1.0, -1.0]])   # one layout: exact
    assert torch.equal(same, R.permute(2, 3, 0, 1) - Z.permute(2, 3, 0, 1))
    cp = torch.empty(o, o, v, v, dtype=torch.float64, device="cuda")
    combine([cp], [Y.permute(1, 2, 0, 3)])
    assert torch.equal(cp, Y.permute(1, 2, 0, 3).contiguous())


def test_broadcast_product_accumulate(gpulib):
    from fricc_gb300.rccsd_dense import combine
    o, v = 6, 9
    S = _r(v, v, seed=4)
    t1 = _r(o, v, seed=5)
    t2 = _r(o, o, v, v, seed=6)
    out = t2.clone()
    combine([out], [], [[1.0]], prod=[S[None, None, :, :], t1[:, None, :, None], t1[None, :, None, :]],
            accumulate=True)
    ref = t2 + S[None, None, :, :] * t1[:, None, :, None] * t1[None, :, None, :]
    assert torch.equal(out, ref)


def test_two_outputs_tt_pattern(gpulib):
    """tt = t2 + t1 (x) t1 in natural order and in [r,p,q,s] order in one pass."""
    from fricc_gb300.rccsd_dense import combine
    o, v = 4, 11
    t1 = _r(o, v, seed=7)
    t2 = _r(o, o, v, v, seed=8)
    tt = torch.empty_like(t2)
    ttp = torch.empty(v, o, o, v, dtype=torch.float64, device="cuda")
    combine([tt, ttp.permute(1, 2, 0, 3)], [t2], [[1.0, 1.0], [1.0, 1.0]],
            prod=[t1[:, None, :, None], t1[None, :, None, :]])
    ref = t2 + torch.einsum("pr,qs->pqrs", t1, t1)
    assert torch.equal(tt, ref)
    assert torch.equal(ttp, ref.permute(2, 0, 1, 3))


def test_three_outputs_and_diagonal(gpulib):
    from fricc_gb300.rccsd_dense import combine, zero
    o, v = 5, 8
    A = _r(v, o, o, v, seed=9)
    B = _r(v, o, v, o, seed=10)
    WA = torch.empty(o, v, o, v, dtype=torch.float64, device="cuda")
    WB = torch.empty_like(WA)
    W2 = torch.empty_like(WA)
    xa, xb = A.permute(1, 3, 2, 0), B.permute(1, 2, 3, 0)
    combine([WA, WB, W2], [xa, xb], [[1.0, 0.0], [0.0, 1.0], [2.0, -1.0]])
    assert torch.equal(WA, xa.contiguous()) and torch.equal(WB, xb.contiguous())
    assert torch.equal(W2, 2.0 * xa - xb)
    F = _r(o, o, seed=11)
    e = _r(o, seed=12)
    G = F.clone()
    combine([G.diagonal()], [e], [[-1.0]], accumulate=True)
    ref = F.clone()
    ref.diagonal().sub_(e)
    assert torch.equal(G, ref)
    zero(G)
    assert not G.any()


def test_bad_arguments_raise(gpulib):
    from fricc_gb300.rccsd_dense import combine
    a = torch.zeros(3, 4, dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError):
        combine([a], [a.float()])
    with pytest.raises(ValueError):
        combine([a], [a], [[1.0, 2.0]])
    with pytest.raises(ValueError):
        combine([a], [])


@pytest.mark.parametrize("shape", [(3, 5, 45, 37), (2, 1, 33, 70), (1, 1, 8, 8), (7, 9, 100, 9)])
def test_transposed_inputs_tiled(gpulib, shape):
    """Inputs contiguous along another dimension than the output's innermost
    one (read through shared-memory tiles), with odd sizes, a direct input,
    a broadcast product and accumulation."""
    from fricc_gb300.rccsd_dense import combine
    a, b, c, d = shape
    X = _r(a, b, d, c, seed=13)            # X.transpose(2, 3): contiguous along dim 2
    Y = _r(c, a, b, d, seed=14)            # Y.permute(1, 2, 0, 3): contiguous along dim 3
    Z = _r(d, c, b, a, seed=15)            # Z.permute(3, 2, 1, 0): contiguous along dim 0
    w = _r(d, seed=16)
    out0 = _r(a, b, c, d, seed=17)
    out = out0.clone()
    xs = [X.transpose(2, 3), Y.permute(1, 2, 0, 3), Z.permute(3, 2, 1, 0)]
    combine([out], xs, [[1.5, -1.0, 1.0, 2.0]], prod=[w[None, None, None, :], X.transpose(2, 3)], accumulate=True)
    ref = out0 + (((1.5 * xs[0] + (-xs[1])) + xs[2]) + 2.0 * (w * xs[0]))
    assert _close(out, ref, out0, 1.5 * xs[0], xs[1], xs[2], 2.0 * w * xs[0])
