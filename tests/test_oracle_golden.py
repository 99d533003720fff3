"""The oracle (oracle/fri_oracle.c + oracle/ccsd_oracle.py) against golden
vectors produced by the reference's own C++ and fricc/friccsd.py
(tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest

from conftest import golden

TERMS = ("0101", "2323", "1302", "1202", "1303", "1203", "1323", "0112", "0113", "0313", "0312")


def test_compress_golden_bitexact(oracle):
    g = golden("compress.npz")
    n = int(g["n_cases"])
    assert n >= 15
    for k in range(n):
        x = g[f"c{k}_x"]
        m = int(g[f"c{k}_m"])
        for kind in ("fri", "largest"):
            rn = float(g[f"c{k}_{kind}_rn"]) if kind == "fri" else None
            t = oracle.SparseTensor4d(x, x.shape, m, kind, "systematic", rn=rn)
            ref_idx, ref_val = g[f"c{k}_{kind}_idx"], g[f"c{k}_{kind}_val"]
            np.testing.assert_array_equal(t.idx4, ref_idx, err_msg=f"case {k} {kind}")
            # bit for bit, NaN/inf included
            assert np.array_equal(t.vals.view(np.int64), ref_val.view(np.int64)), f"case {k} {kind}"


def test_contract_golden_bitexact(oracle):
    g = golden("contract.npz")
    for si in range(3):
        t2 = g[f"s{si}_t2"]
        m = int(g[f"s{si}_m"])
        T = oracle.SparseTensor4d(t2, t2.shape, m, "largest")
        for term in TERMS:
            W = g[f"s{si}_{term}_W"]
            for strided in (0, 1):
                Wuse = W if not strided else np.ascontiguousarray(W.transpose(3, 2, 1, 0)).transpose(3, 2, 1, 0)
                out = g[f"s{si}_{term}_init"].copy()
                oracle.contract_DTSpT(Wuse, T, out, term)
                np.testing.assert_array_equal(out, g[f"s{si}_{term}_out{strided}"], err_msg=f"{si} {term}")


def _iteration_system():
    from oracle import pyscf_standin as P
    g = golden("iteration.npz")

    class Sys:
        pass

    s = Sys()
    s.nocc = int(g["nocc"])
    s.L = g["L"]
    s.mo_energy = g["mo_energy"]
    s.nmo = s.mo_energy.size
    s.nvir = s.nmo - s.nocc
    s.fock = np.diag(s.mo_energy)
    from fricc_gb300.synthetic import SyntheticSystem
    s.eri = lambda b: SyntheticSystem.eri(s, b)
    s._sl = lambda c: SyntheticSystem._sl(s, c)
    s.naux = s.L.shape[0]
    return g, P.make_eris(s)


def test_iteration_golden_teacher_forced(oracle):
    """Every reference iterate, fed to the oracle update with the same draws,
    gives the next reference iterate."""
    from oracle import ccsd_oracle as CO
    g, eris = _iteration_system()
    settings = {"m_keep": int(g["m"]), "compression": "fri", "sampling_method": "systematic",
                "verbose": False, "compressed_contractions": ["O^2V^4", "O^3V^3", "O^4V^2"]}
    rn = list(g["rn"])
    t1s, t2s, E = g["t1"], g["t2"], g["energies"]
    from oracle import pyscf_standin as P
    for it in range(len(E)):
        draws = iter(rn[2 * it: 2 * it + 2])
        t1n, t2n = CO.update_amps(settings, t1s[it], t2s[it], eris, rn_draw=lambda: next(draws))
        np.testing.assert_allclose(t2n, t2s[it + 1], rtol=0, atol=1e-13)
        np.testing.assert_allclose(t1n, t1s[it + 1], rtol=0, atol=1e-13)
        assert abs(P.ccsd_energy(t1n, t2n, eris) - E[it]) < 1e-12


def test_iteration_golden_free_running(oracle):
    """The oracle's own loop, from the MP2 guess with the reference's draws,
    follows the reference trajectory to 1e-10 Eh."""
    from oracle import ccsd_oracle as CO
    g, eris = _iteration_system()
    settings = {"m_keep": int(g["m"]), "compression": "fri", "sampling_method": "systematic",
                "verbose": False, "compressed_contractions": ["O^2V^4", "O^3V^3", "O^4V^2"]}
    draws = iter(list(g["rn"]))
    conv, e, t1, t2, energies = CO.kernel(settings, eris, g["t1"][0], g["t2"][0], max_cycle=len(g["energies"]),
                                          rn_draw=lambda: next(draws))
    assert np.max(np.abs(np.array(energies) - g["energies"])) < 1e-10


LCCSD_VARIANTS = (("shared", False, False), ("independent", True, False), ("lccd", False, True))


def _lccsd_system():
    g = golden("lccsd.npz")
    from oracle import pyscf_standin as P
    from fricc_gb300.synthetic import SyntheticSystem

    class Sys:
        pass

    s = Sys()
    s.nocc = int(g["nocc"])
    s.L = g["L"]
    s.mo_energy = g["mo_energy"]
    s.nmo = s.mo_energy.size
    s.nvir = s.nmo - s.nocc
    s.fock = np.diag(s.mo_energy)
    s.naux = s.L.shape[0]
    s.eri = lambda b: SyntheticSystem.eri(s, b)
    s._sl = lambda c: SyntheticSystem._sl(s, c)
    return g, P.make_eris(s)


def _lccsd_settings(g, lccd, indep):
    return {"m_keep": int(g["m"]), "compression": "fri", "sampling_method": "systematic", "verbose": False,
            "compressed_contractions": ["O^2V^4", "O^3V^3", "O^4V^2"], "LCCD": lccd,
            "Independent Compressions": indep}


@pytest.mark.parametrize("name,indep,lccd", LCCSD_VARIANTS)
def test_lccsd_golden_teacher_forced(oracle, name, indep, lccd):
    """Each fricc/frilccsd.py iterate, fed to the oracle update with the same
    draws, gives the next one; the linear energy matches."""
    from oracle import lccsd_oracle as LO
    g, eris = _lccsd_system()
    settings = _lccsd_settings(g, lccd, indep)
    rn = list(g[f"{name}_rn"])
    per = 6 if indep else 1
    t1s, t2s, E = g[f"{name}_t1"], g[f"{name}_t2"], g[f"{name}_energies"]
    for it in range(len(E)):
        draws = iter(rn[per * it: per * it + per])
        t1n, t2n = LO.update_amps(settings, t1s[it], t2s[it], eris, rn_draw=lambda: next(draws),
                                  independent=indep, lccd=lccd)
        np.testing.assert_allclose(t2n, t2s[it + 1], rtol=0, atol=1e-13)
        np.testing.assert_allclose(t1n, t1s[it + 1], rtol=0, atol=1e-13)
        assert abs(LO.lin_cc_energy(t1n, t2n, eris) - E[it]) < 1e-12
    if lccd:
        assert not np.any(t1s[1:])


@pytest.mark.parametrize("name,indep,lccd", LCCSD_VARIANTS)
def test_lccsd_golden_free_running(oracle, name, indep, lccd):
    from oracle import lccsd_oracle as LO
    g, eris = _lccsd_system()
    draws = iter(list(g[f"{name}_rn"]))
    conv, e, t1, t2, energies = LO.kernel(_lccsd_settings(g, lccd, indep), eris, g[f"{name}_t1"][0],
                                          g[f"{name}_t2"][0], max_cycle=len(g[f"{name}_energies"]),
                                          rn_draw=lambda: next(draws), independent=indep, lccd=lccd)
    assert np.max(np.abs(np.array(energies) - g[f"{name}_energies"])) < 1e-10


def _unbiased_system():
    g = golden("unbiased.npz")
    from oracle import pyscf_standin as P
    from fricc_gb300.synthetic import SyntheticSystem

    class Sys:
        pass

    s = Sys()
    s.nocc = int(g["nocc"])
    s.L = g["L"]
    s.mo_energy = g["mo_energy"]
    s.nmo = s.mo_energy.size
    s.nvir = s.nmo - s.nocc
    s.fock = np.diag(s.mo_energy)
    s.naux = s.L.shape[0]
    s.eri = lambda b: SyntheticSystem.eri(s, b)
    s._sl = lambda c: SyntheticSystem._sl(s, c)
    return g, P.make_eris(s)


def test_unbiased_golden(oracle):
    """The running-average W compression after burn-in (fricc/friccsd.py:108-136):
    the oracle's loop follows the reference's trajectory, and teacher-forced
    steps (the average accumulating the reference's own inputs) match each iterate."""
    from oracle import ccsd_oracle as CO
    g, eris = _unbiased_system()
    settings = {"m_keep": int(g["m"]), "compression": "fri", "sampling_method": "systematic", "verbose": False,
                "compressed_contractions": ["O^2V^4", "O^3V^3", "O^4V^2"], "unbiased": True,
                "burn_in": int(g["burn_in"])}
    draws = iter(list(g["rn"]))
    conv, e, t1, t2, energies = CO.kernel(settings, eris, g["t1"][0], g["t2"][0], max_cycle=len(g["energies"]),
                                          rn_draw=lambda: next(draws))
    assert np.max(np.abs(np.array(energies) - g["energies"])) < 1e-10
    state = {}
    rn = list(g["rn"])
    for it in range(len(g["energies"])):
        d = iter(rn[2 * it: 2 * it + 2])
        t1n, t2n = CO.update_amps(settings, g["t1"][it], g["t2"][it], eris, rn_draw=lambda: next(d), state=state)
        np.testing.assert_allclose(t2n, g["t2"][it + 1], rtol=0, atol=1e-13)
    assert state["iter"] == len(g["energies"])
    # the average after burn-in: it=0 -> T2 input, it=1 -> reset to the input, then (1-1/it) Y + X/it
    b = int(g["burn_in"])
    y = g["t2"][b]
    for k in range(b + 1, len(g["energies"])):
        it = k - b
        y = g["t2"][k] / it + (it - 1) / it * y
    assert np.array_equal(state["t2_avg"], y)


def test_pivotal_golden_bitexact(oracle):
    """Pivotal sampling (the binding's default, src/fri_utils.cpp:63-127): the
    oracle, fed the reference's rand() stream, emits the reference's indices
    and values bit for bit and consumes the same number of draws."""
    from fricc_gb300.rng import GlibcRand
    g = golden("pivotal.npz")
    n = int(g["n_cases"])
    assert n >= 19
    for k in range(n):
        if not int(g[f"c{k}_ok"]):
            continue
        x, m, used = g[f"c{k}_x"], int(g[f"c{k}_m"]), int(g[f"c{k}_used"])
        r = GlibcRand(int(g[f"c{k}_seed"]))
        draws = np.array([r.uniform() for _ in range(x.size)])
        t = oracle.SparseTensor4d(x, x.shape, m, "fri", "pivotal", draws=draws)
        np.testing.assert_array_equal(t.idx4, g[f"c{k}_idx"], err_msg=f"case {k}")
        assert np.array_equal(t.vals.view(np.int64), g[f"c{k}_val"].view(np.int64)), f"case {k}"
        assert t.draws_used == used, (k, t.draws_used, used)


def test_parallel_sample_golden(oracle):
    """parallel_sample (src/fri_utils.cpp:176-362) at one chunk: the oracle fed
    the reference's rand() stream returns the reference's indices and consumes
    the same number of draws."""
    from fricc_gb300.rng import GlibcRand
    g = golden("parallel_sample.npz")
    n = int(g["n_cases"])
    assert n >= 10
    for k in range(n):
        assert int(g[f"c{k}_ok"])
        q, ns, seed = g[f"c{k}_q"], int(g[f"c{k}_n"]), int(g[f"c{k}_seed"])
        r = GlibcRand(seed)
        draws = np.array([r.uniform() for _ in range(q.size + 4)])
        S, used = oracle.parallel_sample(ns, q, 1, draws)
        np.testing.assert_array_equal(S, g[f"c{k}_S"], err_msg=f"case {k}")
        assert used == int(g[f"c{k}_used"]), (k, used)


EINSUM = {"0101": ("klij,klab->ijab", 1.0, "oooo"), "2323": ("abcd,ijcd->ijab", 1.0, "vvvv"),
          "1302": ("akic,kjcb->ijab", 2.0, "voov"), "1202": ("akci,kjcb->ijab", -1.0, "vovo"),
          "1303": ("akic,kjbc->ijab", 1.0, "voov"), "1203": ("bkci,kjac->ijab", 1.0, "vovo"),
          "1323": ("kcld,ijcd->klij", 1.0, "ovov"), "0112": ("ldkc,ilda->akic", -0.5, "ovov"),
          "0113": ("ldkc,ilad->akic", 1.0, "ovov"), "0313": ("lckd,ilad->akic", -0.5, "ovov"),
          "0312": ("lckd,ilda->akci", -0.5, "ovov")}


@pytest.mark.parametrize("no,nv,frac", [(4, 8, 0.1), (5, 10, 0.01), (10, 20, 0.001), (20, 40, 0.001)])
def test_oracle_terms_equal_einsum(oracle, no, nv, frac):
    """The reference's fricc/tests/test_sparse_tensors.py pattern on the
    oracle: every term on a "largest"-compressed T2 that keeps all nonzeros
    equals np.einsum of the dense T2 (:48-269; seed 20 as there)."""
    rng = np.random.default_rng(20)
    d = {"o": no, "v": nv}
    t2 = np.zeros(no * no * nv * nv)
    nnz = max(1, int(t2.size * frac))
    t2[rng.choice(t2.size, nnz, replace=False)] = rng.random(nnz)
    t2 = t2.reshape(no, no, nv, nv)
    T = oracle.SparseTensor4d(t2, t2.shape, nnz, "largest")
    for term in TERMS:
        spec, coef, wshape = EINSUM[term]
        W = rng.random(tuple(d[c] for c in wshape))
        ref = coef * np.einsum(spec, W, t2)
        out = np.zeros(ref.shape)
        oracle.contract_DTSpT(W, T, out, term)
        np.testing.assert_allclose(out, ref, rtol=1e-12, atol=1e-13 * max(1.0, np.abs(ref).max()), err_msg=term)


@pytest.mark.parametrize("no,nv,frac", [(4, 8, 0.1), (10, 15, 0.001), (100, 2, 0.001)])
def test_oracle_largest_elements_exact(oracle, no, nv, frac):
    """test_sparse_tensors.py:18-45: every kept (index, value) of a "largest"
    compression is the dense tensor's element at that index, and they are the
    m largest magnitudes."""
    rng = np.random.default_rng(20)
    a = rng.random((no, no, nv, nv))
    m = max(1, int(a.size * frac))
    T = oracle.SparseTensor4d(a, a.shape, m, "largest")
    for mi in range(m):
        idx, value = T.get_element(mi)
        assert value == a[tuple(idx)]
    kept = np.sort(np.abs(T.vals))
    assert np.array_equal(kept, np.sort(np.abs(a.ravel()))[-m:])


def test_oracle_replays_reference_driver_calls(oracle):
    """Every py_rccsd call of the reference's own fricc/friccsd.py (two
    iterations, tests/golden/dropin.npz) replayed through the oracle: the
    compressions bit for bit, the contractions bit for bit (the oracle keeps
    the reference's loop order)."""
    g = golden("dropin.npz")
    tensors = {}
    for i in range(int(g["n_calls"])):
        c = lambda key: g[f"c{i}_{key}"]  # noqa: E731
        if str(c("kind")) == "sp":
            x = np.ascontiguousarray(c("x"))
            T = oracle.SparseTensor4d(x, tuple(int(d) for d in c("dims")), int(c("m")), str(c("compression")),
                                      str(c("sampling")), rn=float(c("rn")))
            assert np.array_equal(T.idx4, c("idx"))
            assert np.array_equal(T.vals.view(np.int64), c("val").view(np.int64))
            tensors[int(c("k"))] = T
        else:
            W = np.ascontiguousarray(c("W")).copy().transpose(np.argsort(c("wperm")))
            out = np.ascontiguousarray(c("before")).copy().transpose(np.argsort(c("operm")))
            oracle.contract_DTSpT(W, tensors[int(c("sp"))], out, str(c("term")))
            want = np.ascontiguousarray(c("after")).transpose(np.argsort(c("operm")))
            assert np.array_equal(out, want), (i, str(c("term")))
