"""Generate the golden vectors in tests/golden/ from the reference itself.

Runs only where the reference checkout is available (it reads
/root/reference, or $FRICC_REFERENCE).  It compiles the reference's own
py_rccsd module from its sources (``make -C oracle ref``), imports it, and
records:

* compress.npz  -- SparseTensor4d("fri"/"largest") outputs (index slots and
                   values, bit for bit) on seeded inputs, with the libc
                   ``rand()`` draw each "fri" call consumed;
* contract.npz  -- contract_DTSpT outputs for all eleven terms, accumulated
                   in place into a non-zero output, including strided W;
* iteration.npz -- the reference's fricc/friccsd.py ``kernel`` run
                   unmodified (on the PySCF stand-in in oracle/) for a small
                   synthetic system: every iterate, every energy, every draw;
* lccsd.npz     -- the same for fricc/frilccsd.py (FRI-LCCSD): one shared
                   compression, six independent compressions, and LCCD.
* pivotal.npz   -- SparseTensor4d("fri", "pivotal") outputs (pivotal is the
                   binding's default) with the number of rand() draws each
                   consumed, the reference run in a forked child because its
                   sampler exits the process on its own errors;
* parallel_sample.npz -- the reference's parallel_sample (src/fri_utils.cpp:176-362)
                   at one thread, through oracle/_ref/ref_parallel_sample, on FRI
                   probability vectors, with the draws each call consumed;
* unbiased.npz  -- fricc/friccsd.py with "unbiased": True (running-average
                   W compression after burn-in), its missing iteration
                   counter supplied by the loop in this script.
* dropin.npz    -- every SparseTensor4d / contract_DTSpT call the unmodified
                   fricc/friccsd.py makes in two iterations, recorded at the
                   binding (arguments, draw, results), for replay through
                   fricc_gb300.py_rccsd.

Usage:  OMP_NUM_THREADS=1 python tests/golden/make_golden.py [--only-dropin]
"""
from __future__ import annotations

import ctypes
import importlib.util
import os
import subprocess
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("FRICC_REFERENCE", "/root/reference")
sys.path.insert(0, REPO)

from oracle import pyscf_standin  # noqa: E402
from fricc_gb300.synthetic import SyntheticSystem  # noqa: E402

TERMS = ("0101", "2323", "1302", "1202", "1303", "1203", "1323", "0112", "0113", "0313", "0312")
W_SHAPE = {"0101": "oooo", "2323": "vvvv", "1302": "voov", "1202": "vovo", "1303": "voov",
           "1203": "vovo", "1323": "ovov", "0112": "ovov", "0113": "ovov", "0313": "ovov",
           "0312": "ovov"}
OUT_SHAPE = {"1323": "oooo", "0112": "voov", "0113": "voov", "0313": "voov", "0312": "vovo"}


def load_reference_module():
    subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "ref", f"REF_DIR={REF}", "-s"],
                   check=True)
    sys.path.insert(0, os.path.join(REPO, "oracle", "_ref"))
    import py_rccsd  # the reference's own module
    return py_rccsd


def load_reference_friccsd(py_rccsd):
    pyscf_standin.install()
    pkg = types.ModuleType("fricc")
    pkg.__path__ = []
    sys.modules["fricc"] = pkg
    sys.modules["fricc.py_rccsd"] = py_rccsd
    spec = importlib.util.spec_from_file_location("fricc.friccsd",
                                                  os.path.join(REF, "fricc", "friccsd.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules["fricc.friccsd"] = mod
    spec.loader.exec_module(mod)
    return mod


libc = ctypes.CDLL(None)


def draws(seed, n):
    libc.srand(seed)
    return [libc.rand() / 2147483647.0 for _ in range(n)]


def ref_sparse(R, x, m, kind, seed):
    libc.srand(seed)
    t = R.SparseTensor4d(x, x.shape, m, kind, "systematic", False)
    idx = np.array([t.get_element(i)[0] for i in range(m)], dtype=np.int64).reshape(m, 4)
    val = np.array([t.get_element(i)[1] for i in range(m)], dtype=np.float64)
    return idx, val


def compress_cases(R):
    rng = np.random.default_rng(2024)
    cases = []
    # heavy-tailed small tensors, including ties, zeros, m = 1 and m = N
    for c in range(14):
        shp = tuple(int(s) for s in rng.integers(2, 7, size=4))
        n = int(np.prod(shp))
        x = rng.standard_normal(shp) * np.exp(2 * rng.standard_normal(shp))
        if c % 4 == 1:
            x = np.round(x)  # exact ties and zeros
        if c % 4 == 2:
            x[rng.random(shp) < 0.6] = 0.0
        m = {0: 1, 3: n}.get(c, int(rng.integers(1, n + 1)))
        cases.append((x, m))
    # MP2 amplitudes of small synthetic systems
    for (o, v, seed, frac) in ((6, 24, 1, 0.12), (6, 24, 2, 0.05), (5, 20, 3, 0.3)):
        s = SyntheticSystem(o, v, 8 * (o + v), 0.05, seed)
        x = s.mp2_amplitudes()[1]
        cases.append((x, int(frac * x.size)))
    out = {}
    for k, (x, m) in enumerate(cases):
        x = np.ascontiguousarray(x)
        out[f"c{k}_x"] = x
        out[f"c{k}_m"] = np.int64(m)
        for kind in ("fri", "largest"):
            seed = 100 + k
            idx, val = ref_sparse(R, x, m, kind, seed)
            key = f"c{k}_{kind}"
            out[key + "_rn"] = np.float64(draws(seed, 1)[0] if kind == "fri" else -1.0)
            out[key + "_idx"] = idx
            out[key + "_val"] = val
    out["n_cases"] = np.int64(len(cases))
    return out


def _ref_pivotal_child(R, x, m, seed, wfd):
    """In a forked child: the reference's pivotal SparseTensor4d (which may
    exit the process on its own errors); the result goes back through wfd."""
    import pickle
    libc.srand(seed)
    t = R.SparseTensor4d(x, x.shape, m, "fri", "pivotal", False)
    tail = [libc.rand() for _ in range(4)]
    idx = np.array([t.get_element(i)[0] for i in range(m)], dtype=np.int64).reshape(m, 4)
    val = np.array([t.get_element(i)[1] for i in range(m)], dtype=np.float64)
    os.write(wfd, pickle.dumps((idx, val, tail)))


def ref_pivotal(R, x, m, seed):
    """(idx, val, draws consumed) of the reference's pivotal compression, or
    None when the reference exits (its own error paths)."""
    import pickle
    rfd, wfd = os.pipe()
    pid = os.fork()
    if pid == 0:
        os.close(rfd)
        try:
            _ref_pivotal_child(R, x, m, seed, wfd)
        finally:
            os._exit(0)
    os.close(wfd)
    data = b""
    while True:
        chunk = os.read(rfd, 1 << 20)
        if not chunk:
            break
        data += chunk
    os.close(rfd)
    _, status = os.waitpid(pid, 0)
    if status != 0 or not data:
        return None
    idx, val, tail = pickle.loads(data)
    libc.srand(seed)
    stream = [libc.rand() for _ in range(x.size + 8)]
    used = next(k for k in range(len(stream) - 3) if stream[k:k + 4] == tail)
    return idx, val, used


def pivotal_cases(R):
    """Pivotal compressions by the reference (the binding's default sampling),
    on the compress.npz inputs and on larger MP2 amplitudes."""
    g = np.load(os.path.join(HERE, "compress.npz"))
    xs = [(g[f"c{k}_x"], int(g[f"c{k}_m"])) for k in range(int(g["n_cases"]))]
    for (o, v, seed, frac) in ((8, 32, 4, 0.05), (6, 30, 5, 0.2)):
        sys_ = SyntheticSystem(o, v, 8 * (o + v), 0.05, seed)
        x = sys_.mp2_amplitudes()[1]
        xs.append((np.ascontiguousarray(x), int(frac * x.size)))
    out = {"n_cases": np.int64(len(xs))}
    for k, (x, m) in enumerate(xs):
        seed = 500 + k
        r = ref_pivotal(R, x, m, seed)
        out[f"c{k}_x"] = x
        out[f"c{k}_m"] = np.int64(m)
        out[f"c{k}_seed"] = np.int64(seed)
        out[f"c{k}_ok"] = np.int64(r is not None)
        if r is not None:
            idx, val, used = r
            out[f"c{k}_idx"], out[f"c{k}_val"], out[f"c{k}_used"] = idx, val, np.int64(used)
    return out


def parallel_sample_cases():
    """The reference's own parallel_sample (through oracle/_ref/ref_parallel_sample)
    at one thread, on FRI probability vectors: p = |x| / R * m' with p_D = 0
    (the oracle's get_d_largest, itself pinned above)."""
    from oracle import fri_oracle as FO
    import tempfile
    exe = os.path.join(REPO, "oracle", "_ref", "ref_parallel_sample")
    rng = np.random.default_rng(909)
    xs = []
    for c in range(8):
        n = int(rng.integers(20, 3000))
        x = rng.standard_normal(n) * np.exp(2 * rng.standard_normal(n))
        xs.append((x, int(rng.integers(1, max(2, n // 3)))))
    for (o, v, seed, frac) in ((6, 24, 1, 0.12), (8, 32, 4, 0.05)):
        sys_ = SyntheticSystem(o, v, 8 * (o + v), 0.05, seed)
        x = sys_.mp2_amplitudes()[1].ravel()
        xs.append((x, int(frac * x.size)))
    out = {"n_cases": np.int64(len(xs))}
    for k, (x, m) in enumerate(xs):
        D, R = FO.get_d_largest(x, m)
        mp = m - D.size
        p = np.abs(x) / R * float(mp)
        p[D] = 0.0
        seed = 700 + k
        with tempfile.NamedTemporaryFile(suffix=".bin", delete=False) as f:
            f.write(np.ascontiguousarray(p, dtype=np.float64).tobytes())
            path = f.name
        r = subprocess.run([exe, path, str(mp), "1", str(seed)], capture_output=True, text=True)
        os.unlink(path)
        out[f"c{k}_q"] = p
        out[f"c{k}_n"] = np.int64(mp)
        out[f"c{k}_seed"] = np.int64(seed)
        out[f"c{k}_ok"] = np.int64(r.returncode == 0)
        if r.returncode == 0:
            # the reference logs its timings on stdout first; ref_parallel_sample's own two lines come last
            lines = r.stdout.split("\n")[:-1]
            S = np.array([int(t) for t in lines[-2].split()], dtype=np.int64)
            tail = [int(t) for t in lines[-1].split()]
            libc.srand(seed)
            stream = [libc.rand() for _ in range(p.size + 8)]
            used = next(j for j in range(len(stream) - 3) if stream[j:j + 4] == tail)
            out[f"c{k}_S"] = S
            out[f"c{k}_used"] = np.int64(used)
    return out


def contract_cases(R):
    rng = np.random.default_rng(77)
    out = {}
    for si, (no, nv, frac) in enumerate(((4, 8, 0.1), (5, 9, 0.05), (3, 7, 0.4))):
        d = {"o": no, "v": nv}
        t2 = np.zeros(no * no * nv * nv)
        nz = rng.choice(t2.size, size=max(1, int(t2.size * frac)), replace=False)
        t2[nz] = rng.standard_normal(nz.size)
        t2 = t2.reshape(no, no, nv, nv)
        m = nz.size
        T = R.SparseTensor4d(t2, t2.shape, m, "largest")
        for term in TERMS:
            ws = tuple(d[c] for c in W_SHAPE[term])
            osh = tuple(d[c] for c in OUT_SHAPE.get(term, "oovv"))
            W = rng.standard_normal(ws)
            out0 = rng.standard_normal(osh)
            for strided in (0, 1):
                Wuse = W if not strided else np.ascontiguousarray(W.transpose(3, 2, 1, 0)).transpose(3, 2, 1, 0)
                o = out0.copy()
                R.contract_DTSpT(Wuse, T, o, term)
                out[f"s{si}_{term}_out{strided}"] = o
            out[f"s{si}_{term}_W"] = W
            out[f"s{si}_{term}_init"] = out0
            out[f"s{si}_t2"] = t2
            out[f"s{si}_m"] = np.int64(m)
    return out


def iteration_case(R):
    F = load_reference_friccsd(R)
    s = SyntheticSystem(4, 12, 60, 0.05, 7)
    eris = pyscf_standin.make_eris(s)
    settings = {"m_keep": 800, "compression": "fri", "sampling_method": "systematic",
                "verbose": False, "compressed_contractions": ["O^2V^4", "O^3V^3", "O^4V^2"],
                "unbiased": False}

    class Driver(pyscf_standin.CCSD):
        def update_amps(self, t1, t2, eris):
            return F.update_amps(self, t1, t2, eris)

    cc = Driver(eris, settings)
    n_iter = 8
    cc.max_cycle = n_iter
    t1, t2 = pyscf_standin.mp2_guess(eris)
    iterates = [(t1, t2)]

    def record(t1, t2, eris):
        r = F.update_amps(cc, t1, t2, eris)
        iterates.append(r)
        return r

    cc.update_amps = record
    seed = 11
    libc.srand(seed)
    conv, e, _, _ = F.kernel(cc, eris, t1, t2)
    return {
        "L": s.L, "mo_energy": s.mo_energy, "nocc": np.int64(4), "m": np.int64(800),
        "seed": np.int64(seed), "rn": np.array(draws(seed, 2 * n_iter)),
        "energies": np.array(cc.energies),
        "t1": np.stack([a for a, _ in iterates]), "t2": np.stack([b for _, b in iterates]),
    }


def load_reference_frilccsd(F):
    """fricc/frilccsd.py, with a stub for the emcee import it never calls here."""
    if "emcee" not in sys.modules:
        emcee = types.ModuleType("emcee")
        emcee.autocorr = types.ModuleType("emcee.autocorr")

        def integrated_time(*a, **k):
            raise NotImplementedError("emcee is not installed")

        emcee.autocorr.integrated_time = integrated_time
        sys.modules["emcee"] = emcee
        sys.modules["emcee.autocorr"] = emcee.autocorr
    spec = importlib.util.spec_from_file_location("fricc.frilccsd",
                                                  os.path.join(REF, "fricc", "frilccsd.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules["fricc.frilccsd"] = mod
    spec.loader.exec_module(mod)
    return mod


LCCSD_VARIANTS = (("shared", False, False, 6), ("independent", True, False, 6), ("lccd", False, True, 4))


def lccsd_cases(R):
    """FRI-LCCSD trajectories of the reference's own fricc/frilccsd.py:
    one shared compression, six independent compressions, and LCCD."""
    F = load_reference_friccsd(R)
    LF = load_reference_frilccsd(F)
    s = SyntheticSystem(4, 12, 60, 0.05, 7)
    eris = pyscf_standin.make_eris(s)
    out = {"L": s.L, "mo_energy": s.mo_energy, "nocc": np.int64(4), "m": np.int64(800)}
    for vi, (name, indep, lccd, n_iter) in enumerate(LCCSD_VARIANTS):
        settings = {"m_keep": 800, "compression": "fri", "sampling_method": "systematic",
                    "verbose": False, "compressed_contractions": ["O^2V^4", "O^3V^3", "O^4V^2"],
                    "LCCD": lccd, "Independent Compressions": indep}

        class Driver(pyscf_standin.CCSD):
            def energy(self, t1, t2, eris):
                return LF.lin_cc_energy(self, t1, t2, eris)

        cc = Driver(eris, settings)
        cc.max_cycle = n_iter
        t1, t2 = pyscf_standin.mp2_guess(eris)
        iterates = [(t1, t2)]

        def record(t1, t2, eris, cc=cc):
            r = (LF.update_amps_independent_compressions if indep else LF.update_amps)(cc, t1, t2, eris)
            iterates.append(r)
            return r

        cc.update_amps = record
        seed = 21 + vi
        libc.srand(seed)
        F.kernel(cc, eris, t1, t2)
        per = 6 if indep else 1
        out[f"{name}_seed"] = np.int64(seed)
        out[f"{name}_rn"] = np.array(draws(seed, per * (len(iterates) - 1)))
        out[f"{name}_energies"] = np.array(cc.energies)
        out[f"{name}_t1"] = np.stack([a for a, _ in iterates])
        out[f"{name}_t2"] = np.stack([b for _, b in iterates])
    return out


def unbiased_case(R):
    """fricc/friccsd.py with "unbiased": True.  The reference reads an
    iteration counter cc._iter that it never defines; the loop here sets it
    to the number of updates already run before each call, so the
    reference's own running-average code (:108-136) runs unmodified."""
    F = load_reference_friccsd(R)
    s = SyntheticSystem(4, 12, 60, 0.05, 7)
    eris = pyscf_standin.make_eris(s)
    settings = {"m_keep": 800, "compression": "fri", "sampling_method": "systematic",
                "verbose": False, "compressed_contractions": ["O^2V^4", "O^3V^3", "O^4V^2"],
                "unbiased": True, "burn_in": 2}

    class Driver(pyscf_standin.CCSD):
        pass

    cc = Driver(eris, settings)
    n_iter = 7
    cc.max_cycle = n_iter
    cc._iter = 0
    t1, t2 = pyscf_standin.mp2_guess(eris)
    iterates = [(t1, t2)]

    def record(t1, t2, eris):
        r = F.update_amps(cc, t1, t2, eris)
        cc._iter += 1
        iterates.append(r)
        return r

    cc.update_amps = record
    seed = 41
    libc.srand(seed)
    F.kernel(cc, eris, t1, t2)
    return {
        "L": s.L, "mo_energy": s.mo_energy, "nocc": np.int64(4), "m": np.int64(800), "burn_in": np.int64(2),
        "seed": np.int64(seed), "rn": np.array(draws(seed, 2 * (len(iterates) - 1))),
        "energies": np.array(cc.energies),
        "t1": np.stack([a for a, _ in iterates]), "t2": np.stack([b for _, b in iterates]),
    }


def _layout(a):
    """(contiguous data, permutation) such that data.transpose(inverse) has
    a's memory order: a permuted view of a C-contiguous array is rebuilt
    with the same strides by data.transpose(np.argsort(perm))."""
    perm = tuple(int(i) for i in np.argsort([-s for s in a.strides], kind="stable"))
    return np.array(a.transpose(perm), order="C", copy=True), np.array(perm, dtype=np.int64)


def dropin_case(R):
    """Every py_rccsd call the unmodified fricc/friccsd.py makes in two
    iterations of its kernel (on the PySCF stand-in), recorded at the
    binding: each SparseTensor4d(...) with its arguments, the libc draw it
    consumed and its entries (get_element for every slot), and each
    contract_DTSpT(W, T, ouput, term) with W, the output before and after
    the call (W and ouput in their memory layout) and which recorded tensor
    it used.  Replaying the calls through another implementation of the
    binding shows that fricc/friccsd.py would run the same iteration on it."""
    rec = {"calls": []}
    seed = 61
    state = {"draws": 0}

    class Rec(types.ModuleType):
        pass

    mod = Rec("py_rccsd_recorder")

    def SparseTensor4d(tensor_arr, dims, m, compression="fri", sampling_method="pivotal", verbose=False):
        k = sum(1 for c in rec["calls"] if c["kind"] == "sp")
        t = R.SparseTensor4d(tensor_arr, dims, m, compression, sampling_method, verbose)
        rn = -1.0
        if compression == "fri" and sampling_method == "systematic":
            rn = draws(seed, state["draws"] + 1)[-1]
            state["draws"] += 1
        idx = np.array([t.get_element(i)[0] for i in range(m)], dtype=np.int64).reshape(m, 4)
        val = np.array([t.get_element(i)[1] for i in range(m)], dtype=np.float64)
        rec["calls"].append({"kind": "sp", "k": k, "x": np.array(tensor_arr), "dims": np.array(dims, np.int64),
                             "m": int(m), "compression": compression, "sampling": sampling_method,
                             "rn": rn, "idx": idx, "val": val})
        return Tagged(t, k)

    class Tagged:
        """The reference's tensor with the number of its recorded constructor call."""

        def __init__(self, t, k):
            self.t, self.k = t, k

        def __getattr__(self, name):
            return getattr(self.t, name)

    def contract_DTSpT(W, T, ouput, term):
        before, operm = _layout(ouput)
        wdata, wperm = _layout(W)
        R.contract_DTSpT(W, T.t, ouput, term)
        after, _ = _layout(ouput)
        rec["calls"].append({"kind": "ct", "term": term, "sp": T.k, "W": wdata, "wperm": wperm,
                             "before": before, "after": after, "operm": operm})

    mod.SparseTensor4d = SparseTensor4d
    mod.contract_DTSpT = contract_DTSpT
    F = load_reference_friccsd(mod)
    s = SyntheticSystem(4, 12, 60, 0.05, 9)
    eris = pyscf_standin.make_eris(s)
    settings = {"m_keep": 700, "compression": "fri", "sampling_method": "systematic",
                "verbose": False, "compressed_contractions": ["O^2V^4", "O^3V^3", "O^4V^2"],
                "unbiased": False}

    class Driver(pyscf_standin.CCSD):
        def update_amps(self, t1, t2, eris):
            return F.update_amps(self, t1, t2, eris)

    cc = Driver(eris, settings)
    cc.max_cycle = 2
    t1, t2 = pyscf_standin.mp2_guess(eris)
    libc.srand(seed)
    F.kernel(cc, eris, t1, t2)
    out = {"n_calls": np.int64(len(rec["calls"])), "seed": np.int64(seed), "energies": np.array(cc.energies)}
    for i, c in enumerate(rec["calls"]):
        for key, val in c.items():
            out[f"c{i}_{key}"] = np.asarray(val)
    return out


def main():
    if "--only-dropin" in sys.argv:
        R = load_reference_module()
        np.savez_compressed(os.path.join(HERE, "dropin.npz"), **dropin_case(R))
        print("dropin.npz", os.path.getsize(os.path.join(HERE, "dropin.npz")), "bytes")
        return
    R = load_reference_module()
    np.savez_compressed(os.path.join(HERE, "compress.npz"), **compress_cases(R))
    np.savez_compressed(os.path.join(HERE, "contract.npz"), **contract_cases(R))
    np.savez_compressed(os.path.join(HERE, "iteration.npz"), **iteration_case(R))
    np.savez_compressed(os.path.join(HERE, "lccsd.npz"), **lccsd_cases(R))
    np.savez_compressed(os.path.join(HERE, "unbiased.npz"), **unbiased_case(R))
    np.savez_compressed(os.path.join(HERE, "pivotal.npz"), **pivotal_cases(R))
    np.savez_compressed(os.path.join(HERE, "parallel_sample.npz"), **parallel_sample_cases())
    np.savez_compressed(os.path.join(HERE, "dropin.npz"), **dropin_case(R))
    for f in ("compress.npz", "contract.npz", "iteration.npz", "lccsd.npz", "unbiased.npz", "pivotal.npz",
              "parallel_sample.npz", "dropin.npz"):
        print(f, os.path.getsize(os.path.join(HERE, f)), "bytes")


if __name__ == "__main__":
    main()
