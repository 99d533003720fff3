"""An iteration replayed from a CUDA graph (FRICCSDGPU(graph=True)) gives the
same trajectory as eager execution: same kernels in the same order, the
draws read from device memory instead of kernel arguments."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["df64", "fp64"])
def test_graph_replay_matches_eager(gpulib, precision):
    from fricc_gb300.friccsd import FRICCSDGPU
    from fricc_gb300.rccsd_dense import DeviceERIs
    from fricc_gb300.rng import GlibcRand
    from fricc_gb300.synthetic import SyntheticSystem
    s = SyntheticSystem(10, 40, 200, 0.05, 3)
    E = DeviceERIs.from_system(s)
    t1h, t2h = s.mp2_amplitudes()
    res = {}
    for graph in (False, True):
        gs = FRICCSDGPU(E, {"m_keep": 20000}, rn_draw=GlibcRand(11), precision=precision, graph=graph)
        t1, t2 = torch.from_numpy(t1h).cuda(), torch.from_numpy(t2h).cuda()
        es = []
        for _ in range(6):
            t1, t2 = gs.update_amps(t1, t2)
            es.append(gs.read_energy())
        res[graph] = (np.array(es), t1.cpu().numpy(), t2.cpu().numpy())
        if graph:
            assert gs._g is not None  # iterations 2.. ran from the graph
    (ea, t1a, t2a), (eb, t1b, t2b) = res[False], res[True]
    assert np.abs(ea - eb).max() <= 1e-14
    assert np.abs(t2a - t2b).max() <= 1e-14 * np.abs(t2a).max()
    assert np.abs(t1a - t1b).max() <= 1e-14 * max(np.abs(t1a).max(), 1e-300)


def test_graph_replicas_match_eager(gpulib):
    from fricc_gb300.batch import ReplicaBatch
    from fricc_gb300.rccsd_dense import DeviceERIs
    from fricc_gb300.synthetic import SyntheticSystem
    s = SyntheticSystem(8, 32, 160, 0.05, 4)
    E = DeviceERIs.from_system(s)
    out = []
    for graph in (False, True):
        b = ReplicaBatch(E, {"m_keep": 8000}, seeds=[1, 2, 3, 4, 5, 6], n_streams=3, graph=graph)
        for _ in range(4):
            b.step()
        out.append(np.array(b.history))
    assert np.abs(out[0] - out[1]).max() <= 1e-14
