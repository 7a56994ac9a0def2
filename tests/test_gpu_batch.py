"""Batched launch: several grids of different sizes and w-plane sets in one
persistent kernel, each member checked against the oracle (FP32 tolerance),
repeated, and replayed from a CUDA graph."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL32 = 1e-5


def _members(seed=5):
    rng = np.random.default_rng(seed)
    specs = [(128, (8, 12)), (256, (8, 20, 40)), (512, (16, 96)), (256, (64,)), (128, (6, 10, 14))]
    # one shared GCF array: member m's planes follow member m-1's
    gcf_parts, members, base = [], [], 0
    for G, sup in specs:
        sup = np.array(sup, np.int32)
        sizes = 64 * sup.astype(np.int64) ** 2
        offs = base + np.concatenate([[0], np.cumsum(sizes)[:-1]])
        base += int(sizes.sum())
        gcf_parts.append((rng.standard_normal(int(sizes.sum())) +
                          1j * rng.standard_normal(int(sizes.sum()))) / 8)
        n = int(rng.integers(2000, 6000))
        lim = 0.45 * G
        uvw = np.column_stack([rng.uniform(-lim, lim, n), rng.uniform(-lim, lim, n),
                               rng.uniform(-1, 1, n)])
        plane = rng.integers(-1, len(sup), n).astype(np.int32)
        vis = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        members.append(dict(G=G, sup=sup, offs=offs.astype(np.int64), uvw=uvw, plane=plane,
                            vis=vis))
    return members, np.concatenate(gcf_parts)


def _oracle(m, gcf):
    g = np.zeros((m["G"], m["G"]), np.complex128)
    O.scatter_planes(1.0, m["G"], int(m["sup"].max()), m["uvw"], m["vis"], m["plane"], m["sup"],
                     gcf, m["offs"], g)
    return g


def test_batch_matches_oracle_per_member_and_in_a_graph():
    import torch

    from rc_gb300.engine import Batch

    members, gcf = _members()
    keep = []
    spec = []
    for m in members:
        uvw = torch.tensor(m["uvw"], device="cuda")
        plane = torch.tensor(m["plane"], device="cuda")
        keep += [uvw, plane]
        spec.append(dict(uvw=uvw, plane=plane, scale=1.0, grid_size=m["G"],
                         grid_shape=(m["G"], m["G"]), supports=m["sup"], gcf_offsets=m["offs"],
                         margin=int(m["sup"].max())))
    B = Batch(spec)
    st = B.stats()
    assert st["members"] == len(members)
    d_gcf = torch.tensor(gcf, dtype=torch.complex64, device="cuda")
    vis = [torch.tensor(m["vis"], dtype=torch.complex64, device="cuda") for m in members]
    grids = [torch.zeros((m["G"], m["G"]), dtype=torch.complex64, device="cuda") for m in members]
    for rep in range(2):
        for g in grids:
            g.zero_()
        B.grid(vis, d_gcf, grids)
        torch.cuda.synchronize()
        for m, g in zip(members, grids):
            assert rel_l2(g.cpu().numpy(), _oracle(m, gcf)) < TOL32
    models = [torch.tensor(np.random.default_rng(i).standard_normal((m["G"], m["G"])) * (1 + 1j),
                           dtype=torch.complex64, device="cuda") for i, m in enumerate(members)]
    for mode in (0, 1):
        preds = B.degrid(d_gcf, models, mode=mode)
        torch.cuda.synchronize()
        for m, model, p in zip(members, models, preds):
            exp = O.degrid_planes(1.0, m["G"], int(m["sup"].max()), m["uvw"], m["plane"], m["sup"],
                                  gcf, m["offs"], model.cpu().numpy().astype(np.complex128),
                                  mode=mode)
            assert rel_l2(p.cpu().numpy(), exp) < TOL32
    # the whole batched step in a CUDA graph
    preds = [torch.empty(m["uvw"].shape[0], dtype=torch.complex64, device="cuda") for m in members]

    def step():
        for g in grids:
            g.zero_()
        B.grid(vis, d_gcf, grids)
        B.degrid(d_gcf, models, preds=preds)

    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        step()
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        step()
    for g in grids:
        g.fill_(7.0)
    graph.replay()
    torch.cuda.synchronize()
    for m, g in zip(members, grids):
        assert rel_l2(g.cpu().numpy(), _oracle(m, gcf)) < TOL32
    B.close()


def test_batch_rejects_mixed_tiles():
    import torch

    from rc_gb300 import lib
    from rc_gb300.engine import Batch

    members, gcf = _members()
    uvw = torch.tensor(members[0]["uvw"], device="cuda")
    m = dict(uvw=uvw, scale=1.0, grid_size=128, grid_shape=(128, 128),
             supports=members[0]["sup"], gcf_offsets=members[0]["offs"])
    with pytest.raises(AssertionError):
        Batch([m] * (lib.MAX_BATCH + 1))
