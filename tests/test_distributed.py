"""Multi-process (gloo, world size 2, CPU) tests of the sharded atlas's host logic
(deformetrica_code_gb300/distributed.py) and of the benchmark's max-over-ranks timing.

The per-rank iteration is a stand-in with the same interface as deformation.Atlas (a GPU is not
needed for the exchange): subject s contributes terms that depend on s and its momenta only, so
the sharded result must equal the single-process result over all subjects.
"""
import os
import socket

import numpy as np
import pytest

from deformetrica_code_gb300.distributed import assign_subjects

NCP, NV, S = 5, 7, 9


class StandIn:
    """Subject s: loglik term -(s + 1) |p_s|^2 split 1:3 into data and regularity; gradients
    linear in the momenta."""

    def __init__(self, subjects):
        self.subjects = list(subjects)

    def step(self, mom):
        per = np.array([-(s + 1.0) * float(np.sum(m * m)) for s, m in zip(self.subjects, mom)])
        gm = np.stack([-(s + 1.0) * 2.0 * m for s, m in zip(self.subjects, mom)])
        gc = sum(0.1 * (s + 1.0) * m for s, m in zip(self.subjects, mom))
        gt = sum(np.full((NV, 3), 0.01 * (s + 1.0) * float(m.sum())) for s, m in zip(self.subjects, mom))
        tot = 0.0
        for v in per:
            tot += v
        ll = np.concatenate([[tot, 0.25 * per.sum(), 0.75 * per.sum()], per])
        return ll, gm, gc, gt


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    from deformetrica_code_gb300.distributed import ShardedAtlas, max_over_ranks
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        work = np.arange(S, 0, -1) * 10.0 + (np.arange(S) % 3)
        mom = np.random.default_rng(0).standard_normal((S, NCP, 3))
        sa = ShardedAtlas(S, NCP, NV, work, StandIn)
        ll, gm, gc, gt = sa.step(mom)
        t = max_over_ranks(1.5 + rank)
        q.put((rank, sa.mine, ll, gm, gc, gt, t))
    finally:
        dist.destroy_process_group()


def test_assign_subjects_balances_and_covers():
    work = [50, 10, 40, 30, 30, 5]
    shares = assign_subjects(work, 2)
    assert sorted(sum(shares, [])) == list(range(6))
    loads = [sum(work[i] for i in s) for s in shares]
    assert abs(loads[0] - loads[1]) <= max(work)
    assert assign_subjects(work, 2) == shares  # deterministic
    assert assign_subjects(work, 1) == [list(range(6))]
    assert assign_subjects([1, 1], 3)[2] == []


def test_sharded_atlas_gloo_two_ranks():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort(key=lambda o: o[0])
    mom = np.random.default_rng(0).standard_normal((S, NCP, 3))
    ref_ll, ref_gm, ref_gc, ref_gt = StandIn(range(S)).step(mom)
    assert sorted(out[0][1] + out[1][1]) == list(range(S)) and out[0][1] and out[1][1]
    for rank, mine, ll, gm, gc, gt, t in out:
        assert ll[0] == ref_ll[0]  # summed in subject order: the same bits
        np.testing.assert_array_equal(ll[3:], ref_ll[3:])
        np.testing.assert_allclose(ll[1:3], ref_ll[1:3], rtol=1e-14)
        np.testing.assert_array_equal(gm, ref_gm)
        np.testing.assert_allclose(gc, ref_gc, rtol=1e-14, atol=1e-15)
        np.testing.assert_allclose(gt, ref_gt, rtol=1e-14, atol=1e-15)
        assert t == 2.5  # the slowest rank's time
    # both ranks hold identical results
    for a, b in zip(out[0][2:6], out[1][2:6]):
        np.testing.assert_array_equal(a, b)
