"""Atlas subjects sharded over ranks: one process per GPU, torch.distributed for the one exchange.

The reference runs an atlas's subjects on host threads and sums their gradients on the host
(AbstractAtlas.cxx:166-205 for the threads, :489-557 for the sums). Here each rank runs the batched
iteration (`Atlas`) over its share of the subjects; per iteration the ranks exchange

* the per-subject log-likelihood terms (a zero-filled length-S vector, summed): every rank then
  forms the total in subject order, so it is the same bits on every rank;
* the control-point and template gradients (sums over subjects): one all-reduce each;
* the momenta gradients: gathered the same way as the log-likelihood terms.

Subjects are assigned largest first to the rank with the least work so far (work = template
faces x target faces of the data term, the dominant kernel sum), a deterministic rule every rank
computes alike. The exchange is the only collective; nothing else is shared.
"""
from __future__ import annotations

import numpy as np


def assign_subjects(work, world: int) -> list[list[int]]:
    """Largest-first greedy assignment of subjects (by `work`) to `world` ranks; each rank's list
    is in subject order. Ties go to the lower rank and the lower subject index."""
    work = np.asarray(work, dtype=np.float64)
    load = np.zeros(world)
    out: list[list[int]] = [[] for _ in range(world)]
    for s in sorted(range(len(work)), key=lambda i: (-work[i], i)):
        r = int(np.argmin(load))
        out[r].append(s)
        load[r] += work[s]
    return [sorted(o) for o in out]


def _all_reduce_sum(arr: np.ndarray, group=None) -> np.ndarray:
    import torch
    import torch.distributed as dist
    backend = dist.get_backend(group)
    dev = "cuda" if backend == "nccl" else "cpu"
    t = torch.from_numpy(np.ascontiguousarray(arr, dtype=np.float64)).to(dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy()


def max_over_ranks(value: float, group=None) -> float:
    """The largest `value` over the ranks (the benchmark's step time)."""
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


class ShardedAtlas:
    """Deterministic-atlas iteration over all subjects, this rank running its share.

    `make_atlas(subject_indices)` builds the rank's local iteration: an object whose
    `step(mom_local)` returns (loglik[3 + S_local], grad_mom[S_local, ncp, 3], grad_cp[ncp, 3],
    grad_template[nv, 3]) like `deformation.Atlas.step`. `step(mom)` takes the momenta of ALL
    subjects (S x ncp x 3) and returns the same four quantities for all subjects, the same bits on
    every rank: per-subject terms and momenta gradients are gathered, the total log-likelihood is
    summed in subject order from them, and the data / regularity split and the control-point and
    template gradients are all-reduced.
    """

    def __init__(self, n_subjects: int, ncp: int, nv: int, work, make_atlas, group=None):
        import torch.distributed as dist
        self.group = group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)
        self.S, self.ncp, self.nv = int(n_subjects), int(ncp), int(nv)
        self.shares = assign_subjects(work, self.world)
        self.mine = self.shares[self.rank]
        self.local = make_atlas(self.mine) if self.mine else None

    def step(self, mom):
        mom = np.asarray(mom, dtype=np.float64)
        S = self.S
        per = np.zeros(S)
        gm = np.zeros((S, self.ncp, 3))
        gc = np.zeros((self.ncp, 3))
        gt = np.zeros((self.nv, 3))
        split = np.zeros(2)
        if self.local is not None:
            ll, gml, gcl, gtl = self.local.step(np.ascontiguousarray(mom[self.mine]))
            per[self.mine] = ll[3:]
            gm[self.mine] = gml
            gc[:] = gcl
            gt[:] = gtl
            split[:] = ll[1:3]
        # the same collectives, in the same order, on every rank
        per = _all_reduce_sum(per, self.group)
        gm = _all_reduce_sum(gm, self.group)
        gc = _all_reduce_sum(gc, self.group)
        gt = _all_reduce_sum(gt, self.group)
        split = _all_reduce_sum(split, self.group)
        total = 0.0
        for v in per:  # subject order, as the single-GPU iteration sums them
            total += float(v)
        ll = np.concatenate([[total], split, per])
        return ll, gm, gc, gt
