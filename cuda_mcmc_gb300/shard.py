"""Sharding independent sequences of one or many fits across ranks.

Replica exchange never crosses a sequence, and fits are independent, so a
multi-GPU run needs no collective during the sweep: the (fit, sequence) work
items are split across ranks, every rank runs its shards, and the records
(pout, tout, chi2, final state) are gathered once at the end.

* :func:`item_costs` -- the cost of one (fit, sequence) item: proposals per
  iteration x model terms per proposal;
* :func:`partition` -- contiguous sequence ranges per (rank, fit) with
  balanced total cost: items are laid out fit by fit, sequence by sequence,
  and rank r takes the items whose cost midpoints fall in
  [r, r + 1) * total / world;
* :func:`shard_jobs` -- the DeviceJobs of one rank (``DeviceJob.from_workload``
  with ``seqs``: each shard seeds its generators with the subsequences it has
  in the unsharded run, so the shards together walk exactly the unsharded
  chains);
* :func:`gather` -- rank 0 reassembles every fit's arrays along the sequence
  axis from the ranks' shards (torch.distributed object gather: any backend,
  gloo on CPU included).
"""
from __future__ import annotations

import numpy as np

# sequence axis of each gatherable array (reference layouts)
SEQ_AXIS = {"pout": 2, "tout": 1, "chi2": 0, "pcur": 1, "chi2c": 1, "flag": 1, "ptent": 1,
            "ptentn": 1, "pstp": 2, "n_acpt": 2, "n_exch": 1, "n_cnt": 2, "n_hist": 3,
            "tcur": 1, "rndst": 1, "chi2m": 1}


def item_costs(fits):
    """Cost of one sequence of each fit: nprm * nbeta proposals per
    iteration, each over the fit's ndat model terms."""
    return [float(w.nprm * w.nbeta * max(w.ndat, 1)) for w in fits]


def partition(nseqs, costs, world):
    """Split fits f (nseqs[f] sequences of cost costs[f] each) over `world`
    ranks.  Returns, per rank, a list of (fit, s0, s1) contiguous sequence
    ranges; every sequence is in exactly one range."""
    if world < 1:
        raise ValueError("world must be >= 1")
    total = float(sum(n * c for n, c in zip(nseqs, costs)))
    per = total / world if total > 0 else 1.0
    out = [[] for _ in range(world)]
    acc = 0.0
    for f, (n, c) in enumerate(zip(nseqs, costs)):
        cur, s0 = None, 0
        for s in range(n):
            r = min(int((acc + 0.5 * c) / per), world - 1) if total > 0 else (s * world) // n
            acc += c
            if cur is None:
                cur, s0 = r, s
            elif r != cur:
                out[cur].append((f, s0, s))
                cur, s0 = r, s
        if cur is not None:
            out[cur].append((f, s0, n))
    return out


def rank_cost(parts, costs):
    """Total cost of each rank's ranges."""
    return [sum((s1 - s0) * costs[f] for f, s0, s1 in p) for p in parts]


def shard_jobs(fits, parts_of_rank, niter_total=None, seed=1234, **kw):
    """DeviceJobs of one rank's shards: [(fit, s0, s1, job)] (fit f seeded
    with seed + f)."""
    from .device import DeviceJob
    return [(f, s0, s1, DeviceJob.from_workload(fits[f], niter_total=niter_total, seed=seed + f,
                                                seqs=(s0, s1), **kw))
            for f, s0, s1 in parts_of_rank]


def gather(local, nfits, fields=("pout", "tout", "chi2"), group=None, dst=0):
    """Reassemble shards.  ``local``: this rank's [(fit, s0, s1, {field:
    array})].  Rank ``dst`` gets {fit: {field: array over all sequences}};
    the other ranks get None.  Without an initialised process group the local
    shards are assembled (a single rank)."""
    import torch.distributed as dist
    payload = [(f, s0, s1, {k: np.asarray(a[k]) for k in fields}) for f, s0, s1, a in local]
    if dist.is_available() and dist.is_initialized():
        rank = dist.get_rank(group)
        got = [None] * dist.get_world_size(group) if rank == dst else None
        dist.gather_object(payload, got, dst=dst, group=group)
        if rank != dst:
            return None
        shards = [x for part in got for x in part]
    else:
        shards = payload
    out = {}
    for f in range(nfits):
        mine = sorted((s for s in shards if s[0] == f), key=lambda s: s[1])
        if not mine:
            continue
        pos = 0
        for _, s0, s1, _ in mine:
            if s0 != pos:
                raise ValueError("fit %d: sequences %d..%d missing from the shards" % (f, pos, s0))
            pos = s1
        out[f] = {k: np.concatenate([s[3][k] for s in mine], axis=SEQ_AXIS[k]) for k in fields}
    return out
