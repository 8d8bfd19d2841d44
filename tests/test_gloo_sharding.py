"""Sharded assembly on 2 CPU ranks (gloo): partition + Export-ADD = global result.

Each rank takes its brick partition (the reference's CartesianConnManager
split), reads its elements' LIDs from the product's host numbering
(DOFManager without a device), builds the export plan of the interface rows,
assembles its elements with the oracle (the kernels need a GPU) and sums the
interface rows with the other rank; the result must equal the one-rank
assembly, and only interface rows may travel.  Runs without a GPU.
"""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from tianxin_gb300 import sharding


def test_brick_ranges_follow_reference_split():
    # 7 bricks over 3 ranks: the first `remainder` ranks get one more
    assert [sharding.brick_range(7, 3, p) for p in range(3)] == [(0, 3), (3, 5), (5, 7)]
    assert sharding.rank_triplet(5, (2, 2, 2)) == (1, 0, 1)
    got = sorted(b for r in range(8) for b in sharding.owned_bricks((4, 3, 5), (2, 2, 2), r))
    assert got == list(range(4 * 3 * 5))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import tianxin_gb300 as tx
        from oracle import oracle as O
        from tianxin_gb300 import _abi as A
        n = (4, 4, 6)
        q = A.equation_set(A.TX_PHYS_ELASTICITY, params=(1.0, 0.3, 0.0, 0.0, -1.0, 0.0))
        o = O.Oracle(A.mesh_desc(n, jitter=0.1, seed=8), q)
        dof = tx.DOFManager(tx.CartesianConnManager(*n, jitter=0.1, seed=8), q, require_device=False)
        x = np.random.default_rng(0).uniform(-1, 1, o.n_dofs)
        mine = sharding.owned_bricks(n, (1, 1, world), rank)
        lo, hi = min(mine), max(mine) + 1
        assert hi - lo == len(mine)  # z-split: a contiguous element range
        rowptr, _ = o.graph()
        plan = sharding.ExportPlan([dof.getElementLIDs(0)[lo:hi]], dof.n_dofs, rowptr)
        f, v = o.evaluate(x, block=0, elem_range=(lo, hi))
        ft, vt = torch.from_numpy(f), torch.from_numpy(v)
        sharding.export_add(plan, ft, vt)
        if rank == 0:
            f_ref, v_ref = o.evaluate(x)
            # every row this rank holds is complete after the exchange
            rows = plan.local_rows
            ents = np.concatenate([np.arange(rowptr[r], rowptr[r + 1]) for r in rows])
            # the interface is the node layer z = 3 (5 x 5 nodes, 3 DOFs each)
            out.put((float(np.abs(ft.numpy()[rows] - f_ref[rows]).max() / np.abs(f_ref).max()),
                     float(np.abs(vt.numpy()[ents] - v_ref[ents]).max() / np.abs(v_ref).max()),
                     len(plan.all_rows), plan.volume(), o.n_dofs + o.nnz))
    finally:
        dist.destroy_process_group()


def test_two_rank_assembly_equals_one_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    ef, ev, rows, volume, full = q.get(timeout=5)
    assert ef <= 1e-14 and ev <= 1e-14
    assert rows == 5 * 5 * 3
    assert volume < full / 3  # the interface, not the whole arrays
