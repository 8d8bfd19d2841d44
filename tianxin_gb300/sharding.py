"""Element partition of the brick lattice over ranks, and the exchange it needs.

The reference distributes bricks over px x py x pz MPI ranks
(CartesianConnManager::buildLocalElements, dof-mgr/test/cartesian_topology/
CartesianConnManager.cpp:499-575): rank (i,j,k) owns an even split of the
bricks in each direction, the first `remainder` ranks one more.  Each rank
assembles its own elements into ghosted f/A, and one exchange step sums the
ghosted contributions into the owners (Tpetra Export ADD,
disc-fe/src/lof/Panzer_TpetraLinearObjFactory_impl.hpp:176-205).

On one GPU per box the bench runs independent replicas; this module gives the
partition and a sum-exchange (torch.distributed all_reduce of the partial
residual/CRS values) so the sharded form is testable with gloo on CPU.
"""


def rank_triplet(rank, procs):
    px, py, pz = procs
    k = rank // (px * py)
    j = (rank - px * py * k) // px
    i = rank - px * py * k - px * j
    return i, j, k


def brick_range(n_total, n_procs, p):
    """[start, stop) of the bricks rank coordinate p owns along one direction."""
    even, rem = divmod(n_total, n_procs)
    start = p * even + min(rem, p)
    return start, start + even + (1 if rem > p else 0)


def owned_bricks(totals, procs, rank):
    """Global brick ids (x fastest) owned by rank, in the reference's local order."""
    ijk = rank_triplet(rank, procs)
    rx, ry, rz = (brick_range(totals[d], procs[d], ijk[d]) for d in range(3))
    NX, NY = totals[0], totals[1]
    return [x + NX * (y + NY * z) for z in range(*rz) for y in range(*ry) for x in range(*rx)]


def export_add(tensors, group=None):
    """Sum the ranks' ghosted contributions (Export ADD onto one owner map)."""
    import torch.distributed as dist
    for t in tensors:
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return tensors
