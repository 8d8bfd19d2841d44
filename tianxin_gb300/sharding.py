"""Element partition of the brick lattice over ranks, and the exchange it needs.

The reference distributes bricks over px x py x pz MPI ranks
(CartesianConnManager::buildLocalElements, dof-mgr/test/cartesian_topology/
CartesianConnManager.cpp:499-575): rank (i,j,k) owns an even split of the
bricks in each direction, the first `remainder` ranks one more.  Each rank
assembles its own elements into ghosted f/A, and one exchange step sums the
ghosted contributions into the owners (Tpetra Export ADD,
disc-fe/src/lof/Panzer_TpetraLinearObjFactory_impl.hpp:176-205).

Here the exchange moves the interface only: ExportPlan finds, from each
rank's element LIDs (the DOF manager's host numbering), the rows more than
one rank touches; export_add packs those rows of f and of the CRS values
into one buffer, sums it over the ranks (torch.distributed all_reduce) and
unpacks it, so rows interior to a rank never travel.  On one GPU per box the
bench runs independent replicas; the sharded form is tested with gloo on CPU.
"""
import numpy as np
import torch


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


class ExportPlan:
    """The rows touched by more than one rank (every rank holds the same plan).

    local_lids: this rank's element LID arrays (one [E][n] array per block it
    assembles); n_rows: DOF rows of the ghosted map; rowptr: the CRS row
    pointer (numpy int64), for the matrix part of the exchange."""

    def __init__(self, local_lids, n_rows, rowptr=None, group=None):
        import torch.distributed as dist
        touched = np.zeros(n_rows, np.int32)
        for lids in local_lids:
            touched[np.unique(np.asarray(lids).ravel())] = 1
        count = torch.from_numpy(touched.copy())
        dist.all_reduce(count, op=dist.ReduceOp.SUM, group=group)
        shared = count.numpy() > 1
        self.local_rows = np.nonzero(touched)[0]                     # rows this rank holds (owned + ghosted)
        self.rows = np.nonzero(shared & (touched > 0))[0]          # interface rows this rank holds
        self.all_rows = np.nonzero(shared)[0]                        # the same on every rank
        self.n_rows = n_rows
        self.vals_index = None
        if rowptr is not None:
            rp = np.asarray(rowptr, np.int64)
            starts, ends = rp[self.all_rows], rp[self.all_rows + 1]
            self.vals_index = np.concatenate([np.arange(a, b) for a, b in zip(starts, ends)]) if len(starts) \
                else np.zeros(0, np.int64)

    def volume(self):
        """Values the exchange moves per rank: interface entries of f and of the CRS values."""
        return len(self.all_rows) + (0 if self.vals_index is None else len(self.vals_index))


def export_add(plan, f=None, vals=None, group=None):
    """Sum the ranks' contributions to the interface rows of f and the CRS values in place (Export ADD).

    Every rank contributes its partial sums of the interface rows (zero where it touches none) and receives
    the total; rows only one rank touches already hold their final values."""
    import torch.distributed as dist
    parts = []
    if f is not None:
        parts.append(f[torch.from_numpy(plan.all_rows)])
    if vals is not None:
        parts.append(vals[torch.from_numpy(plan.vals_index)])
    if not parts:
        return
    buf = torch.cat(parts)
    dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
    k = 0
    if f is not None:
        f[torch.from_numpy(plan.all_rows)] = buf[:len(plan.all_rows)]
        k = len(plan.all_rows)
    if vals is not None:
        vals[torch.from_numpy(plan.vals_index)] = buf[k:]
