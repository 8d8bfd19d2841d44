"""Lattice meshes as explicit meshes: the same nodes (lattice node order),
elements (block order), box sides as side sets and node sets, so that the
explicit path can be compared with the lattice path, which the oracle pins."""
import numpy as np

import tianxin_gb300 as tx
from tianxin_gb300 import _abi as A

HEX_FACES = [[0, 1, 5, 4], [1, 2, 6, 5], [2, 3, 7, 6], [0, 4, 7, 3], [0, 3, 2, 1], [4, 5, 6, 7]]
TET_FACES = [[0, 1, 3], [1, 2, 3], [0, 3, 2], [0, 2, 1]]
SIDE_NAMES = ["xmin", "xmax", "ymin", "ymax", "zmin", "zmax"]


def lattice_as_explicit(conn, n):
    """(coords, blocks, side_sets, node_sets) of a CartesianConnManager with n = (NX, NY, NZ) bricks."""
    coords = conn.coordinates()
    nx, ny, nz = n
    node_ijk = np.stack(np.unravel_index(np.arange(len(coords)), (nz + 1, ny + 1, nx + 1))[::-1], axis=1)
    lim = np.array([nx, ny, nz])
    on_side = [node_ijk[:, s // 2] == (lim[s // 2] if s % 2 else 0) for s in range(6)]
    blocks, pairs, first = [], [[] for _ in range(6)], 0
    for b in range(conn.numElementBlocks()):
        cn = conn.getElementVertices(b)
        topo = A.TX_TOPO_HEX if cn.shape[1] == 8 else A.TX_TOPO_TET
        blocks.append((topo, cn, b + 1, f"block_{b + 1}"))
        faces = HEX_FACES if topo == A.TX_TOPO_HEX else TET_FACES
        for e in range(len(cn)):
            for s, fv in enumerate(faces):
                for side in range(6):
                    if on_side[side][cn[e][fv]].all():
                        pairs[side].append((first + e, s))
        first += len(cn)
    side_sets = [(SIDE_NAMES[s], s + 1, pairs[s]) for s in range(6)]
    node_sets = [(SIDE_NAMES[s], s + 1, np.flatnonzero(on_side[s])) for s in range(6)]
    return coords, blocks, side_sets, node_sets


def box(n=(3, 2, 2), blocks=(1, 1, 1), topo=A.TX_TOPO_HEX, jitter=0.1, seed=5):
    bricks = tuple(a * b for a, b in zip(n, blocks))
    conn = tx.CartesianConnManager(*n, *blocks, topology=topo, jitter=jitter, seed=seed)
    return conn, lattice_as_explicit(conn, bricks)
