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


# quadratic nodes in shards order (Hexahedron<27>, Tetrahedron<10>), which are
# also Exodus II's HEX27 / TETRA10 orders: the mid-edge node of edge c, the
# mid-face node of face c, the centre
HEX_EDGES = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6), (3, 7)]
HEX_EDGE_NODE = [8, 9, 10, 11, 16, 17, 18, 19, 12, 13, 14, 15]
HEX_FACE_NODE = [25, 24, 26, 23, 21, 22]
TET_EDGES = [(0, 1), (1, 2), (2, 0), (0, 3), (1, 3), (2, 3)]


def side_nodes(topo, s):
    """Quadratic node ordinals on side s."""
    if topo == A.TX_TOPO_HEX:
        fv = HEX_FACES[s]
        return fv + [HEX_EDGE_NODE[c] for c, (a, b) in enumerate(HEX_EDGES) if a in fv and b in fv] + \
            [HEX_FACE_NODE[s]]
    fv = TET_FACES[s]
    return fv + [4 + c for c, (a, b) in enumerate(TET_EDGES) if a in fv and b in fv]


def quadratic_lattice_as_explicit(conn, n, q):
    """A lattice mesh with a TX_HGRAD_C2 field as hex27 / tet10 blocks whose node k
    is the lattice's DOF entity k (GID // fields), so that the explicit numbering
    equals the lattice numbering; mid-edge / mid-face / centre nodes sit at the
    means of their vertices.  Returns (coords, blocks, side_sets, node_sets)."""
    dof = tx.DOFManager(conn, q, require_device=False)
    nf = dof.n_fields
    coords_v, blocks_v, ss, _ = lattice_as_explicit(conn, n)
    coords = np.zeros((dof.n_dofs // nf, 3))
    blocks, conns = [], []
    for b, (topo, cv, bid, name) in enumerate(blocks_v):
        g = dof.getElementGIDs(b)[:, dof.getGIDFieldOffsets(b, 0)] // nf  # [E][nodes] in basis order
        pv = coords_v[cv]
        coords[g[:, :cv.shape[1]]] = pv
        if topo == A.TX_TOPO_HEX:
            for c, (a, e) in enumerate(HEX_EDGES):
                coords[g[:, HEX_EDGE_NODE[c]]] = 0.5 * (pv[:, a] + pv[:, e])
            for s, fv in enumerate(HEX_FACES):
                coords[g[:, HEX_FACE_NODE[s]]] = pv[:, fv].mean(axis=1)
            coords[g[:, 20]] = pv.mean(axis=1)
        else:
            for c, (a, e) in enumerate(TET_EDGES):
                coords[g[:, 4 + c]] = 0.5 * (pv[:, a] + pv[:, e])
        blocks.append((topo, g, bid, name))
        conns += [(topo, row) for row in g]
    node_sets = []
    for name, sid, pairs in ss:
        nodes = {int(conns[e][1][k]) for e, s in pairs for k in side_nodes(conns[e][0], s)}
        node_sets.append((name, sid, np.array(sorted(nodes), dtype=np.int64)))
    return coords, blocks, ss, node_sets
