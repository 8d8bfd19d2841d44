"""Exodus II mesh output in the NetCDF classic container (STK_Interface::writeToExodus's
role for the mesh itself: adapters-stk/src/Panzer_STK_Interface.cpp).

Writes coordinates, hex8/tet4/hex27/tet10 element blocks, side sets and node sets with
the Exodus II variable names (1-based element and node numbers, 1-based side
ordinals) in CDF-1 or CDF-2; no results variables.  Host-side utility: the
file is what the library's reader (tx_mesh_create_exodus) and other Exodus
tools read.
"""
import struct

import numpy as np

_NC_DIMENSION, _NC_VARIABLE, _NC_ATTRIBUTE = 0x0A, 0x0B, 0x0C
_NC_CHAR, _NC_INT, _NC_FLOAT, _NC_DOUBLE = 2, 4, 5, 6
_SIZE = {_NC_CHAR: 1, _NC_INT: 4, _NC_FLOAT: 4, _NC_DOUBLE: 8}
_FMT = {_NC_INT: ">i4", _NC_FLOAT: ">f4", _NC_DOUBLE: ">f8"}
_ELEM_TYPE = {(0, 8): "HEX8", (1, 4): "TETRA4", (0, 27): "HEX27", (1, 10): "TETRA10"}  # (topology, nodes)
_LEN_NAME = 33


def _pad(b):
    return b + b"\0" * (-len(b) % 4)


def _name(s):
    b = s.encode()
    return struct.pack(">i", len(b)) + _pad(b)


def _attr(name, nc_type, value):
    if nc_type == _NC_CHAR:
        data = value.encode()
        n = len(data)
    else:
        arr = np.asarray(value, dtype=_FMT[nc_type]).reshape(-1)
        data, n = arr.tobytes(), arr.size
    return _name(name) + struct.pack(">ii", nc_type, n) + _pad(data)


def _names_array(names):
    out = np.zeros((len(names), _LEN_NAME), dtype="S1")
    for i, s in enumerate(names):
        b = s.encode()[: _LEN_NAME - 1]
        out[i, : len(b)] = np.frombuffer(b, dtype="S1")
    return out


def write_exodus(path, coords, blocks, side_sets=(), node_sets=(), node_num_map=None, version=2, title="tianxin"):
    """Write a 3-D mesh.

    coords [n][3]; blocks [(topology, conn[E][nodes] 0-based, id, name)] with the vertices (hex8 / tet4) or
    the quadratic nodes (hex27 / tet10, shards order);
    side_sets [(name, id, [(element, side), ...])] with 0-based elements over
    the whole mesh and 0-based shards sides; node_sets [(name, id, nodes)];
    node_num_map: optional global node ids (1-based, any order).
    """
    coords = np.asarray(coords, dtype=np.float64).reshape(-1, 3)
    dims, variables = [], []

    def dim(name, n):
        if n <= 0:
            raise ValueError(f"dimension {name} must be positive")
        dims.append((name, int(n)))
        return len(dims) - 1

    def var(name, dimids, nc_type, data, attrs=()):
        variables.append((name, dimids, nc_type, data, attrs))

    d_name = dim("len_name", _LEN_NAME)
    dim("four", 4)
    d_dim = dim("num_dim", 3)
    d_nodes = dim("num_nodes", len(coords))
    dim("num_elem", sum(len(np.asarray(b[1])) for b in blocks))
    d_blk = dim("num_el_blk", len(blocks))
    side_sets = [s for s in side_sets if len(s[2])]
    node_sets = [s for s in node_sets if len(s[2])]
    d_ss = dim("num_side_sets", len(side_sets)) if side_sets else None
    d_ns = dim("num_node_sets", len(node_sets)) if node_sets else None
    var("coordx", [d_nodes], _NC_DOUBLE, coords[:, 0])
    var("coordy", [d_nodes], _NC_DOUBLE, coords[:, 1])
    var("coordz", [d_nodes], _NC_DOUBLE, coords[:, 2])
    var("coor_names", [d_dim, d_name], _NC_CHAR, _names_array(["x", "y", "z"]))
    if node_num_map is not None:
        var("node_num_map", [d_nodes], _NC_INT, np.asarray(node_num_map, dtype=np.int64))
    var("eb_names", [d_blk, d_name], _NC_CHAR, _names_array([b[3] or "" for b in blocks]))
    var("eb_status", [d_blk], _NC_INT, np.ones(len(blocks), np.int64))
    var("eb_prop1", [d_blk], _NC_INT, np.array([b[2] for b in blocks]), [("name", _NC_CHAR, "ID")])
    for k, (topo, conn, _, _) in enumerate(blocks, 1):
        c = np.asarray(conn, dtype=np.int64)
        c = c.reshape(len(c), -1)
        de = dim(f"num_el_in_blk{k}", len(c))
        dn = dim(f"num_nod_per_el{k}", c.shape[1])
        var(f"connect{k}", [de, dn], _NC_INT, c + 1, [("elem_type", _NC_CHAR, _ELEM_TYPE[(topo, c.shape[1])])])
    if side_sets:
        var("ss_names", [d_ss, d_name], _NC_CHAR, _names_array([s[0] for s in side_sets]))
        var("ss_status", [d_ss], _NC_INT, np.ones(len(side_sets), np.int64))
        var("ss_prop1", [d_ss], _NC_INT, np.array([s[1] for s in side_sets]), [("name", _NC_CHAR, "ID")])
        for k, (_, _, pairs) in enumerate(side_sets, 1):
            p = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
            ds = dim(f"num_side_ss{k}", len(p))
            var(f"elem_ss{k}", [ds], _NC_INT, p[:, 0] + 1)
            var(f"side_ss{k}", [ds], _NC_INT, p[:, 1] + 1)
    if node_sets:
        var("ns_names", [d_ns, d_name], _NC_CHAR, _names_array([s[0] for s in node_sets]))
        var("ns_status", [d_ns], _NC_INT, np.ones(len(node_sets), np.int64))
        var("ns_prop1", [d_ns], _NC_INT, np.array([s[1] for s in node_sets]), [("name", _NC_CHAR, "ID")])
        for k, (_, _, nodes) in enumerate(node_sets, 1):
            nd = np.asarray(nodes, dtype=np.int64).reshape(-1)
            dk = dim(f"num_nod_ns{k}", len(nd))
            var(f"node_ns{k}", [dk], _NC_INT, nd + 1)

    # data blocks, then the header with their offsets (offset width fixed by the version)
    blobs = []
    for name, dimids, nc_type, data, attrs in variables:
        if nc_type == _NC_CHAR:
            raw = np.asarray(data, dtype="S1").tobytes()
        else:
            raw = np.asarray(data).astype(_FMT[nc_type]).tobytes()
        blobs.append(_pad(raw))
    off_fmt = ">i" if version == 1 else ">q"
    gatts = [("api_version", _NC_FLOAT, 8.0), ("version", _NC_FLOAT, 8.0),
             ("floating_point_word_size", _NC_INT, 8), ("file_size", _NC_INT, 1), ("title", _NC_CHAR, title)]

    def header(begins):
        h = b"CDF" + bytes([version]) + struct.pack(">i", 0)
        h += struct.pack(">ii", _NC_DIMENSION, len(dims))
        for name, n in dims:
            h += _name(name) + struct.pack(">i", n)
        h += struct.pack(">ii", _NC_ATTRIBUTE, len(gatts))
        for a in gatts:
            h += _attr(*a)
        h += struct.pack(">ii", _NC_VARIABLE, len(variables))
        for (name, dimids, nc_type, _, attrs), blob, begin in zip(variables, blobs, begins):
            h += _name(name) + struct.pack(">i", len(dimids)) + b"".join(struct.pack(">i", d) for d in dimids)
            h += struct.pack(">ii", _NC_ATTRIBUTE, len(attrs)) + b"".join(_attr(*a) for a in attrs) \
                if attrs else struct.pack(">ii", 0, 0)
            h += struct.pack(">ii", nc_type, len(blob)) + struct.pack(off_fmt, begin)
        return h

    size = len(header([0] * len(variables)))
    begins, at = [], size
    for blob in blobs:
        begins.append(at)
        at += len(blob)
    if version == 1 and at >= 2 ** 31:
        raise ValueError("file too large for CDF-1; use version=2")
    with open(path, "wb") as f:
        f.write(header(begins))
        for blob in blobs:
            f.write(blob)
    return path
