"""Panzer/Tianxin-shaped host API over the C-ABI (device memory via torch).

Class and method names follow the reference so a caller of the reference's
assembly path finds the same objects:

  CartesianConnManager      dof-mgr/test/cartesian_topology/CartesianConnManager.hpp
  DOFManager                dof-mgr/src/Panzer_DOFManager.hpp (GlobalIndexer queries)
  TpetraLinearObjFactory    disc-fe/src/lof/Panzer_TpetraLinearObjFactory_decl.hpp
  CrsMatrix                 Tpetra::CrsMatrix local layout (rowptr, colind, values)
  DirichletBC               TianXin::DirichletEvalautor parameter list
  NeumannBC                 "Neumann Conditions" entry of Type "Flux" (TianXin::Flux,
                            disc-fe/src/evaluators/TianXin_Neumann_impl.hpp:146-166)
  ModelEvaluator.evalModel  disc-fe/src/Panzer_ModelEvaluator_impl.hpp:1714-1882
  AssemblyEngine.evaluate   disc-fe/src/Panzer_AssemblyEngine_impl.hpp:65-182

Errors from the library raise TxError (the reference throws std::logic_error /
TEUCHOS_TEST_FOR_EXCEPTION in the same places).
"""
import ctypes as C

import numpy as np
import torch

from . import _abi
from ._lib import TxError, check, load

HEX, TET = _abi.TX_TOPO_HEX, _abi.TX_TOPO_TET


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _np_ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def _element_vertices(conn, block):
    nv, n = C.c_int32(), len(conn.getElementBlock(block))
    check(conn.h, conn.lib.tx_mesh_element_vertices(conn.h, block, C.byref(nv), None))
    out = np.zeros((n, nv.value), np.int64)
    check(conn.h, conn.lib.tx_mesh_element_vertices(conn.h, block, C.byref(nv), _np_ptr(out)))
    return out


class CartesianConnManager:
    """Brick lattice on one rank; blocks named eblock-i_j_k (i slowest)."""

    def __init__(self, nx, ny, nz, bx=1, by=1, bz=1, topology=HEX, lengths=(1.0, 1.0, 1.0), jitter=0.0, seed=0):
        self.lib = load()
        self.desc = _abi.mesh_desc((nx, ny, nz), (bx, by, bz), topology, lengths, jitter, seed)
        h = C.c_void_p()
        rc = self.lib.tx_mesh_create(C.byref(self.desc), C.byref(h))
        if rc != 0:
            raise TxError(rc, "tx_mesh_create: " + self.lib.tx_last_error(None).decode())
        self.h = h
        ne, nv, nb = C.c_int64(), C.c_int64(), C.c_int32()
        self.lib.tx_mesh_sizes(self.h, C.byref(ne), C.byref(nv), C.byref(nb))
        self.n_elements, self.n_vertices, self.n_blocks = ne.value, nv.value, nb.value

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.tx_destroy(self.h)
            self.h = None

    def numElementBlocks(self):
        return self.n_blocks

    def getElementBlockIds(self):
        d = self.desc
        return [f"eblock-{i}_{j}_{k}" for i in range(d.bx) for j in range(d.by) for k in range(d.bz)]

    def getElementBlock(self, block):
        n = C.c_int64()
        check(self.h, self.lib.tx_mesh_block_elements(self.h, block, C.byref(n), None))
        out = np.zeros(n.value, np.int64)
        check(self.h, self.lib.tx_mesh_block_elements(self.h, block, C.byref(n), _np_ptr(out)))
        return out

    def coordinates(self):
        out = np.zeros((self.n_vertices, 3))
        check(self.h, self.lib.tx_mesh_coordinates(self.h, _np_ptr(out)))
        return out

    def getElementVertices(self, block):
        """Vertex node numbers [E][nv] of a block's elements (shards order)."""
        return _element_vertices(self, block)


class ExplicitConnManager:
    """An unstructured hex8/tet4 mesh (nodal fields) from arrays or an Exodus II file.

    Node numbers are 0-based and are the vertex GIDs of the numbering.  Side
    sets hold (element, side) pairs (element over the whole mesh, 0-based
    shards side); node sets hold node numbers.  Blocks, side sets and node
    sets are addressed by index or name.
    """

    def __init__(self, h, lib):
        self.h, self.lib = h, lib
        ne, nv, nb = C.c_int64(), C.c_int64(), C.c_int32()
        self.lib.tx_mesh_sizes(self.h, C.byref(ne), C.byref(nv), C.byref(nb))
        self.n_elements, self.n_vertices, self.n_blocks = ne.value, nv.value, nb.value

    @classmethod
    def from_arrays(cls, coords, blocks, side_sets=(), node_sets=()):
        """blocks: [(topology, conn[E][nodes], id, name)] with the vertices or the hex27 / tet10 nodes (shards order);
        side_sets: [(name, id, [(elem, side), ...])];
        node_sets: [(name, id, nodes)]."""
        lib = load()
        xyz = np.ascontiguousarray(coords, dtype=np.float64).reshape(-1, 3)
        keep = [xyz]
        bl = (_abi.ExplicitBlock * len(blocks))()
        for k, (topo, conn, bid, name) in enumerate(blocks):
            c = np.ascontiguousarray(conn, dtype=np.int64)
            keep.append(c)
            bl[k].topology, bl[k].n_elem, bl[k].conn, bl[k].id = topo, c.shape[0], _np_ptr(c), bid
            bl[k].nodes_per_elem = c.shape[1] if c.ndim == 2 else 0  # vertices, or hex27 / tet10 nodes
            bl[k].name = name.encode() if name else None

        def sets(items, per):
            arr = (_abi.ExplicitSet * max(len(items), 1))()
            for k, (name, sid, entries) in enumerate(items):
                e = np.ascontiguousarray(entries, dtype=np.int64).reshape(-1)
                keep.append(e)
                arr[k].n, arr[k].entries, arr[k].id = len(e) // per, _np_ptr(e), sid
                arr[k].name = name.encode() if name else None
            return arr

        d = _abi.MeshExplicitDesc()
        d.n_nodes, d.coords, d.n_blocks, d.blocks = len(xyz), _np_ptr(xyz), len(blocks), bl
        d.n_side_sets, d.side_sets = len(side_sets), sets(side_sets, 2)
        d.n_node_sets, d.node_sets = len(node_sets), sets(node_sets, 1)
        h, err = C.c_void_p(), C.create_string_buffer(512)
        rc = lib.tx_mesh_create_explicit(C.byref(d), C.byref(h), err, 512)
        if rc != 0:
            raise TxError(rc, "tx_mesh_create_explicit: " + err.value.decode())
        return cls(h, lib)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.tx_destroy(self.h)
            self.h = None

    def _names(self, kind):
        n = C.c_int64()
        check(self.h, self.lib.tx_mesh_set_info(self.h, kind, -1, None, None, 0, C.byref(n)))
        out = []
        for k in range(n.value):
            buf = C.create_string_buffer(256)
            check(self.h, self.lib.tx_mesh_set_info(self.h, kind, k, None, buf, 256, None))
            out.append(buf.value.decode())
        return out

    def _entries(self, kind, k):
        n = C.c_int64()
        check(self.h, self.lib.tx_mesh_set_info(self.h, kind, k, None, None, 0, C.byref(n)))
        out = np.zeros(n.value * (2 if kind == 1 else 1), np.int64)
        if len(out):
            check(self.h, self.lib.tx_mesh_set_entries(self.h, kind, k, _np_ptr(out)))
        return out.reshape(-1, 2) if kind == 1 else out

    def _index(self, kind, key):
        return key if isinstance(key, (int, np.integer)) else self._names(kind).index(key)

    def numElementBlocks(self):
        return self.n_blocks

    def getElementBlockIds(self):
        return self._names(0)

    def getSidesetNames(self):
        return self._names(1)

    def getNodesetNames(self):
        return self._names(2)

    def getElementBlock(self, block):
        return self._entries(0, self._index(0, block))

    def getSideset(self, key):
        """(element, side) pairs of a side set."""
        return self._entries(1, self._index(1, key))

    def getNodeset(self, key):
        return self._entries(2, self._index(2, key))

    def sideSetIndex(self, key):
        return self._index(1, key)

    def nodeSetIndex(self, key):
        return self._index(2, key)

    def coordinates(self):
        out = np.zeros((self.n_vertices, 3))
        check(self.h, self.lib.tx_mesh_coordinates(self.h, _np_ptr(out)))
        return out

    def getElementVertices(self, block):
        """Vertex node numbers [E][nv] of a block's elements (shards order)."""
        return _element_vertices(self, block)


class ExodusReaderFactory:
    """STK_ExodusReaderFactory: "File Name" of a 3-D Exodus II mesh (NetCDF classic).

    linear=True keeps the vertex nodes of quadratic elements (the
    QuadraticToLinearMeshFactory conversion)."""

    def __init__(self, file_name, linear=False):
        self.file_name, self.linear = str(file_name), linear

    def buildMesh(self):
        lib = load()
        h, err = C.c_void_p(), C.create_string_buffer(512)
        rc = lib.tx_mesh_create_exodus(self.file_name.encode(), int(self.linear), C.byref(h), err, 512)
        if rc != 0:
            raise TxError(rc, "tx_mesh_create_exodus: " + err.value.decode())
        return ExplicitConnManager(h, lib)


def exodus_summary(file_name):
    """Sizes of an Exodus file of any dimension: version, dim, n_nodes, n_elem, n_blocks, n_side_sets, n_node_sets."""
    s, err = _abi.ExodusSummary(), C.create_string_buffer(512)
    rc = load().tx_exodus_inspect(str(file_name).encode(), C.byref(s), err, 512)
    if rc != 0:
        raise TxError(rc, "tx_exodus_inspect: " + err.value.decode())
    return {k: getattr(s, k) for k, _ in _abi.ExodusSummary._fields_}


class DOFManager:
    """buildGlobalUnknowns for the fields of one equation set on a mesh."""

    def __init__(self, conn, eqset, require_device=True):
        self.conn, self.eqset, self.lib, self.h = conn, eqset, conn.lib, conn.h
        rc = self.lib.tx_dof_build(self.h, C.byref(eqset))
        if rc != 0 and (require_device or rc != _abi.TX_ECUDA):
            check(self.h, rc, "tx_dof_build")
        self.device_ready = rc == 0
        n, ndm, nnz, nf = C.c_int64(), C.c_int32(), C.c_int64(), C.c_int32()
        check(self.h, self.lib.tx_dof_sizes(self.h, C.byref(n), C.byref(ndm), C.byref(nnz), C.byref(nf)))
        self.n_dofs, self.max_gid_count, self.nnz, self.n_fields = n.value, ndm.value, nnz.value, nf.value
        self.field_names = _abi.field_names(eqset.physics)

    # GlobalIndexer queries --------------------------------------------------
    def getFieldNum(self, name):
        return self.field_names.index(name)

    def getFieldString(self, num):
        return self.field_names[num]

    def getNumFields(self):
        return self.n_fields

    def getOwnedIndices(self):
        out = np.zeros(self.n_dofs, np.int64)
        check(self.h, self.lib.tx_dof_owned_gids(self.h, _np_ptr(out)))
        return out

    def getElementBlockGIDCount(self, block):
        n = C.c_int32()
        check(self.h, self.lib.tx_dof_block_gid_count(self.h, block, C.byref(n)))
        return n.value

    def getElementGIDs(self, block):
        ne = len(self.conn.getElementBlock(block))
        out = np.zeros((ne, self.getElementBlockGIDCount(block)), np.int64)
        check(self.h, self.lib.tx_dof_element_gids(self.h, block, _np_ptr(out)))
        return out

    def getElementLIDs(self, block):
        ne = len(self.conn.getElementBlock(block))
        out = np.zeros((ne, self.getElementBlockGIDCount(block)), np.int32)
        check(self.h, self.lib.tx_dof_element_lids(self.h, block, _np_ptr(out)))
        return out

    def getGIDFieldOffsets(self, block, field):
        n = C.c_int32()
        check(self.h, self.lib.tx_dof_field_offsets(self.h, block, field, C.byref(n), None))
        out = np.zeros(n.value, np.int32)
        check(self.h, self.lib.tx_dof_field_offsets(self.h, block, field, C.byref(n), _np_ptr(out)))
        return out

    def dirichletDofsNodeSet(self, node_set, field_mask=0x7):
        """Sorted local DOF ids of the fields in field_mask at the nodes of a node set (explicit meshes)."""
        k = self.conn.nodeSetIndex(node_set)
        n = C.c_int64()
        check(self.h, self.lib.tx_dirichlet_dofs_node_set(self.h, k, field_mask, C.byref(n), None))
        out = np.zeros(n.value, np.int32)
        check(self.h, self.lib.tx_dirichlet_dofs_node_set(self.h, k, field_mask, C.byref(n), _np_ptr(out)))
        return out

    def dirichletDofs(self, side_mask, field_mask=0x7):
        """Sorted local DOF ids of the fields in field_mask on the given box sides."""
        n = C.c_int64()
        check(self.h, self.lib.tx_dirichlet_dofs(self.h, side_mask, field_mask, C.byref(n), None))
        out = np.zeros(n.value, np.int32)
        check(self.h, self.lib.tx_dirichlet_dofs(self.h, side_mask, field_mask, C.byref(n), _np_ptr(out)))
        return out


class CrsMatrix:
    """Tpetra local CRS on the device: rowptr int64, colind int32, values f64.

    on_handle_graph: rowptr/colind are the graph the DOF manager's handle
    built (TpetraLinearObjFactory), so apply and the solver may take the
    entity-block form (one column index per nf x nf block); apply_form is
    "entity" or "crs".
    """

    def __init__(self, dof, rowptr, colind, values=None, on_handle_graph=False):
        self.dof, self.rowptr, self.colind = dof, rowptr, colind
        self.values = values if values is not None else torch.zeros(colind.numel(), dtype=torch.float64,
                                                                      device=colind.device)
        self.n_rows = rowptr.numel() - 1
        self.on_handle_graph = on_handle_graph
        self.apply_form = "entity" if on_handle_graph else "crs"

    def initializeMatrix(self, v=0.0):
        self.values.fill_(v)

    def apply(self, x, y=None, alpha=1.0, beta=0.0, values=None):
        """y = alpha A x + beta y (Tpetra::CrsMatrix::apply); f64 or f32 by dtype of values."""
        vals = self.values if values is None else values
        prec = _abi.TX_SPMV_F64 if vals.dtype == torch.float64 else _abi.TX_SPMV_F32
        if self.apply_form == "entity":
            prec |= _abi.TX_SPMV_ENTITY_BLOCKS
        if y is None:
            y = torch.zeros(self.n_rows, dtype=vals.dtype, device=vals.device)
        lib = self.dof.lib
        lib.tx_set_stream(self.dof.h, C.c_void_p(torch.cuda.current_stream().cuda_stream))
        check(self.dof.h, lib.tx_spmv(self.dof.h, prec, self.n_rows, _ptr(self.rowptr), _ptr(self.colind), _ptr(vals),
                                      _ptr(x), _ptr(y), alpha, beta), "tx_spmv")
        return y

    def setApplyShape(self, lanes=0, unroll=0):
        """Launch shape of apply (and of the solver's SpMV) on this handle: lanes per row, loads per lane; 0, 0 = auto."""
        check(self.dof.h, self.dof.lib.tx_set_spmv_shape(self.dof.h, lanes, unroll), "tx_set_spmv_shape")

    def setEntityApplyShape(self, lanes=0, unroll=0):
        """Launch shape of the entity-block form: lanes per entity, blocks per lane pass; 0, 0 = auto."""
        check(self.dof.h, self.dof.lib.tx_set_spmv_entity_shape(self.dof.h, lanes, unroll),
              "tx_set_spmv_entity_shape")

    def setApplyForm(self, form):
        """"entity" (the handle's graph only) or "crs"."""
        if form not in ("entity", "crs") or (form == "entity" and not self.on_handle_graph):
            raise ValueError(f"apply form {form!r} not available for this matrix")
        self.apply_form = form

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.values.cpu().numpy(), self.colind.cpu().numpy(), self.rowptr.cpu().numpy()),
                             shape=(self.n_rows, self.n_rows))


class TpetraLinearObjFactory:
    """Owns the CRS graph (buildGhostedGraph; one rank: ghosted == owned)."""

    def __init__(self, dof, device="cuda"):
        self.dof, self.device = dof, device
        self.rowptr = torch.empty(dof.n_dofs + 1, dtype=torch.int64, device=device)
        self.colind = torch.empty(dof.nnz, dtype=torch.int32, device=device)
        dof.lib.tx_set_stream(dof.h, C.c_void_p(torch.cuda.current_stream().cuda_stream))
        check(dof.h, dof.lib.tx_graph_build(dof.h, _ptr(self.rowptr), _ptr(self.colind)), "tx_graph_build")

    def buildGraph(self):
        return self.rowptr, self.colind

    def getTpetraMatrix(self):
        return CrsMatrix(self.dof, self.rowptr, self.colind, on_handle_graph=True)

    def getTpetraVector(self):
        return torch.zeros(self.dof.n_dofs, dtype=torch.float64, device=self.device)


def _ptr_array(tensors):
    """Host array of device pointers (NULL for None), kept alive by the caller."""
    arr = (C.c_void_p * len(tensors))(*[None if t is None else t.data_ptr() for t in tensors])
    return arr


class BlockedDOFManager:
    """BlockedDOFManager: the fields of one equation set grouped into field blocks.

    blocks lists the field names of each block, e.g. [["UX"], ["UY"], ["UZ"]]
    (every field in exactly one block; inside a block the fields take the
    equation set's field order).  Block i numbers its DOFs
    b_i * entity + k (k = the field's place in the block) over the entities
    of the interleaved DOFManager in its LID order, as a DOFManager built on
    the block's fields alone numbers them.
    """

    def __init__(self, dof, blocks):
        self.dof, self.lib, self.h = dof, dof.lib, dof.h
        # within a block the fields keep the equation set's field order
        self.blocks = [sorted(b, key=dof.getFieldNum) for b in blocks]
        fb = np.full(dof.n_fields, -1, np.int32)
        for i, names in enumerate(self.blocks):
            for name in names:
                f = dof.getFieldNum(name)
                if fb[f] >= 0:
                    raise ValueError(f"field {name} in two blocks")
                fb[f] = i
        if (fb < 0).any():
            raise ValueError("every field must be in a block")
        self._fb = fb
        check(self.h, self.lib.tx_blocked_layout(self.h, len(self.blocks), _np_ptr(fb)), "tx_blocked_layout")
        self.n_entities = dof.n_dofs // dof.n_fields

    def getNumFieldBlocks(self):
        return len(self.blocks)

    def getFieldBlocks(self):
        return self.blocks

    def getFieldBlock(self, name):
        return int(self._fb[self.dof.getFieldNum(name)])

    def getBlockSize(self, i):
        return len(self.blocks[i]) * self.n_entities

    def getFieldDOFs(self, i, name):
        """Block-i LIDs of field name (entity order)."""
        k = self.blocks[i].index(name)
        return np.arange(self.n_entities, dtype=np.int64) * len(self.blocks[i]) + k

    def getOwnedIndices(self, i):
        """Block-i GIDs in block-LID order: ascending entity GID, the block's fields interleaved."""
        g = self.dof.getOwnedIndices()
        nf = self.dof.n_fields
        ent_rank, f = g // nf, g % nf
        keep = self._fb[f] == i
        pos = np.array([self.blocks[i].index(self.dof.getFieldString(k)) if self._fb[k] == i else -1
                        for k in range(nf)])
        return ent_rank[keep] * len(self.blocks[i]) + pos[f[keep]]


class BlockedCrsMatrix:
    """The blocked operator [A_ij] (Thyra blocked linear op of Tpetra CRS blocks; None = excluded pair)."""

    def __init__(self, blof, blocks):
        self.blof, self.blocks = blof, blocks

    def getBlock(self, i, j):
        return self.blocks[i][j]

    def initializeMatrix(self, v=0.0):
        for row in self.blocks:
            for m in row:
                if m is not None:
                    m.initializeMatrix(v)

    def apply(self, xb, yb=None, alpha=1.0, beta=0.0):
        """y_i = alpha sum_j A_ij x_j + beta y_i over the blocks not excluded."""
        bd = self.blof.bdof
        if yb is None:
            yb = [torch.zeros(bd.getBlockSize(i), dtype=torch.float64, device=xb[0].device)
                  for i in range(bd.getNumFieldBlocks())]
        vals = [m.values if m is not None else None for row in self.blocks for m in row]
        lib = bd.lib
        lib.tx_set_stream(bd.h, C.c_void_p(torch.cuda.current_stream().cuda_stream))
        pv, px, py = _ptr_array(vals), _ptr_array(xb), _ptr_array(yb)
        check(bd.h, lib.tx_blocked_spmv(bd.h, pv, px, py, alpha, beta), "tx_blocked_spmv")
        return yb


class BlockedTpetraLinearObjFactory:
    """BlockedTpetraLinearObjFactory: block graphs, block vectors and the blocked operator of a BlockedDOFManager."""

    def __init__(self, bdof, device="cuda"):
        self.bdof, self.device = bdof, device
        self.excluded = set()
        self._graphs = {}

    def getBlockRowCount(self):
        return self.bdof.getNumFieldBlocks()

    def getBlockColCount(self):
        return self.bdof.getNumFieldBlocks()

    def addExcludedPair(self, i, j):
        self.excluded.add((i, j))

    def addExcludedPairs(self, pairs):
        for i, j in pairs:
            self.addExcludedPair(i, j)

    def getGraph(self, i, j):
        if (i, j) not in self._graphs:
            bd = self.bdof
            rows, cols, nnz = C.c_int64(), C.c_int64(), C.c_int64()
            check(bd.h, bd.lib.tx_blocked_sizes(bd.h, i, j, C.byref(rows), C.byref(cols), C.byref(nnz)),
                  "tx_blocked_sizes")
            rp = torch.empty(rows.value + 1, dtype=torch.int64, device=self.device)
            ci = torch.empty(nnz.value, dtype=torch.int32, device=self.device)
            bd.lib.tx_set_stream(bd.h, C.c_void_p(torch.cuda.current_stream().cuda_stream))
            check(bd.h, bd.lib.tx_blocked_graph_build(bd.h, i, j, _ptr(rp), _ptr(ci)), "tx_blocked_graph_build")
            self._graphs[(i, j)] = (rp, ci)
        return self._graphs[(i, j)]

    def getTpetraMatrix(self, i, j):
        rp, ci = self.getGraph(i, j)
        return CrsMatrix(self.bdof.dof, rp, ci)

    def getTpetraDomainVector(self, i):
        return torch.zeros(self.bdof.getBlockSize(i), dtype=torch.float64, device=self.device)

    getTpetraRangeVector = getTpetraDomainVector

    def getBlockedVector(self):
        return [self.getTpetraDomainVector(i) for i in range(self.getBlockRowCount())]

    def getBlockedMatrix(self):
        n = self.getBlockRowCount()
        return BlockedCrsMatrix(self, [[None if (i, j) in self.excluded else self.getTpetraMatrix(i, j)
                                        for j in range(n)] for i in range(n)])

    def splitVector(self, x, xb=None):
        """Interleaved vector -> block vectors."""
        xb = self.getBlockedVector() if xb is None else xb
        bd = self.bdof
        bd.lib.tx_set_stream(bd.h, C.c_void_p(torch.cuda.current_stream().cuda_stream))
        check(bd.h, bd.lib.tx_blocked_split_vector(bd.h, _ptr(x), _ptr_array(xb)), "tx_blocked_split_vector")
        return xb

    def mergeVector(self, xb, x=None):
        """Block vectors -> interleaved vector."""
        x = torch.zeros(self.bdof.dof.n_dofs, dtype=torch.float64, device=self.device) if x is None else x
        bd = self.bdof
        bd.lib.tx_set_stream(bd.h, C.c_void_p(torch.cuda.current_stream().cuda_stream))
        check(bd.h, bd.lib.tx_blocked_merge_vector(bd.h, _ptr_array(xb), _ptr(x)), "tx_blocked_merge_vector")
        return x

    def splitMatrix(self, W, Wb):
        """Interleaved CRS values (the DOFManager's graph) -> the blocks of Wb (excluded blocks skipped)."""
        bd = self.bdof
        vals = [m.values if m is not None else None for row in Wb.blocks for m in row]
        bd.lib.tx_set_stream(bd.h, C.c_void_p(torch.cuda.current_stream().cuda_stream))
        check(bd.h, bd.lib.tx_blocked_split_matrix(bd.h, _ptr(W.values), _ptr_array(vals)),
              "tx_blocked_split_matrix")
        return Wb


class DirichletBC:
    """Dirichlet parameter list: DOF Names on the box sides (a side mask) or, on an explicit
    mesh, on a node set (name or index), value g."""

    def __init__(self, dof, side_mask=None, fields=None, value=0.0, node_set=None):
        names = fields if fields is not None else dof.field_names
        mask = 0
        for n in names:
            mask |= 1 << dof.getFieldNum(n)
        if node_set is not None:
            self.lids_host = dof.dirichletDofsNodeSet(node_set, mask)
        else:
            self.lids_host = dof.dirichletDofs(side_mask, mask)
        self.lids = torch.from_numpy(self.lids_host).to("cuda")
        if np.isscalar(value):
            self.g = None if value == 0.0 else torch.full((len(self.lids_host),), float(value), dtype=torch.float64,
                                                           device="cuda")
        else:
            self.g = torch.as_tensor(value, dtype=torch.float64, device="cuda")


_VALUE_TYPES = {"Constant": _abi.TX_VALUE_CONSTANT, "Linear": _abi.TX_VALUE_LINEAR,
                "TimeTable": _abi.TX_VALUE_TIME_TABLE}


def neumann_desc(block, side_mask, field, value_type="Constant", value=0.0, times=None, values=None, side_set=-1):
    """tx_neumann_desc from the reference's parameter names; the table arrays stay referenced by the result.
    side_set >= 0 names a side set of an explicit mesh by index (then side_mask is unused)."""
    d = _abi.NeumannDesc()
    d.block, d.side_mask, d.field = block, side_mask, field
    d.side_set = side_set + 1
    d.value_type = _VALUE_TYPES[value_type] if isinstance(value_type, str) else int(value_type)
    d.value = float(value)
    if times is not None:
        tt = np.ascontiguousarray(times, dtype=np.float64)
        tv = np.ascontiguousarray(values, dtype=np.float64)
        if tt.shape != tv.shape:
            raise ValueError("Time Values and BC Values differ in length")
        d.n_table, d.table_t, d.table_v = len(tt), _np_ptr(tt), _np_ptr(tv)
        d._keep = (tt, tv)
    return d


def neumann_value(value_type="Constant", value=0.0, times=None, values=None, t=0.0):
    """WorksetFunctor value at time t (host only; TianXin_WorksetFunctor_impl.hpp)."""
    d = neumann_desc(0, 1, 0, value_type, value, times, values)
    out = C.c_double()
    rc = load().tx_neumann_value(C.byref(d), t, C.byref(out))
    if rc != 0:
        raise TxError(rc, "tx_neumann_value")
    return out.value


class NeumannBC:
    """A "Neumann Conditions" sublist of Type "Flux": Element Block Name (block), SideSet Name (side mask),
    DOF Name, Value Type (Constant / Linear / TimeTable) and its value or table.

    Creating it builds the side workset and side tables on the device; evaluate(f, t) adds the flux to f.
    """

    def __init__(self, dof, side_mask=0, dof_name=None, value_type="Constant", value=0.0, times=None, values=None,
                 block=0, side_set=None):
        field = dof.getFieldNum(dof_name) if dof_name is not None else 0
        self.dof = dof
        ss = dof.conn.sideSetIndex(side_set) if side_set is not None else -1
        self.desc = neumann_desc(block, side_mask, field, value_type, value, times, values, side_set=ss)
        sid, ns = C.c_int32(), C.c_int64()
        check(dof.h, dof.lib.tx_neumann_create(dof.h, C.byref(self.desc), C.byref(sid), C.byref(ns)),
              "tx_neumann_create")
        self.id, self.n_sides = sid.value, ns.value

    def value(self, t=0.0):
        out = C.c_double()
        check(self.dof.h, self.dof.lib.tx_neumann_value(C.byref(self.desc), t, C.byref(out)), "tx_neumann_value")
        return out.value

    def evaluate(self, f, t=0.0):
        lib = self.dof.lib
        lib.tx_set_stream(self.dof.h, C.c_void_p(torch.cuda.current_stream().cuda_stream))
        check(self.dof.h, lib.tx_neumann_eval(self.dof.h, self.id, t, _ptr(f)), "tx_neumann_eval")
        return f


def eval_args(x, x_dot=None, aux=None, alpha=0.0, beta=1.0, t=0.0, f=None, W=None, mixed=False, block=-1,
              workset=(0, -1), deterministic=False, persistent=False, scatter_direct=False):
    a = _abi.EvalArgs()
    a.x, a.x_dot, a.aux = _ptr(x), _ptr(x_dot), _ptr(aux)
    a.alpha, a.beta, a.t = alpha, beta, t
    a.f = _ptr(f)
    a.crs_vals = _ptr(W.values) if W is not None else None
    a.block = block
    a.elem_begin, a.elem_end = workset
    a.flags = ((_abi.TX_EVAL_MIXED if mixed else 0) | (_abi.TX_EVAL_DETERMINISTIC if deterministic else 0) |
               (_abi.TX_EVAL_PERSISTENT if persistent else 0) |
               (_abi.TX_EVAL_SCATTER_DIRECT if scatter_direct else 0))
    return a


class AssemblyEngine:
    """Volume fill of every block (or one workset range of a block)."""

    def __init__(self, lof):
        self.lof, self.dof = lof, lof.dof
        self.scatter_direct = False  # set by the autotuner
        self.gather = False          # two-phase evaluation (TX_EVAL_GATHER), set by the autotuner
        self._gather_fits = None     # whether TX_EVAL_GATHER holds the handle's rows (asked once)

    def setWorksetSize(self, min_size, max_size=None, seed=0):
        """Worksets of the persistent evaluation: sizes uniform in [min_size, max_size]."""
        check(self.dof.h, self.dof.lib.tx_set_worksets(self.dof.h, min_size, max_size or min_size, seed),
              "tx_set_worksets")

    def setGridCap(self, max_ctas):
        check(self.dof.h, self.dof.lib.tx_set_grid_cap(self.dof.h, max_ctas), "tx_set_grid_cap")

    def setVariant(self, variant):
        """Assembly kernel: 0 automatic, 1 CTA-staged, 2 warp per element (hex8 elasticity, mixed), 3 the
        element contractions on the tensor cores (hex8 elasticity, mixed R+J; tcgen05 TF32 with hi/lo splitting)."""
        check(self.dof.h, self.dof.lib.tx_set_assembly_variant(self.dof.h, variant), "tx_set_assembly_variant")

    def setCtaThreads(self, threads):
        """Threads a CTA of the staged Jacobian kernel (64, 128 or 256; elements per CTA = threads / the
        element's basis count rounded up to a power of two); 0 restores 128."""
        check(self.dof.h, self.dof.lib.tx_set_cta_threads(self.dof.h, threads), "tx_set_cta_threads")

    def gather_supported(self):
        """Whether the two-phase form holds this handle's rows (not, e.g., quadratic elasticity's)."""
        if self._gather_fits is None:
            ok = C.c_int32()
            check(self.dof.h, self.dof.lib.tx_eval_gather_supported(self.dof.h, C.byref(ok)), "tx_eval_gather_supported")
            self._gather_fits = bool(ok.value)
        return self._gather_fits

    def gather_form(self):
        """The form of TX_EVAL_GATHER with mixed precision: "lattice" (owner-computes rows of a hex8 elasticity
        lattice), "two-phase" (element rows to scratch, then the row gather) or None."""
        form = C.c_int32()
        check(self.dof.h, self.dof.lib.tx_eval_gather_form(self.dof.h, C.byref(form)), "tx_eval_gather_form")
        return {_abi.TX_GATHER_LATTICE: "lattice", _abi.TX_GATHER_TWO_PHASE: "two-phase"}.get(form.value)

    def gather_applies(self, W, block=-1, workset=(0, -1), deterministic=False, persistent=False):
        """Whether evaluate() with these arguments takes the two-phase form (f and W overwritten)."""
        return (self.gather and W is not None and block < 0 and tuple(workset) == (0, -1) and not deterministic
                and not persistent and self.gather_supported())

    def evaluate(self, x, x_dot=None, aux=None, alpha=0.0, beta=1.0, t=0.0, f=None, W=None, mixed=False,
                 block=-1, workset=(0, -1), deterministic=False, persistent=False, scatter_direct=None, gather=None):
        """Volume fill.  Summed into f and W, except in the two-phase form (gather=True, or the tuned
        default for whole-handle Jacobian evaluations), which overwrites them."""
        if scatter_direct is None:
            scatter_direct = self.scatter_direct
        if gather is None:
            gather = self.gather_applies(W, block, workset, deterministic, persistent)
        a = eval_args(x, x_dot, aux, alpha, beta, t, f, W, mixed, block, workset, deterministic, persistent,
                      scatter_direct)
        if gather:
            a.flags |= _abi.TX_EVAL_GATHER
        lib = self.dof.lib
        lib.tx_set_stream(self.dof.h, C.c_void_p(torch.cuda.current_stream().cuda_stream))
        check(self.dof.h, lib.tx_eval(self.dof.h, C.byref(a)), "tx_eval")

    def evaluateDfdp(self, x, param, dfdp, x_dot=None, aux=None, t=0.0, block=-1, workset=(0, -1)):
        """dfdp += df/dp for the equation set's parameter params[param] (the Tangent type's dfdp vector)."""
        a = eval_args(x, x_dot, aux, 0.0, 1.0, t, None, None, False, block, workset)
        lib = self.dof.lib
        lib.tx_set_stream(self.dof.h, C.c_void_p(torch.cuda.current_stream().cuda_stream))
        check(self.dof.h, lib.tx_eval_dfdp(self.dof.h, C.byref(a), int(param), _ptr(dfdp)), "tx_eval_dfdp")
        return dfdp

    def evaluateTangent(self, x, tangent, dfdp, x_dot=None, aux=None, alpha=0.0, beta=1.0, t=0.0, block=-1,
                        workset=(0, -1), deterministic=False):
        """Tangent evaluation type: dfdp[i] += (beta dR/dx + alpha dR/dxdot) tangent[i] for the rows of the
        2-D tensors tangent and dfdp ([n_tangent, N], n_tangent <= 4); f and W are not touched."""
        a = eval_args(x, x_dot, aux, alpha, beta, t, None, None, False, block, workset, deterministic)
        a.flags |= _abi.TX_EVAL_TANGENT
        a.tangent, a.dfdp, a.n_tangent = _ptr(tangent), _ptr(dfdp), int(tangent.shape[0])
        lib = self.dof.lib
        lib.tx_set_stream(self.dof.h, C.c_void_p(torch.cuda.current_stream().cuda_stream))
        check(self.dof.h, lib.tx_eval(self.dof.h, C.byref(a)), "tx_eval (Tangent)")
        return dfdp


class ModelEvaluator:
    """evalModel(inArgs{x, x_dot, alpha, beta, t}, outArgs{f, W}) on the device."""

    def __init__(self, lof, dirichlet=(), neumann=()):
        self.lof, self.dof = lof, lof.dof
        self.ae = AssemblyEngine(lof)
        self.dirichlet = list(dirichlet)
        self.neumann = list(neumann)

    def create_W_op(self):
        return self.lof.getTpetraMatrix()

    def evalModel(self, x, x_dot=None, alpha=0.0, beta=1.0, t=0.0, f=None, W=None, aux=None, mixed=False,
                  zero=True, deterministic=False, persistent=False):
        # A Jacobian evaluation from zero may take the two-phase form, which overwrites f and W (no zeroing):
        # when the autotuner chose it, and for deterministic evaluations, where its fixed-order row sums
        # are faster than the coloured launches.  zero=False sums into f and W: the atomic forms.
        gather = zero and W is not None and not persistent and (self.ae.gather or deterministic) and \
            self.ae.gather_supported()
        if zero and not gather:
            if f is not None:
                f.zero_()
            if W is not None:
                W.initializeMatrix(0.0)
        self.ae.evaluate(x, x_dot, aux, alpha, beta, t, f, W, mixed, deterministic=deterministic and not gather,
                         persistent=persistent, gather=gather)
        if f is not None:  # Neumann sums into equations before Dirichlet overwrites rows
            for bc in self.neumann:
                bc.evaluate(f, t)
        self.applyDirichlet(x, f, W)
        return f, W

    def applyDirichlet(self, x, f=None, W=None):
        lib = self.dof.lib
        for bc in self.dirichlet:
            check(self.dof.h, lib.tx_dirichlet_apply(self.dof.h, len(bc.lids_host), _ptr(bc.lids), _ptr(bc.g), _ptr(x),
                                                     _ptr(f), _ptr(W.values) if W is not None else None),
                  "tx_dirichlet_apply")

    def dirichlet_lids(self):
        if not self.dirichlet:
            return torch.zeros(0, dtype=torch.int32, device="cuda"), None
        lids = torch.cat([bc.lids for bc in self.dirichlet])
        gs = [bc.g if bc.g is not None else torch.zeros(len(bc.lids_host), dtype=torch.float64, device="cuda")
              for bc in self.dirichlet]
        return lids, torch.cat(gs)

    def solve(self, W, x, b=None, rtol=1e-10, inner_rtol=1e-5, max_outer=50, max_inner=100000, matrix_free=False,
              x_dot=None, alpha=0.0, beta=1.0, t=0.0, fixed=False, reuse_operator=False, stats_device=None,
              x_pred=None, x_dot_coef=0.0, block_jacobi=False):
        """FP64 iterative refinement around FP32 Jacobi-CG; x updated in place. Returns stats.

        block_jacobi=True preconditions with the 3x3 entity diagonal blocks when W applies in the
        entity-block form (three-field problems), the diagonal otherwise.

        fixed=True runs exactly max_outer x max_inner iterations without host
        reads (capturable); its statistics go to stats_device (device f64[4]).
        """
        if not hasattr(self, "_dir"):
            self._dir = self.dirichlet_lids()  # kept alive: captured graphs read these
        lids, g = self._dir
        a = _abi.SolveArgs()
        a.rowptr, a.colind, a.vals = _ptr(W.rowptr), _ptr(W.colind), _ptr(W.values)
        a.b, a.x = _ptr(b), _ptr(x)
        a.n_dirichlet, a.dirichlet_lids, a.dirichlet_g = lids.numel(), _ptr(lids), _ptr(g)
        a.rtol, a.inner_rtol, a.max_outer, a.max_inner = rtol, inner_rtol, max_outer, max_inner
        a.flags = ((_abi.TX_SOLVE_MATRIX_FREE_RESIDUAL if matrix_free else 0) |
                   (_abi.TX_SOLVE_FIXED_ITERATIONS if fixed else 0) |
                   (_abi.TX_SOLVE_REUSE_OPERATOR if reuse_operator else 0) |
                   (_abi.TX_SOLVE_ENTITY_BLOCKS if getattr(W, "apply_form", "crs") == "entity" else 0) |
                   (_abi.TX_SOLVE_BLOCK_JACOBI if block_jacobi else 0))
        a.x_dot, a.alpha, a.beta, a.t = _ptr(x_dot), alpha, beta, t
        a.stats_device = _ptr(stats_device)
        a.x_pred, a.x_dot_coef = _ptr(x_pred), x_dot_coef
        ids = np.array([bc.id for bc in self.neumann], dtype=np.int32)
        a.n_neumann, a.neumann_ids = len(ids), _np_ptr(ids) if len(ids) else None
        lib = self.dof.lib
        lib.tx_set_stream(self.dof.h, C.c_void_p(torch.cuda.current_stream().cuda_stream))
        check(self.dof.h, lib.tx_solve_cg_ir(self.dof.h, C.byref(a)), "tx_solve_cg_ir")
        return {"outer": int(a.stats[0]), "inner": int(a.stats[1]), "relres": a.stats[2], "r0": a.stats[3]}


class BlockedModelEvaluator:
    """evalModel on blocked containers: x, x_dot and f as lists of block vectors, W a BlockedCrsMatrix.

    The gather from the product vector, the volume fill with its scatter, the
    Neumann fluxes and the Dirichlet rows run as in ModelEvaluator on the
    interleaved layout (the blocked numbering is a permutation of it), and
    the results are split into the blocks; excluded blocks are not written.
    """

    def __init__(self, me, blof):
        self.me, self.blof = me, blof
        lof = me.lof
        self._x, self._xd, self._f = lof.getTpetraVector(), lof.getTpetraVector(), lof.getTpetraVector()
        self._W = None

    def create_W_op(self):
        return self.blof.getBlockedMatrix()

    def evalModel(self, xb, x_dot=None, alpha=0.0, beta=1.0, t=0.0, f=None, W=None, mixed=False, **kw):
        blof = self.blof
        x = blof.mergeVector(xb, self._x)
        xd = blof.mergeVector(x_dot, self._xd) if x_dot is not None else None
        Wi = None
        if W is not None:
            if self._W is None:
                self._W = self.me.create_W_op()
            Wi = self._W
        self.me.evalModel(x, x_dot=xd, alpha=alpha, beta=beta, t=t, f=self._f if f is not None else None, W=Wi,
                          mixed=mixed, **kw)
        if f is not None:
            blof.splitVector(self._f, f)
        if W is not None:
            blof.splitMatrix(Wi, W)
        return f, W


_INTEGRANDS = {"Field": _abi.TX_INTEGRAND_FIELD, "L2 Error": _abi.TX_INTEGRAND_L2_ERROR,
               "H1 Error": _abi.TX_INTEGRAND_H1_ERROR, "Max": _abi.TX_INTEGRAND_MAX, "Min": _abi.TX_INTEGRAND_MIN,
               "Probe": _abi.TX_INTEGRAND_PROBE}


class Response:
    """A response (TianXin Response_Integral / panzer Functional, ExtremeValue, Probe).

    "Field" integrates a DOF field over the cells, or over sides with side_mask (box sides) or side_set
    (explicit meshes, name or index); "L2 Error" and "H1 Error" integrate the Poisson example's error
    integrands against the manufactured solution of TX_SOURCE_SINE; "Max" / "Min" are the ExtremeValue
    response of the field at the cubature points; "Probe" is the field's value at point.  evaluate()
    leaves the value in a device scalar and can add the gradient (the Jacobian evaluation type);
    value() returns it on the host."""

    def __init__(self, dof, integrand="Field", dof_name=None, block=-1, cubature_degree=0, side_mask=0,
                 side_set=None, point=None):
        self.dof = dof
        d = _abi.ResponseDesc()
        d.block = block
        d.field = dof.getFieldNum(dof_name) if dof_name is not None else 0
        d.integrand = _INTEGRANDS[integrand] if isinstance(integrand, str) else int(integrand)
        d.cubature_degree = cubature_degree
        d.side_mask = side_mask
        d.side_set = dof.conn.sideSetIndex(side_set) + 1 if side_set is not None else 0
        if point is not None:
            d.point[0], d.point[1], d.point[2] = (float(v) for v in point)
        rid = C.c_int32()
        check(dof.h, dof.lib.tx_response_create(dof.h, C.byref(d), C.byref(rid)), "tx_response_create")
        self.id = rid.value
        self.out = torch.zeros(1, dtype=torch.float64, device="cuda")

    def evaluate(self, x, dgdx=None):
        lib = self.dof.lib
        lib.tx_set_stream(self.dof.h, C.c_void_p(torch.cuda.current_stream().cuda_stream))
        check(self.dof.h, lib.tx_response_eval(self.dof.h, self.id, _ptr(x), _ptr(self.out), _ptr(dgdx)),
              "tx_response_eval")
        return self.out

    def value(self, x):
        return float(self.evaluate(x).item())


def ip_coordinates(dof, block, cubature_degree=0):
    """IPCoordinates response: the physical cubature points [E][nq][3] of a block (device tensor)."""
    nq = C.c_int32()
    check(dof.h, dof.lib.tx_ip_coordinates(dof.h, block, cubature_degree, C.byref(nq), None), "tx_ip_coordinates")
    ne = len(dof.conn.getElementBlock(block))
    out = torch.empty((ne, nq.value, 3), dtype=torch.float64, device="cuda")
    dof.lib.tx_set_stream(dof.h, C.c_void_p(torch.cuda.current_stream().cuda_stream))
    check(dof.h, dof.lib.tx_ip_coordinates(dof.h, block, cubature_degree, C.byref(nq), _ptr(out)), "tx_ip_coordinates")
    return out


class HostEvaluator:
    """evalModel for a caller whose Tpetra vectors and matrix live in host memory (pinned), pipelined: step k's
    f and CRS values are copied back on a copy stream while step k + 1 assembles into the other of two device
    buffer sets.  Every step still copies its x in and its f and W out; synchronize() waits for the last copy.
    The host link (about 0.2 TB/s on this machine) bounds the step, the assembly overlaps it."""

    def __init__(self, me, mixed=True):
        self.me, self.lof, self.mixed = me, me.lof, mixed
        self.sets = [(self.lof.getTpetraVector(), self.lof.getTpetraVector(), me.create_W_op()) for _ in range(2)]
        self.copy = torch.cuda.Stream()
        self.done = [torch.cuda.Event(), torch.cuda.Event()]   # copy-back of set i finished
        self.ready = [torch.cuda.Event(), torch.cuda.Event()]  # assembly of set i finished
        self.k = 0

    def step(self, x_host, f_host, W_host, **kw):
        i = self.k & 1
        x, f, W = self.sets[i]
        cur = torch.cuda.current_stream()
        cur.wait_event(self.done[i])          # the set's previous copy-back has left the device
        x.copy_(x_host, non_blocking=True)
        self.me.evalModel(x, f=f, W=W, mixed=self.mixed, **kw)
        self.ready[i].record(cur)
        with torch.cuda.stream(self.copy):
            self.copy.wait_event(self.ready[i])
            f_host.copy_(f, non_blocking=True)
            W_host.copy_(W.values, non_blocking=True)
            self.done[i].record(self.copy)
        self.k += 1

    def synchronize(self):
        torch.cuda.current_stream().wait_stream(self.copy)


class CapturedGraph:
    """fn()'s library work recorded into a CUDA graph owned by the handle (tx_graph_capture_begin/end) and
    replayed by launch().  fn may only make launch-only calls (evalModel, NeumannBC.evaluate, apply,
    solve(fixed=True) after one uncaptured solve) and in-place tensor ops; their pointers are frozen."""

    def __init__(self, dof, fn):
        self.dof, self.id = dof, None
        self.stream = torch.cuda.Stream()
        self.stream.wait_stream(torch.cuda.current_stream())
        lib, gid = dof.lib, C.c_int32(-1)
        with torch.cuda.stream(self.stream):
            lib.tx_set_stream(dof.h, C.c_void_p(self.stream.cuda_stream))
            check(dof.h, lib.tx_graph_capture_begin(dof.h), "tx_graph_capture_begin")
            try:
                fn()
            finally:
                rc = lib.tx_graph_capture_end(dof.h, C.byref(gid))
            check(dof.h, rc, "tx_graph_capture_end")
        self.id = gid.value

    def launch(self):
        lib = self.dof.lib
        self.stream.wait_stream(torch.cuda.current_stream())
        lib.tx_set_stream(self.dof.h, C.c_void_p(self.stream.cuda_stream))
        check(self.dof.h, lib.tx_graph_launch(self.dof.h, self.id), "tx_graph_launch")
        torch.cuda.current_stream().wait_stream(self.stream)

    def __del__(self):
        if self.id is not None:
            self.dof.lib.tx_graph_destroy(self.dof.h, self.id)
            self.id = None


class Batch:
    """Many independent meshes (DOFManagers) evaluated by one persistent launch."""

    def __init__(self, dofs, workset=(512, 512), seed=0, max_ctas=0):
        self.dofs = list(dofs)
        self.lib = self.dofs[0].lib
        hs = (C.c_void_p * len(self.dofs))(*[d.h for d in self.dofs])
        b = C.c_void_p()
        rc = self.lib.tx_batch_create(hs, len(self.dofs), C.byref(b))
        if rc:
            raise TxError(rc, "tx_batch_create")
        self.b = b
        self.setWorksets(*workset, seed=seed, max_ctas=max_ctas)

    def __del__(self):
        if getattr(self, "b", None):
            self.lib.tx_batch_destroy(self.b)
            self.b = None

    def setWorksets(self, min_size, max_size, seed=0, max_ctas=0):
        rc = self.lib.tx_batch_set_worksets(self.b, min_size, max_size, seed, max_ctas)
        if rc:
            raise TxError(rc, "tx_batch_set_worksets")

    def evaluate(self, xs, fs, Ws=None, x_dots=None, auxs=None, alpha=0.0, beta=1.0, t=0.0, mixed=False,
                 scatter_direct=False):
        """One persistent launch over every instance's worksets (staged Jacobian scatter unless scatter_direct)."""
        n = len(self.dofs)
        args = (_abi.EvalArgs * n)()
        for i in range(n):
            args[i] = eval_args(xs[i], None if x_dots is None else x_dots[i], None if auxs is None else auxs[i],
                                alpha, beta, t, fs[i], None if Ws is None else Ws[i], mixed,
                                scatter_direct=scatter_direct)
        self.lib.tx_set_stream(self.dofs[0].h, C.c_void_p(torch.cuda.current_stream().cuda_stream))
        rc = self.lib.tx_batch_eval(self.b, args)
        if rc:
            raise TxError(rc, "tx_batch_eval: " + (self.lib.tx_batch_last_error(self.b) or b"").decode())


def synchronize(dof):
    check(dof.h, dof.lib.tx_synchronize(dof.h), "tx_synchronize")
