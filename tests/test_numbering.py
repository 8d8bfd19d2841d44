"""Product host set-up vs the oracle, bit for bit (CPU only; no kernels run).

Numbering facts checked: owned_ GIDs in LID order, element GID and LID
vectors, per-field offsets (Panzer_DOFManager.cpp:449-716,1293-1372,
Panzer_FieldAggPattern.cpp:369-413), Dirichlet DOF sets
(TianXin_PointEvaluator_impl.hpp:104,196-202) and vertex coordinates.
The numbering itself is pinned by the reference's one-rank CubeHex fixture
(adapters-stk/test/stk_connmngr/tCubeHexMeshDOFManager.cpp:137-193).
"""
import json
import os

import numpy as np
import pytest

import tianxin_gb300 as tx
from oracle import oracle as O
from tianxin_gb300 import _abi as A

CASES = [
    ("poisson_hex8", (3, 2, 2), (1, 1, 1), A.TX_TOPO_HEX, A.TX_PHYS_POISSON, A.TX_HGRAD_C1),
    ("elasticity_hex8", (2, 2, 3), (1, 1, 1), A.TX_TOPO_HEX, A.TX_PHYS_ELASTICITY, A.TX_HGRAD_C1),
    ("poisson_tet4", (2, 3, 2), (1, 1, 1), A.TX_TOPO_TET, A.TX_PHYS_POISSON, A.TX_HGRAD_C1),
    ("elasticity_tet4", (2, 3, 2), (1, 1, 1), A.TX_TOPO_TET, A.TX_PHYS_ELASTICITY, A.TX_HGRAD_C1),
    ("poisson_hex27", (2, 2, 2), (1, 1, 1), A.TX_TOPO_HEX, A.TX_PHYS_POISSON, A.TX_HGRAD_C2),
    ("heat_tet10", (2, 2, 2), (1, 1, 1), A.TX_TOPO_TET, A.TX_PHYS_HEAT, A.TX_HGRAD_C2),
    ("heat_hex27_tet10", (2, 2, 2), (2, 1, 1), [A.TX_TOPO_HEX, A.TX_TOPO_TET], A.TX_PHYS_HEAT, A.TX_HGRAD_C2),
    ("multiblock_hex8", (2, 1, 2), (2, 2, 1), A.TX_TOPO_HEX, A.TX_PHYS_POISSON, A.TX_HGRAD_C1),
    ("maxwell_nedelec", (2, 2, 2), (1, 1, 1), A.TX_TOPO_HEX, A.TX_PHYS_MAXWELL, A.TX_HCURL_I1),
]


def build(n, blocks, topo, phys, basis, jitter=0.1, seed=3):
    m = A.mesh_desc(n, blocks, topo, jitter=jitter, seed=seed)
    q = A.equation_set(phys, basis)
    o = O.Oracle(m, q)
    conn = tx.CartesianConnManager(*n, *blocks, topology=topo, jitter=jitter, seed=seed)
    dof = tx.DOFManager(conn, q, require_device=False)
    return o, conn, dof


@pytest.mark.parametrize("name,n,blocks,topo,phys,basis", CASES, ids=[c[0] for c in CASES])
def test_numbering_bit_exact(name, n, blocks, topo, phys, basis):
    o, conn, dof = build(n, blocks, topo, phys, basis)
    assert dof.n_dofs == o.n_dofs
    assert dof.nnz == o.nnz
    assert np.array_equal(dof.getOwnedIndices(), o.owned_gids())
    for b in range(o.n_blocks):
        assert np.array_equal(conn.getElementBlock(b), o.block_elements(b))
        assert dof.getElementBlockGIDCount(b) == o.block_gid_count(b)
        assert np.array_equal(dof.getElementGIDs(b), o.element_gids(b))
        assert np.array_equal(dof.getElementLIDs(b), o.element_lids(b))
        for f in range(o.n_fields):
            assert np.array_equal(dof.getGIDFieldOffsets(b, f), o.field_offsets(b, f))
    assert np.array_equal(conn.coordinates(), o.coordinates())


@pytest.mark.parametrize("name,n,blocks,topo,phys,basis", CASES, ids=[c[0] for c in CASES])
def test_dirichlet_sets(name, n, blocks, topo, phys, basis):
    o, _, dof = build(n, blocks, topo, phys, basis)
    for sides in (A.ALL_SIDES, A.SIDE_ZMIN, A.SIDE_XMAX | A.SIDE_YMIN):
        for fmask in (0x7, 0x1):
            assert np.array_equal(dof.dirichletDofs(sides, fmask), o.dirichlet_dofs(sides, fmask))


def test_lid_differs_from_gid():
    # LID = first-touch order, not GID order (Appendix fact of the numbering)
    o, _, dof = build((2, 2, 2), (1, 1, 1), A.TX_TOPO_HEX, A.TX_PHYS_POISSON, A.TX_HGRAD_C1, jitter=0.0)
    g = dof.getOwnedIndices()
    assert not np.array_equal(g, np.arange(len(g)))
    assert np.array_equal(np.sort(g), np.arange(len(g)))


def test_elasticity_offsets_interleaved():
    _, _, dof = build((1, 1, 1), (1, 1, 1), A.TX_TOPO_HEX, A.TX_PHYS_ELASTICITY, A.TX_HGRAD_C1)
    assert list(dof.getGIDFieldOffsets(0, 0)) == list(range(0, 24, 3))
    assert list(dof.getGIDFieldOffsets(0, 1)) == list(range(1, 24, 3))
    assert list(dof.getGIDFieldOffsets(0, 2)) == list(range(2, 24, 3))


def test_hex27_offsets_follow_subcell_map():
    # one Q2 field: offsets[basis] = position of the basis' sub-cell in geometric order
    _, _, dof = build((1, 1, 1), (1, 1, 1), A.TX_TOPO_HEX, A.TX_PHYS_POISSON, A.TX_HGRAD_C2)
    off = dof.getGIDFieldOffsets(0, 0)
    order = list(range(8)) + [8, 9, 10, 11, 16, 17, 18, 19, 12, 13, 14, 15] + [25, 24, 26, 23, 21, 22] + [20]
    assert [int(off[b]) for b in order] == list(range(27))


def test_mixed_interface_is_conforming():
    # hex27 block and tet10 block share the 97x97-like lattice points of the interface
    o, _, dof = build((2, 2, 2), (2, 1, 1), [A.TX_TOPO_HEX, A.TX_TOPO_TET], A.TX_PHYS_HEAT, A.TX_HGRAD_C2)
    ga = set(dof.getElementGIDs(0).ravel())
    gb = set(dof.getElementGIDs(1).ravel())
    assert len(ga & gb) == 5 * 5  # (2*2+1)^2 Q2/P2 points on the interface face
    assert dof.n_dofs == 5 * 5 * 5 * 2 - 25


def test_invalid_descriptions_raise():
    with pytest.raises(tx.TxError):
        tx.CartesianConnManager(0, 1, 1)
    conn = tx.CartesianConnManager(1, 1, 1, topology=A.TX_TOPO_TET)
    with pytest.raises(tx.TxError):
        tx.DOFManager(conn, A.equation_set(A.TX_PHYS_MAXWELL, A.TX_HCURL_I1), require_device=False)


def _cube_hex_fixture():
    with open(os.path.join(os.path.dirname(__file__), "golden", "reference_known_answers.json")) as fh:
        return json.load(fh)["cube_hex_dof_numbering"]


def _cube_hex_explicit(n):
    """The CubeHex factory's mesh as an explicit mesh: nodes x-fastest, elements x-fastest, shards vertex order."""
    nx, ny, nz = n
    idx = lambda i, j, k: i + (nx + 1) * (j + (ny + 1) * k)
    coords = [(i / nx, j / ny, k / nz) for k in range(nz + 1) for j in range(ny + 1) for i in range(nx + 1)]
    conn = [[idx(i, j, k), idx(i + 1, j, k), idx(i + 1, j + 1, k), idx(i, j + 1, k),
             idx(i, j, k + 1), idx(i + 1, j, k + 1), idx(i + 1, j + 1, k + 1), idx(i, j + 1, k + 1)]
            for k in range(nz) for j in range(ny) for i in range(nx)]
    return tx.ExplicitConnManager.from_arrays(coords, [(A.TX_TOPO_HEX, conn, 1, "eblock-0_0_0")])


def test_cube_hex_numbering_fixture_of_the_reference():
    # tCubeHexMeshDOFManager's one-rank element GIDs (three nodal fields interleaved per node, GIDs ascending by
    # node GID) on the oracle, the lattice numbering and the explicit-mesh numbering of the same mesh
    g = _cube_hex_fixture()
    n = tuple(g["mesh"])
    q = A.equation_set(A.TX_PHYS_ELASTICITY)  # three HGRAD_C1 fields, like ux, uy, p
    assert len(A.field_names(A.TX_PHYS_ELASTICITY)) == g["n_fields"]
    o = O.Oracle(A.mesh_desc(n), q)
    lattice = tx.DOFManager(tx.CartesianConnManager(*n), q, require_device=False)
    explicit = tx.DOFManager(_cube_hex_explicit(n), q, require_device=False)
    for source in (o.element_gids(0), lattice.getElementGIDs(0), explicit.getElementGIDs(0)):
        for e, gids in g["element_gids"].items():
            assert list(source[int(e)]) == gids, e
    for e, nodes in g["element_nodes"].items():
        assert list(o.element_conn(int(e))) == nodes, e


def test_gather_form_query():
    # the owner-computes lattice form applies to one hex8 elasticity block on the whole lattice only
    import ctypes as C
    form = C.c_int32()
    cases = [((3, 2, 2), (1, 1, 1), A.TX_TOPO_HEX, A.TX_PHYS_ELASTICITY, A.TX_GATHER_LATTICE),
             ((3, 2, 2), (1, 1, 1), A.TX_TOPO_HEX, A.TX_PHYS_POISSON, A.TX_GATHER_TWO_PHASE),
             ((3, 2, 2), (1, 1, 1), A.TX_TOPO_TET, A.TX_PHYS_ELASTICITY, A.TX_GATHER_TWO_PHASE),
             ((2, 1, 2), (2, 1, 1), A.TX_TOPO_HEX, A.TX_PHYS_ELASTICITY, A.TX_GATHER_TWO_PHASE)]
    for n, blocks, topo, phys, expect in cases:
        conn = tx.CartesianConnManager(*n, *blocks, topology=topo)
        dof = tx.DOFManager(conn, A.equation_set(phys), require_device=False)
        assert dof.lib.tx_eval_gather_form(dof.h, C.byref(form)) == 0
        assert form.value == expect, (n, blocks, topo, phys)
