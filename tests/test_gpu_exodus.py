"""Evaluation on explicit meshes (Exodus files and arrays) on the GPU.

The explicit path must reproduce the lattice path on the same mesh: a
lattice mesh written to an Exodus file (lattice node order, box sides as side
sets and node sets) and read back gives the same numbering, so the
deterministic (coloured) evaluation gives the same bits in f and W (linear
fields on hex8 / tet4, quadratic fields on hex27 / tet10), with
Dirichlet rows from node sets and Neumann fluxes from side sets in place of
box sides (f to 1e-15: the flux sums with atomics).  With the nodes renumbered
(node_num_map), the first-touch LIDs and so f and W in LID order are
unchanged.  The lattice path is pinned to the oracle elsewhere.
"""
import numpy as np
import pytest
import torch

import tianxin_gb300 as tx
from tianxin_gb300 import _abi as A
from tianxin_gb300.exodus import write_exodus

import exodus_cases as X

pytestmark = pytest.mark.gpu
ELAST = (1.0, 0.3, 0.1, -0.2, -1.0, 0.7)


def _evaluate(conn, q, explicit, x_np, nblocks):
    dof = tx.DOFManager(conn, q)
    lof = tx.TpetraLinearObjFactory(dof)
    if explicit:
        dbc = [tx.DirichletBC(dof, node_set="zmin")]
        nbc = [tx.NeumannBC(dof, dof_name=dof.field_names[-1], value=-0.3, block=b, side_set="zmax")
               for b in range(nblocks)]
    else:
        dbc = [tx.DirichletBC(dof, A.SIDE_ZMIN)]
        nbc = [tx.NeumannBC(dof, A.SIDE_ZMAX, dof.field_names[-1], value=-0.3, block=b) for b in range(nblocks)]
    me = tx.ModelEvaluator(lof, dbc, nbc)
    x, f, W = torch.from_numpy(x_np).cuda(), lof.getTpetraVector(), me.create_W_op()
    me.evalModel(x, x_dot=0.5 * x, alpha=0.5, beta=1.0, f=f, W=W, deterministic=True)
    return dof, f.cpu().numpy(), W.values.cpu().numpy(), (me, lof)


@pytest.mark.parametrize("topo,phys", [(A.TX_TOPO_HEX, A.TX_PHYS_ELASTICITY), (A.TX_TOPO_TET, A.TX_PHYS_POISSON)])
def test_exodus_mesh_reproduces_the_lattice_path(cuda, tmp_path, topo, phys):
    conn, (coords, blocks, ss, ns) = X.box(n=(3, 2, 2), blocks=(1, 2, 1), topo=topo)
    path = write_exodus(tmp_path / "box.exo", coords, blocks, ss, ns)
    mesh = tx.ExodusReaderFactory(path).buildMesh()
    q = A.equation_set(phys, params=ELAST if phys == A.TX_PHYS_ELASTICITY else (1.0, 0.5, 1.0, 2.0))
    nf = 3 if phys == A.TX_PHYS_ELASTICITY else 1
    x_np = np.random.default_rng(2).uniform(-1, 1, nf * len(coords))
    d0, f0, v0, _ = _evaluate(conn, q, False, x_np, len(blocks))
    d1, f1, v1, _ = _evaluate(mesh, q, True, x_np, len(blocks))
    assert np.array_equal(v0, v1)
    assert np.abs(f0 - f1).max() <= 1e-15 * np.abs(f0).max()


@pytest.mark.parametrize("topo,phys", [(A.TX_TOPO_HEX, A.TX_PHYS_HEAT), (A.TX_TOPO_TET, A.TX_PHYS_POISSON)])
def test_quadratic_exodus_mesh_reproduces_the_lattice_path(cuda, tmp_path, topo, phys):
    """TX_HGRAD_C2 fields on HEX27 / TETRA10 blocks read from an Exodus file: the
    same bits as the lattice's quadratic path (node sets with the mid-side nodes
    for Dirichlet, side sets for Neumann)."""
    n, nb = (2, 2, 1), (1, 1, 2)
    conn = tx.CartesianConnManager(*n, *nb, topology=topo, jitter=0.1, seed=5)
    q = A.equation_set(phys, A.TX_HGRAD_C2, params=(1.0, 0.5, 1.0) if phys == A.TX_PHYS_HEAT else (1.0, 0.5, 1.0, 2.0))
    coords, blocks, ss, ns = X.quadratic_lattice_as_explicit(conn, tuple(a * b for a, b in zip(n, nb)), q)
    mesh = tx.ExodusReaderFactory(write_exodus(tmp_path / "quad.exo", coords, blocks, ss, ns)).buildMesh()
    x_np = np.random.default_rng(3).uniform(-1, 1, len(coords))
    d0, f0, v0, _ = _evaluate(conn, q, False, x_np, len(blocks))
    d1, f1, v1, _ = _evaluate(mesh, q, True, x_np, len(blocks))
    assert np.array_equal(d0.getOwnedIndices(), d1.getOwnedIndices())
    assert np.array_equal(v0, v1)
    assert np.abs(f0 - f1).max() <= 1e-15 * np.abs(f0).max()
    # responses over the quadratic field: block integrals, a side-set integral, the extreme value
    x = torch.from_numpy(x_np).cuda()
    for b in range(len(blocks)):
        r0 = tx.Response(d0, "Field", block=b).value(x)
        r1 = tx.Response(d1, "Field", block=b).value(x)
        assert abs(r0 - r1) <= 1e-14 * max(1.0, abs(r0))
        s0 = tx.Response(d0, "Field", block=b, side_mask=A.SIDE_ZMAX).value(x)
        s1 = tx.Response(d1, "Field", block=b, side_set="zmax").value(x)
        assert abs(s0 - s1) <= 1e-14 * max(1.0, abs(s0))
    assert tx.Response(d0, "Max").value(x) == tx.Response(d1, "Max").value(x)


def test_renumbered_nodes_keep_lid_order_results(cuda, tmp_path):
    conn, (coords, blocks, ss, ns) = X.box(n=(3, 3, 2))
    q = A.equation_set(A.TX_PHYS_ELASTICITY, params=ELAST)
    gid = np.random.default_rng(7).permutation(len(coords)) + 1
    m0 = tx.ExodusReaderFactory(write_exodus(tmp_path / "a.exo", coords, blocks, ss, ns)).buildMesh()
    m1 = tx.ExodusReaderFactory(write_exodus(tmp_path / "b.exo", coords, blocks, ss, ns, node_num_map=gid)).buildMesh()
    x_np = np.random.default_rng(8).uniform(-1, 1, 3 * len(coords))
    d0, f0, v0, _ = _evaluate(m0, q, True, x_np, 1)
    d1, f1, v1, _ = _evaluate(m1, q, True, x_np, 1)
    assert np.array_equal(v0, v1)
    assert np.abs(f0 - f1).max() <= 1e-15 * np.abs(f0).max()
    rank = np.argsort(np.argsort(gid))
    # owned GIDs follow the renumbered nodes: node n's DOFs are 3 rank[n] + field
    g0, g1 = d0.getOwnedIndices(), d1.getOwnedIndices()
    assert np.array_equal(g1, 3 * rank[g0 // 3] + g0 % 3)


def test_solve_on_an_exodus_mesh(cuda, tmp_path):
    conn, (coords, blocks, ss, ns) = X.box(n=(6, 5, 4), jitter=0.05)
    mesh = tx.ExodusReaderFactory(write_exodus(tmp_path / "c.exo", coords, blocks, ss, ns)).buildMesh()
    q = A.equation_set(A.TX_PHYS_ELASTICITY, params=(1.0, 0.3, 0.0, 0.0, -1.0))
    sols = []
    for c, explicit in ((conn, False), (mesh, True)):
        dof = tx.DOFManager(c, q)
        lof = tx.TpetraLinearObjFactory(dof)
        bc = tx.DirichletBC(dof, node_set="zmin") if explicit else tx.DirichletBC(dof, A.SIDE_ZMIN)
        me = tx.ModelEvaluator(lof, [bc])
        x, f, W = lof.getTpetraVector(), lof.getTpetraVector(), me.create_W_op()
        me.evalModel(x, f=f, W=W, mixed=True)
        st = me.solve(W, x, rtol=1e-11, matrix_free=True)
        assert st["relres"] <= 1e-11
        sols.append(x.cpu().numpy())
    assert np.abs(sols[0] - sols[1]).max() <= 1e-10 * np.abs(sols[0]).max()


def test_side_set_and_probe_responses_on_an_exodus_mesh(cuda, tmp_path):
    conn, (coords, blocks, ss, ns) = X.box(n=(3, 2, 2), blocks=(1, 2, 1))
    mesh = tx.ExodusReaderFactory(write_exodus(tmp_path / "r.exo", coords, blocks, ss, ns)).buildMesh()
    q = A.equation_set(A.TX_PHYS_POISSON, params=(1.0, 0.0, 0.0, 1.0))
    d_lat, d_exp = tx.DOFManager(conn, q), tx.DOFManager(mesh, q)
    x = torch.from_numpy(np.random.default_rng(4).uniform(-1, 1, d_lat.n_dofs)).cuda()
    for b in range(len(blocks)):
        v0 = tx.Response(d_lat, "Field", block=b, side_mask=A.SIDE_ZMAX).value(x)
        v1 = tx.Response(d_exp, "Field", block=b, side_set="zmax").value(x)
        assert abs(v0 - v1) <= 1e-14 * max(1.0, abs(v0))
    p = (0.4, 0.7, 0.3)
    assert tx.Response(d_lat, "Probe", point=p).value(x) == tx.Response(d_exp, "Probe", point=p).value(x)


def test_empty_block_and_empty_sets_change_nothing(cuda):
    """An element block with no elements, an empty side set and an empty node set (ragged inputs the
    reference's meshes can hold): every evaluation form, Neumann, Dirichlet and the responses give what
    the mesh without them gives."""
    conn, (coords, blocks, ss, ns) = X.box(n=(3, 2, 2))
    empty = (A.TX_TOPO_TET, np.zeros((0, 4), np.int64), 9, "empty")
    m0 = tx.ExplicitConnManager.from_arrays(coords, blocks, ss, ns)
    m1 = tx.ExplicitConnManager.from_arrays(coords, [empty] + list(blocks), ss + [("none", 7, [])],
                                            ns + [("nonodes", 8, [])])
    q = A.equation_set(A.TX_PHYS_ELASTICITY, params=ELAST)
    x_np = np.random.default_rng(9).uniform(-1, 1, 3 * len(coords))
    outs = []
    for m, nb in ((m0, 1), (m1, 2)):
        dof = tx.DOFManager(m, q)
        lof = tx.TpetraLinearObjFactory(dof)
        dbc = [tx.DirichletBC(dof, node_set="zmin")] + ([tx.DirichletBC(dof, node_set="nonodes")] if nb == 2 else [])
        nbc = [tx.NeumannBC(dof, dof_name="UZ", value=-0.3, block=b, side_set=s)
               for b in range(nb) for s in (("zmax", "none") if nb == 2 else ("zmax",))]
        me = tx.ModelEvaluator(lof, dbc, nbc)
        x = torch.from_numpy(x_np).cuda()
        res = []
        for kw in (dict(deterministic=True), dict(mixed=True), dict(persistent=True)):
            f, W = lof.getTpetraVector(), me.create_W_op()
            me.evalModel(x, x_dot=0.5 * x, alpha=0.5, beta=1.0, f=f, W=W, **kw)
            res.append((f.cpu().numpy(), W.values.cpu().numpy()))
        me.ae.gather = True
        f, W = lof.getTpetraVector(), me.create_W_op()
        me.evalModel(x, f=f, W=W)
        res.append((f.cpu().numpy(), W.values.cpu().numpy()))
        last = nb - 1  # the non-empty block
        resp = [tx.Response(dof, "Field", block=last).value(x),
                tx.Response(dof, "Max", dof_name="UX").value(x),
                tx.Response(dof, "Field", block=last, side_set="zmax").value(x)]
        if nb == 2:
            assert tx.Response(dof, "Field", block=0).value(x) == 0.0
            assert tuple(tx.ip_coordinates(dof, 0).shape)[0] == 0
        outs.append((dof.getOwnedIndices(), res, resp))
    (g0, r0, p0), (g1, r1, p1) = outs
    assert np.array_equal(g0, g1)
    assert np.array_equal(r0[0][1], r1[0][1])  # deterministic: same bits
    for (f0, v0), (f1, v1) in zip(r0, r1):
        assert np.abs(f0 - f1).max() <= 1e-14 * np.abs(f0).max()
        assert np.abs(v0 - v1).max() <= 1e-14 * np.abs(v0).max()
    assert p0[1] == p1[1] and abs(p0[0] - p1[0]) <= 1e-14 * abs(p0[0]) and abs(p0[2] - p1[2]) <= 1e-14 * abs(p0[2])
