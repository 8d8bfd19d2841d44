"""Blocked linear objects (BlockedDOFManager + BlockedTpetraLinearObjFactory)
on the GPU against the oracle.

Block (i, j) of the operator must be the submatrix of the oracle's
interleaved Jacobian on block i's rows and block j's columns, both numbered
b * entity + k (k = the field's place in its block), with the graph's
columns ascending; block vectors are the matching pieces of the product
vector.  Layouts: field-split elasticity [[UX], [UY], [UZ]], a grouping with
a gap [[UX, UZ], [UY]], and a single block.  Bars: graphs, splits and
merges bit-exact (they move values); the blocked evaluation 1e-12 relative
to the oracle (FP64); the blocked apply 1e-13 relative to the interleaved
product (summation order).
"""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

import tianxin_gb300 as tx
from oracle import oracle as O
from tianxin_gb300 import _abi as A

pytestmark = pytest.mark.gpu

ELAST = (1.0, 0.3, 0.1, -0.2, -1.0, 0.7)
LAYOUTS = {"split": [["UX"], ["UY"], ["UZ"]], "gap": [["UX", "UZ"], ["UY"]], "one": [["UX", "UY", "UZ"]]}


def _setup(n=(4, 3, 3), topo=A.TX_TOPO_HEX, jitter=0.1, seed=5):
    m = A.mesh_desc(n, (1, 1, 1), topo, jitter=jitter, seed=seed)
    q = A.equation_set(A.TX_PHYS_ELASTICITY, A.TX_HGRAD_C1, params=ELAST)
    conn = tx.CartesianConnManager(*n, topology=topo, jitter=jitter, seed=seed)
    dof = tx.DOFManager(conn, q)
    return O.Oracle(m, q), dof


def _rows(bd, i):
    """Interleaved LIDs of block i's rows in block-LID order."""
    dof = bd.dof
    ne, fields = bd.n_entities, bd.getFieldBlocks()[i]
    nums = [dof.getFieldNum(f) for f in fields]
    return (np.arange(ne)[:, None] * dof.n_fields + np.array(nums)[None, :]).reshape(-1)


def _block(Acsr, bd, i, j):
    B = Acsr[_rows(bd, i)][:, _rows(bd, j)].tocsr()
    B.sort_indices()
    return B


@pytest.mark.parametrize("layout", list(LAYOUTS))
def test_blocked_graphs_and_evaluation_match_the_oracle(cuda, layout):
    o, dof = _setup()
    bd = tx.BlockedDOFManager(dof, LAYOUTS[layout])
    blof = tx.BlockedTpetraLinearObjFactory(bd)
    lof = tx.TpetraLinearObjFactory(dof)
    me = tx.ModelEvaluator(lof, [tx.DirichletBC(dof, A.SIDE_ZMIN)])
    bme = tx.BlockedModelEvaluator(me, blof)
    rng = np.random.default_rng(4)
    x, xd = rng.uniform(-1, 1, o.n_dofs), rng.uniform(-1, 1, o.n_dofs)
    xt, xdt = torch.from_numpy(x).cuda(), torch.from_numpy(xd).cuda()
    xb, xdb = blof.splitVector(xt), blof.splitVector(xdt)
    assert torch.equal(blof.mergeVector(xb), xt)  # split/merge round trip
    fb, Wb = blof.getBlockedVector(), bme.create_W_op()
    bme.evalModel(xb, x_dot=xdb, alpha=0.5, beta=1.0, f=fb, W=Wb)
    # oracle: interleaved f and W with the same Dirichlet rows (f_d = x_d, row d = e_d)
    f_ref, v_ref = o.evaluate(x, xd, None, alpha=0.5, beta=1.0)
    rp, ci = o.graph()
    lids = tx.DirichletBC(dof, A.SIDE_ZMIN).lids_host
    f_ref[lids] = x[lids]
    Aref = sp.csr_matrix((v_ref, ci, rp), shape=(o.n_dofs, o.n_dofs)).tolil()
    for d in lids:
        Aref.rows[d] = list(Aref.rows[d]); Aref.data[d] = [1.0 if c == d else 0.0 for c in Aref.rows[d]]
    Aref = Aref.tocsr()
    nb = bd.getNumFieldBlocks()
    scale = np.abs(v_ref).max()
    for i in range(nb):
        r = _rows(bd, i)
        assert np.abs(fb[i].cpu().numpy() - f_ref[r]).max() <= 1e-12 * np.abs(f_ref).max()
        for j in range(nb):
            B = _block(Aref, bd, i, j)
            brp, bci = blof.getGraph(i, j)
            assert np.array_equal(brp.cpu().numpy(), B.indptr) and np.array_equal(bci.cpu().numpy(), B.indices)
            assert np.abs(Wb.getBlock(i, j).values.cpu().numpy() - B.data).max() <= 1e-12 * scale, (i, j)


def test_blocked_apply_and_excluded_pairs(cuda):
    o, dof = _setup(n=(5, 4, 3))
    bd = tx.BlockedDOFManager(dof, LAYOUTS["gap"])
    blof = tx.BlockedTpetraLinearObjFactory(bd)
    lof = tx.TpetraLinearObjFactory(dof)
    W = lof.getTpetraMatrix()
    rng = np.random.default_rng(6)
    W.values.copy_(torch.from_numpy(rng.uniform(-1, 1, dof.nnz)))
    Wb = blof.getBlockedMatrix()
    blof.splitMatrix(W, Wb)
    # the split is a permutation: bit-exact against scipy's submatrices
    Acsr = sp.csr_matrix((W.values.cpu().numpy(), W.colind.cpu().numpy(), W.rowptr.cpu().numpy()),
                         shape=(dof.n_dofs, dof.n_dofs))
    for i in range(2):
        for j in range(2):
            assert np.array_equal(Wb.getBlock(i, j).values.cpu().numpy(), _block(Acsr, bd, i, j).data)
    x = rng.uniform(-1, 1, dof.n_dofs)
    xb = blof.splitVector(torch.from_numpy(x).cuda())
    y0 = [torch.from_numpy(rng.uniform(-1, 1, bd.getBlockSize(i))).cuda() for i in range(2)]
    yb = [t.clone() for t in y0]
    Wb.apply(xb, yb, alpha=-1.5, beta=0.25)
    y_ref = Acsr @ x
    for i in range(2):
        r = _rows(bd, i)
        ref = -1.5 * y_ref[r] + 0.25 * y0[i].cpu().numpy()
        assert np.abs(yb[i].cpu().numpy() - ref).max() <= 1e-13 * np.abs(ref).max()
    # excluded pair (0, 1): y_0 = A_00 x_0 only; a row of excluded pairs scales y by beta
    blof2 = tx.BlockedTpetraLinearObjFactory(bd)
    blof2.addExcludedPairs([(0, 1), (1, 0), (1, 1)])
    We = blof2.getBlockedMatrix()
    assert We.getBlock(0, 1) is None and We.getBlock(1, 1) is None
    blof2.splitMatrix(W, We)
    yb = [t.clone() for t in y0]
    We.apply(xb, yb, alpha=1.0, beta=0.5)
    B00 = _block(Acsr, bd, 0, 0)
    ref0 = B00 @ x[_rows(bd, 0)] + 0.5 * y0[0].cpu().numpy()
    assert np.abs(yb[0].cpu().numpy() - ref0).max() <= 1e-13 * np.abs(ref0).max()
    assert torch.equal(yb[1], 0.5 * y0[1])


def test_blocked_layout_errors(cuda):
    _, dof = _setup(n=(2, 2, 2))
    with pytest.raises(ValueError):
        tx.BlockedDOFManager(dof, [["UX", "UY"], ["UY", "UZ"]])
    with pytest.raises(ValueError):
        tx.BlockedDOFManager(dof, [["UX"], ["UY"]])
    bd = tx.BlockedDOFManager(dof, LAYOUTS["split"])
    with pytest.raises(tx.TxError) as e:
        tx.BlockedTpetraLinearObjFactory(bd).getGraph(3, 0)
    assert e.value.code == A.TX_ERANGE
