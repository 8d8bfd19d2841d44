"""Owner-computes lattice assembly (single-block hex8 elasticity on the brick
lattice, mixed precision, TX_EVAL_GATHER): every CRS value and residual entry
written once by the CTA that owns the node.

Checked against the oracle's FP64 residual and Jacobian (forward-mode AD) at
the mixed tolerance, against the atomic mixed kernel, for bitwise
repeatability and for overwriting (no zeroing needed), on lattices whose
sizes cut the 4 x 4 node tiles and the z chunks unevenly, with and without
the time-derivative (mass) terms.
"""
import numpy as np
import pytest
import torch

import tianxin_gb300 as tx
from oracle import oracle as O
from tianxin_gb300 import _abi as A

pytestmark = pytest.mark.gpu

TOL_MIXED = 2e-5  # FP32 element arithmetic and FP32 sums of the eight element contributions


def rel(a, ref):
    return float(np.abs(a - ref).max() / np.abs(ref).max())


def setup(n, params, jitter=0.1, seed=5):
    m = A.mesh_desc(n, jitter=jitter, seed=seed)
    q = A.equation_set(A.TX_PHYS_ELASTICITY, params=params)
    conn = tx.CartesianConnManager(*n, jitter=jitter, seed=seed)
    dof = tx.DOFManager(conn, q)
    lof = tx.TpetraLinearObjFactory(dof)
    return O.Oracle(m, q), dof, lof


CASES = [
    ((1, 1, 1), (1.0, 0.3, 0.0, 0.0, -1.0, 0.0)),
    ((6, 5, 7), (1.0, 0.3, 0.0, 0.0, -1.0, 0.0)),
    ((9, 4, 3), (2.0, 0.25, 0.5, -0.25, 1.0, 0.0)),
    ((13, 6, 5), (1.0, 0.3, 0.1, 0.2, 0.3, 1.5)),  # density: mass terms through x_dot and alpha
]


@pytest.mark.parametrize("n,params", CASES, ids=["1x1x1", "6x5x7", "9x4x3", "13x6x5_mass"])
def test_lattice_gather_against_oracle(cuda, n, params):
    o, dof, lof = setup(n, params)
    rng = np.random.default_rng(1)
    x_h = rng.uniform(-1, 1, o.n_dofs)
    xd_h = rng.uniform(-1, 1, o.n_dofs)
    alpha, beta = 0.75, 1.25
    f_ref, v_ref = o.evaluate(x_h, xd_h, alpha=alpha, beta=beta)
    x, xd = torch.from_numpy(x_h).cuda(), torch.from_numpy(xd_h).cuda()
    ae = tx.AssemblyEngine(lof)
    f, W = lof.getTpetraVector(), lof.getTpetraMatrix()
    f.fill_(7.0)  # overwritten, not summed into
    W.initializeMatrix(-3.0)
    ae.evaluate(x, xd, alpha=alpha, beta=beta, f=f, W=W, mixed=True, gather=True)
    fg, wg = f.cpu().numpy(), W.values.cpu().numpy()
    assert rel(fg, f_ref) <= TOL_MIXED and rel(wg, v_ref) <= TOL_MIXED, (rel(fg, f_ref), rel(wg, v_ref))
    # the atomic mixed kernel: same FP32 element arithmetic, FP64 sums
    fa, Wa = lof.getTpetraVector(), lof.getTpetraMatrix()
    ae.evaluate(x, xd, alpha=alpha, beta=beta, f=fa, W=Wa, mixed=True, gather=False)
    assert rel(fg, fa.cpu().numpy()) <= 2e-6 and rel(wg, Wa.values.cpu().numpy()) <= 2e-6
    # the same bits on every call
    f2, W2 = lof.getTpetraVector(), lof.getTpetraMatrix()
    ae.evaluate(x, xd, alpha=alpha, beta=beta, f=f2, W=W2, mixed=True, gather=True)
    assert torch.equal(f2, f) and torch.equal(W2.values, W.values)


def test_lattice_gather_multi_layer_chunks_against_oracle(cuda):
    # 26 x 22 x 30: 7 x 6 node tiles, several node layers per z chunk
    o, dof, lof = setup((26, 22, 30), (1.0, 0.3, 0.0, 0.0, -1.0, 0.0), jitter=0.05, seed=9)
    x_h = np.random.default_rng(2).uniform(-1e-3, 1e-3, o.n_dofs)
    f_ref, v_ref = o.evaluate(x_h, threads=8)
    f, W = lof.getTpetraVector(), lof.getTpetraMatrix()
    tx.AssemblyEngine(lof).evaluate(torch.from_numpy(x_h).cuda(), f=f, W=W, mixed=True, gather=True)
    assert rel(f.cpu().numpy(), f_ref) <= TOL_MIXED
    assert rel(W.values.cpu().numpy(), v_ref) <= TOL_MIXED


def test_lattice_gather_with_dirichlet_model_evaluator(cuda):
    # ModelEvaluator's deterministic evaluation takes the two-phase form, i.e. the lattice kernel here
    n = (7, 6, 5)
    o, dof, lof = setup(n, (1.0, 0.3, 0.0, 0.0, -1.0, 0.0))
    me = tx.ModelEvaluator(lof, [tx.DirichletBC(dof, A.SIDE_ZMIN)])
    x_h = np.random.default_rng(3).uniform(-1, 1, o.n_dofs)
    bd = o.dirichlet_dofs(A.SIDE_ZMIN)
    f_ref, v_ref = o.evaluate(x_h)
    o.dirichlet_apply(bd, np.zeros(len(bd)), x_h, f_ref, v_ref)
    f, W = lof.getTpetraVector(), me.create_W_op()
    me.evalModel(torch.from_numpy(x_h).cuda(), f=f, W=W, mixed=True, deterministic=True)
    assert rel(f.cpu().numpy(), f_ref) <= TOL_MIXED
    assert rel(W.values.cpu().numpy(), v_ref) <= TOL_MIXED


def test_lattice_gather_regular_lattice_zero_entries(cuda):
    # no jitter: some couplings of the regular lattice cancel to exact zeros, which the copy-out widens exactly
    o, dof, lof = setup((5, 4, 6), (1.0, 0.25, 0.0, 0.0, -1.0, 0.0), jitter=0.0)
    x_h = np.random.default_rng(6).uniform(-1, 1, o.n_dofs)
    f_ref, v_ref = o.evaluate(x_h)
    x = torch.from_numpy(x_h).cuda()
    ae = tx.AssemblyEngine(lof)
    f, W = lof.getTpetraVector(), lof.getTpetraMatrix()
    ae.evaluate(x, f=f, W=W, mixed=True, gather=True)
    wg = W.values.cpu().numpy()
    assert rel(f.cpu().numpy(), f_ref) <= TOL_MIXED and rel(wg, v_ref) <= TOL_MIXED
    assert np.isfinite(wg).all()
    tiny = np.abs(v_ref) <= 1e-14 * np.abs(v_ref).max()
    assert np.abs(wg[tiny]).max() <= 1e-6 * np.abs(v_ref).max()


@pytest.mark.parametrize("n,params,alpha", [
    ((1, 7, 3), (1.0, 0.3, 0.0, 0.0, -1.0, 0.0), 0.75),      # one element wide: most node tiles half empty
    ((2, 2, 64), (1.0, 0.3, 0.0, 0.0, -1.0, 0.0), 0.75),     # tall: many z chunks of one node column
    ((7, 5, 4), (1.0, 0.3, 0.1, 0.2, 0.3, 2.0), 0.0),        # density with alpha = 0: mass terms in R only
], ids=["1x7x3", "2x2x64", "7x5x4_alpha0"])
def test_lattice_gather_edge_shapes_against_oracle(cuda, n, params, alpha):
    o, dof, lof = setup(n, params, seed=8)
    rng = np.random.default_rng(11)
    x_h = rng.uniform(-1, 1, o.n_dofs)
    xd_h = rng.uniform(-1, 1, o.n_dofs)
    f_ref, v_ref = o.evaluate(x_h, xd_h, alpha=alpha, beta=1.0)
    f, W = lof.getTpetraVector(), lof.getTpetraMatrix()
    f.fill_(-5.0)
    W.initializeMatrix(9.0)
    ae = tx.AssemblyEngine(lof)
    assert ae.gather_form() == "lattice"
    ae.evaluate(torch.from_numpy(x_h).cuda(), torch.from_numpy(xd_h).cuda(), alpha=alpha, beta=1.0, f=f, W=W,
                mixed=True, gather=True)
    assert rel(f.cpu().numpy(), f_ref) <= TOL_MIXED and rel(W.values.cpu().numpy(), v_ref) <= TOL_MIXED
