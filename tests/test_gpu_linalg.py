"""GPU SpMV and the FP64-refined FP32 Jacobi-CG against the oracle.

Bars: SpMV FP64 within 1e-13 relative (reassociated sums), FP32 SpMV within
1e-6; converged solutions within 1e-10 relative of the oracle's FP64 CG
solution (both solved to a 1e-13 relative residual).
"""
import numpy as np
import pytest
import torch

import tianxin_gb300 as tx
from oracle import oracle as O
from tianxin_gb300 import _abi as A

pytestmark = pytest.mark.gpu


def poisson_c1(n=8, jitter=0.1, seed=1):
    m = A.mesh_desc(n, jitter=jitter, seed=seed)
    q = A.equation_set(A.TX_PHYS_POISSON, params=(1.0, 0.0, 0.0, 0.0), source_kind=A.TX_SOURCE_SINE)
    o = O.Oracle(m, q)
    dof = tx.DOFManager(tx.CartesianConnManager(n, n, n, jitter=jitter, seed=seed), q)
    lof = tx.TpetraLinearObjFactory(dof)
    return o, dof, lof


def elasticity(n=6, jitter=0.05, seed=2):
    m = A.mesh_desc(n, jitter=jitter, seed=seed)
    q = A.equation_set(A.TX_PHYS_ELASTICITY, params=(1.0, 0.3, 0.0, 0.0, -1.0, 0.0))
    o = O.Oracle(m, q)
    dof = tx.DOFManager(tx.CartesianConnManager(n, n, n, jitter=jitter, seed=seed), q)
    lof = tx.TpetraLinearObjFactory(dof)
    return o, dof, lof


def test_spmv_f64_f32(cuda):
    o, dof, lof = elasticity(5)
    rng = np.random.default_rng(0)
    x = rng.uniform(-1, 1, o.n_dofs)
    _, vals = o.evaluate(x)
    rp, ci = o.graph()
    y_ref = O.spmv(rp, ci, vals, x)
    W = lof.getTpetraMatrix()
    W.values.copy_(torch.from_numpy(vals))
    y = W.apply(torch.from_numpy(x).cuda()).cpu().numpy()
    assert np.abs(y - y_ref).max() <= 1e-13 * np.abs(y_ref).max()
    # y = 2 A x - 0.5 y0
    y0 = rng.uniform(-1, 1, o.n_dofs)
    yy = torch.from_numpy(y0.copy()).cuda()
    W.apply(torch.from_numpy(x).cuda(), yy, alpha=2.0, beta=-0.5)
    assert np.abs(yy.cpu().numpy() - (2 * y_ref - 0.5 * y0)).max() <= 1e-12 * np.abs(y_ref).max()
    v32 = W.values.float()
    y32 = W.apply(torch.from_numpy(x).float().cuda(), values=v32).cpu().numpy()
    assert np.abs(y32 - y_ref).max() <= 1e-5 * np.abs(y_ref).max()


def _oracle_solution(o, bd, g=0.0):
    """Newton step from x0 (Dirichlet values set): A dx = -f(x0), A with unit Dirichlet rows."""
    x0 = np.zeros(o.n_dofs)
    x0[bd] = g
    f, vals = o.evaluate(x0)
    o.dirichlet_apply(bd, np.full(len(bd), g), x0, f, vals)
    rp, ci = o.graph()
    dx, it, rr = O.cg(rp, ci, vals, -f, rtol=1e-13, maxit=200000)
    return x0 + dx, rr


def test_poisson_solve_matches_oracle(cuda):
    o, dof, lof = poisson_c1(8)
    bd = o.dirichlet_dofs(A.ALL_SIDES)
    x_ref, rr = _oracle_solution(o, bd)
    assert rr <= 1e-12
    me = tx.ModelEvaluator(lof, [tx.DirichletBC(dof, A.ALL_SIDES)])
    x = lof.getTpetraVector()
    f = lof.getTpetraVector()
    W = me.create_W_op()
    me.evalModel(x, f=f, W=W)
    b = -f
    st = me.solve(W, x, b=b, rtol=1e-13)
    err = np.abs(x.cpu().numpy() - x_ref).max() / np.abs(x_ref).max()
    assert st["relres"] <= 1e-13
    assert err <= 1e-10, (err, st)


def test_elasticity_mixed_assembly_matrix_free_refinement(cuda):
    # mixed (FP32-contraction) Jacobian + FP64 matrix-free residual: solution at FP64 accuracy
    o, dof, lof = elasticity(6)
    bd = o.dirichlet_dofs(A.SIDE_ZMIN)
    x_ref, rr = _oracle_solution(o, bd)
    me = tx.ModelEvaluator(lof, [tx.DirichletBC(dof, A.SIDE_ZMIN)])
    x = lof.getTpetraVector()
    f = lof.getTpetraVector()
    W = me.create_W_op()
    me.evalModel(x, f=f, W=W, mixed=True)
    st = me.solve(W, x, rtol=1e-12, matrix_free=True)
    err = np.abs(x.cpu().numpy() - x_ref).max() / np.abs(x_ref).max()
    assert st["relres"] <= 1e-12
    assert err <= 1e-10, (err, st)


def test_solver_rejects_missing_rhs(cuda):
    o, dof, lof = poisson_c1(3)
    me = tx.ModelEvaluator(lof)
    W = me.create_W_op()
    with pytest.raises(tx.TxError) as e:
        me.solve(W, lof.getTpetraVector(), b=None)
    assert e.value.code == A.TX_EINVAL


@pytest.mark.parametrize("n", [6, 14])
def test_block_jacobi_same_solution_fewer_iterations(cuda, n):
    # entity-block form, 3x3 block-Jacobi inner preconditioner (Dirichlet rows and columns eliminated in
    # the blocks): the FP64-refined solution equals the oracle's as with point Jacobi, in no more inner
    # iterations; a capturable fixed-iteration solve after it reuses the block inverses
    o, dof, lof = elasticity(n)
    bd = o.dirichlet_dofs(A.SIDE_ZMIN)
    x_ref, rr = _oracle_solution(o, bd)
    me = tx.ModelEvaluator(lof, [tx.DirichletBC(dof, A.SIDE_ZMIN)])
    f, W = lof.getTpetraVector(), me.create_W_op()
    me.evalModel(lof.getTpetraVector(), f=f, W=W, mixed=True)
    W.setApplyForm("entity")
    inner = {}
    for blk in (False, True):
        x = lof.getTpetraVector()
        st = me.solve(W, x, rtol=1e-12, matrix_free=True, block_jacobi=blk)
        err = np.abs(x.cpu().numpy() - x_ref).max() / np.abs(x_ref).max()
        assert st["relres"] <= 1e-12 and err <= 1e-10, (blk, err, st)
        inner[blk] = st["inner"]
    assert inner[True] <= inner[False], inner
    x = lof.getTpetraVector()
    stats = torch.zeros(4, dtype=torch.float64, device="cuda")
    me.solve(W, x, matrix_free=True, fixed=True, reuse_operator=True, max_outer=4, max_inner=inner[True],
             stats_device=stats, block_jacobi=True)
    err = np.abs(x.cpu().numpy() - x_ref).max() / np.abs(x_ref).max()
    assert err <= 1e-9, err
