"""Neumann "Flux" boundary conditions on the GPU against the oracle.

The reference adds val(t) * integral of N_b over the side set to the
residual of one DOF field (TianXin::Flux, disc-fe/src/evaluators/
TianXin_Neumann_impl.hpp:146-166), after the volume fill and before the
Dirichlet rows (disc-fe/src/Panzer_AssemblyEngine_impl.hpp:93-115), and the
Jacobian is unchanged.  Bars: 1e-13 relative to the largest entry against
the oracle (FP64, summation order differs); the side totals at full size
equal value x area to 1e-12.
"""
import numpy as np
import pytest
import torch

import tianxin_gb300 as tx
from oracle import oracle as O
from tianxin_gb300 import _abi as A

pytestmark = pytest.mark.gpu

TOL = 1e-13

CASES = {
    "poisson_hex8": dict(n=(4, 3, 5), blocks=(1, 1, 1), topo=A.TX_TOPO_HEX, phys=A.TX_PHYS_POISSON,
                         basis=A.TX_HGRAD_C1, params=(1.0, 0.0, 0.0, 1.0), sides=A.SIDE_XMIN | A.SIDE_ZMAX,
                         field="U", block=0),
    "elasticity_traction_hex8": dict(n=(3, 4, 3), blocks=(1, 1, 1), topo=A.TX_TOPO_HEX, phys=A.TX_PHYS_ELASTICITY,
                                     basis=A.TX_HGRAD_C1, params=(1.0, 0.3, 0.0, 0.0, -1.0), sides=A.SIDE_ZMAX,
                                     field="UZ", block=0),
    "heat_hex27_block0": dict(n=(2, 3, 2), blocks=(2, 1, 1), topo=[A.TX_TOPO_HEX, A.TX_TOPO_TET],
                              phys=A.TX_PHYS_HEAT, basis=A.TX_HGRAD_C2, params=(1.0, 0.5, 1.0),
                              sides=A.SIDE_XMIN | A.SIDE_YMIN | A.SIDE_ZMAX, field="T", block=0),
    "heat_tet10_block1": dict(n=(2, 3, 2), blocks=(2, 1, 1), topo=[A.TX_TOPO_HEX, A.TX_TOPO_TET],
                              phys=A.TX_PHYS_HEAT, basis=A.TX_HGRAD_C2, params=(1.0, 0.5, 1.0),
                              sides=A.ALL_SIDES, field="T", block=1),
    "poisson_tet4_all": dict(n=(3, 3, 3), blocks=(1, 1, 1), topo=A.TX_TOPO_TET, phys=A.TX_PHYS_POISSON,
                             basis=A.TX_HGRAD_C1, params=(1.0, 0.0, 0.0, 1.0), sides=A.ALL_SIDES, field="U",
                             block=0),
}


def _setup(c, jitter=0.15, seed=9, lengths=(1.0, 1.0, 1.0)):
    m = A.mesh_desc(c["n"], c["blocks"], c["topo"], lengths=lengths, jitter=jitter, seed=seed)
    q = A.equation_set(c["phys"], c["basis"], params=c["params"])
    o = O.Oracle(m, q)
    conn = tx.CartesianConnManager(*c["n"], *c["blocks"], topology=c["topo"], lengths=lengths, jitter=jitter,
                                   seed=seed)
    dof = tx.DOFManager(conn, q)
    return o, dof, tx.TpetraLinearObjFactory(dof)


@pytest.mark.parametrize("name", list(CASES))
def test_neumann_flux_matches_oracle(cuda, name):
    c = CASES[name]
    o, dof, lof = _setup(c)
    bc = tx.NeumannBC(dof, c["sides"], c["field"], "Constant", value=-2.5, block=c["block"])
    f_ref, n_ref = o.neumann(c["block"], c["sides"], dof.getFieldNum(c["field"]), -2.5)
    assert bc.n_sides == n_ref > 0
    f = lof.getTpetraVector()
    bc.evaluate(f)
    got = f.cpu().numpy()
    assert np.abs(got - f_ref).max() <= TOL * np.abs(f_ref).max()
    # rows outside the side set stay exactly zero on hex blocks
    if (c["topo"] if isinstance(c["topo"], int) else c["topo"][c["block"]]) == A.TX_TOPO_HEX:
        assert np.all(got[f_ref == 0.0] == 0.0)


def test_neumann_time_table_and_linear_values(cuda):
    c = CASES["poisson_hex8"]
    o, dof, lof = _setup(c)
    tt, tv = [0.0, 1.0, 2.0], [0.0, 3.0, -1.0]
    bc = tx.NeumannBC(dof, A.SIDE_YMAX, "U", "TimeTable", times=tt, values=tv)
    lin = tx.NeumannBC(dof, A.SIDE_YMAX, "U", "Linear", value=4.0)
    unit, _ = o.neumann(0, A.SIDE_YMAX, 0, 1.0)
    for t in (0.5, 1.5, 2.0):
        for b, ty, kw in ((bc, "TimeTable", dict(times=tt, values=tv)), (lin, "Linear", dict(value=4.0))):
            f = lof.getTpetraVector()
            b.evaluate(f, t)
            v = O.workset_functor(ty, t=t, **kw)
            assert np.abs(f.cpu().numpy() - v * unit).max() <= TOL * max(abs(v), 1.0) * np.abs(unit).max()
    with pytest.raises(tx.TxError) as e:
        bc.evaluate(lof.getTpetraVector(), 2.5)
    assert e.value.code == A.TX_ERANGE


def test_eval_model_adds_flux_before_dirichlet_and_keeps_the_jacobian(cuda):
    c = CASES["elasticity_traction_hex8"]
    o, dof, lof = _setup(c)
    rng = np.random.default_rng(1)
    x = rng.uniform(-0.1, 0.1, o.n_dofs)
    bd = o.dirichlet_dofs(A.SIDE_ZMIN)
    x[bd] = 0.0
    f_ref, v_ref = o.evaluate(x)
    o.neumann(0, A.SIDE_ZMAX, 2, 0.7, f_ref)
    o.dirichlet_apply(bd, None, x, f_ref, v_ref)
    me = tx.ModelEvaluator(lof, [tx.DirichletBC(dof, A.SIDE_ZMIN)],
                           [tx.NeumannBC(dof, A.SIDE_ZMAX, "UZ", value=0.7)])
    xd = torch.from_numpy(x).cuda()
    f, W = lof.getTpetraVector(), me.create_W_op()
    me.evalModel(xd, f=f, W=W)
    assert np.abs(f.cpu().numpy() - f_ref).max() <= 1e-12 * np.abs(f_ref).max()
    assert np.abs(W.values.cpu().numpy() - v_ref).max() <= 1e-12 * np.abs(v_ref).max()


def test_solve_with_flux_matches_oracle(cuda):
    # Poisson: u = 0 on z = 0, flux 2 on z = 1 (a linear profile in z for k = 1);
    # the matrix-free refinement residual carries the flux as evalModel does.
    c = dict(CASES["poisson_hex8"], params=(1.0, 0.0, 0.0, 0.0))
    o, dof, lof = _setup(c, jitter=0.1)
    bd = o.dirichlet_dofs(A.SIDE_ZMIN)
    x0 = np.zeros(o.n_dofs)
    f, vals = o.evaluate(x0)
    o.neumann(0, A.SIDE_ZMAX, 0, 2.0, f)
    o.dirichlet_apply(bd, None, x0, f, vals)
    rp, ci = o.graph()
    dx, _, rr = O.cg(rp, ci, vals, -f, rtol=1e-13, maxit=100000)
    x_ref = x0 + dx
    me = tx.ModelEvaluator(lof, [tx.DirichletBC(dof, A.SIDE_ZMIN)], [tx.NeumannBC(dof, A.SIDE_ZMAX, "U", value=2.0)])
    x, fd, W = lof.getTpetraVector(), lof.getTpetraVector(), me.create_W_op()
    me.evalModel(x, f=fd, W=W)
    st = me.solve(W, x, rtol=1e-12, matrix_free=True)
    assert st["relres"] <= 1e-12
    err = np.abs(x.cpu().numpy() - x_ref).max() / np.abs(x_ref).max()
    assert err <= 1e-10
    # the flux drives u = -2 z (R = grad u . grad v + 2 * v on the top side)
    X = o.dof_coordinates()
    assert np.abs(x_ref + 2.0 * X[:, 2]).max() <= 1e-9


def test_neumann_totals_at_size(cuda):
    # 64^3 elasticity, traction on z = lz: the side total is value * lx * ly
    # (the side vertices stay on the lattice), independent of the interior jitter.
    n, L, val = 64, (2.0, 1.0, 1.5), -0.125
    conn = tx.CartesianConnManager(n, n, n, lengths=L, jitter=0.05, seed=2024)
    dof = tx.DOFManager(conn, A.equation_set(A.TX_PHYS_ELASTICITY, params=(1.0, 0.3, 0.0, 0.0, -1.0)))
    lof = tx.TpetraLinearObjFactory(dof)
    bc = tx.NeumannBC(dof, A.SIDE_ZMAX, "UZ", value=val)
    assert bc.n_sides == n * n
    f = lof.getTpetraVector()
    bc.evaluate(f)
    fz = f.view(-1, 3)
    assert abs(float(fz[:, 2].sum()) - val * L[0] * L[1]) <= 1e-12
    assert float(fz[:, :2].abs().max()) == 0.0
    # interior side nodes carry val * h^2
    h2 = (L[0] / n) * (L[1] / n)
    top = fz[:, 2][fz[:, 2] != 0].cpu().numpy()
    assert np.isclose(top.min(), val * h2, rtol=1e-13) or np.isclose(top.max(), val * h2, rtol=1e-13)


def test_neumann_argument_errors(cuda):
    conn = tx.CartesianConnManager(2, 2, 2)
    dof = tx.DOFManager(conn, A.equation_set(A.TX_PHYS_MAXWELL, A.TX_HCURL_I1, params=(1.0, 1.0)))
    with pytest.raises(tx.TxError) as e:
        tx.NeumannBC(dof, A.SIDE_XMIN, "E")
    assert e.value.code == A.TX_EINVAL
    conn = tx.CartesianConnManager(2, 2, 2)
    dof = tx.DOFManager(conn, A.equation_set(A.TX_PHYS_POISSON, params=(1.0, 0.0, 0.0, 1.0)))
    with pytest.raises(tx.TxError) as e:
        tx.NeumannBC(dof, A.SIDE_XMIN, "U", block=3)
    assert e.value.code == A.TX_ERANGE
    with pytest.raises(tx.TxError) as e:
        tx.NeumannBC(dof, 0, "U")
    assert e.value.code == A.TX_EINVAL
    with pytest.raises(tx.TxError) as e:
        tx.NeumannBC(dof, A.SIDE_XMIN, "U", "TimeTable", times=[0.0, 0.0], values=[1.0, 2.0])
    assert e.value.code == A.TX_EINVAL


def test_captured_eval_model_step_replays(cuda):
    # tx_graph_capture_begin/end around zeroing + volume fill + flux + Dirichlet;
    # replays after x changes in place equal direct evaluations.
    c = CASES["elasticity_traction_hex8"]
    o, dof, lof = _setup(c)
    me = tx.ModelEvaluator(lof, [tx.DirichletBC(dof, A.SIDE_ZMIN)], [tx.NeumannBC(dof, A.SIDE_ZMAX, "UZ", value=0.3)])
    x = lof.getTpetraVector()
    f, W = lof.getTpetraVector(), me.create_W_op()
    me.evalModel(x, f=f, W=W, mixed=True)  # first launches set kernel attributes outside the capture
    g = tx.CapturedGraph(dof, lambda: me.evalModel(x, f=f, W=W, mixed=True))
    f2, W2 = lof.getTpetraVector(), me.create_W_op()
    gen = torch.Generator(device="cuda").manual_seed(4)
    for _ in range(3):
        x.copy_(torch.rand(x.shape, dtype=torch.float64, device="cuda", generator=gen) * 0.01)
        g.launch()
        me.evalModel(x, f=f2, W=W2, mixed=True)
        torch.cuda.synchronize()
        assert float((f - f2).abs().max()) <= 1e-12 * float(f2.abs().max())
        assert float((W.values - W2.values).abs().max()) <= 1e-12 * float(W2.values.abs().max())
