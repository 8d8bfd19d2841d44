"""Integral responses on the GPU against the oracle, and the reference's
convergence-rate check (adapters-stk/example/PoissonExample/convergence_rate.py:
L2 and H1 errors of refined solves fall like h^2 and h for linear elements).

Bars: values 1e-12 relative to the oracle (FP64, summation order differs),
the same bits on repeated calls, gradients 1e-12 relative to their largest
entry; rates within 0.15 of 2 and 1.
"""
import numpy as np
import pytest
import torch

import tianxin_gb300 as tx
from oracle import oracle as O
from tianxin_gb300 import _abi as A

pytestmark = pytest.mark.gpu

CASES = {
    "poisson_hex8": dict(n=(4, 3, 5), blocks=(1, 1, 1), topo=A.TX_TOPO_HEX, phys=A.TX_PHYS_POISSON,
                         basis=A.TX_HGRAD_C1, params=(1.0, 0.0, 0.0, 1.0), field="U"),
    "heat_hex27_tet10": dict(n=(2, 3, 2), blocks=(2, 1, 1), topo=[A.TX_TOPO_HEX, A.TX_TOPO_TET],
                             phys=A.TX_PHYS_HEAT, basis=A.TX_HGRAD_C2, params=(1.0, 0.5, 1.0), field="T"),
    "poisson_tet4": dict(n=(3, 3, 3), blocks=(1, 1, 1), topo=A.TX_TOPO_TET, phys=A.TX_PHYS_POISSON,
                         basis=A.TX_HGRAD_C1, params=(1.0, 0.0, 0.0, 1.0), field="U"),
    "elasticity_uy_hex8": dict(n=(3, 4, 3), blocks=(1, 1, 1), topo=A.TX_TOPO_HEX, phys=A.TX_PHYS_ELASTICITY,
                               basis=A.TX_HGRAD_C1, params=(1.0, 0.3, 0.0, 0.0, -1.0), field="UY"),
}


def _setup(c, jitter=0.15, seed=7):
    m = A.mesh_desc(c["n"], c["blocks"], c["topo"], jitter=jitter, seed=seed)
    q = A.equation_set(c["phys"], c["basis"], params=c["params"])
    conn = tx.CartesianConnManager(*c["n"], *c["blocks"], topology=c["topo"], jitter=jitter, seed=seed)
    dof = tx.DOFManager(conn, q)
    return O.Oracle(m, q), dof


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("integrand", ["Field", "L2 Error", "H1 Error"])
def test_response_matches_oracle(cuda, name, integrand):
    c = CASES[name]
    o, dof = _setup(c)
    field = dof.getFieldNum(c["field"])
    deg = 2 if "tet" in name else 4
    x = np.random.default_rng(5).uniform(-1, 1, o.n_dofs)
    v_ref, g_ref = o.response(integrand, field=field, degree=deg, x=x, gradient=True)
    r = tx.Response(dof, integrand, c["field"], cubature_degree=deg)
    xd = torch.from_numpy(x).cuda()
    g = torch.zeros(o.n_dofs, dtype=torch.float64, device="cuda")
    v = float(r.evaluate(xd, g).item())
    assert abs(v - v_ref) <= 1e-12 * max(abs(v_ref), 1e-300)
    assert np.abs(g.cpu().numpy() - g_ref).max() <= 1e-12 * np.abs(g_ref).max()
    bits = {r.evaluate(xd).clone().view(torch.int64).item() for _ in range(3)}
    assert len(bits) == 1  # fixed summation order


def test_response_per_block(cuda):
    c = CASES["heat_hex27_tet10"]
    o, dof = _setup(c)
    x = np.random.default_rng(6).uniform(0, 1, o.n_dofs)
    xd = torch.from_numpy(x).cuda()
    parts = []
    for block in (0, 1):
        v_ref = o.response("Field", block=block, degree=2, x=x)
        v = tx.Response(dof, "Field", "T", block=block, cubature_degree=2).value(xd)
        assert abs(v - v_ref) <= 1e-12 * abs(v_ref)
        parts.append(v)
    whole = tx.Response(dof, "Field", "T", cubature_degree=2).value(xd)
    assert abs(whole - sum(parts)) <= 1e-13 * abs(whole)


def _solve_error(n):
    conn = tx.CartesianConnManager(n, n, n, jitter=0.1, seed=3)
    dof = tx.DOFManager(conn, A.equation_set(A.TX_PHYS_POISSON, params=(1.0, 0.0, 0.0, 0.0),
                                             source_kind=A.TX_SOURCE_SINE))
    lof = tx.TpetraLinearObjFactory(dof)
    me = tx.ModelEvaluator(lof, [tx.DirichletBC(dof, A.ALL_SIDES)])
    x, f, W = lof.getTpetraVector(), lof.getTpetraVector(), me.create_W_op()
    me.evalModel(x, f=f, W=W)
    st = me.solve(W, x, rtol=1e-12, matrix_free=True)
    assert st["relres"] <= 1e-12
    l2 = tx.Response(dof, "L2 Error", cubature_degree=6).value(x) ** 0.5
    h1 = tx.Response(dof, "H1 Error", cubature_degree=6).value(x) ** 0.5
    return l2, h1


def test_convergence_rates_of_refined_solves(cuda):
    errs = [_solve_error(n) for n in (8, 16, 32)]
    for (l2a, h1a), (l2b, h1b) in zip(errs, errs[1:]):
        assert abs(np.log2(l2a / l2b) - 2.0) <= 0.15
        assert abs(np.log2(h1a / h1b) - 1.0) <= 0.15


def test_response_errors(cuda):
    conn = tx.CartesianConnManager(2, 2, 2)
    dof = tx.DOFManager(conn, A.equation_set(A.TX_PHYS_MAXWELL, A.TX_HCURL_I1, params=(1.0, 1.0)))
    with pytest.raises(tx.TxError) as e:
        tx.Response(dof, "Field")
    assert e.value.code == A.TX_EINVAL
    conn = tx.CartesianConnManager(2, 2, 2, topology=A.TX_TOPO_TET)
    dof = tx.DOFManager(conn, A.equation_set(A.TX_PHYS_POISSON, params=(1.0, 0.0, 0.0, 1.0)))
    with pytest.raises(tx.TxError):
        tx.Response(dof, "Field", cubature_degree=4)  # tet rules: degree 2


# ExtremeValue, side-set integrals, probes and integration-point coordinates against the oracle.
# u(q) sums the same basis terms in the same order on both sides; the bars allow the GPU's fused
# multiply-adds: 1e-14 relative for values, exact winner locations (random data has no ties).
@pytest.mark.parametrize("name", ["poisson_hex8", "heat_hex27_tet10", "elasticity_uy_hex8"])
@pytest.mark.parametrize("kind", ["Max", "Min"])
def test_extreme_value_matches_oracle(cuda, name, kind):
    c = CASES[name]
    o, dof = _setup(c)
    field = dof.getFieldNum(c["field"])
    x = np.random.default_rng(11).uniform(-1, 1, o.n_dofs)
    v_ref, g_ref = o.extreme(kind == "Max", field=field, degree=2, x=x, gradient=True)
    r = tx.Response(dof, kind, c["field"], cubature_degree=2)
    g = torch.zeros(o.n_dofs, dtype=torch.float64, device="cuda")
    v = float(r.evaluate(torch.from_numpy(x).cuda(), g).item())
    assert abs(v - v_ref) <= 1e-14 * abs(v_ref)
    gn = g.cpu().numpy()
    assert np.array_equal(np.flatnonzero(gn), np.flatnonzero(g_ref))  # the same winning cell and point
    assert np.abs(gn - g_ref).max() <= 1e-14


@pytest.mark.parametrize("name", ["poisson_hex8", "heat_hex27_tet10", "poisson_tet4", "elasticity_uy_hex8"])
def test_side_integral_matches_oracle(cuda, name):
    c = CASES[name]
    o, dof = _setup(c)
    field = dof.getFieldNum(c["field"])
    x = np.random.default_rng(12).uniform(-1, 1, o.n_dofs)
    for block in ((0, 1) if name == "heat_hex27_tet10" else (-1,)):
        mask = A.SIDE_XMIN | A.SIDE_YMAX | A.SIDE_ZMAX
        v_ref, g_ref = o.side_response(mask, field=field, block=block, x=x, gradient=True)
        r = tx.Response(dof, "Field", c["field"], block=block, side_mask=mask)
        g = torch.zeros(o.n_dofs, dtype=torch.float64, device="cuda")
        v = float(r.evaluate(torch.from_numpy(x).cuda(), g).item())
        assert abs(v - v_ref) <= 1e-13 * np.abs(g_ref).sum()
        assert np.abs(g.cpu().numpy() - g_ref).max() <= 1e-14 * np.abs(g_ref).max()


@pytest.mark.parametrize("name", ["poisson_hex8", "heat_hex27_tet10", "poisson_tet4"])
def test_probe_matches_oracle(cuda, name):
    c = CASES[name]
    o, dof = _setup(c)
    field = dof.getFieldNum(c["field"])
    x = np.random.default_rng(13).uniform(-1, 1, o.n_dofs)
    rng = np.random.default_rng(14)
    for _ in range(4):
        p = rng.uniform(0.05, 0.95, 3)  # the lattice spans the unit cube
        v_ref, e, g_ref = o.probe(p, field=field, x=x, gradient=True)
        assert e >= 0
        r = tx.Response(dof, "Probe", c["field"], point=p)
        g = torch.zeros(o.n_dofs, dtype=torch.float64, device="cuda")
        v = float(r.evaluate(torch.from_numpy(x).cuda(), g).item())
        assert abs(v - v_ref) <= 1e-12 * max(1.0, abs(v_ref))
        assert np.abs(g.cpu().numpy() - g_ref).max() <= 1e-12
    with pytest.raises(tx.TxError) as err:
        tx.Response(dof, "Probe", c["field"], point=(5.0, 0.5, 0.5))
    assert err.value.code == A.TX_ERANGE


def test_ip_coordinates_match_oracle(cuda):
    c = CASES["heat_hex27_tet10"]
    o, dof = _setup(c)
    xyz = o.coordinates()
    for b, topo in ((0, A.TX_TOPO_HEX), (1, A.TX_TOPO_TET)):
        pts = tx.ip_coordinates(dof, b, cubature_degree=2).cpu().numpy()
        conn = dof.conn.getElementVertices(b)
        assert pts.shape[0] == len(conn)
        for e in (0, len(conn) // 2, len(conn) - 1):
            ip = np.zeros((pts.shape[1], 3))
            n = O.lib().orc_cell_values(topo, 2, O._p(np.ascontiguousarray(xyz[conn[e]])), None, O._p(ip))
            assert n == pts.shape[1]
            assert np.abs(pts[e] - ip).max() <= 1e-14


def test_response_kind_errors(cuda):
    o, dof = _setup(CASES["poisson_hex8"])
    with pytest.raises(tx.TxError):
        tx.Response(dof, "L2 Error", side_mask=A.SIDE_ZMAX)  # side responses integrate the field
    with pytest.raises(tx.TxError):
        tx.Response(dof, "Max", side_mask=A.SIDE_ZMAX)
