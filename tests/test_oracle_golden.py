"""The oracle against the reference's own known answers (CPU only).

Each test restates one of the reference's unit tests on the oracle:
  Q1 mass matrix       adapters-stk/test/model_evaluator/model_evaluator_mass_check.cpp:195-211
  two-hex integrals    disc-fe/test/evaluator_tests/integrator_scalar.cpp:393-410,500-501
  first IP coordinate  disc-fe/test/core_tests/integration_values2.cpp:103-110
  hex27 sub-cell map   dof-mgr/test/dofmngr_test/tIntrepidFieldPattern.cpp:527-573
  HCurl quadrilateral  disc-fe/test/core_tests/basis_values2.cpp:289-426 (and the hex I1 functions' face traces)
  scatter pattern      adapters-stk/test/evaluator_tests/tpetra_scatter_residual.cpp:281-305
  reproduction         dof-mgr/test/fe_assembly/test_fe_assembly_HEX.hpp:672-677 (||b-Ax|| <= 1e-10)
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from tianxin_gb300 import _abi as A

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def dense(o, vals):
    rp, ci = o.graph()
    M = np.zeros((o.n_dofs, o.n_dofs))
    for r in range(o.n_dofs):
        M[r, ci[rp[r]:rp[r + 1]]] = vals[rp[r]:rp[r + 1]]
    return M


def unit_hex_mass():
    # transient Poisson term only (k = 0, c = 0, udot multiplier 1): W = alpha*M with alpha=1, beta=0
    o = O.Oracle(A.mesh_desc(1), A.equation_set(A.TX_PHYS_POISSON, params=(0.0, 0.0, 1.0, 0.0)))
    _, v = o.evaluate(np.zeros(o.n_dofs), np.zeros(o.n_dofs), alpha=1.0, beta=0.0)
    M = dense(o, v)
    # node positions by LID to classify neighbours
    X = o.dof_coordinates()
    return M, X


def test_mass_matrix_known_answer_3d():
    M, X = unit_hex_mass()
    for i in range(8):
        for j in range(8):
            d = int(round(np.abs(X[i] - X[j]).sum()))  # lattice distance 0..3
            expect = {0: 1 / 27, 1: 1 / 54, 2: 1 / 108, 3: 1 / 216}[d]
            assert abs(M[i, j] - expect) <= 1e-15 * 1 / 27


def test_mass_matrix_known_answer_reference_2d_values():
    # Summing the unit-cube hex mass over its two z-layers gives the unit-square
    # Q1 mass of the reference test: 1/9 diagonal, 1/18 edge, 1/36 opposite.
    M, X = unit_hex_mass()
    bottom = [i for i in range(8) if X[i, 2] == 0.0]
    top_of = {i: [j for j in range(8) if X[j, 2] == 1.0 and np.allclose(X[j, :2], X[i, :2])][0] for i in bottom}
    g = json.load(open(os.path.join(GOLDEN, "reference_known_answers.json")))["q1_mass_2d"]
    for i in bottom:
        for j in bottom:
            m2 = M[i, j] + M[i, top_of[j]] + M[top_of[i], j] + M[top_of[i], top_of[j]]
            d = int(round(np.abs(X[i] - X[j]).sum()))
            expect = {0: g["diag"], 1: g["edge"], 2: g["opposite"]}[d]
            assert m2 == pytest.approx(expect, rel=1e-15, abs=0)


def test_two_hex_integrals():
    g = json.load(open(os.path.join(GOLDEN, "reference_known_answers.json")))["two_hex"]
    for X, expect in zip(g["coords"], g["integral_2x_length"]):
        wdet, _ = O.cell_values(A.TX_TOPO_HEX, g["quad_order"], np.array(X, float))
        assert 2.0 * wdet.sum() == pytest.approx(expect, rel=1e-15)


def test_first_integration_point():
    X = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float)
    _, ip = O.cell_values(A.TX_TOPO_HEX, 2, X)
    assert len(ip) == 8
    expect = (1.0 / np.sqrt(3.0) + 1.0) / 2.0
    assert np.allclose(ip[0], expect, rtol=1e-8, atol=0)


def test_hex27_subcell_map():
    g = json.load(open(os.path.join(GOLDEN, "reference_known_answers.json")))["hex27_subcells"]
    for dim, name in ((0, "nodes"), (1, "edges"), (2, "faces"), (3, "cell")):
        got = [O.basis_subcell(A.TX_TOPO_HEX, A.TX_HGRAD_C2, dim, c) for c in range(len(g[name]))]
        assert got == g[name]


def test_partition_of_unity_and_gradients():
    rng = np.random.default_rng(0)
    for topo, basis in ((A.TX_TOPO_HEX, A.TX_HGRAD_C1), (A.TX_TOPO_HEX, A.TX_HGRAD_C2), (A.TX_TOPO_TET, A.TX_HGRAD_C1),
                        (A.TX_TOPO_TET, A.TX_HGRAD_C2)):
        for _ in range(5):
            xi = rng.uniform(-1, 1, 3) if topo == A.TX_TOPO_HEX else rng.dirichlet([1, 1, 1, 1])[1:]
            v, g = O.basis_eval(topo, basis, xi)
            assert v.sum() == pytest.approx(1.0, abs=1e-14)
            assert np.allclose(g.sum(axis=0), 0.0, atol=1e-13)


HEX_V = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1], [-1, -1, 1], [1, -1, 1], [1, 1, 1],
                  [-1, 1, 1]], float)
HEX_EDGES = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6), (3, 7)]
QUAD_V = np.array([[-1, -1], [1, -1], [1, 1], [-1, 1]], float)


def quad_i1(x, y):
    """Lowest-order Nedelec on [-1,1]^2, shards edges 0..3 (v0->v1, v1->v2, v2->v3, v3->v0): values (4, 2) and
    scalar curls (4,), dual to u(edge midpoint) . (half edge vector)."""
    val = np.array([[0.5 * (1 - y), 0.0], [0.0, 0.5 * (1 + x)], [-0.5 * (1 + y), 0.0], [0.0, -0.5 * (1 - x)]])
    curl = np.full(4, 0.5)
    return val, curl


def test_hcurl_quad_fixture_of_the_reference():
    # basis_values2.cpp's HCurl quadrilateral test, restated: reference values and curl of function 0, and the
    # covariant transforms on its 0.5 x 0.5 cells (value J^-T v, curl c / det J, weights w det J)
    g = json.load(open(os.path.join(GOLDEN, "reference_known_answers.json")))["hcurl_quad_i1"]
    s, w1 = np.polynomial.legendre.leggauss(3)  # degree 4 rule: 3 x 3 Gauss points
    h = g["cell_size"]
    J = np.eye(2) * h / 2
    det = np.linalg.det(J)
    assert det == g["rel_cell_vol"]
    for i, xq in enumerate(s):
        for j, yq in enumerate(s):
            val, curl = quad_i1(xq, yq)
            assert val[0, 0] == -0.5 * (yq - 1.0) and val[0, 1] == 0.0
            assert curl[0] == g["function0_curl"]
            phys = val @ np.linalg.inv(J)  # rows: J^-T v
            pcurl = curl / det
            weight = w1[i] * w1[j]
            assert np.allclose(val, g["value_scale"] * phys, rtol=0, atol=1e-15)
            assert np.allclose(curl, g["rel_cell_vol"] * pcurl, rtol=0, atol=1e-15)
            assert np.allclose(weight * det * phys, g["rel_cell_vol"] * weight * phys, rtol=0, atol=1e-15)
    # the restated functions are dual to the midpoint tangential values
    for k in range(4):
        a, b = QUAD_V[k], QUAD_V[(k + 1) % 4]
        val, _ = quad_i1(*((a + b) / 2))
        assert np.allclose(val @ ((b - a) / 2), np.eye(4)[k], atol=1e-15)


def test_nedelec_hex_dual_to_midpoint_tangential_values():
    # the oracle's hex functions: u_i(m_j) . t_j = delta_ij (t_j half the edge vector), and the line integral
    # of every function along its own edge is 2 (the edge length), along the others 0
    s, w = np.polynomial.legendre.leggauss(3)
    for k, (a, b) in enumerate(HEX_EDGES):
        t = (HEX_V[b] - HEX_V[a]) / 2
        val, _ = O.basis_eval(A.TX_TOPO_HEX, A.TX_HCURL_I1, (HEX_V[a] + HEX_V[b]) / 2)
        assert np.allclose(val @ t, np.eye(12)[k], atol=1e-15)
        line = np.zeros(12)
        for sj, wj in zip(s, w):
            v, _ = O.basis_eval(A.TX_TOPO_HEX, A.TX_HCURL_I1, HEX_V[a] + (sj + 1) / 2 * (HEX_V[b] - HEX_V[a]))
            line += wj * v @ t
        assert np.allclose(line, 2.0 * np.eye(12)[k], atol=1e-14)


def test_nedelec_hex_face_traces_are_the_pinned_quad_functions():
    # on each face, the tangential trace of the hex edge functions is the quadrilateral I1 function of the face's
    # edge (orientation included) and the trace of every other function vanishes: the hex normalisation follows
    # from the reference's quadrilateral fixture
    faces = [(0, 1, 5, 4), (1, 2, 6, 5), (2, 3, 7, 6), (0, 4, 7, 3), (0, 3, 2, 1), (4, 5, 6, 7)]  # shards
    rng = np.random.default_rng(0)
    for fv in faces:
        P = HEX_V[list(fv)]
        eu, ev = (P[1] - P[0]) / 2, (P[3] - P[0]) / 2  # local axes: face vertex 0 at (-1, -1)
        centre = P.mean(axis=0)
        quad_edge_of = {}
        for q in range(4):
            a, b = fv[q], fv[(q + 1) % 4]
            k = [i for i, e in enumerate(HEX_EDGES) if set(e) == {a, b}][0]
            quad_edge_of[k] = (q, 1.0 if HEX_EDGES[k] == (a, b) else -1.0)
        for _ in range(4):
            uv = rng.uniform(-1, 1, 2)
            val, _ = O.basis_eval(A.TX_TOPO_HEX, A.TX_HCURL_I1, centre + uv[0] * eu + uv[1] * ev)
            qv, _ = quad_i1(*uv)
            for k in range(12):
                trace = np.array([val[k] @ eu, val[k] @ ev])
                expect = quad_edge_of[k][1] * qv[quad_edge_of[k][0]] if k in quad_edge_of else np.zeros(2)
                assert np.allclose(trace, expect, atol=1e-15), (fv, k)


@pytest.mark.parametrize("h", [1.0, 0.25])
def test_nedelec_hex_physical_transforms(h):
    # one hex of side h: the oracle's Maxwell Jacobian is (1/mu) int curl N . curl N + sigma int N . N with
    # N = J^-T N_ref and curl N = J curl N_ref / det J (the transforms the quadrilateral fixture pins), J = h/2 I,
    # and the edge signs of the lattice's vertex GIDs
    inv_mu, sigma = 1.5, 0.75
    o = O.Oracle(A.mesh_desc(1, lengths=(h, h, h)), A.equation_set(A.TX_PHYS_MAXWELL, A.TX_HCURL_I1,
                                                                     params=(inv_mu, sigma)))
    z = np.zeros(o.n_dofs)
    _, v = o.evaluate(z, aux=z)
    W = dense(o, v)
    lids = o.element_lids(0)[0]
    K = W[np.ix_(lids, lids)]
    gid = lambda p: int((p[0] > 0) + 2 * (p[1] > 0) + 4 * (p[2] > 0))
    sign = np.array([1.0 if gid(HEX_V[a]) < gid(HEX_V[b]) else -1.0 for a, b in HEX_EDGES])
    s, w = np.polynomial.legendre.leggauss(2)
    A_ref, B_ref = np.zeros((12, 12)), np.zeros((12, 12))
    for i, xq in enumerate(s):
        for j, yq in enumerate(s):
            for k, zq in enumerate(s):
                val, curl = O.basis_eval(A.TX_TOPO_HEX, A.TX_HCURL_I1, np.array([xq, yq, zq]))
                wq = w[i] * w[j] * w[k]
                A_ref += wq * curl @ curl.T
                B_ref += wq * val @ val.T
    det = (h / 2) ** 3
    expect = np.outer(sign, sign) * (inv_mu * (h / 2) ** 2 / det ** 2 * det * A_ref + sigma * (2 / h) ** 2 * det * B_ref)
    assert np.allclose(K, expect, rtol=0, atol=1e-14 * np.abs(expect).max())


def test_scatter_pattern_counts():
    # constant source on an undistorted mesh: every hex8 basis integrates to h^3/8,
    # so f = -s h^3/8 * (number of elements sharing the node): v, 2v, 4v or 8v
    n = 3
    o = O.Oracle(A.mesh_desc(n), A.equation_set(A.TX_PHYS_POISSON, params=(0.0, 0.0, 0.0, 1.0)))
    f, _ = o.evaluate(np.zeros(o.n_dofs), jacobian=False)
    v = -(1.0 / n) ** 3 / 8
    ratio = f / v
    assert set(np.round(ratio).astype(int)) == {1, 2, 4, 8}
    assert np.allclose(ratio, np.round(ratio), rtol=0, atol=1e-12)


@pytest.mark.parametrize("topo,basis", [(A.TX_TOPO_HEX, A.TX_HGRAD_C1), (A.TX_TOPO_HEX, A.TX_HGRAD_C2),
                                        (A.TX_TOPO_TET, A.TX_HGRAD_C1), (A.TX_TOPO_TET, A.TX_HGRAD_C2)])
def test_reproduction_of_in_space_solution(topo, basis):
    # -lap u + u = f with u = 1 + x + 2y + 3z (in every space here), Dirichlet u on the boundary:
    # the nodal interpolant solves the discrete system, so f(u_h) = b - A u_h = 0 (test_fe_assembly_HEX)
    m = A.mesh_desc((2, 3, 2), topology=topo, jitter=0.15, seed=7)
    q = A.equation_set(A.TX_PHYS_POISSON, basis, params=(1.0, 1.0, 0.0, 0.0), source_kind=A.TX_SOURCE_AFFINE,
                       integration_order=4 if topo == A.TX_TOPO_HEX else 2)
    if topo == A.TX_TOPO_TET and basis == A.TX_HGRAD_C1:
        pass
    o = O.Oracle(m, q)
    X = o.dof_coordinates()
    u = 1 + X[:, 0] + 2 * X[:, 1] + 3 * X[:, 2]
    f, vals = o.evaluate(u)
    bd = o.dirichlet_dofs(A.ALL_SIDES)
    o.dirichlet_apply(bd, u[bd], u, f, vals)
    assert np.linalg.norm(f) <= 1e-10 * np.linalg.norm(u)


# ------------------------------------------------------------------ Neumann
def test_neumann_flux_known_answer_reference_2d_values():
    # The reference's flux test: value 5 on the left side of [0,2]x[0,1] (2x1
    # quads, integration order 1) gives cell 0 the residual (2.5, 0, 0, 2.5).
    # Extruded one brick in z, each 2-D node is a pair of hex nodes; their sum
    # is the 2-D value.
    g = json.load(open(os.path.join(GOLDEN, "reference_known_answers.json")))["neumann_flux_left"]
    o = O.Oracle(A.mesh_desc((2, 1, 1), lengths=(2.0, 1.0, 1.0)),
                 A.equation_set(A.TX_PHYS_POISSON, params=(1.0, 0.0, 0.0, 0.0), integration_order=g["integration_order"]))
    f, n = o.neumann(0, A.SIDE_XMIN, 0, g["value"])
    assert n == 1
    X = o.dof_coordinates()
    quad = [(0.0, 0.0), (1.0, 0.0), (1.0, 1.0), (0.0, 1.0)]  # cell 0's nodes in quad order
    for k, (x, y) in enumerate(quad):
        pair = [i for i in range(o.n_dofs) if X[i, 0] == x and X[i, 1] == y]
        assert len(pair) == 2
        assert abs(f[pair].sum() - g["cell0_residual"][k]) <= g["tol"] * g["value"]
    assert abs(f.sum() - g["value"] * 1.0) <= 1e-14  # the flux times the side's area


@pytest.mark.parametrize("topo,basis,order", [(A.TX_TOPO_HEX, A.TX_HGRAD_C1, 2), (A.TX_TOPO_HEX, A.TX_HGRAD_C2, 4),
                                              (A.TX_TOPO_TET, A.TX_HGRAD_C1, 2), (A.TX_TOPO_TET, A.TX_HGRAD_C2, 2)])
def test_neumann_flux_closed_forms(topo, basis, order):
    # Boundary vertices keep their lattice positions under the interior jitter,
    # so every box side is tiled by exact rectangles (hex) or right triangles
    # (tet), where the side rules integrate the traces exactly:
    # sum of the flux = value * area, and the per-node shares of a rectangle
    # (Q1: A/4; Q2 tensor weights (1,4,1)/6 squared) and of a triangle
    # (P1: A/3; P2: 0 at vertices, A/3 at edge midpoints).
    n, L, val = 3, (1.5, 1.0, 2.0), -0.75
    o = O.Oracle(A.mesh_desc(n, topology=topo, lengths=L, jitter=0.2, seed=4),
                 A.equation_set(A.TX_PHYS_POISSON, basis, params=(1.0, 0.0, 0.0, 0.0), integration_order=order))
    f, cnt = o.neumann(0, A.SIDE_YMAX, 0, val)
    area = L[0] * L[2]
    assert cnt == (n * n if topo == A.TX_TOPO_HEX else 2 * n * n)
    assert abs(f.sum() - val * area) <= 1e-13 * abs(val * area)
    X = o.dof_coordinates()
    on = np.abs(X[:, 1] - L[1]) < 1e-12
    # off the side: exact zeros on hex sides (the side map keeps the fixed
    # coordinate at exactly +-1); rounding of 1 - x - y - z on tet sides
    assert np.abs(f[~on]).max() <= (0.0 if topo == A.TX_TOPO_HEX else 1e-16 * abs(val))
    h = (L[0] / n, L[2] / n)
    if topo == A.TX_TOPO_HEX and basis == A.TX_HGRAD_C1:
        # an interior node of the side touches 4 rectangles
        i = np.where(on & (np.abs(X[:, 0] - h[0]) < 1e-12) & (np.abs(X[:, 2] - h[1]) < 1e-12))[0]
        assert abs(f[i[0]] - val * h[0] * h[1]) <= 1e-14
    if topo == A.TX_TOPO_TET and basis == A.TX_HGRAD_C2:
        verts = on & np.isclose(np.mod(X[:, 0], h[0]), 0) & np.isclose(np.mod(X[:, 2], h[1]), 0)
        verts |= on & np.isclose(np.mod(X[:, 0], h[0]), h[0]) & np.isclose(np.mod(X[:, 2], h[1]), h[1])
        assert np.abs(f[verts]).max() <= 1e-15


def test_workset_functor_values():
    # Constant; Linear with the elapse time read from "Value" (the reference's
    # LinearWorksetFunctor); TimeTable interpolation and its error past the end.
    assert O.workset_functor("Constant", 3.5, t=9.0) == 3.5
    assert O.workset_functor("Linear", 4.0, t=1.0) == 1.0   # 4 * 1 / 4
    assert O.workset_functor("Linear", 4.0, t=6.0) == 4.0
    assert O.workset_functor("Linear", 4.0, t=-1.0) == 0.0
    tt, tv = [0.0, 1.0, 3.0], [2.0, 4.0, 0.0]
    assert O.workset_functor("TimeTable", times=tt, values=tv, t=0.0) == 2.0
    assert O.workset_functor("TimeTable", times=tt, values=tv, t=0.5) == 3.0
    assert O.workset_functor("TimeTable", times=tt, values=tv, t=2.0) == 2.0
    assert O.workset_functor("TimeTable", times=tt, values=tv, t=-1.0) == 2.0
    with pytest.raises(ValueError):
        O.workset_functor("TimeTable", times=tt, values=tv, t=3.5)


# ---------------------------------------------------------------- responses
@pytest.mark.parametrize("topo,basis", [(A.TX_TOPO_HEX, A.TX_HGRAD_C1), (A.TX_TOPO_HEX, A.TX_HGRAD_C2),
                                        (A.TX_TOPO_TET, A.TX_HGRAD_C1), (A.TX_TOPO_TET, A.TX_HGRAD_C2)])
def test_response_closed_forms_and_gradient(topo, basis):
    # Every basis here reproduces linear fields on the jittered (trilinear or
    # affine) cells, so the integral of x over the box is exact; the "Field"
    # gradient sums to the volume; the error integrands are quadratic in x, so a
    # central difference checks their gradients to rounding.
    L = (1.5, 1.0, 0.75)
    o = O.Oracle(A.mesh_desc(2, topology=topo, lengths=L, jitter=0.2, seed=3),
                 A.equation_set(A.TX_PHYS_POISSON, basis, params=(1.0, 0.0, 0.0, 0.0)))
    X = o.dof_coordinates()
    vol = L[0] * L[1] * L[2]
    v, g = o.response("Field", x=np.ones(o.n_dofs), gradient=True)
    assert abs(v - vol) <= 1e-14 and abs(g.sum() - vol) <= 1e-13
    assert abs(o.response("Field", x=X[:, 0].copy()) - vol * L[0] / 2) <= 1e-14
    rng = np.random.default_rng(0)
    x = rng.uniform(-1, 1, o.n_dofs)
    for kind in ("L2 Error", "H1 Error"):
        v, g = o.response(kind, x=x, gradient=True)
        for i in rng.choice(o.n_dofs, 5, replace=False):
            h = 1e-3
            xp, xm = x.copy(), x.copy()
            xp[i] += h
            xm[i] -= h
            fd = (o.response(kind, x=xp) - o.response(kind, x=xm)) / (2 * h)
            assert abs(fd - g[i]) <= 1e-8 * max(1.0, abs(g[i])), (kind, i)


@pytest.mark.parametrize("topo,basis", [(A.TX_TOPO_HEX, A.TX_HGRAD_C1), (A.TX_TOPO_HEX, A.TX_HGRAD_C2),
                                        (A.TX_TOPO_TET, A.TX_HGRAD_C1)])
def test_extreme_side_and_probe_closed_forms(topo, basis):
    # u = x + 2y + 3z lies in every basis here, so: the integral of u over the
    # z = 1 face is 0.5 + 1 + 3 = 4.5 and the face area 1 (ExtremeValue, side
    # and probe responses of the restatement); the probe returns u exactly at
    # any point, even on jittered cells, with a gradient that sums to 1
    # (partition of unity); on the unjittered hex lattice the max over the
    # Gauss points sits at the point nearest (1,1,1): each coordinate
    # 1 - h/2 + h/(2 sqrt 3) for the 2-point rule.
    n = 4
    h = 1.0 / n
    o = O.Oracle(A.mesh_desc(n, topology=topo), A.equation_set(A.TX_PHYS_POISSON, basis, params=(1.0, 0.0, 0.0, 0.0)))
    X = o.dof_coordinates()
    u = X[:, 0] + 2 * X[:, 1] + 3 * X[:, 2]
    assert abs(o.side_response(A.SIDE_ZMAX, x=u) - 4.5) <= 1e-13
    v, g = o.side_response(A.SIDE_ZMAX, x=np.ones(o.n_dofs), gradient=True)
    assert abs(v - 1.0) <= 1e-14 and abs(g.sum() - 1.0) <= 1e-13
    if topo == A.TX_TOPO_HEX and basis == A.TX_HGRAD_C1:
        c = 1 - h / 2 + h / (2 * np.sqrt(3))
        vmax, gmax = o.extreme(True, x=u, degree=2, gradient=True)
        assert abs(vmax - 6 * c) <= 1e-13 and abs(gmax.sum() - 1.0) <= 1e-14
        assert abs(o.extreme(False, x=u, degree=2) - 6 * (1 - c)) <= 1e-13
    oj = O.Oracle(A.mesh_desc(n, topology=topo, jitter=0.2, seed=9),
                  A.equation_set(A.TX_PHYS_POISSON, basis, params=(1.0, 0.0, 0.0, 0.0)))
    Xj = oj.dof_coordinates()
    uj = Xj[:, 0] + 2 * Xj[:, 1] + 3 * Xj[:, 2]
    for p in ((0.31, 0.47, 0.52), (0.9, 0.05, 0.66)):
        val, e, gp = oj.probe(p, x=uj, gradient=True)
        assert e >= 0 and abs(val - (p[0] + 2 * p[1] + 3 * p[2])) <= 1e-12 and abs(gp.sum() - 1.0) <= 1e-12
    assert oj.probe((1.5, 0.5, 0.5), x=uj)[1] == -1


def test_dirichlet_rows_and_columns_keep_symmetry():
    # RowsAndColumns (no residual) keeps a symmetric Jacobian symmetric; rows only does not
    import scipy.sparse as sp
    o = O.Oracle(A.mesh_desc(3, jitter=0.1, seed=2), A.equation_set(A.TX_PHYS_ELASTICITY, params=(1.0, 0.3, 0.0, 0.0, -1.0)))
    x = np.random.default_rng(1).uniform(-1, 1, o.n_dofs)
    _, v = o.evaluate(x, None, None)
    rp, ci = o.graph()
    lids = np.flatnonzero(o.dof_coordinates()[:, 2] == 0.0).astype(np.int32)
    for with_f, symmetric in ((False, True), (True, False)):
        vv = v.copy()
        f = np.zeros(o.n_dofs) if with_f else None
        o.dirichlet_apply(lids, None, x, f, vv)
        K = sp.csr_matrix((vv, ci, rp), shape=(o.n_dofs, o.n_dofs))
        assert (abs(K - K.T).max() <= 1e-14 * abs(K).max()) == symmetric
        assert np.all(K.diagonal()[lids] == 1.0)
