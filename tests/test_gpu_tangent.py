"""Tangent evaluation type against the oracle.

GatherSolution_Tpetra<Tangent> seeds the derivative slots with tangent
vectors and ScatterResidual_Tpetra<Tangent> sums those slots into dfdp
(disc-fe/src/evaluators/Panzer_GatherSolution_Tpetra_impl.hpp:336-389,
Panzer_ScatterResidual_Tpetra_impl.hpp:237-270), so dfdp_i = W t_i with
W = beta dR/dx + alpha dR/dxdot.  The oracle's W comes from its forward-mode
AD Jacobian, applied with its own CRS product.  Bar: 1e-12 relative to the
largest entry.
"""
import numpy as np
import pytest
import torch

import tianxin_gb300 as tx
from oracle import oracle as O
from tianxin_gb300 import _abi as A

pytestmark = pytest.mark.gpu

CASES = {
    "elasticity_hex8": dict(n=(3, 3, 4), blocks=(1, 1, 1), topo=A.TX_TOPO_HEX, phys=A.TX_PHYS_ELASTICITY,
                            basis=A.TX_HGRAD_C1, params=(1.0, 0.3, 0.0, 0.0, -1.0, 2.0)),
    "heat_hex27_tet10": dict(n=(2, 2, 2), blocks=(2, 1, 1), topo=[A.TX_TOPO_HEX, A.TX_TOPO_TET],
                             phys=A.TX_PHYS_HEAT, basis=A.TX_HGRAD_C2, params=(1.0, 0.5, 1.0)),
    "poisson_tet4": dict(n=(3, 3, 3), blocks=(1, 1, 1), topo=A.TX_TOPO_TET, phys=A.TX_PHYS_POISSON,
                         basis=A.TX_HGRAD_C1, params=(1.0, 0.5, 2.0, 1.0)),
    "maxwell_hex": dict(n=(2, 3, 2), blocks=(1, 1, 1), topo=A.TX_TOPO_HEX, phys=A.TX_PHYS_MAXWELL,
                        basis=A.TX_HCURL_I1, params=(1.0, 2.0)),
}


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("alpha,beta", [(0.0, 1.0), (1.0, 0.0), (0.5, 2.0)])
@pytest.mark.parametrize("deterministic", [False, True])
def test_tangent_equals_jacobian_times_directions(cuda, name, alpha, beta, deterministic):
    c = CASES[name]
    m = A.mesh_desc(c["n"], c["blocks"], c["topo"], jitter=0.12, seed=8)
    q = A.equation_set(c["phys"], c["basis"], params=c["params"])
    o = O.Oracle(m, q)
    dof = tx.DOFManager(tx.CartesianConnManager(*c["n"], *c["blocks"], topology=c["topo"], jitter=0.12, seed=8), q)
    lof = tx.TpetraLinearObjFactory(dof)
    rng = np.random.default_rng(4)
    x, xd, aux = (rng.uniform(0, 1, o.n_dofs) for _ in range(3))
    _, vals = o.evaluate(x, xd, aux=aux, alpha=alpha, beta=beta)
    rp, ci = o.graph()
    T = rng.uniform(-1, 1, (3, o.n_dofs))
    ref = np.stack([O.spmv(rp, ci, vals, T[i]) for i in range(3)])
    dfdp = torch.zeros(3, o.n_dofs, dtype=torch.float64, device="cuda")
    cu = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    tx.AssemblyEngine(lof).evaluateTangent(cu(x), cu(T), dfdp, x_dot=cu(xd), aux=cu(aux), alpha=alpha, beta=beta,
                                           deterministic=deterministic)
    got = dfdp.cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


def test_tangent_argument_errors(cuda):
    dof = tx.DOFManager(tx.CartesianConnManager(2, 2, 2), A.equation_set(A.TX_PHYS_POISSON, params=(1, 0, 0, 1)))
    lof = tx.TpetraLinearObjFactory(dof)
    x = lof.getTpetraVector()
    ae = tx.AssemblyEngine(lof)
    with pytest.raises(tx.TxError):
        ae.evaluateTangent(x, torch.zeros(5, dof.n_dofs, dtype=torch.float64, device="cuda"),
                           torch.zeros(5, dof.n_dofs, dtype=torch.float64, device="cuda"))


PARAM_CASES = [
    ("poisson_tet4", (1.0, 0.5, 2.0, 1.0), A.TX_SOURCE_CONST, A.TX_PHYS_POISSON, A.TX_TOPO_TET, A.TX_HGRAD_C1, range(4)),
    ("poisson_affine_hex8", (1.0, 0.7, 2.0, 1.0), A.TX_SOURCE_AFFINE, A.TX_PHYS_POISSON, A.TX_TOPO_HEX, A.TX_HGRAD_C1,
     range(4)),
    ("elasticity_hex8", (1.3, 0.3, 0.2, -0.1, -1.0, 2.0), A.TX_SOURCE_CONST, A.TX_PHYS_ELASTICITY, A.TX_TOPO_HEX,
     A.TX_HGRAD_C1, range(6)),
    ("heat_hex27", (1.0, 0.5, 1.5), A.TX_SOURCE_CONST, A.TX_PHYS_HEAT, A.TX_TOPO_HEX, A.TX_HGRAD_C2, range(3)),
    ("maxwell_hex", (1.5, 2.0), A.TX_SOURCE_CONST, A.TX_PHYS_MAXWELL, A.TX_TOPO_HEX, A.TX_HCURL_I1, range(2)),
]


@pytest.mark.parametrize("name,params,source,phys,topo,basis,indices", PARAM_CASES, ids=[c[0] for c in PARAM_CASES])
def test_parameter_sensitivities_match_oracle_differences(cuda, name, params, source, phys, topo, basis, indices):
    # df/dp_i against the oracle's residual difference: exact for the parameters the
    # residual is affine in (unit step), a central difference for Poisson's ratio
    n = (3, 2, 3)
    m = A.mesh_desc(n, topology=topo, jitter=0.12, seed=5)
    rng = np.random.default_rng(3)
    q = A.equation_set(phys, basis, params=params, source_kind=source)
    o = O.Oracle(m, q)
    x, xd, aux = (rng.uniform(-1, 1, o.n_dofs) for _ in range(3))
    dof = tx.DOFManager(tx.CartesianConnManager(*n, topology=topo, jitter=0.12, seed=5), q)
    lof = tx.TpetraLinearObjFactory(dof)
    cu = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    def central(i, h):
        fs = []
        for sgn in (1.0, -1.0):
            pp = list(params)
            pp[i] += sgn * h
            oo = O.Oracle(m, A.equation_set(phys, basis, params=pp, source_kind=source))
            fs.append(oo.evaluate(x, xd, aux=aux, jacobian=False)[0])
        return (fs[0] - fs[1]) / (2 * h)

    for i in indices:
        nonlinear = phys == A.TX_PHYS_ELASTICITY and i == 1  # Poisson's ratio, through the Lame parameters
        h = 1e-3 if nonlinear else 1.0
        ref = central(i, h)
        if nonlinear:  # Richardson: O(h^4)
            ref = (4.0 * central(i, h / 2) - ref) / 3.0
        dfdp = torch.zeros(o.n_dofs, dtype=torch.float64, device="cuda")
        tx.AssemblyEngine(lof).evaluateDfdp(cu(x), i, dfdp, x_dot=cu(xd), aux=cu(aux))
        got = dfdp.cpu().numpy()
        tol = 1e-9 if nonlinear else 1e-12  # Richardson truncation near 1e-10
        assert np.abs(got - ref).max() <= tol * max(np.abs(ref).max(), 1e-300), (name, i)
    with pytest.raises(tx.TxError):
        tx.AssemblyEngine(lof).evaluateDfdp(cu(x), 7, torch.zeros(o.n_dofs, dtype=torch.float64, device="cuda"))
