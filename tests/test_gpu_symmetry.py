"""Symmetric forming of the FP64 element matrices (run on a GB300).

The staged FP64 kernels form each symmetric element matrix (elasticity,
Poisson, Nedelec Maxwell) as its upper blocks and write every block with its
transpose, and split the heat rows into a symmetric conduction part and the
N_b term.  Checked on small meshes: the assembled Jacobian against the
oracle's forward-mode AD Jacobian at the FP64 bar, and, for the symmetric
families, against its own transpose (the element matrices are transposes of
each other bit for bit, so only the order of the FP64 sums into an entry can
differ); the heat Jacobian is not symmetric and its transpose is not close.
"""
import numpy as np
import pytest
import torch

import tianxin_gb300 as tx
from oracle import oracle as O
from tianxin_gb300 import _abi as A

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12

CASES = [
    # name, bricks, topology, physics, basis, params, symmetric
    ("elasticity_hex8", (3, 4, 3), A.TX_TOPO_HEX, A.TX_PHYS_ELASTICITY, A.TX_HGRAD_C1, (1.0, 0.3, 0.1, -0.2, -1.0, 0.7), True),
    ("elasticity_tet4", (2, 3, 3), A.TX_TOPO_TET, A.TX_PHYS_ELASTICITY, A.TX_HGRAD_C1, (1.0, 0.3, 0.0, 0.0, -1.0, 0.0), True),
    ("poisson_hex8", (4, 3, 3), A.TX_TOPO_HEX, A.TX_PHYS_POISSON, A.TX_HGRAD_C1, (1.0, 0.5, 1.0, 2.0), True),
    ("maxwell_nedelec", (3, 2, 3), A.TX_TOPO_HEX, A.TX_PHYS_MAXWELL, A.TX_HCURL_I1, (1.0, 1.0), True),
    ("heat_hex27", (2, 2, 3), A.TX_TOPO_HEX, A.TX_PHYS_HEAT, A.TX_HGRAD_C2, (1.0, 0.5, 1.0), False),
    ("heat_tet10", (2, 2, 2), A.TX_TOPO_TET, A.TX_PHYS_HEAT, A.TX_HGRAD_C2, (1.0, 0.5, 1.0), False),
]


def dense(lof, W):
    rp, ci = lof.rowptr.cpu().numpy(), lof.colind.cpu().numpy()
    n = rp.size - 1
    K = np.zeros((n, n))
    K[np.repeat(np.arange(n), np.diff(rp)), ci] = W.values.cpu().numpy()
    return K


@pytest.mark.parametrize("name,n,topo,phys,basis,params,sym", CASES, ids=[c[0] for c in CASES])
def test_fp64_staged_jacobian_symmetry(cuda, name, n, topo, phys, basis, params, sym):
    m = A.mesh_desc(n, topology=topo, jitter=0.1, seed=7)
    q = A.equation_set(phys, basis, params=params)
    o = O.Oracle(m, q)
    conn = tx.CartesianConnManager(*n, topology=topo, jitter=0.1, seed=7)
    lof = tx.TpetraLinearObjFactory(tx.DOFManager(conn, q))
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, o.n_dofs)
    aux = rng.standard_normal(o.n_dofs) if phys == A.TX_PHYS_MAXWELL else None
    f_ref, v_ref = o.evaluate(x, None, aux, alpha=0.0, beta=1.0)
    ae = tx.AssemblyEngine(lof)
    ae.setVariant(1)  # the CTA-staged kernel
    f, W = lof.getTpetraVector(), lof.getTpetraMatrix()
    ae.evaluate(torch.from_numpy(x).cuda(), aux=None if aux is None else torch.from_numpy(aux).cuda(),
                f=f, W=W, mixed=False, gather=False)
    wv = W.values.cpu().numpy()
    assert np.abs(wv - v_ref).max() <= FP64_TOL * np.abs(v_ref).max()
    K = dense(lof, W)
    asym = float(np.abs(K - K.T).max() / np.abs(K).max())
    if sym:
        assert asym <= 1e-14, asym
    else:
        assert asym > 1e-6, asym  # the dk/dT term: the heat Jacobian is not symmetric
