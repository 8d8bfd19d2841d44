"""Newmark elastodynamics (beta=1/4, gamma=1/2) with graph-captured steps
against an FP64 Newmark on the oracle's matrices.

Bar: displacement after 10 steps within 1e-10 relative of the oracle; every
step's FP64 relative residual (from the captured solver) <= 1e-10.
"""
import numpy as np
import pytest
import torch

import tianxin_gb300 as tx
from oracle import oracle as O
from tianxin_gb300 import _abi as A
from tianxin_gb300.newmark import NewmarkElastodynamics

pytestmark = pytest.mark.gpu


def dense(o, vals):
    rp, ci = o.graph()
    M = np.zeros((o.n_dofs, o.n_dofs))
    for r in range(o.n_dofs):
        M[r, ci[rp[r]:rp[r + 1]]] = vals[rp[r]:rp[r + 1]]
    return M


@pytest.mark.parametrize("linear", [True, False])
def test_newmark_graph_steps_match_oracle(cuda, linear):
    n, dt, beta, gamma = 5, 1e-3, 0.25, 0.5
    params = (1.0, 0.25, 0.0, 0.0, 0.0, 1.0)  # E, nu, body force, rho
    q = A.equation_set(A.TX_PHYS_ELASTICITY, params=params)
    o = O.Oracle(A.mesh_desc(n, jitter=0.05, seed=3), q)
    dof = tx.DOFManager(tx.CartesianConnManager(n, n, n, jitter=0.05, seed=3), q)
    lof = tx.TpetraLinearObjFactory(dof)
    me = tx.ModelEvaluator(lof)
    u0 = np.random.default_rng(0).normal(0.0, 1e-3, o.n_dofs)

    # oracle FP64 Newmark (dense): M a + K u = F
    z = np.zeros(o.n_dofs)
    f0, kv = o.evaluate(z, z, alpha=0.0, beta=1.0)
    _, mv = o.evaluate(z, z, alpha=1.0, beta=0.0, residual=False)
    K, M, F = dense(o, kv), dense(o, mv), -f0
    c = 1.0 / (beta * dt * dt)
    u, v = u0.copy(), np.zeros(o.n_dofs)
    a = np.linalg.solve(M, F - K @ u)
    Keff = K + c * M
    for _ in range(10):
        up = u + dt * v + dt * dt * (0.5 - beta) * a
        vp = v + dt * (1 - gamma) * a
        u = np.linalg.solve(Keff, F + c * M @ up)
        a = c * (u - up)
        v = vp + gamma * dt * a

    nm = NewmarkElastodynamics(me, dt, beta, gamma, mixed=True, outer=3, inner=24, linear=linear)
    nm.initialize(torch.from_numpy(u0).cuda())
    nm.capture()
    worst = 0.0
    for _ in range(10):
        st = nm.step()
        worst = max(worst, float(st[2]))
    torch.cuda.synchronize()
    err = np.abs(nm.u.cpu().numpy() - u).max() / np.abs(u).max()
    assert worst <= 1e-10, worst
    assert err <= 1e-10, err
