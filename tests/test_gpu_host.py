"""HostEvaluator: evalModel with host-resident (pinned) x, f and CRS values,
pipelined over two device buffer sets.  Each step's host results equal a
direct device evaluation of that step's x (the copy-back of step k runs
while step k + 1 assembles)."""
import numpy as np
import pytest
import torch

import tianxin_gb300 as tx
from tianxin_gb300 import _abi as A

pytestmark = pytest.mark.gpu


def test_host_pipeline_matches_device_evaluations(cuda):
    conn = tx.CartesianConnManager(6, 5, 4, jitter=0.1, seed=3)
    dof = tx.DOFManager(conn, A.equation_set(A.TX_PHYS_ELASTICITY, params=(1.0, 0.3, 0.0, 0.0, -1.0)))
    lof = tx.TpetraLinearObjFactory(dof)
    me = tx.ModelEvaluator(lof, [tx.DirichletBC(dof, A.SIDE_ZMIN)])
    hev = tx.HostEvaluator(me, mixed=True)
    g = torch.Generator().manual_seed(6)
    steps = 5
    xs = [(torch.rand(dof.n_dofs, dtype=torch.float64, generator=g) * 0.01).pin_memory() for _ in range(steps)]
    fh = [torch.empty(dof.n_dofs, dtype=torch.float64).pin_memory() for _ in range(steps)]
    Wh = [torch.empty(dof.nnz, dtype=torch.float64).pin_memory() for _ in range(steps)]
    for k in range(steps):
        hev.step(xs[k], fh[k], Wh[k])
    hev.synchronize()
    torch.cuda.synchronize()
    f, W = lof.getTpetraVector(), me.create_W_op()
    for k in range(steps):
        me.evalModel(xs[k].cuda(), f=f, W=W, mixed=True)
        torch.cuda.synchronize()
        assert torch.equal(fh[k], f.cpu()) or float((fh[k] - f.cpu()).abs().max()) <= 1e-12 * float(f.abs().max())
        assert float((Wh[k] - W.values.cpu()).abs().max()) <= 1e-12 * float(W.values.abs().max())
