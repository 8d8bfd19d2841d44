"""Element contractions on the tensor cores (TX_VARIANT_TENSOR): hex8 elasticity
mixed R+J with P = sum_q W grad N_a grad N_b^T and M = sum_q W N_a N_b formed by
tcgen05 TF32 MMAs (hi/lo split, three products), the rest of the element on the
CUDA cores, atomic scatter.

Checked against the oracle's FP64 residual and Jacobian (forward-mode AD) at the
mixed tolerance, against the CUDA-core staged kernel, with and without the mass
terms, on lattices whose element counts leave the last batch of four partly
empty, and with the status word read by tx_synchronize.
"""
import numpy as np
import pytest
import torch

import tianxin_gb300 as tx
from oracle import oracle as O
from tianxin_gb300 import _abi as A

pytestmark = pytest.mark.gpu

TOL_MIXED = 2e-5  # FP32 element arithmetic, TF32 hi/lo products (~2^-22), FP64 sums
TOL_CUDA_CORES = 5e-6  # against the FP32 CUDA-core kernel: the splitting error and summation order


def rel(a, ref):
    return float(np.abs(a - ref).max() / np.abs(ref).max())


CASES = [
    ((1, 1, 1), (1.0, 0.3, 0.0, 0.0, -1.0, 0.0)),
    ((6, 5, 7), (1.0, 0.3, 0.0, 0.0, -1.0, 0.0)),  # 210 elements: the last batch of four holds two
    ((13, 6, 5), (1.0, 0.3, 0.1, 0.2, 0.3, 1.5)),  # density: mass terms through x_dot and alpha
    ((24, 20, 18), (2.0, 0.25, 0.5, -0.25, 1.0, 0.0)),  # 8640 elements: several batches a CTA
]


@pytest.mark.parametrize("n,params", CASES, ids=["1x1x1", "6x5x7", "13x6x5_mass", "24x20x18"])
def test_tensor_core_contractions_against_oracle(cuda, n, params):
    m = A.mesh_desc(n, jitter=0.1, seed=5)
    q = A.equation_set(A.TX_PHYS_ELASTICITY, params=params)
    o = O.Oracle(m, q)
    conn = tx.CartesianConnManager(*n, jitter=0.1, seed=5)
    dof = tx.DOFManager(conn, q)
    lof = tx.TpetraLinearObjFactory(dof)
    rng = np.random.default_rng(1)
    x_h = rng.uniform(-1, 1, o.n_dofs)
    xd_h = rng.uniform(-1, 1, o.n_dofs)
    alpha, beta = 0.75, 1.25
    f_ref, v_ref = o.evaluate(x_h, xd_h, alpha=alpha, beta=beta, threads=8)
    x, xd = torch.from_numpy(x_h).cuda(), torch.from_numpy(xd_h).cuda()
    ae = tx.AssemblyEngine(lof)
    out = {}
    for variant in (3, 1):
        ae.setVariant(variant)
        f, W = lof.getTpetraVector(), lof.getTpetraMatrix()
        ae.evaluate(x, xd, alpha=alpha, beta=beta, f=f, W=W, mixed=True)
        tx.synchronize(dof)  # raises TX_ETIMEDOUT if an MMA wait gave up
        out[variant] = (f.cpu().numpy(), W.values.cpu().numpy())
    ft, wt = out[3]
    assert rel(ft, f_ref) <= TOL_MIXED and rel(wt, v_ref) <= TOL_MIXED, (rel(ft, f_ref), rel(wt, v_ref))
    fc, wc = out[1]
    assert rel(wt, wc) <= TOL_CUDA_CORES and rel(ft, fc) <= TOL_CUDA_CORES
    assert np.abs(wt - wc).max() > 0.0  # a different kernel ran: TF32 products, not FP32 FMAs


def test_bounded_wait_gives_up_and_reports(cuda):
    # the give-up path of the bounded mbarrier waits: nothing arrives, the wait ends, tx_synchronize reports it once
    conn = tx.CartesianConnManager(2, 2, 2)
    dof = tx.DOFManager(conn, A.equation_set(A.TX_PHYS_ELASTICITY))
    lib = dof.lib
    assert lib.tx_selftest_wait_timeout(dof.h) == 0
    assert lib.tx_synchronize(dof.h) == A.TX_ETIMEDOUT
    assert b"gave up" in lib.tx_last_error(dof.h)
    assert lib.tx_synchronize(dof.h) == 0
