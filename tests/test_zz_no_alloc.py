"""tx_eval_noalloc: the volume fill for callers that may not allocate device memory.

Applications that reserve all device memory up front in their own pool
cannot accept a driver allocation outside it, and step loops that must not
stall the device cannot afford the cudaFree of grown scratch.  For them the
library offers tx_eval_noalloc, which keeps the persistent evaluation's
scratch (work counter, parameter tables, work list) in a fixed static device
array instead of allocating it.  These tests call it through the C-ABI and
check it against tx_eval with TX_EVAL_PERSISTENT, the existing entry point,
on two calls in a row.  This file is collected last so that a failure here
leaves every other test already run.
"""
import ctypes as C

import numpy as np
import pytest
import torch

import tianxin_gb300 as tx
from tianxin_gb300 import _abi as A
from tianxin_gb300 import _lib
from tianxin_gb300.panzer import eval_args

pytestmark = pytest.mark.gpu

TOL = 1e-12  # both paths do the same element arithmetic; only the FP64 summation order differs


def _setup(n, blocks, topo, phys, basis, params, ws):
    conn = tx.CartesianConnManager(*n, *blocks, topology=topo, jitter=0.1, seed=12)
    dof = tx.DOFManager(conn, A.equation_set(phys, basis, params=params))
    lof = tx.TpetraLinearObjFactory(dof)
    tx.AssemblyEngine(lof).setWorksetSize(ws, ws)
    return conn, dof, lof


def _call(lib, dof, args):
    lib.tx_set_stream(dof.h, C.c_void_p(torch.cuda.current_stream().cuda_stream))
    return lib.tx_eval_noalloc(dof.h, C.byref(args))


@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("case", ["heat_hex27_tet10", "elasticity_hex8"])
def test_noalloc_matches_persistent_twice(cuda, case, mixed):
    lib = _lib.load()
    if case == "heat_hex27_tet10":
        conn, dof, lof = _setup((3, 2, 2), (2, 1, 1), [A.TX_TOPO_HEX, A.TX_TOPO_TET], A.TX_PHYS_HEAT,
                                A.TX_HGRAD_C2, (1.0, 0.5, 1.0), ws=7)
    else:
        conn, dof, lof = _setup((6, 5, 4), (1, 1, 1), A.TX_TOPO_HEX, A.TX_PHYS_ELASTICITY, A.TX_HGRAD_C1,
                                (1.0, 0.3, 0.0, 0.0, -1.0, 0.5), ws=16)
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.rand(dof.n_dofs, dtype=torch.float64, device="cuda", generator=g)
    xd = torch.rand(dof.n_dofs, dtype=torch.float64, device="cuda", generator=g)
    # reference: the existing entry point, tx_eval with TX_EVAL_PERSISTENT
    f_ref, W_ref = lof.getTpetraVector(), lof.getTpetraMatrix()
    tx.AssemblyEngine(lof).evaluate(x, xd, alpha=0.5, beta=1.0, f=f_ref, W=W_ref, mixed=mixed, persistent=True)
    f, W = lof.getTpetraVector(), lof.getTpetraMatrix()
    for call in range(2):  # the static scratch keeps the last call's contents
        f.zero_()
        W.initializeMatrix(0.0)
        rc = _call(lib, dof, eval_args(x, xd, None, 0.5, 1.0, 0.0, f, W, mixed))
        assert rc == 0, lib.tx_last_error(dof.h)
        torch.cuda.synchronize()
        assert float((f - f_ref).abs().max()) <= TOL * float(f_ref.abs().max()), call
        assert float((W.values - W_ref.values).abs().max()) <= TOL * float(W_ref.values.abs().max()), call


def test_noalloc_rejects_work_lists_beyond_the_limit(cuda):
    lib = _lib.load()
    n = 41  # 68,921 elements: one-element worksets exceed the 65,536-item limit
    conn, dof, lof = _setup((n, n, n), (1, 1, 1), A.TX_TOPO_HEX, A.TX_PHYS_POISSON, A.TX_HGRAD_C1,
                            (1.0, 0.0, 0.0, 1.0), ws=1)
    x, f = lof.getTpetraVector(), lof.getTpetraVector()
    rc = _call(lib, dof, eval_args(x, f=f))
    assert rc == A.TX_ERANGE
    assert b"65536" in lib.tx_last_error(dof.h)
    tx.AssemblyEngine(lof).setWorksetSize(64, 64)  # 1,077 worksets of one item each: accepted
    assert _call(lib, dof, eval_args(x, f=f)) == 0
    f_ref = lof.getTpetraVector()
    tx.AssemblyEngine(lof).evaluate(x, f=f_ref)
    torch.cuda.synchronize()
    assert float((f - f_ref).abs().max()) <= TOL * float(f_ref.abs().max())


def test_noalloc_argument_errors(cuda):
    lib = _lib.load()
    conn, dof, lof = _setup((2, 2, 2), (1, 1, 1), A.TX_TOPO_HEX, A.TX_PHYS_POISSON, A.TX_HGRAD_C1,
                            (1.0, 0.0, 0.0, 1.0), ws=4)
    x, f = lof.getTpetraVector(), lof.getTpetraVector()
    assert _call(lib, dof, eval_args(x, f=f, block=0)) == A.TX_EINVAL
    assert _call(lib, dof, eval_args(x, f=f, deterministic=True)) == A.TX_EINVAL
    assert _call(lib, dof, eval_args(None, f=f)) == A.TX_EINVAL
