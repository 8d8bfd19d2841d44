"""The C-ABI from plain C (cudaMalloc'd buffers, no torch) gives the same
evaluation as the Python path; its Newton step reaches 1e-10."""
import os
import subprocess

import pytest
import torch

import tianxin_gb300 as tx
from tianxin_gb300 import _abi as A
from tianxin_gb300 import _lib

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_plain_c_caller(cuda, tmp_path):
    build = os.path.join(ROOT, "tianxin_gb300", "_build")
    exe = str(tmp_path / "capi_smoke")
    subprocess.run(["gcc", "-O2", "-I", os.path.join(ROOT, "include"), "-I", "/usr/local/cuda/include",
                    os.path.join(ROOT, "tests", "capi", "capi_smoke.c"), "-L", build, "-ltianxin_gb300",
                    "-L", "/usr/local/cuda/lib64", "-lcudart", "-lm", f"-Wl,-rpath,{build}", "-o", exe], check=True)
    out = subprocess.run([exe, "6"], check=True, capture_output=True, text=True).stdout.split()
    assert out[:2] == ["capi", "ok"]
    N, nnz, sf, sv, relres = int(out[2]), int(out[3]), float(out[4]), float(out[5]), float(out[6])
    # same evaluation through the Python host API
    conn = tx.CartesianConnManager(6, 6, 6, jitter=0.05, seed=2024)
    dof = tx.DOFManager(conn, A.equation_set(A.TX_PHYS_ELASTICITY, params=(1.0, 0.3, 0.0, 0.0, -1.0)))
    lof = tx.TpetraLinearObjFactory(dof)
    me = tx.ModelEvaluator(lof, [tx.DirichletBC(dof, A.SIDE_ZMIN)])
    f, W = lof.getTpetraVector(), me.create_W_op()
    me.evalModel(lof.getTpetraVector(), f=f, W=W, mixed=True)
    assert (N, nnz) == (dof.n_dofs, dof.nnz)
    assert abs(float(f.abs().sum()) - sf) <= 1e-12 * sf
    assert abs(float(W.values.abs().sum()) - sv) <= 1e-12 * sv
    assert relres <= 1e-10
