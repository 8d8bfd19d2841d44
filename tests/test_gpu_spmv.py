"""CRS SpMV (Tpetra::CrsMatrix::apply) on graphs of every row-length class.

Without a tuned shape the kernel picks the lanes per row from the mean row
length: Poisson tet4 (about 11 entries a row) 4 lanes; Poisson hex8 (about
23), heat on hex27 + tet10 (about 60; vertex rows of 125 take several
passes) and elasticity hex8 (about 69) 8 lanes.  A random CSR matrix with
empty and long rows covers the shape used when the mean is unknown, and
every tunable shape is checked on two graphs.  Matrices on the handle's
graph also take the entity-block form (one column index per 3 x 3 block of
elasticity; nf = 1 graphs run the CRS form under that flag), checked in every
shape, on a Dirichlet-modified Jacobian, and inside the solver.  Bars: FP64
within 1e-13 relative (reassociated sums), FP32 within 1e-5.
"""
import ctypes as C

import numpy as np
import pytest
import torch

import tianxin_gb300 as tx
from tianxin_gb300 import _abi as A
from tianxin_gb300 import _lib

pytestmark = pytest.mark.gpu


def _csr_ref(rp, ci, vals, x):
    y = np.zeros(len(rp) - 1)
    for r in range(len(rp) - 1):
        y[r] = np.dot(vals[rp[r]:rp[r + 1]], x[ci[rp[r]:rp[r + 1]]])
    return y


GRAPHS = {
    "poisson_tet4": dict(n=(5, 5, 5), blocks=(1, 1, 1), topo=A.TX_TOPO_TET, phys=A.TX_PHYS_POISSON,
                         basis=A.TX_HGRAD_C1, params=(1.0, 0.0, 0.0, 1.0)),
    "poisson_hex8": dict(n=(7, 6, 5), blocks=(1, 1, 1), topo=A.TX_TOPO_HEX, phys=A.TX_PHYS_POISSON,
                         basis=A.TX_HGRAD_C1, params=(1.0, 0.0, 0.0, 1.0)),
    "heat_hex27_tet10": dict(n=(4, 3, 3), blocks=(2, 1, 1), topo=[A.TX_TOPO_HEX, A.TX_TOPO_TET],
                             phys=A.TX_PHYS_HEAT, basis=A.TX_HGRAD_C2, params=(1.0, 0.5, 1.0)),
    "elasticity_hex8": dict(n=(12, 12, 12), blocks=(1, 1, 1), topo=A.TX_TOPO_HEX, phys=A.TX_PHYS_ELASTICITY,
                            basis=A.TX_HGRAD_C1, params=(1.0, 0.3, 0.0, 0.0, -1.0, 0.0)),
}


@pytest.mark.parametrize("form", ["crs", "entity"])
@pytest.mark.parametrize("name", list(GRAPHS))
def test_spmv_on_assembly_graphs(cuda, name, form):
    g = GRAPHS[name]
    conn = tx.CartesianConnManager(*g["n"], *g["blocks"], topology=g["topo"], jitter=0.1, seed=5)
    dof = tx.DOFManager(conn, A.equation_set(g["phys"], g["basis"], params=g["params"]))
    lof = tx.TpetraLinearObjFactory(dof)
    W = lof.getTpetraMatrix()
    W.setApplyForm(form)
    rng = np.random.default_rng(11)
    vals = rng.uniform(-1, 1, dof.nnz)
    x = rng.uniform(-1, 1, dof.n_dofs)
    W.values.copy_(torch.from_numpy(vals))
    rp, ci = W.rowptr.cpu().numpy(), W.colind.cpu().numpy()
    y_ref = _csr_ref(rp, ci, vals, x)
    scale = np.abs(y_ref).max()
    y = W.apply(torch.from_numpy(x).cuda()).cpu().numpy()
    assert np.abs(y - y_ref).max() <= 1e-13 * scale
    y0 = rng.uniform(-1, 1, dof.n_dofs)
    yy = torch.from_numpy(y0.copy()).cuda()
    W.apply(torch.from_numpy(x).cuda(), yy, alpha=-1.5, beta=0.25)
    assert np.abs(yy.cpu().numpy() - (-1.5 * y_ref + 0.25 * y0)).max() <= 1e-13 * scale
    y32 = W.apply(torch.from_numpy(x).float().cuda(), values=W.values.float()).cpu().numpy()
    assert np.abs(y32 - y_ref).max() <= 1e-5 * scale


def test_spmv_random_rows_with_empty_and_long_rows(cuda):
    lib = _lib.load()
    conn = tx.CartesianConnManager(2, 2, 2)
    dof = tx.DOFManager(conn, A.equation_set(A.TX_PHYS_POISSON, params=(1.0, 0.0, 0.0, 1.0)))
    rng = np.random.default_rng(3)
    n = 1001  # differs from the handle's DOF count: no mean row length is known
    lens = rng.integers(0, 150, n)
    lens[rng.choice(n, 50, replace=False)] = 0
    rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    ci = rng.integers(0, n, int(rp[-1])).astype(np.int32)
    vals = rng.uniform(-1, 1, int(rp[-1]))
    x = rng.uniform(-1, 1, n)
    y_ref = _csr_ref(rp, ci, vals, x)
    d = {k: torch.from_numpy(v).cuda() for k, v in dict(rp=rp, ci=ci, vals=vals, x=x).items()}
    y = torch.full((n,), 7.0, dtype=torch.float64, device="cuda")
    lib.tx_set_stream(dof.h, C.c_void_p(torch.cuda.current_stream().cuda_stream))
    rc = lib.tx_spmv(dof.h, A.TX_SPMV_F64, n, d["rp"].data_ptr(), d["ci"].data_ptr(), d["vals"].data_ptr(),
                     d["x"].data_ptr(), y.data_ptr(), 1.0, 0.0)
    assert rc == 0
    out = y.cpu().numpy()
    assert np.abs(out - y_ref).max() <= 1e-13 * np.abs(y_ref).max()
    assert np.all(out[lens == 0] == 0.0)  # empty rows: beta = 0 overwrites


@pytest.mark.parametrize("name", ["poisson_hex8", "elasticity_hex8"])
def test_spmv_every_launch_shape(cuda, name):
    # the autotuner's knob changes only the summation order
    g = GRAPHS[name]
    conn = tx.CartesianConnManager(*g["n"], *g["blocks"], topology=g["topo"], jitter=0.1, seed=5)
    dof = tx.DOFManager(conn, A.equation_set(g["phys"], g["basis"], params=g["params"]))
    W = tx.TpetraLinearObjFactory(dof).getTpetraMatrix()
    rng = np.random.default_rng(2)
    vals = rng.uniform(-1, 1, dof.nnz)
    x = rng.uniform(-1, 1, dof.n_dofs)
    W.values.copy_(torch.from_numpy(vals))
    y_ref = _csr_ref(W.rowptr.cpu().numpy(), W.colind.cpu().numpy(), vals, x)
    xd = torch.from_numpy(x).cuda()
    x32 = xd.float()
    v32 = W.values.float()
    W.setApplyForm("crs")
    for lanes in (4, 8, 16, 32):
        for unroll in (1, 2, 4, 16):  # 16: aligned 16-byte loads
            W.setApplyShape(lanes, unroll)
            y = W.apply(xd).cpu().numpy()
            assert np.abs(y - y_ref).max() <= 1e-13 * np.abs(y_ref).max(), (lanes, unroll)
            y32 = W.apply(x32, values=v32).cpu().numpy()
            assert np.abs(y32 - y_ref).max() <= 1e-5 * np.abs(y_ref).max(), (lanes, unroll)
    W.setApplyShape(0, 0)
    W.setApplyForm("entity")
    for lanes, unroll in [(3, 1), (3, 2), (3, 3), (4, 4), (8, 4)] + \
            [(lanes, unroll) for lanes in (4, 8, 16, 32) for unroll in (1, 2)]:
        if True:
            W.setEntityApplyShape(lanes, unroll)
            y = W.apply(xd).cpu().numpy()
            assert np.abs(y - y_ref).max() <= 1e-13 * np.abs(y_ref).max(), ("entity", lanes, unroll)
            y32 = W.apply(x32, values=v32).cpu().numpy()
            assert np.abs(y32 - y_ref).max() <= 1e-5 * np.abs(y_ref).max(), ("entity", lanes, unroll)
    W.setEntityApplyShape(0, 0)


def test_entity_form_on_assembled_dirichlet_jacobian_and_in_the_solver(cuda):
    # tet4 elasticity: entity degrees vary (4 to about 27 neighbours); Dirichlet rows keep the pattern
    conn = tx.CartesianConnManager(6, 5, 4, topology=A.TX_TOPO_TET, jitter=0.1, seed=4)
    q = A.equation_set(A.TX_PHYS_ELASTICITY, params=(1.0, 0.3, 0.0, 0.0, -1.0, 0.0))
    dof = tx.DOFManager(conn, q)
    lof = tx.TpetraLinearObjFactory(dof)
    me = tx.ModelEvaluator(lof, [tx.DirichletBC(dof, A.SIDE_ZMIN)])
    x, f, W = lof.getTpetraVector(), lof.getTpetraVector(), me.create_W_op()
    me.evalModel(x, f=f, W=W)
    vals = W.values.cpu().numpy()
    rp, ci = W.rowptr.cpu().numpy(), W.colind.cpu().numpy()
    xs = np.random.default_rng(9).uniform(-1, 1, dof.n_dofs)
    y_ref = _csr_ref(rp, ci, vals, xs)
    y = W.apply(torch.from_numpy(xs).cuda()).cpu().numpy()
    assert W.apply_form == "entity"
    assert np.abs(y - y_ref).max() <= 1e-13 * np.abs(y_ref).max()
    sols = {}
    for form in ("crs", "entity"):
        W.setApplyForm(form)
        xx = lof.getTpetraVector()
        st = me.solve(W, xx, rtol=1e-11, matrix_free=False, b=-f)
        assert st["relres"] <= 1e-11, form
        sols[form] = xx.cpu().numpy()
    assert np.abs(sols["crs"] - sols["entity"]).max() <= 1e-9 * np.abs(sols["crs"]).max()


def test_entity_form_needs_the_handle_graph(cuda):
    lib = _lib.load()
    g = GRAPHS["elasticity_hex8"]
    conn = tx.CartesianConnManager(3, 3, 3)
    dof = tx.DOFManager(conn, A.equation_set(g["phys"], g["basis"], params=g["params"]))
    W = tx.TpetraLinearObjFactory(dof).getTpetraMatrix()
    x = torch.ones(dof.n_dofs, dtype=torch.float64, device="cuda")
    y = torch.zeros(dof.n_dofs, dtype=torch.float64, device="cuda")
    rc = lib.tx_spmv(dof.h, A.TX_SPMV_F64 | A.TX_SPMV_ENTITY_BLOCKS, dof.n_dofs - 3, W.rowptr.data_ptr(),
                     W.colind.data_ptr(), W.values.data_ptr(), x.data_ptr(), y.data_ptr(), 1.0, 0.0)
    assert rc == A.TX_EINVAL
    other = tx.CrsMatrix(dof, W.rowptr.clone(), W.colind.clone())
    assert other.apply_form == "crs"
    with pytest.raises(ValueError):
        other.setApplyForm("entity")


def test_spmv_vector_shape_on_unaligned_arrays(cuda):
    # values starting 8 bytes past a 16-byte boundary: the 16-byte form falls back to single loads
    lib = _lib.load()
    conn = tx.CartesianConnManager(2, 2, 2)
    dof = tx.DOFManager(conn, A.equation_set(A.TX_PHYS_POISSON, params=(1.0, 0.0, 0.0, 1.0)))
    rng = np.random.default_rng(8)
    n = 300
    lens = rng.integers(0, 90, n)
    rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    ci = rng.integers(0, n, int(rp[-1])).astype(np.int32)
    vals = rng.uniform(-1, 1, int(rp[-1]))
    x = rng.uniform(-1, 1, n)
    y_ref = _csr_ref(rp, ci, vals, x)
    vbuf = torch.zeros(len(vals) + 1, dtype=torch.float64, device="cuda")
    vbuf[1:] = torch.from_numpy(vals).cuda()
    cbuf = torch.zeros(len(ci) + 1, dtype=torch.int32, device="cuda")
    cbuf[1:] = torch.from_numpy(ci).cuda()
    d_rp, d_x = torch.from_numpy(rp).cuda(), torch.from_numpy(x).cuda()
    y = torch.zeros(n, dtype=torch.float64, device="cuda")
    lib.tx_set_stream(dof.h, C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert lib.tx_set_spmv_shape(dof.h, 8, 16) == 0
    rc = lib.tx_spmv(dof.h, A.TX_SPMV_F64, n, d_rp.data_ptr(), cbuf.data_ptr() + 4, vbuf.data_ptr() + 8,
                     d_x.data_ptr(), y.data_ptr(), 1.0, 0.0)
    assert rc == 0
    assert np.abs(y.cpu().numpy() - y_ref).max() <= 1e-13 * np.abs(y_ref).max()
