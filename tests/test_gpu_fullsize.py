"""Parity with the oracle at the workloads' stated sizes.

Every named workload is compared with the oracle (the CPU restatement of the
reference path, FP64, forward-mode AD Jacobians) on the same mesh and state,
at full size:

* elasticity hex8 128^3 (2,097,152 elements, 6,440,067 DOFs, 513,599,625 CRS
  entries): owned GIDs, element GID/LID vectors, Dirichlet set and the CRS
  graph bit-exact; FP64 residual and Jacobian within 1e-12 of the oracle's
  (relative to the largest entry); the mixed Jacobian, atomic, owner-computes
  lattice and tensor-core forms, within its stated 2e-5;
  the GPU's converged solution has an oracle-computed FP64 residual
  ||f(x)|| <= 1e-10 ||f(0)||, as the reference's fe_assembly test checks
  ||b - Ax|| (dof-mgr/test/fe_assembly/test_fe_assembly_HEX.hpp:672-677);
* nonlinear heat, hex27 48^3 + tet10 48^3 (774,144 elements): numbering and
  graph bit-exact, the persistent launch over uneven worksets of 256-1024
  elements within 1e-12 (FP64) and 2e-5 (mixed) of the oracle;
* Newmark elastodynamics hex8 96^3: ten graph-captured steps against ten
  steps of an FP64 Newmark on the oracle's K and M (oracle CG to 1e-13),
  displacements within 1e-10;
* the 256-mesh batch: every instance of the one-launch batch within 1e-12
  (FP64) and 2e-5 (mixed) of the oracle.

These run for minutes (the 128^3 oracle holds about 14 GB of host memory).
"""
import os

import numpy as np
import pytest
import torch

import tianxin_gb300 as tx
from oracle import oracle as O
from tianxin_gb300 import _abi as A
from tianxin_gb300 import workloads as WL
from tianxin_gb300.newmark import NewmarkElastodynamics
from tianxin_gb300.panzer import AssemblyEngine, Batch

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count()
TOL_FP64 = 1e-12   # FP64 path vs the oracle, relative to the largest entry
TOL_MIXED = 2e-5   # FP32 element arithmetic with FP64 sums, relative to the largest entry
TOL_SOLUTION = 1e-10


def rel(a, ref):
    return float(np.abs(a - ref).max() / np.abs(ref).max())


def numbering_and_graph_equal(w, o):
    dof = w.dof
    assert dof.n_dofs == o.n_dofs and dof.nnz == o.nnz
    assert np.array_equal(dof.getOwnedIndices(), o.owned_gids())
    for b in range(o.n_blocks):
        assert np.array_equal(dof.getElementGIDs(b), o.element_gids(b)), b
        assert np.array_equal(dof.getElementLIDs(b), o.element_lids(b)), b
        for f in range(o.n_fields):
            assert np.array_equal(dof.getGIDFieldOffsets(b, f), o.field_offsets(b, f))
    rp, ci = o.graph()
    assert np.array_equal(w.lof.rowptr.cpu().numpy(), rp)
    assert np.array_equal(w.lof.colind.cpu().numpy(), ci)


# ------------------------------------------------------------ elasticity 128^3
@pytest.fixture(scope="module")
def c2(cuda):
    w = WL.elasticity_hex8(128)
    o = O.Oracle(w.mesh_desc, w.eqset)
    yield w, o
    del o


def test_elasticity_128_numbering_graph_dirichlet_bit_exact(c2):
    w, o = c2
    assert o.n_elements == 128 ** 3 and o.nnz == 9 * (3 * 128 + 1) ** 3
    numbering_and_graph_equal(w, o)
    assert np.array_equal(w.dof.dirichletDofs(A.SIDE_ZMIN), o.dirichlet_dofs(A.SIDE_ZMIN))


def test_elasticity_128_residual_jacobian_against_oracle(c2):
    w, o = c2
    x_h = np.random.default_rng(7).uniform(-1e-3, 1e-3, o.n_dofs)
    bd = o.dirichlet_dofs(A.SIDE_ZMIN)
    x_h[bd] = 0.0
    f_ref, v_ref = o.evaluate(x_h, threads=THREADS)
    o.dirichlet_apply(bd, np.zeros(len(bd)), x_h, f_ref, v_ref)
    x = torch.from_numpy(x_h).cuda()
    f, W = w.lof.getTpetraVector(), w.me.create_W_op()
    # FP64 and mixed atomic forms, the mixed owner-computes lattice form (deterministic evaluations take
    # the gather form, which on this lattice is k_lattice_gather) and the tensor-core contractions
    assert w.me.ae.gather_form() == "lattice"
    for mixed, det, variant, tol in ((False, False, 0, TOL_FP64), (True, False, 0, TOL_MIXED),
                                     (True, True, 0, TOL_MIXED), (True, False, 3, TOL_MIXED)):
        w.me.ae.setVariant(variant)
        w.me.evalModel(x, f=f, W=W, mixed=mixed, deterministic=det)
        tx.synchronize(w.dof)
        ef = rel(f.cpu().numpy(), f_ref)
        ew = rel(W.values.cpu().numpy(), v_ref)
        assert ef <= tol and ew <= tol, (mixed, det, variant, ef, ew)
    w.me.ae.setVariant(0)


def test_elasticity_128_converged_solution_oracle_residual(c2):
    w, o = c2
    f, W = w.lof.getTpetraVector(), w.me.create_W_op()
    x = w.lof.getTpetraVector()
    w.me.evalModel(x, f=f, W=W, mixed=True)
    st = w.me.solve(W, x, rtol=1e-11, inner_rtol=1e-5, matrix_free=True, max_outer=40, block_jacobi=True)
    assert st["relres"] <= 1e-11, st
    x_h = x.cpu().numpy()
    bd = o.dirichlet_dofs(A.SIDE_ZMIN)
    z = np.zeros(o.n_dofs)
    f0, _ = o.evaluate(z, jacobian=False, threads=THREADS)
    o.dirichlet_apply(bd, np.zeros(len(bd)), z, f0)
    fx, _ = o.evaluate(x_h, jacobian=False, threads=THREADS)
    o.dirichlet_apply(bd, np.zeros(len(bd)), x_h, fx)
    relres = float(np.linalg.norm(fx) / np.linalg.norm(f0))
    assert relres <= TOL_SOLUTION, relres


# ------------------------------------------------------ heat hex27 + tet10 48^3
def test_heat_hex27_tet10_48_against_oracle(cuda):
    w = WL.heat_hex27_tet10(48)
    o = O.Oracle(w.mesh_desc, w.eqset)
    assert o.n_dofs == 2 * 97 ** 3 - 97 ** 2
    numbering_and_graph_equal(w, o)
    T_h = np.random.default_rng(2).uniform(0.0, 1.0, o.n_dofs)
    f_ref, v_ref = o.evaluate(T_h, threads=THREADS)
    T = torch.from_numpy(T_h).cuda()
    ae = AssemblyEngine(w.lof)
    ae.setWorksetSize(256, 1024, seed=11)
    f, W = w.lof.getTpetraVector(), w.lof.getTpetraMatrix()
    for mixed, tol in ((False, TOL_FP64), (True, TOL_MIXED)):
        f.zero_()
        W.initializeMatrix(0.0)
        ae.evaluate(T, f=f, W=W, mixed=mixed, persistent=True)
        ef = rel(f.cpu().numpy(), f_ref)
        ew = rel(W.values.cpu().numpy(), v_ref)
        assert ef <= tol and ew <= tol, (mixed, ef, ew)


# ------------------------------------------------- Newmark elastodynamics 96^3
def test_elastodynamics_96_ten_steps_against_oracle_newmark(cuda):
    dt, beta, gamma = 1e-3, 0.25, 0.5
    c = 1.0 / (beta * dt * dt)
    w = WL.elastodynamics_hex8(96)
    o = O.Oracle(w.mesh_desc, w.eqset)
    n = o.n_dofs
    u0 = np.random.default_rng(4).normal(0.0, 1e-3, n)

    # oracle: K, M and F in FP64; M a + K u = F stepped with the same Newmark scheme
    z = np.zeros(n)
    f0, kv = o.evaluate(z, z, alpha=0.0, beta=1.0, threads=THREADS)
    _, mv = o.evaluate(z, z, alpha=1.0, beta=0.0, residual=False, threads=THREADS)
    rp, ci = o.graph()
    F = -f0
    keff = kv + c * mv
    del f0
    a, _, rr = O.cg(rp, ci, mv, F - O.spmv(rp, ci, kv, u0), rtol=1e-13)
    assert rr <= 1e-12
    u, v = u0.copy(), np.zeros(n)
    for _ in range(10):
        up = u + dt * v + dt * dt * (0.5 - beta) * a
        vp = v + dt * (1.0 - gamma) * a
        u, _, rr = O.cg(rp, ci, keff, F + c * O.spmv(rp, ci, mv, up), x0=up, rtol=1e-13)
        assert rr <= 1e-12
        a = c * (u - up)
        v = vp + gamma * dt * a
    del kv, mv, keff, rp, ci

    nm = NewmarkElastodynamics(w.me, dt, beta, gamma, mixed=True, outer=3, inner=24)
    nm.initialize(torch.from_numpy(u0).cuda())
    nm.capture()
    worst = 0.0
    for _ in range(10):
        worst = max(worst, float(nm.step()[2]))
    torch.cuda.synchronize()
    assert worst <= TOL_SOLUTION, worst
    err = rel(nm.u.cpu().numpy(), u)
    assert err <= TOL_SOLUTION, err


# ------------------------------------------------------------ 256-mesh batch
def test_mixed_batch_256_every_instance_against_oracle(cuda):
    ws = WL.mixed_batch(256)
    assert [w.name for w in ws] == [k for k, _ in WL.batch_plan(256)]
    rng = np.random.default_rng(5)
    xs_h = [rng.uniform(-1.0, 1.0, w.dof.n_dofs) for w in ws]
    xs = [torch.from_numpy(x).cuda() for x in xs_h]
    auxs = [w.extras.get("J") for w in ws]
    out = {}
    batch = Batch([w.dof for w in ws], workset=(512, 512))
    for mixed in (False, True):
        fs = [w.lof.getTpetraVector() for w in ws]
        Ws = [w.lof.getTpetraMatrix() for w in ws]
        batch.evaluate(xs, fs, Ws, auxs=auxs, mixed=mixed)
        torch.cuda.synchronize()
        out[mixed] = [(f.cpu().numpy(), W.values.cpu().numpy()) for f, W in zip(fs, Ws)]
        del fs, Ws
    worst = {False: 0.0, True: 0.0}
    for i, w in enumerate(ws):
        o = O.Oracle(w.mesh_desc, w.eqset)
        J = auxs[i]
        f_ref, v_ref = o.evaluate(xs_h[i], aux=None if J is None else J.cpu().numpy(), threads=THREADS)
        for mixed, tol in ((False, TOL_FP64), (True, TOL_MIXED)):
            f, v = out[mixed][i]
            e = max(rel(f, f_ref), rel(v, v_ref))
            worst[mixed] = max(worst[mixed], e)
            assert e <= tol, (i, w.name, mixed, e)
        del o
    assert worst[False] <= TOL_FP64 and worst[True] <= TOL_MIXED, worst
