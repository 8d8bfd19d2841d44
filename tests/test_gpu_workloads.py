"""The named workloads at full size on the GPU.

Where the oracle is too slow at full size, size-independent properties stand
in (symmetry, rigid-body modes, linearity, reproducibility, agreement of the
persistent / batched launches with the per-block path, which the oracle pins
at small sizes in test_gpu_assembly.py).
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tianxin_gb300 import _abi as A
from tianxin_gb300 import workloads as WL
from tianxin_gb300.newmark import NewmarkElastodynamics
from tianxin_gb300.panzer import AssemblyEngine, Batch

pytestmark = pytest.mark.gpu


def trel(a, b):
    return float((a - b).abs().max() / b.abs().max())


def test_poisson_hex8_16_against_oracle(cuda):
    w = WL.poisson_hex8(16)
    o = O.Oracle(w.mesh_desc, w.eqset)
    x_h = np.random.default_rng(0).uniform(-1, 1, o.n_dofs)
    x = torch.from_numpy(x_h).cuda()
    f, W = w.lof.getTpetraVector(), w.me.create_W_op()
    w.me.evalModel(x, f=f, W=W)
    f_ref, v_ref = o.evaluate(x_h)
    bd = o.dirichlet_dofs(A.ALL_SIDES)
    o.dirichlet_apply(bd, np.zeros(len(bd)), x_h, f_ref, v_ref)
    assert np.abs(f.cpu().numpy() - f_ref).max() <= 1e-12 * np.abs(f_ref).max()
    assert np.abs(W.values.cpu().numpy() - v_ref).max() <= 1e-12 * np.abs(v_ref).max()


@pytest.fixture(scope="module")
def elasticity128(cuda):
    return WL.elasticity_hex8(128)


def test_elasticity_128_properties(elasticity128):
    w = elasticity128
    N = w.dof.n_dofs
    g = torch.Generator(device="cuda").manual_seed(1)
    x = (torch.rand(N, dtype=torch.float64, device="cuda", generator=g) * 2 - 1) * 1e-3
    ae = AssemblyEngine(w.lof)
    f, f0 = w.lof.getTpetraVector(), w.lof.getTpetraVector()
    W = w.lof.getTpetraMatrix()
    ae.evaluate(x, f=f, W=W)                       # FP64, no Dirichlet rows
    ae.evaluate(torch.zeros_like(x), f=f0)
    # linearity: f(x) - f(0) = A x
    Ax = W.apply(x)
    assert trel(f - f0, Ax) <= 1e-12
    # symmetry: y.(A z) = z.(A y)
    y = torch.rand(N, dtype=torch.float64, device="cuda", generator=g)
    z = torch.rand(N, dtype=torch.float64, device="cuda", generator=g)
    a1, a2 = float(y @ W.apply(z)), float(z @ W.apply(y))
    assert abs(a1 - a2) <= 1e-12 * abs(a1)
    # rigid translations are in the kernel of K
    for c in range(3):
        t = torch.zeros(N, dtype=torch.float64, device="cuda")
        t[c::3] = 1.0
        assert float(W.apply(t).abs().max()) <= 1e-12 * float(W.values.abs().max())
    # mixed Jacobian: FP32 element contractions, stated error
    Wm = w.lof.getTpetraMatrix()
    fm = w.lof.getTpetraVector()
    ae.evaluate(x, f=fm, W=Wm, mixed=True)
    assert trel(Wm.values, W.values) <= 2e-5
    assert trel(fm, f) <= 2e-5


def test_elasticity_128_deterministic_scatter(elasticity128):
    w = elasticity128
    N = w.dof.n_dofs
    x = torch.full((N,), 1e-3, dtype=torch.float64, device="cuda")
    ae = AssemblyEngine(w.lof)
    f1, f2, fa = (w.lof.getTpetraVector() for _ in range(3))
    W1, W2, Wa = (w.lof.getTpetraMatrix() for _ in range(3))
    ae.evaluate(x, f=f1, W=W1, mixed=True, deterministic=True)
    ae.evaluate(x, f=f2, W=W2, mixed=True, deterministic=True)
    ae.evaluate(x, f=fa, W=Wa, mixed=True)
    assert torch.equal(W1.values, W2.values) and torch.equal(f1, f2)
    assert trel(W1.values, Wa.values) <= 1e-12


def test_heat_hex27_tet10_48_persistent_uneven_worksets(cuda):
    w = WL.heat_hex27_tet10(48)
    assert w.dof.n_dofs == 2 * 97 ** 3 - 97 ** 2
    N = w.dof.n_dofs
    g = torch.Generator(device="cuda").manual_seed(2)
    T = torch.rand(N, dtype=torch.float64, device="cuda", generator=g)
    ae = AssemblyEngine(w.lof)
    ae.setWorksetSize(256, 1024, seed=11)
    f_ref, W_ref = w.lof.getTpetraVector(), w.lof.getTpetraMatrix()
    ae.evaluate(T, f=f_ref, W=W_ref)                # per-block launches, FP64
    for mixed, tol in ((False, 1e-12), (True, 2e-5)):
        f, W = w.lof.getTpetraVector(), w.lof.getTpetraMatrix()
        ae.evaluate(T, f=f, W=W, mixed=mixed, persistent=True)
        assert trel(f, f_ref) <= tol and trel(W.values, W_ref.values) <= tol


def test_heat_hex27_tet10_small_against_oracle(cuda):
    w = WL.heat_hex27_tet10(3)
    o = O.Oracle(w.mesh_desc, w.eqset)
    T = np.random.default_rng(3).uniform(0, 1, o.n_dofs)
    ae = AssemblyEngine(w.lof)
    ae.setWorksetSize(4, 13, seed=1)
    f, W = w.lof.getTpetraVector(), w.lof.getTpetraMatrix()
    ae.evaluate(torch.from_numpy(T).cuda(), f=f, W=W, persistent=True)
    f_ref, v_ref = o.evaluate(T)
    assert np.abs(f.cpu().numpy() - f_ref).max() <= 1e-12 * np.abs(f_ref).max()
    assert np.abs(W.values.cpu().numpy() - v_ref).max() <= 1e-12 * np.abs(v_ref).max()


def test_elastodynamics_96_graph_steps(cuda):
    w = WL.elastodynamics_hex8(96)
    g = torch.Generator(device="cuda").manual_seed(4)
    u0 = torch.randn(w.dof.n_dofs, dtype=torch.float64, device="cuda", generator=g) * 1e-3
    nm = NewmarkElastodynamics(w.me, 1e-3, 0.25, 0.5, mixed=True, outer=3, inner=24)
    nm.initialize(u0)
    nm.capture()
    worst = 0.0
    for _ in range(10):
        worst = max(worst, float(nm.step()[2]))
    assert worst <= 1e-10, worst
    assert torch.isfinite(nm.u).all()


def test_mixed_batch_256_one_launch(cuda):
    ws = WL.mixed_batch(256)
    assert len(ws) == 256
    g = torch.Generator(device="cuda").manual_seed(5)
    xs = [(torch.rand(w.dof.n_dofs, dtype=torch.float64, device="cuda", generator=g) * 2 - 1) for w in ws]
    auxs = [w.extras.get("J") for w in ws]
    for mixed, tol in ((False, 1e-12), (True, 2e-5)):
        fs = [w.lof.getTpetraVector() for w in ws]
        Ws = [w.lof.getTpetraMatrix() for w in ws]
        Batch([w.dof for w in ws], workset=(512, 512)).evaluate(xs, fs, Ws, auxs=auxs, mixed=mixed)
        for i, w in enumerate(ws):
            f_ref, W_ref = w.lof.getTpetraVector(), w.lof.getTpetraMatrix()
            AssemblyEngine(w.lof).evaluate(xs[i], aux=auxs[i], f=f_ref, W=W_ref)
            assert trel(fs[i], f_ref) <= tol, (i, w.name)
            assert trel(Ws[i].values, W_ref.values) <= tol, (i, w.name)


def test_mixed_batch_small_instances_against_oracle(cuda):
    plan = [p for p in WL.batch_plan(256) if p[1] <= 8][:6]
    for i, (kind, n) in enumerate(plan):
        w = WL.batch_instance(kind, n, 77 + i)
        o = O.Oracle(w.mesh_desc, w.eqset)
        x_h = np.random.default_rng(i).uniform(-1, 1, o.n_dofs)
        J = w.extras.get("J")
        f, W = w.lof.getTpetraVector(), w.lof.getTpetraMatrix()
        Batch([w.dof]).evaluate([torch.from_numpy(x_h).cuda()], [f], [W], auxs=[J])
        f_ref, v_ref = o.evaluate(x_h, aux=None if J is None else J.cpu().numpy())
        assert np.abs(f.cpu().numpy() - f_ref).max() <= 1e-12 * np.abs(f_ref).max(), kind
        assert np.abs(W.values.cpu().numpy() - v_ref).max() <= 1e-12 * np.abs(v_ref).max(), kind
