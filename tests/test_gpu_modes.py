"""Deterministic (coloured), persistent (one-launch worksets) and batched
(many meshes, one launch) evaluation against the oracle on the GPU."""
import numpy as np
import pytest
import torch

import tianxin_gb300 as tx
from oracle import oracle as O
from tianxin_gb300 import _abi as A

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_TOL = 2e-5

PARAMS = {
    A.TX_PHYS_POISSON: (1.0, 0.5, 1.0, 2.0),
    A.TX_PHYS_ELASTICITY: (1.0, 0.3, 0.1, -0.2, -1.0, 0.7),
    A.TX_PHYS_HEAT: (1.0, 0.5, 1.0),
    A.TX_PHYS_MAXWELL: (1.0, 1.0),
}


def build(n, blocks, topo, phys, basis, source=0, jitter=0.1, seed=5):
    m = A.mesh_desc(n, blocks, topo, jitter=jitter, seed=seed)
    q = A.equation_set(phys, basis, params=PARAMS[phys], source_kind=source)
    o = O.Oracle(m, q)
    conn = tx.CartesianConnManager(*n, *blocks, topology=topo, jitter=jitter, seed=seed)
    dof = tx.DOFManager(conn, q)
    lof = tx.TpetraLinearObjFactory(dof)
    return o, dof, lof


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def run(dof, lof, x, xd, aux, mixed=False, **kw):
    dev = lambda a: torch.from_numpy(a).cuda()
    f = lof.getTpetraVector()
    W = lof.getTpetraMatrix()
    tx.AssemblyEngine(lof).evaluate(dev(x), dev(xd), dev(aux), 0.5, 1.0, 0.0, f, W, mixed, **kw)
    torch.cuda.synchronize()
    return f.cpu().numpy(), W.values.cpu().numpy()


@pytest.mark.parametrize("topo,phys,basis", [(A.TX_TOPO_HEX, A.TX_PHYS_ELASTICITY, A.TX_HGRAD_C1),
                                             (A.TX_TOPO_TET, A.TX_PHYS_POISSON, A.TX_HGRAD_C1),
                                             (A.TX_TOPO_TET, A.TX_PHYS_HEAT, A.TX_HGRAD_C2)])
def test_deterministic_is_bitwise_reproducible(cuda, topo, phys, basis):
    o, dof, lof = build((4, 3, 3), (1, 1, 1), topo, phys, basis)
    rng = np.random.default_rng(1)
    x, xd, aux = rng.uniform(-1, 1, o.n_dofs), rng.uniform(-1, 1, o.n_dofs), rng.standard_normal(o.n_dofs)
    f1, v1 = run(dof, lof, x, xd, aux, deterministic=True)
    f2, v2 = run(dof, lof, x, xd, aux, deterministic=True)
    assert np.array_equal(f1, f2) and np.array_equal(v1, v2)
    f_ref, v_ref = o.evaluate(x, xd, aux, alpha=0.5, beta=1.0)
    assert rel(f1, f_ref) <= FP64_TOL and rel(v1, v_ref) <= FP64_TOL


@pytest.mark.parametrize("mixed", [False, True])
def test_persistent_mixed_families_uneven_worksets(cuda, mixed):
    # hex27 + tet10 blocks, worksets of 5..17 elements, one launch
    o, dof, lof = build((2, 3, 2), (2, 1, 1), [A.TX_TOPO_HEX, A.TX_TOPO_TET], A.TX_PHYS_HEAT, A.TX_HGRAD_C2)
    rng = np.random.default_rng(2)
    x, xd, aux = rng.uniform(0, 1, o.n_dofs), np.zeros(o.n_dofs), np.zeros(o.n_dofs)
    ae = tx.AssemblyEngine(lof)
    ae.setWorksetSize(5, 17, seed=3)
    f, v = run(dof, lof, x, xd, aux, mixed=mixed, persistent=True)
    f_ref, v_ref = o.evaluate(x, xd, aux, alpha=0.5, beta=1.0)
    tol = MIXED_TOL if mixed else FP64_TOL
    assert rel(f, f_ref) <= tol and rel(v, v_ref) <= tol


def test_batch_of_meshes_one_launch(cuda):
    cases = [((3, 2, 2), A.TX_TOPO_HEX, A.TX_PHYS_POISSON, A.TX_HGRAD_C1),
             ((2, 2, 3), A.TX_TOPO_TET, A.TX_PHYS_ELASTICITY, A.TX_HGRAD_C1),
             ((2, 3, 2), A.TX_TOPO_HEX, A.TX_PHYS_MAXWELL, A.TX_HCURL_I1),
             ((4, 4, 4), A.TX_TOPO_HEX, A.TX_PHYS_POISSON, A.TX_HGRAD_C1)]
    rng = np.random.default_rng(4)
    built, xs, xds, auxs, fs, Ws, refs = [], [], [], [], [], [], []
    for i, (n, topo, phys, basis) in enumerate(cases):
        o, dof, lof = build(n, (1, 1, 1), topo, phys, basis, seed=10 + i)
        x, xd, aux = rng.uniform(-1, 1, o.n_dofs), rng.uniform(-1, 1, o.n_dofs), rng.standard_normal(o.n_dofs)
        built.append((o, dof, lof))
        xs.append(torch.from_numpy(x).cuda())
        xds.append(torch.from_numpy(xd).cuda())
        auxs.append(torch.from_numpy(aux).cuda())
        fs.append(lof.getTpetraVector())
        Ws.append(lof.getTpetraMatrix())
        refs.append(o.evaluate(x, xd, aux, alpha=0.5, beta=1.0))
    batch = tx.Batch([b[1] for b in built], workset=(3, 11), seed=9)
    batch.evaluate(xs, fs, Ws, xds, auxs, alpha=0.5, beta=1.0)
    torch.cuda.synchronize()
    for i, (f_ref, v_ref) in enumerate(refs):
        assert rel(fs[i].cpu().numpy(), f_ref) <= FP64_TOL, i
        assert rel(Ws[i].values.cpu().numpy(), v_ref) <= FP64_TOL, i


@pytest.mark.parametrize("jitter", [0.0, 0.2])
def test_warp_per_element_kernel_matches_cta_kernel_and_oracle(cuda, jitter):
    # TX_VARIANT_WARP (hex8 elasticity, mixed) against the CTA-staged kernel and
    # the FP64 oracle, with a time-derivative vector (alpha mass term) and the
    # residual-only form; several blocks and uneven block sizes.
    o, dof, lof = build((5, 4, 3), (2, 1, 2), A.TX_TOPO_HEX, A.TX_PHYS_ELASTICITY, A.TX_HGRAD_C1, jitter=jitter)
    rng = np.random.default_rng(9)
    x, xd, aux = (rng.uniform(-0.2, 0.2, o.n_dofs) for _ in range(3))
    f_ref, v_ref = o.evaluate(x, xd, alpha=0.5, beta=1.0)
    ae = tx.AssemblyEngine(lof)
    out = {}
    for variant in (1, 2):
        ae.setVariant(variant)
        out[variant] = run(dof, lof, x, xd, aux, mixed=True)
        assert rel(out[variant][0], f_ref) <= MIXED_TOL
        assert rel(out[variant][1], v_ref) <= MIXED_TOL
        # residual-only evaluation
        f = lof.getTpetraVector()
        dev = lambda a: torch.from_numpy(a).cuda()
        ae.evaluate(dev(x), dev(xd), None, 0.5, 1.0, 0.0, f, None, True)
        assert rel(f.cpu().numpy(), f_ref) <= MIXED_TOL
    assert rel(out[2][1], out[1][1]) <= 1e-5
    ae.setVariant(0)


def test_warp_and_tensor_variants_fall_back_where_no_such_kernel(cuda):
    o, dof, lof = build((3, 3, 3), (1, 1, 1), A.TX_TOPO_TET, A.TX_PHYS_POISSON, A.TX_HGRAD_C1)
    rng = np.random.default_rng(1)
    x, xd, aux = (rng.uniform(-1, 1, o.n_dofs) for _ in range(3))
    ae = tx.AssemblyEngine(lof)
    ae.setVariant(2)
    f2, v2 = run(dof, lof, x, xd, aux, mixed=True)
    ae.setVariant(1)
    f1, v1 = run(dof, lof, x, xd, aux, mixed=True)
    assert rel(v2, v1) <= 1e-6 and rel(f2, f1) <= 1e-6
    ae.setVariant(3)  # no tensor-core kernel for tet Poisson either: the CTA-staged kernel
    f3, v3 = run(dof, lof, x, xd, aux, mixed=True)
    assert rel(v3, v1) <= 1e-6 and rel(f3, f1) <= 1e-6
    with pytest.raises(tx.TxError):
        ae.setVariant(4)


# ------------------------------------------------------------ two-phase (gather) evaluation
@pytest.mark.parametrize("topo,phys,basis,blocks", [
    (A.TX_TOPO_HEX, A.TX_PHYS_ELASTICITY, A.TX_HGRAD_C1, (1, 1, 1)),
    (A.TX_TOPO_TET, A.TX_PHYS_ELASTICITY, A.TX_HGRAD_C1, (1, 1, 1)),
    ([A.TX_TOPO_HEX, A.TX_TOPO_TET], A.TX_PHYS_HEAT, A.TX_HGRAD_C2, (2, 1, 1)),
    (A.TX_TOPO_HEX, A.TX_PHYS_POISSON, A.TX_HGRAD_C1, (1, 1, 2)),
    (A.TX_TOPO_HEX, A.TX_PHYS_MAXWELL, A.TX_HCURL_I1, (1, 1, 1)),
])
def test_gather_overwrites_and_matches_oracle(cuda, topo, phys, basis, blocks):
    # f and W start as NaN: the two-phase form writes every entry; the sums have a fixed order, so
    # two evaluations give the same bits
    o, dof, lof = build((3, 3, 2), blocks, topo, phys, basis)
    rng = np.random.default_rng(5)
    x, xd, aux = rng.uniform(-1, 1, o.n_dofs), rng.uniform(-1, 1, o.n_dofs), rng.standard_normal(o.n_dofs)
    f_ref, v_ref = o.evaluate(x, xd, aux, alpha=0.5, beta=1.0)
    dev = lambda a: torch.from_numpy(a).cuda()
    for mixed, tol in ((False, FP64_TOL), (True, MIXED_TOL)):
        outs = []
        for _ in range(2):
            f = torch.full((o.n_dofs,), float("nan"), dtype=torch.float64, device="cuda")
            W = lof.getTpetraMatrix()
            W.values.fill_(float("nan"))
            tx.AssemblyEngine(lof).evaluate(dev(x), dev(xd), dev(aux), 0.5, 1.0, 0.0, f, W, mixed, gather=True)
            outs.append((f.cpu().numpy(), W.values.cpu().numpy()))
        (f1, v1), (f2, v2) = outs
        assert np.array_equal(f1, f2) and np.array_equal(v1, v2)
        assert rel(f1, f_ref) <= tol and rel(v1, v_ref) <= tol, (mixed, rel(f1, f_ref), rel(v1, v_ref))


def test_gather_in_the_model_evaluator_and_its_limits(cuda):
    o, dof, lof = build((4, 3, 3), (1, 1, 1), A.TX_TOPO_HEX, A.TX_PHYS_ELASTICITY, A.TX_HGRAD_C1)
    me = tx.ModelEvaluator(lof, [tx.DirichletBC(dof, A.SIDE_ZMIN)])
    x = torch.from_numpy(np.random.default_rng(2).uniform(-1, 1, o.n_dofs)).cuda()
    res = []
    for gather in (False, True):
        me.ae.gather = gather
        f, W = lof.getTpetraVector(), me.create_W_op()
        f.fill_(7.0)
        W.values.fill_(7.0)
        me.evalModel(x, f=f, W=W)  # zeroes first only in the atomic form
        res.append((f.cpu().numpy(), W.values.cpu().numpy()))
    assert rel(res[1][0], res[0][0]) <= 1e-13 and rel(res[1][1], res[0][1]) <= 1e-13
    ae = tx.AssemblyEngine(lof)
    f, W = lof.getTpetraVector(), lof.getTpetraMatrix()
    for kw in (dict(block=0), dict(deterministic=True)):
        with pytest.raises(tx.TxError):
            ae.evaluate(x, f=f, W=W, gather=True, **kw)
    with pytest.raises(tx.TxError):
        ae.evaluate(x, f=f, W=None, gather=True)


@pytest.mark.parametrize("topo,phys,basis,shapes", [(A.TX_TOPO_HEX, A.TX_PHYS_ELASTICITY, A.TX_HGRAD_C1, (64, 256)),
                                                    (A.TX_TOPO_HEX, A.TX_PHYS_HEAT, A.TX_HGRAD_C2, (64,)),
                                                    (A.TX_TOPO_TET, A.TX_PHYS_HEAT, A.TX_HGRAD_C2, (64, 256))])
def test_cta_tile_shapes_against_oracle(cuda, topo, phys, basis, shapes):
    # the staged kernel at 64 and 256 threads a CTA (half and twice the elements a CTA) gives the oracle's
    # values in both precisions; shapes whose FP64 tables do not fit a CTA (hex27 at 256) and others are refused
    o, dof, lof = build((5, 4, 3), (1, 1, 1), topo, phys, basis)
    rng = np.random.default_rng(4)
    x, xd, aux = rng.uniform(-1, 1, o.n_dofs), rng.uniform(-1, 1, o.n_dofs), rng.standard_normal(o.n_dofs)
    f_ref, v_ref = o.evaluate(x, xd, aux, alpha=0.5, beta=1.0)
    ae = tx.AssemblyEngine(lof)
    for threads in (64, 256):
        if threads not in shapes:
            with pytest.raises(tx.TxError):
                ae.setCtaThreads(threads)
            continue
        ae.setCtaThreads(threads)
        for mixed, tol in ((False, FP64_TOL), (True, MIXED_TOL)):
            f, v = run(dof, lof, x, xd, aux, mixed=mixed)
            assert rel(f, f_ref) <= tol and rel(v, v_ref) <= tol, (threads, mixed)
    ae.setCtaThreads(0)
    with pytest.raises(tx.TxError):
        ae.setCtaThreads(96)


def test_cta_tile_shape_refused_without_a_family(cuda):
    o, dof, lof = build((2, 2, 2), (1, 1, 1), A.TX_TOPO_TET, A.TX_PHYS_POISSON, A.TX_HGRAD_C1)
    with pytest.raises(tx.TxError):
        tx.AssemblyEngine(lof).setCtaThreads(64)
