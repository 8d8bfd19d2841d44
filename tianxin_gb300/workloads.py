"""The synthetic workloads of the assembly path, by name.

  poisson_hex8        -lap u = 3 pi^2 sin sin sin on the unit cube, hex8 Q1, n^3 bricks,
                      interior vertices jittered +-0.1h, homogeneous Dirichlet, 2x2x2 Gauss
  elasticity_hex8     linear elasticity, E=1 nu=0.3, b=(0,0,-1), clamped z=0, jitter 0.05h
  heat_hex27_tet10    k(T)=1+0.5T^2 heat, block A hex27 Q2 (27-point Gauss) on [0,1]^3,
                      block B hex split into 6 tet10 P2 (4-point rule) on [1,2]x[0,1]^2,
                      conforming interface, q=1
  elastodynamics_hex8 rho=1 E=1 nu=0.25, Newmark beta=1/4 gamma=1/2, dt=1e-3
  mixed_batch         many independent meshes, element counts log-uniform in [6^3, 40^3],
                      each Poisson hex8, elasticity tet4 (6 per brick) or curl-curl Maxwell
                      on lowest-order Nedelec hexes (sigma=1, J ~ N(0,1) per edge)

Inputs are seeded synthetic data (no dataset is involved).
"""
import math

import numpy as np
import torch

from . import _abi as A
from .panzer import CartesianConnManager, DirichletBC, DOFManager, ModelEvaluator, TpetraLinearObjFactory


class Workload:
    def __init__(self, name, conn, dof, lof, me, mesh_desc, eqset, extras=None):
        self.name, self.conn, self.dof, self.lof, self.me = name, conn, dof, lof, me
        self.mesh_desc, self.eqset = mesh_desc, eqset
        self.extras = extras or {}

    @property
    def n_elements(self):
        return self.conn.n_elements


def _make(name, n, blocks, topo, eqset, jitter, seed, lengths=(1.0, 1.0, 1.0), dirichlet=()):
    m = A.mesh_desc(n, blocks, topo, lengths, jitter, seed)
    conn = CartesianConnManager(*(n if isinstance(n, tuple) else (n, n, n)), *blocks, topology=topo, lengths=lengths,
                                jitter=jitter, seed=seed)
    dof = DOFManager(conn, eqset)
    lof = TpetraLinearObjFactory(dof)
    me = ModelEvaluator(lof, [DirichletBC(dof, sides, fields) for sides, fields in dirichlet])
    return Workload(name, conn, dof, lof, me, m, eqset)


def poisson_hex8(n=16, seed=1):
    q = A.equation_set(A.TX_PHYS_POISSON, params=(1.0, 0.0, 0.0, 0.0), source_kind=A.TX_SOURCE_SINE)
    return _make("poisson_hex8", n, (1, 1, 1), A.TX_TOPO_HEX, q, 0.1, seed, dirichlet=[(A.ALL_SIDES, None)])


def elasticity_hex8(n=128, seed=2024):
    q = A.equation_set(A.TX_PHYS_ELASTICITY, params=(1.0, 0.3, 0.0, 0.0, -1.0, 0.0))
    return _make("elasticity_hex8", n, (1, 1, 1), A.TX_TOPO_HEX, q, 0.05, seed, dirichlet=[(A.SIDE_ZMIN, None)])


def heat_hex27_tet10(n=48, seed=3):
    q = A.equation_set(A.TX_PHYS_HEAT, A.TX_HGRAD_C2, params=(1.0, 0.5, 1.0), integration_order=[4, 2])
    return _make("heat_hex27_tet10", (n, n, n), (2, 1, 1), [A.TX_TOPO_HEX, A.TX_TOPO_TET], q, 0.0, seed,
                 lengths=(2.0, 1.0, 1.0))


def elastodynamics_hex8(n=96, seed=4):
    q = A.equation_set(A.TX_PHYS_ELASTICITY, params=(1.0, 0.25, 0.0, 0.0, 0.0, 1.0))
    return _make("elastodynamics_hex8", n, (1, 1, 1), A.TX_TOPO_HEX, q, 0.0, seed)


def batch_plan(count=256, seed=5, lo=6 ** 3, hi=40 ** 3):
    """(kind, n) per instance: n = round(N^(1/3)), N log-uniform in [lo, hi]."""
    rng = np.random.default_rng(seed)
    kinds = ["poisson_hex8", "elasticity_tet4", "maxwell_nedelec"]
    out = []
    for _ in range(count):
        N = math.exp(rng.uniform(math.log(lo), math.log(hi)))
        out.append((kinds[int(rng.integers(0, 3))], max(1, int(round(N ** (1.0 / 3.0))))))
    return out


def batch_instance(kind, n, seed):
    if kind == "poisson_hex8":
        q = A.equation_set(A.TX_PHYS_POISSON, params=(1.0, 0.0, 0.0, 0.0), source_kind=A.TX_SOURCE_SINE)
        return _make(kind, n, (1, 1, 1), A.TX_TOPO_HEX, q, 0.1, seed, dirichlet=[(A.ALL_SIDES, None)])
    if kind == "elasticity_tet4":
        q = A.equation_set(A.TX_PHYS_ELASTICITY, params=(1.0, 0.3, 0.0, 0.0, -1.0, 0.0))
        return _make(kind, n, (1, 1, 1), A.TX_TOPO_TET, q, 0.1, seed, dirichlet=[(A.SIDE_ZMIN, None)])
    q = A.equation_set(A.TX_PHYS_MAXWELL, A.TX_HCURL_I1, params=(1.0, 1.0))
    w = _make(kind, n, (1, 1, 1), A.TX_TOPO_HEX, q, 0.1, seed)
    g = torch.Generator(device="cuda").manual_seed(seed)
    w.extras["J"] = torch.randn(w.dof.n_dofs, dtype=torch.float64, device="cuda", generator=g)
    return w


def mixed_batch(count=256, seed=5):
    return [batch_instance(k, n, seed * 1000 + i) for i, (k, n) in enumerate(batch_plan(count, seed))]


# ---------------------------------------------------------------- timing
def _events():
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def time_eval(ae, x, f, W, reps=5, **kw):
    """Mean ms of one R+J evaluation (f, W zeroed inside the timed region)."""
    for _ in range(2):
        f.zero_(); W.initializeMatrix(0.0); ae.evaluate(x, f=f, W=W, **kw)
    torch.cuda.synchronize()
    s, e = _events()
    s.record()
    for _ in range(reps):
        f.zero_(); W.initializeMatrix(0.0); ae.evaluate(x, f=f, W=W, **kw)
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / reps


def assembly_bytes(n_vertices, n_dofs, nnz, conn_entries):
    """Algorithmic bytes of one residual + Jacobian evaluation: vertex coordinates, x, element connectivity
    (DOF entities of every element), f written, CRS values written, column indices and rowptr read."""
    return 24 * n_vertices + 8 * n_dofs + 4 * conn_entries + 8 * n_dofs + 12 * nnz + 8 * (n_dofs + 1)


def _lattice_vertices(w):
    d = w.mesh_desc
    return (d.nx * d.bx + 1) * (d.ny * d.by + 1) * (d.nz * d.bz + 1)


def _conn_entries(w):
    return sum(len(w.conn.getElementBlock(b)) * w.dof.getElementBlockGIDCount(b) // w.dof.n_fields
               for b in range(w.conn.n_blocks))


def _time_kernel(fn, prep, reps):
    """Mean ms of fn() with CUDA events around each call only (prep() runs outside the events)."""
    for _ in range(2):
        prep()
        fn()
    torch.cuda.synchronize()
    total = 0.0
    for _ in range(reps):
        prep()
        s, e = _events()
        s.record()
        fn()
        e.record()
        e.synchronize()
        total += s.elapsed_time(e)
    return total / reps


def _assembly_legs(w, ae, x, f, W, peak_gbs, reps, persistent=False, aux=None, x_dot=None, alpha=0.0):
    """FP64 and mixed R+J of one workload: each precision's tuned kernel, timed alone (zeroing outside);
    x_dot and alpha as given (a transient Jacobian's mass terms)."""
    from . import autotune
    E, N = w.n_elements, w.dof.n_dofs
    bytes_ = assembly_bytes(_lattice_vertices(w), N, w.dof.nnz, _conn_entries(w))
    out = {"elements": E, "dofs": N, "nnz": w.dof.nnz, "algorithmic_bytes": bytes_}
    for tag, mixed in (("fp64", False), ("mixed", True)):
        # per-block launches: the tuned kernel; the persistent launch keeps the workload's worksets
        cfg = {} if persistent else autotune.tune(ae, x, f, W, mixed=mixed, aux=aux, force=True, reps=2,
                                                  x_dot=x_dot, alpha=alpha)
        gather = ae.gather and not persistent

        def prep():
            if not gather:
                f.zero_()
                W.initializeMatrix(0.0)
        ms = _time_kernel(lambda: ae.evaluate(x, x_dot=x_dot, aux=aux, alpha=alpha, f=f, W=W, mixed=mixed,
                                              persistent=persistent), prep, reps)
        form = ("lattice" if gather and mixed and ae.gather_form() == "lattice" else "two-phase" if gather
                else "persistent" if persistent else "staged" if cfg.get("variant") != 2 else "warp")
        gbs = bytes_ / ms / 1e6
        out[tag] = {"ms": ms, "elements_per_s": E / ms * 1e3, "form": form, "achieved_gbs": gbs,
                    "frac": gbs / peak_gbs}
    out["mixed_vs_fp64"] = out["fp64"]["ms"] / out["mixed"]["ms"]
    return out


def newton_heat(w, mixed, tol=1e-10, max_it=12):
    """Newton on the nonlinear heat workload with T = 0 on the box sides, from T = 0: iterations until
    ||f|| <= tol ||f(T0)||.  The residual is always FP64; the Jacobian is FP64 or mixed (FP32 element
    arithmetic), and each linear step J dT = -f is solved by the FP64-refined FP32 CG."""
    from .panzer import DirichletBC, ModelEvaluator
    me = ModelEvaluator(w.lof, [DirichletBC(w.dof, A.ALL_SIDES)])
    T = w.lof.getTpetraVector()
    f, W, dT = w.lof.getTpetraVector(), me.create_W_op(), w.lof.getTpetraVector()
    norms = []
    for _ in range(max_it + 1):
        me.evalModel(T, f=f)  # FP64 residual
        norms.append(float(f.norm()))
        if norms[-1] <= tol * norms[0]:
            break
        me.evalModel(T, W=W, mixed=mixed)
        dT.zero_()
        me.solve(W, dT, b=-f, rtol=1e-12, inner_rtol=1e-5, max_outer=60)
        T.add_(dT)
    return {"iterations": len(norms) - 1, "residual_norms": norms}


def measure_configs(peak_gbs, reps=5):
    """The other named workloads at their stated sizes: FP64 and mixed (or batched) R+J elements/s with the
    roofline fraction of each precision's tuned kernel (algorithmic bytes / kernel time / HBM peak), the
    Newmark step of the elastodynamics workload and Newton iteration counts of the nonlinear heat workload."""
    import gc
    from .newmark import NewmarkElastodynamics
    from .panzer import AssemblyEngine, Batch
    out = {}
    # Poisson hex8 16^3 (launch-latency bound at this size)
    w = poisson_hex8(16)
    ae, x = AssemblyEngine(w.lof), w.lof.getTpetraVector()
    x.uniform_(-1.0, 1.0)
    f, W = w.lof.getTpetraVector(), w.lof.getTpetraMatrix()
    out["poisson_hex8_16"] = _assembly_legs(w, ae, x, f, W, peak_gbs, reps)
    del w, ae, x, f, W
    # nonlinear heat, hex27 48^3 + tet10 48^3, uneven worksets in one persistent launch
    w = heat_hex27_tet10(48)
    ae = AssemblyEngine(w.lof)
    ae.setWorksetSize(256, 1024, seed=11)
    g = torch.Generator(device="cuda").manual_seed(2)
    x = torch.rand(w.dof.n_dofs, dtype=torch.float64, device="cuda", generator=g)
    f, W = w.lof.getTpetraVector(), w.lof.getTpetraMatrix()
    r = _assembly_legs(w, ae, x, f, W, peak_gbs, reps, persistent=True)
    ae.setWorksetSize(256, 1024, seed=11)
    r["newton"] = {"mixed": newton_heat(w, True), "fp64": newton_heat(w, False)}
    out["heat_hex27_tet10_48"] = r
    del w, ae, x, f, W
    gc.collect()
    torch.cuda.empty_cache()
    # elastodynamics hex8 96^3: K_eff assembly and the graph-captured Newmark step
    w = elastodynamics_hex8(96)
    ae = AssemblyEngine(w.lof)
    g = torch.Generator(device="cuda").manual_seed(4)
    u0 = torch.randn(w.dof.n_dofs, dtype=torch.float64, device="cuda", generator=g) * 1e-3
    f, W = w.lof.getTpetraVector(), w.lof.getTpetraMatrix()
    # K_eff = K + c rho M, c = 1 / (beta dt^2) of the step below: the evaluation the Newmark step assembles
    dt, nb_beta = 1e-3, 0.25
    zero = torch.zeros_like(u0)
    r = _assembly_legs(w, ae, u0, f, W, peak_gbs, reps, x_dot=zero, alpha=1.0 / (nb_beta * dt * dt))
    del f, W, zero
    nm = NewmarkElastodynamics(w.me, dt, nb_beta, 0.5, mixed=True, outer=3, inner=24)
    nm.initialize(u0)
    nm.capture()
    nm.step()
    torch.cuda.synchronize()
    s, e = _events()
    s.record()
    rel = [nm.step()[2] for _ in range(10)]
    e.record()
    torch.cuda.synchronize()
    r["newmark"] = {"steps": 10, "ms_per_step": s.elapsed_time(e) / 10,
                    "max_step_relres": max(float(v) for v in rel)}
    out["elastodynamics_hex8_96"] = r
    del w, ae, u0, nm
    gc.collect()
    torch.cuda.empty_cache()
    # 256 independent meshes in one persistent launch
    ws = mixed_batch(256)
    g = torch.Generator(device="cuda").manual_seed(5)
    xs = [torch.rand(w.dof.n_dofs, dtype=torch.float64, device="cuda", generator=g) for w in ws]
    auxs = [w.extras.get("J") for w in ws]
    fs = [w.lof.getTpetraVector() for w in ws]
    Ws = [w.lof.getTpetraMatrix() for w in ws]
    b = Batch([w.dof for w in ws], workset=(512, 512))
    nel = sum(w.n_elements for w in ws)
    bytes_ = sum(assembly_bytes(_lattice_vertices(w), w.dof.n_dofs, w.dof.nnz, _conn_entries(w)) for w in ws)
    r = {"instances": len(ws), "elements": nel, "algorithmic_bytes": bytes_}
    for tag, mixed in (("fp64", False), ("mixed", True)):
        def prep():
            for f_, W_ in zip(fs, Ws):
                f_.zero_()
                W_.initializeMatrix(0.0)
        ms = _time_kernel(lambda: b.evaluate(xs, fs, Ws, auxs=auxs, mixed=mixed), prep, reps)
        gbs = bytes_ / ms / 1e6
        r[tag] = {"ms": ms, "elements_per_s": nel / ms * 1e3, "form": "batched persistent", "achieved_gbs": gbs,
                  "frac": gbs / peak_gbs}
    r["mixed_vs_fp64"] = r["fp64"]["ms"] / r["mixed"]["ms"]
    out["mixed_batch_256"] = r
    return out


def report(names=("poisson_hex8", "heat_hex27_tet10", "elastodynamics_hex8", "mixed_batch")):
    """Elements/s of the non-headline workloads (one JSON object)."""
    import json
    import time
    from .newmark import NewmarkElastodynamics
    from .panzer import AssemblyEngine, Batch
    out = {}
    if "poisson_hex8" in names:
        w = poisson_hex8(16)
        ae, x = AssemblyEngine(w.lof), w.lof.getTpetraVector()
        f, W = w.lof.getTpetraVector(), w.lof.getTpetraMatrix()
        out["poisson_hex8_16"] = {"elements": w.n_elements,
                                  "fp64_ms": time_eval(ae, x, f, W), "mixed_ms": time_eval(ae, x, f, W, mixed=True)}
    if "heat_hex27_tet10" in names:
        w = heat_hex27_tet10(48)
        ae = AssemblyEngine(w.lof)
        ae.setWorksetSize(256, 1024, seed=11)
        g = torch.Generator(device="cuda").manual_seed(2)
        x = torch.rand(w.dof.n_dofs, dtype=torch.float64, device="cuda", generator=g)
        f, W = w.lof.getTpetraVector(), w.lof.getTpetraMatrix()
        r = {"elements": w.n_elements, "dofs": w.dof.n_dofs, "nnz": w.dof.nnz}
        for tag, kw in (("fp64_blocks", {}), ("mixed_blocks", {"mixed": True}),
                        ("fp64_persistent", {"persistent": True}), ("mixed_persistent", {"persistent": True, "mixed": True}),
                        ("mixed_persistent_direct", {"persistent": True, "mixed": True, "scatter_direct": True})):
            r[tag + "_ms"] = time_eval(ae, x, f, W, **kw)
        out["heat_hex27_tet10_48"] = r
    if "elastodynamics_hex8" in names:
        w = elastodynamics_hex8(96)
        g = torch.Generator(device="cuda").manual_seed(4)
        u0 = torch.randn(w.dof.n_dofs, dtype=torch.float64, device="cuda", generator=g) * 1e-3
        nm = NewmarkElastodynamics(w.me, 1e-3, 0.25, 0.5, mixed=True, outer=3, inner=24)
        t0 = time.perf_counter()
        nm.initialize(u0)
        torch.cuda.synchronize()
        t_init = time.perf_counter() - t0
        nm.capture()
        s, e = _events()
        s.record()
        rel = []
        for _ in range(10):
            rel.append(nm.step()[2])
        e.record()
        torch.cuda.synchronize()
        out["elastodynamics_hex8_96"] = {"elements": w.n_elements, "dofs": w.dof.n_dofs, "steps": 10,
                                         "ms_per_step": s.elapsed_time(e) / 10,
                                         "max_step_relres": max(float(v) for v in rel),
                                         "init_s": t_init}
    if "mixed_batch" in names:
        ws = mixed_batch(256)
        g = torch.Generator(device="cuda").manual_seed(5)
        xs = [torch.rand(w.dof.n_dofs, dtype=torch.float64, device="cuda", generator=g) for w in ws]
        auxs = [w.extras.get("J") for w in ws]
        fs = [w.lof.getTpetraVector() for w in ws]
        Ws = [w.lof.getTpetraMatrix() for w in ws]
        b = Batch([w.dof for w in ws], workset=(512, 512))
        nel = sum(w.n_elements for w in ws)
        r = {"instances": len(ws), "elements": nel}
        for tag, mixed, direct in (("fp64", False, False), ("mixed", True, False), ("mixed_direct", True, True)):
            for _ in range(2):
                b.evaluate(xs, fs, Ws, auxs=auxs, mixed=mixed, scatter_direct=direct)
            torch.cuda.synchronize()
            s, e = _events()
            s.record()
            for _ in range(5):
                b.evaluate(xs, fs, Ws, auxs=auxs, mixed=mixed, scatter_direct=direct)
            e.record()
            torch.cuda.synchronize()
            r[tag + "_one_launch_ms"] = s.elapsed_time(e) / 5
        # the same work as one launch per mesh
        s, e = _events()
        s.record()
        for i, w in enumerate(ws):
            AssemblyEngine(w.lof).evaluate(xs[i], aux=auxs[i], f=fs[i], W=Ws[i], mixed=True)
        e.record()
        torch.cuda.synchronize()
        r["mixed_per_mesh_launches_ms"] = s.elapsed_time(e)
        out["mixed_batch_256"] = r
    print(json.dumps(out), flush=True)
    return out


if __name__ == "__main__":
    report()
