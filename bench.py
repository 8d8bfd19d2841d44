#!/usr/bin/env python
"""Benchmark: Jacobian-assembly elements/s + SpMV GB/s on one GB300, mixed vs FP64.

Workload (one GPU): 3-D linear elasticity on a 128^3 hex8 brick mesh
(2,097,152 elements, 6,440,067 DOFs, 513,599,625 CRS entries), E=1, nu=0.3,
body force (0,0,-1), clamped at z=0, 2x2x2 Gauss, interior vertices jittered
+-0.05h (seeded).  A step is one evalModel(f, W) = residual + Jacobian over
every element (zero f and W, fused gather/geometry/integrator/scatter
kernel, Dirichlet rows).  The headline `value` is the mixed path (FP32 element
contractions, FP64 scatter); the FP64-plain path, the CRS SpMV (FP64 and
FP32), the FP64-refined FP32 block-Jacobi CG solve to 1e-10 and, after the
timed legs, the mixed-vs-FP64 solution check are measured beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With --impl reference the CPU restatement of the reference path (the oracle,
forward-mode AD Jacobians, OpenMP over all host cores) is timed on a bounded
sample of the same workload and reported in the same metric.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Jacobian-assembly elems/s + SpMV GB/s on 1 GB300, mixed vs FP64 at <=1e-10 rel"
UNIT = "elements/s"
E2E_WINDOWS = 7


def args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=128, help="bricks per direction (default: the 128^3 workload)")
    p.add_argument("--no-solve", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-configs", action="store_true", help="skip the other named workloads")
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="budget of the CPU-baseline sample")
    p.add_argument("--spmv-shape", default=None,
                   help="fixed SpMV launch shape instead of the autotuner: lanes,unroll (both precisions) "
                        "or lanes,unroll/lanes,unroll (FP64/FP32)")
    p.add_argument("--spmv-form", default="crs", choices=["crs", "entity"],
                   help="SpMV form used with --spmv-shape")
    return p.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def e2e_summary(windows_s, links_s, steps, elements, h2d, d2h):
    """The e2e object from the timed windows (seconds for `steps` steps each, max over ranks) and the link-only
    copies (seconds per step's copy-back): the median window is the value, every window is listed."""
    te = sorted(windows_s)[len(windows_s) // 2]
    link_s = sorted(links_s)[len(links_s) // 2]
    return {"value": elements * steps / te, "unit": UNIT, "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h, "steps": steps, "windows": len(windows_s),
            "statistic": f"median of {len(windows_s)} windows of {steps} steps",
            "window_ms_per_step": [round(t / steps * 1e3, 3) for t in windows_s],
            "link_d2h_gbs": d2h / link_s / 1e9, "link_bound_frac": link_s / (te / steps),
            "path": "host x -> tx_eval(mixed) + Dirichlet -> host f and CRS values (HostEvaluator: copy-back "
                    "of step k overlapped with the assembly of step k+1)"}


def workload_desc(n):
    return {"workload": f"elasticity hex8 {n}^3 (E=1, nu=0.3, b=(0,0,-1), clamp z=0, 2x2x2 Gauss, jitter 0.05h)",
            "elements": n ** 3, "dofs": 3 * (n + 1) ** 3, "nnz": 9 * (3 * n + 1) ** 3}


def algorithmic_bytes(n_nodes, n_dofs, nnz, n_elem, n_vert=8):
    """Per R+J evaluation: coords + x + connectivity + f + A values + colind + rowptr."""
    return 24 * n_nodes + 8 * n_dofs + 4 * n_vert * n_elem + 8 * n_dofs + 8 * nnz + 4 * nnz + 8 * (n_dofs + 1)


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", delete=False, suffix=".csv")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        rows = []
        with open(self.file.name) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 7:
                    rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return None
        sm = sorted(float(r[0]) for r in rows if r[0].replace(".", "").isdigit())
        mx = max((float(r[1]) for r in rows if r[1].replace(".", "").isdigit()), default=None)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[3 + i].lower() == "active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


# --------------------------------------------------------------------------- CPU
def cpu_sample(budget_s, threads=None):
    """The oracle (CPU restatement, AD Jacobians) on an elasticity hex8 sub-lattice of the same workload."""
    import numpy as np

    from oracle import oracle as O
    from tianxin_gb300 import _abi as A
    threads = threads or os.cpu_count()
    n = 20
    q = A.equation_set(A.TX_PHYS_ELASTICITY, params=(1.0, 0.3, 0.0, 0.0, -1.0, 0.0))
    o = O.Oracle(A.mesh_desc(n, jitter=0.05, seed=2024), q)
    x = np.random.default_rng(0).uniform(-1e-3, 1e-3, o.n_dofs)
    o.evaluate(x, threads=threads)  # warm-up
    t0 = time.perf_counter()
    reps = 0
    while True:
        o.evaluate(x, threads=threads)
        reps += 1
        if time.perf_counter() - t0 >= budget_s:
            break
    dt = time.perf_counter() - t0
    return {"value": reps * n ** 3 / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"R+J of elasticity hex8 {n}^3 sub-lattice ({n ** 3} elements, same physics/jitter), "
                      f"{reps} evaluations in {dt:.1f} s, oracle CPU restatement, OpenMP"}


def _oracle_rate(o, x, budget_s, threads, **kw):
    """Elements/s of the oracle's R+J on one mesh, repeated for about budget_s."""
    o.evaluate(x, threads=threads, **kw)
    t0 = time.perf_counter()
    reps = 0
    while True:
        o.evaluate(x, threads=threads, **kw)
        reps += 1
        if time.perf_counter() - t0 >= budget_s:
            break
    return reps * o.n_elements / (time.perf_counter() - t0), reps


def config_cpu_baselines(budget_s=3.0):
    """The oracle (CPU restatement, AD Jacobians) on bounded samples of the other named workloads."""
    import numpy as np

    from oracle import oracle as O
    from tianxin_gb300 import _abi as A
    from tianxin_gb300 import workloads as WL
    cores = os.cpu_count()
    out = {}
    # Poisson hex8 16^3: the whole mesh on one thread (the Kokkos Serial equivalent)
    q = A.equation_set(A.TX_PHYS_POISSON, params=(1.0, 0.0, 0.0, 0.0), source_kind=A.TX_SOURCE_SINE)
    o = O.Oracle(A.mesh_desc(16, jitter=0.1, seed=1), q)
    v, reps = _oracle_rate(o, np.random.default_rng(0).uniform(-1, 1, o.n_dofs), budget_s, 1)
    out["poisson_hex8_16"] = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
                              "sample": f"the whole 16^3 mesh (4096 elements), {reps} R+J evaluations, one thread"}
    # heat: 8^3 hex27 + 8^3 tet10 bricks of the same two-block layout
    q = A.equation_set(A.TX_PHYS_HEAT, A.TX_HGRAD_C2, params=(1.0, 0.5, 1.0), integration_order=[4, 2])
    o = O.Oracle(A.mesh_desc((8, 8, 8), (2, 1, 1), [A.TX_TOPO_HEX, A.TX_TOPO_TET], (2.0, 1.0, 1.0), 0.0, 3), q)
    v, reps = _oracle_rate(o, np.random.default_rng(0).uniform(0, 1, o.n_dofs), budget_s, cores)
    out["heat_hex27_tet10_48"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                  "sample": f"8^3 hex27 + 8^3 bricks of tet10 ({o.n_elements} elements), {reps} R+J "
                                            "evaluations, OpenMP"}
    # elastodynamics: K + c M on a 16^3 sub-lattice (x_dot and alpha = 1 / (beta dt^2))
    q = A.equation_set(A.TX_PHYS_ELASTICITY, params=(1.0, 0.25, 0.0, 0.0, 0.0, 1.0))
    o = O.Oracle(A.mesh_desc(16, jitter=0.0, seed=4), q)
    rng = np.random.default_rng(0)
    x = rng.normal(0, 1e-3, o.n_dofs)
    v, reps = _oracle_rate(o, x, budget_s, cores, x_dot=rng.normal(0, 1.0, o.n_dofs), alpha=4e6, beta=1.0)
    out["elastodynamics_hex8_96"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                     "sample": f"K + M/(beta dt^2) of a 16^3 sub-lattice (4096 elements), {reps} "
                                               "R+J evaluations, OpenMP"}
    # batch: the first instances of the 256-mesh plan, each evaluated once, until the budget is spent
    done, nel, t_eval = 0, 0, 0.0
    for i, (kind, n) in enumerate(WL.batch_plan(256)):
        if kind == "poisson_hex8":
            q = A.equation_set(A.TX_PHYS_POISSON, params=(1.0, 0.0, 0.0, 0.0), source_kind=A.TX_SOURCE_SINE)
            m, aux = A.mesh_desc(n, jitter=0.1, seed=5000 + i), None
        elif kind == "elasticity_tet4":
            q = A.equation_set(A.TX_PHYS_ELASTICITY, params=(1.0, 0.3, 0.0, 0.0, -1.0, 0.0))
            m, aux = A.mesh_desc(n, topology=A.TX_TOPO_TET, jitter=0.1, seed=5000 + i), None
        else:
            q = A.equation_set(A.TX_PHYS_MAXWELL, A.TX_HCURL_I1, params=(1.0, 1.0))
            m, aux = A.mesh_desc(n, jitter=0.1, seed=5000 + i), True
        o = O.Oracle(m, q)
        x = np.random.default_rng(i).uniform(0, 1, o.n_dofs)
        kw = {"aux": np.random.default_rng(i + 1).normal(0, 1, o.n_dofs)} if aux else {}
        t0 = time.perf_counter()
        o.evaluate(x, threads=cores, **kw)
        t_eval += time.perf_counter() - t0
        done += 1
        nel += o.n_elements
        if t_eval >= budget_s:
            break
    out["mixed_batch_256"] = {"value": nel / t_eval, "unit": UNIT, "cores": cores, "kind": "port",
                              "sample": f"the first {done} instances of the plan ({nel} elements), one R+J "
                                        "evaluation each, OpenMP"}
    return out


def run_reference(a):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    import numpy as np

    from oracle import oracle as O
    from tianxin_gb300 import _abi as A
    threads = os.cpu_count()
    n = 16
    q = A.equation_set(A.TX_PHYS_ELASTICITY, params=(1.0, 0.3, 0.0, 0.0, -1.0, 0.0))
    o = O.Oracle(A.mesh_desc(n, jitter=0.05, seed=2024), q)
    x = np.random.default_rng(0).uniform(-1e-3, 1e-3, o.n_dofs)
    for _ in range(a.warmup):
        o.evaluate(x, threads=threads)
    t0 = time.perf_counter()
    for _ in range(a.steps):
        o.evaluate(x, threads=threads)
    dt = time.perf_counter() - t0
    value = a.steps * n ** 3 / dt
    sample = (f"each step: R+J of an elasticity hex8 {n}^3 sub-lattice ({n ** 3} elements) of the 128^3 workload, "
              "oracle CPU restatement (AD Jacobians), OpenMP")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": 1e3 * dt / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": workload_desc(a.n) | {"workload": workload_desc(a.n)["workload"] +
                                            f"; each step a {n}^3 sample ({n ** 3} elements) of it",
                                            "parallelism": "cpu", "sample_elements": n ** 3},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------- GPU
def run_ours(a):
    import numpy as np
    import torch

    import tianxin_gb300 as tx
    from tianxin_gb300 import _abi as A

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    def maxall(v):
        if not dist:
            return v
        t = torch.tensor([v], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    n = a.n
    t_setup = time.perf_counter()
    conn = tx.CartesianConnManager(n, n, n, jitter=0.05, seed=2024)
    q = A.equation_set(A.TX_PHYS_ELASTICITY, params=(1.0, 0.3, 0.0, 0.0, -1.0, 0.0))
    dof = tx.DOFManager(conn, q)
    lof = tx.TpetraLinearObjFactory(dof)
    bc = tx.DirichletBC(dof, A.SIDE_ZMIN)
    me = tx.ModelEvaluator(lof, [bc])
    torch.cuda.synchronize()
    t_setup = time.perf_counter() - t_setup
    E, N, nnz = conn.n_elements, dof.n_dofs, dof.nnz
    gen = torch.Generator(device="cuda").manual_seed(7 + rank)
    x = (torch.rand(N, dtype=torch.float64, device="cuda", generator=gen) * 2 - 1) * 1e-3
    x[bc.lids.long()] = 0.0
    f = lof.getTpetraVector()
    W = me.create_W_op()
    stream = torch.cuda.current_stream()

    def timed_steps(mixed, steps, warmup):
        for _ in range(warmup):
            me.evalModel(x, f=f, W=W, mixed=mixed)
        kev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        barrier()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for i in range(steps):
            if not me.ae.gather_applies(W):  # the two-phase form overwrites f and W
                f.zero_()
                W.initializeMatrix(0.0)
            kev[i][0].record(stream)
            me.ae.evaluate(x, f=f, W=W, mixed=mixed)
            kev[i][1].record(stream)
            me.applyDirichlet(x, f, W)
        t1.record(stream)
        barrier()
        total = maxall(t0.elapsed_time(t1) / 1e3)
        kern = [s.elapsed_time(e) / 1e3 for s, e in kev]
        return total, sum(kern) / len(kern)

    # tile shapes: the project's autotuner times staged/direct scatter x CTA caps on this workload
    from tianxin_gb300 import autotune
    tuned = autotune.tune(me.ae, x, f, W, mixed=True, force=True)
    gather = bool(tuned.get("gather", False))
    clocks = ClockSampler(local)
    clocks.start()
    t_mixed, k_mixed = timed_steps(True, a.steps, a.warmup)
    clk = clocks.stop()
    W_mixed = W.values.clone()
    K64 = max(3, min(a.steps, 8))
    tuned64 = autotune.tune(me.ae, x, f, W, mixed=False, force=True, reps=1)
    t_fp64, k_fp64 = timed_steps(False, K64, 3)
    jac_diff = float((W.values - W_mixed).abs().max() / W.values.abs().max())
    del W_mixed

    value = ws * E * a.steps / t_mixed
    value64 = ws * E * K64 / t_fp64

    # ---- SpMV (Tpetra CrsMatrix::apply) FP64 and FP32
    v32 = W.values.float()
    xs = torch.rand(N, dtype=torch.float64, device="cuda", generator=gen)
    ys = torch.zeros(N, dtype=torch.float64, device="cuda")
    xs32, ys32 = xs.float(), ys.float()

    def time_spmv(vals, xv, yv, reps):
        for _ in range(3):
            W.apply(xv, yv, values=vals)
        barrier()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        for _ in range(reps):
            W.apply(xv, yv, values=vals)
        e.record(stream)
        barrier()
        return maxall(s.elapsed_time(e) / 1e3 / reps)

    reps = max(10, a.steps)
    # forms and launch shapes: CRS (lanes per row x loads per lane, 16 shapes) and entity-block
    # (lanes per entity x blocks per pass, 8 shapes); the autotuner times all of them per precision
    def fix_shape(shape):
        W.setApplyForm(a.spmv_form)
        (W.setApplyShape if a.spmv_form == "crs" else W.setEntityApplyShape)(*shape)
        return {"form": a.spmv_form, "shape": shape, "candidates": []}

    if a.spmv_shape:
        parts = [tuple(int(v) for v in p.split(",")) for p in a.spmv_shape.split("/")]
        sh64 = fix_shape(parts[0])
    else:
        sh64 = autotune.tune_spmv(W, W.values, xs, ys)
    t_s64 = time_spmv(W.values, xs, ys, reps)
    sh32 = fix_shape(parts[-1]) if a.spmv_shape else autotune.tune_spmv(W, v32, xs32, ys32)
    t_s32 = time_spmv(v32, xs32, ys32, reps)  # the FP32 form and shape stay set for the solver's inner SpMV
    n_ent = N // 3

    def spmv_bytes(form, vbytes):
        # CRS: values, column indices, rowptr, x once, y written; entity-block: one column index per
        # 3x3 block and the entity rowptr instead of the DOF rowptr
        if form == "entity":
            return (vbytes * nnz + 4 * (nnz // 9) + 8 * (n_ent + 1) + 2 * vbytes * N)
        return (vbytes + 4) * nnz + 8 * (N + 1) + 2 * vbytes * N

    b64, b32 = spmv_bytes(sh64["form"], 8), spmv_bytes(sh32["form"], 4)
    crs64, crs32 = spmv_bytes("crs", 8), spmv_bytes("crs", 4)

    def best_crs_ms(sh):
        ts = [t for c, t in sh["candidates"] if c[0] == "crs"]
        return round(min(ts), 4) if ts else None
    del v32

    peak, peak_kind = measured_peaks()
    bytes_alg = algorithmic_bytes((n + 1) ** 3, N, nnz, E)
    achieved = bytes_alg / k_mixed / 1e9
    traffic = None
    warp_kernel = tuned.get("variant") == 2
    lattice = gather and me.ae.gather_form() == "lattice"
    # the two-phase form is two kernels: element rows to scratch, then the row gather; the lattice
    # form gathers x into node order, then owns and writes each node's rows once
    kernel_name = ("k_lattice_gather_u + k_lattice_gather<hex8,elasticity,f32>" if lattice
                   else "k_assemble<hex8,elasticity,f32,jac,scratch> + k_gather_rows<float>" if gather
                   else "k_assemble_wpe<hex8,elasticity,f32,jac>" if warp_kernel
                   else "k_assemble<hex8,elasticity,f32,jac>")
    tf = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    if os.path.exists(tf):
        try:
            traffic = json.load(open(tf)).get(("lattice" if lattice else "gather" if gather else
                                               "assemble_wpe" if warp_kernel else "assemble")
                                              + "_elasticity_hex8_mixed_bytes_per_launch_128")
        except Exception:
            traffic = None

    # ---- solve: mixed Jacobian + FP64 matrix-free residual, block-Jacobi CG (FP32) inside FP64 refinement
    solve = None
    if not a.no_solve:
        autotune.tune(me.ae, x, f, W, mixed=True)  # the Jacobian of the timed mixed step (the FP64 leg tuned its own)
        xsol = lof.getTpetraVector()
        me.evalModel(xsol, f=f, W=W, mixed=True)
        barrier()
        ts = time.perf_counter()
        st = me.solve(W, xsol, rtol=1e-10, inner_rtol=1e-5, matrix_free=True, max_outer=30, block_jacobi=True)
        torch.cuda.synchronize()
        ts = time.perf_counter() - ts
        solve = {"rtol": 1e-10, "relres_fp64": st["relres"], "outer": st["outer"], "inner_cg": st["inner"],
                 "seconds": ts, "residual": "FP64 matrix-free (Residual evaluation)",
                 "inner": "FP32 CG, 3x3 block-Jacobi preconditioner (point Jacobi without the entity form)",
                 "max_u": float(xsol.abs().max())}
        del xsol

    # ---- e2e through the public API with host buffers
    e2e = None
    if not a.no_e2e:
        # host-resident x, f and CRS values (pinned, reused every step as a Newton loop's containers are);
        # HostEvaluator overlaps step k's copy-back with step k + 1's assembly
        xh = x.cpu().pin_memory()
        fh = torch.empty(N, dtype=torch.float64).pin_memory()
        Wh = torch.empty(nnz, dtype=torch.float64).pin_memory()
        autotune.tune(me.ae, x, f, W, mixed=True)  # the mixed configuration again (the FP64 leg tuned its own)
        hev = tx.HostEvaluator(me, mixed=True)
        K2 = max(3, min(a.steps, 5))
        for k in range(2):
            hev.step(xh, fh, Wh)
        hev.synchronize()
        # The host link is shared with the machine's other work: a window of K2 steps now and then runs at a
        # fraction of its usual rate, so the leg times E2E_WINDOWS windows and reports the median window (every
        # window's step time is listed beside it).
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        win = []
        for _ in range(E2E_WINDOWS):
            barrier()
            s.record(stream)
            for k in range(K2):
                hev.step(xh, fh, Wh)
            hev.synchronize()
            e.record(stream)
            barrier()
            win.append(maxall(s.elapsed_time(e) / 1e3))
        # the host link alone: the same step's bytes copied back with nothing else running (its bound; median of
        # three)
        links = []
        for _ in range(3):
            s.record(stream)
            for k in range(2):
                fh.copy_(f, non_blocking=True)
                Wh.copy_(W.values, non_blocking=True)
            e.record(stream)
            e.synchronize()
            links.append(s.elapsed_time(e) / 2e3)
        e2e = e2e_summary(win, links, K2, ws * E, 8 * N, 8 * N + 8 * nnz)
        del Wh, hev

    # the mixed path against the FP64 path at full size (after the timed legs): both Jacobians (FP32 element
    # math with FP64 sums, and FP64-plain) refined with the same FP64 residual to 1e-12; their solutions' difference
    if solve is not None:
        sols = []
        for mixed in (True, False):
            xs = lof.getTpetraVector()
            me.evalModel(xs, f=f, W=W, mixed=mixed)
            st2 = me.solve(W, xs, rtol=1e-12, inner_rtol=1e-5, matrix_free=True, max_outer=40, block_jacobi=True)
            sols.append((xs, st2["relres"]))
        (xm, rm), (xd, rd) = sols
        solve["mixed_vs_fp64"] = {"rtol": 1e-12, "relres": [rm, rd],
                                  "solution_maxrel": float((xm - xd).abs().max() / xd.abs().max())}
        del xm, xd, sols

    # the other named workloads at their stated sizes (after the headline legs)
    configs = None
    if not a.no_configs:
        from tianxin_gb300 import workloads as WL
        configs = WL.measure_configs(peak)

    cpu = None
    if rank == 0 and ws == 1:
        try:
            cpu = cpu_sample(a.cpu_seconds)
        except Exception as ex:  # the baseline is reported, not required
            cpu = {"value": None, "error": str(ex)}
        if configs is not None:
            try:
                for k, v in config_cpu_baselines().items():
                    configs[k]["cpu_baseline"] = v
            except Exception as ex:
                configs["cpu_baseline_error"] = str(ex)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": 1e3 * t_mixed / a.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 element math, f64 accumulation", "data": "synthetic",
            "config": workload_desc(n) | {"elements": E, "dofs": N, "nnz": nnz, "parallelism": "replicas",
                                          "l2": "inputs larger than L2 (CRS values 8*nnz bytes)",
                                          "setup_seconds": round(t_setup, 2)},
            "fp64_plain": {"value": value64, "unit": UNIT, "ms_per_step": 1e3 * t_fp64 / K64,
                           "kernel_ms": 1e3 * k_fp64, "steps": K64},
            "mixed_vs_fp64": value / value64,
            "mixed_kernel_ms": 1e3 * k_mixed,
            "jacobian_mixed_vs_fp64_maxrel": jac_diff,
            "spmv": {"f64_gbs": b64 / t_s64 / 1e9, "f32_gbs": b32 / t_s32 / 1e9, "f64_ms": 1e3 * t_s64,
                     "f32_ms": 1e3 * t_s32, "f64_frac": b64 / t_s64 / 1e9 / peak, "f32_frac": b32 / t_s32 / 1e9 / peak,
                     "bytes_f64": b64, "bytes_f32": b32, "form_f64": sh64["form"], "form_f32": sh32["form"],
                     "shape_f64": sh64["shape"], "shape_f32": sh32["shape"],
                     "crs_bytes_f64": crs64, "crs_bytes_f32": crs32,
                     "crs_equivalent_gbs": {"f64": crs64 / t_s64 / 1e9, "f32": crs32 / t_s32 / 1e9},
                     "best_crs_form_ms": {"f64": best_crs_ms(sh64), "f32": best_crs_ms(sh32)},
                     "shape_candidates_ms": {"f64": [(c, round(t, 3)) for c, t in sh64["candidates"]],
                                             "f32": [(c, round(t, 3)) for c, t in sh32["candidates"]]}},
            "solve": solve,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "peak_source": peak_kind, "kernel": kernel_name,
                         "algorithmic_bytes_per_launch": bytes_alg},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": (3 if gather else 2) * a.steps,
            "autotune": {"mixed": {k: v for k, v in tuned.items() if k != "candidates"},
                         "mixed_candidates": "(variant, scatter_direct, gather, cta_threads, grid_cap, ms)",
                         "mixed_candidates_ms": [(c.get("variant"), c.get("scatter_direct"), c.get("gather", False),
                                                  c.get("cta_threads", 0), c.get("grid_cap"), round(c["ms"], 3))
                                                 for c in tuned.get("candidates", [])],
                         "fp64": {k: v for k, v in tuned64.items() if k != "candidates"}},
            "clocks": clk,
            "configs": configs,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    a = args()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
