"""Tile-shape autotuner for the assembly launches.

The knobs play the role of Panzer's HierarchicParallelism team/vector sizes
(disc-fe/src/Panzer_HierarchicParallelism.hpp:78-128):

  * scatter   staged CTA-wide scatter vs per-thread row reductions
  * grid_cap  CTAs of the per-block launch (0 = occupancy x SMs x 4)
  * workset   elements per work item of the persistent / batched launch
  * gather    two-phase evaluation (element rows to scratch, rows gathered and
              written once; on a hex8 elasticity lattice the owner-computes
              lattice kernel) against the atomic scatter; atomic candidates are
              timed with the zeroing of f and W they need, the gather forms
              overwrite them
  * threads   threads a CTA of the staged kernel, 64 / 128 / 256: elements per
              CTA (threads over the element's basis count rounded up to a
              power of two), Panzer's team size

Each candidate is timed with CUDA events on the real evaluation (outputs in
scratch vectors), the fastest is kept, and results are cached in
_build/autotune.json keyed by GPU name, element family, physics, precision
and size.
"""
import json
import os

import torch

from . import _abi as A
from ._lib import TxError as tx_error

CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "autotune.json")


def _key(dof, mixed, mode):
    q = dof.eqset
    return "|".join(str(v) for v in (torch.cuda.get_device_name(), q.physics, list(q.block_basis)[:dof.conn.n_blocks],
                                     list(dof.conn.desc.block_topology)[:dof.conn.n_blocks], dof.conn.n_elements,
                                     int(mixed), mode))


def _load():
    try:
        with open(CACHE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save(d):
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    tmp = CACHE + ".tmp"
    with open(tmp, "w") as f:
        json.dump(d, f, indent=1, sort_keys=True)
    os.replace(tmp, CACHE)


def _time(fn, reps=3):
    fn()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(reps):
        fn()
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / reps


def tune(ae, x, f, W, mixed=True, persistent=False, aux=None, reps=3, force=False, verbose=False, x_dot=None,
         alpha=0.0):
    """Pick and apply the fastest configuration for ae's handle; returns it.  x_dot and alpha are timed as
    given (the mass terms of a transient Jacobian run only with alpha != 0 or x_dot)."""
    dof = ae.dof
    mode = "persistent" if persistent else "block"
    if x_dot is not None or alpha != 0.0:
        mode += "+mass"
    key = _key(dof, mixed, mode)
    cache = _load()
    if key in cache and not force:
        cfg = cache[key]
    else:
        sms = torch.cuda.get_device_properties(0).multi_processor_count
        results = []
        if persistent:
            ae.setGridCap(0)
            for direct in (False, True):  # staged or per-thread Jacobian scatter
                for ws in (128, 256, 512, 1024, 2048):
                    ae.setWorksetSize(ws, ws)
                    t = _time(lambda: ae.evaluate(x, x_dot=x_dot, aux=aux, alpha=alpha, f=f, W=W, mixed=mixed,
                                                  persistent=True, scatter_direct=direct), reps)
                    results.append(({"workset": ws, "grid_cap": 0, "scatter_direct": direct}, t))
        else:
            # kernel variant (warp per element / CTA-staged / CTA direct scatter / tensor-core contractions /
            # two-phase) x CTA tile
            # shape (threads a CTA of the staged kernel: elements per CTA) x CTA cap
            kernels = [(2, False, False, 0), (1, False, False, 0), (1, True, False, 0)] if mixed else \
                [(1, False, False, 0), (1, True, False, 0)]
            if W is not None:
                kernels += [(1, False, False, 64), (1, False, False, 256)]
                if mixed:  # the element contractions on the tensor cores (hex8 elasticity; elsewhere a repeat)
                    kernels.append((3, False, False, 0))
            if W is not None and ae.gather_supported():
                kernels.append((1, False, True, 0))

            def step(direct, gather):
                if not gather:  # the atomic forms sum into f and W, which a step zeroes first
                    W.initializeMatrix(0.0)
                    if f is not None:
                        f.zero_()
                ae.evaluate(x, x_dot=x_dot, aux=aux, alpha=alpha, f=f, W=W, mixed=mixed, scatter_direct=direct,
                            gather=gather)

            for variant, direct, gather, threads in kernels:
                ae.setVariant(variant)
                try:
                    ae.setCtaThreads(threads)
                except tx_error:  # no block of this handle has the tile shape
                    continue
                for cap in (0, sms * 2, sms * 4, sms * 8):
                    ae.setGridCap(cap)
                    try:
                        t = _time(lambda: step(direct, gather), reps)
                    except tx_error:  # a configuration the handle refuses
                        continue
                    results.append(({"variant": variant, "scatter_direct": direct, "gather": gather,
                                     "cta_threads": threads, "grid_cap": cap}, t))
            ae.setCtaThreads(0)
        best = min(results, key=lambda r: r[1])
        cfg = dict(best[0], ms=best[1], candidates=[dict(c, ms=t) for c, t in results])
        cache[key] = cfg
        _save(cache)
        if verbose:
            for c, t in results:
                print(f"  {c}: {t:.3f} ms")
    ae.setGridCap(cfg.get("grid_cap", 0))
    ae.setVariant(cfg.get("variant", 0))
    ae.setCtaThreads(cfg.get("cta_threads", 0))
    ae.gather = bool(cfg.get("gather", False))
    ae.scatter_direct = bool(cfg.get("scatter_direct", False))
    if "workset" in cfg:
        ae.setWorksetSize(cfg["workset"], cfg["workset"])
    return cfg


SPMV_SHAPES = [(lanes, unroll) for lanes in (4, 8, 16, 32) for unroll in (1, 2, 4, 16)]  # 16: 16-byte loads
ENTITY_SHAPES = [(3, 1), (3, 2), (3, 3)] + [(lanes, unroll) for lanes in (4, 8, 16, 32) for unroll in (1, 2)] + \
    [(4, 4), (8, 4)]


def tune_spmv(W, vals, x, y, reps=5):
    """Time W.apply in every launch shape of each form it has and apply the fastest.

    CRS form: lanes per row x loads per lane; entity-block form (matrices on
    the handle's graph): lanes per entity x blocks per lane pass.  Returns
    {"form": f, "shape": (lanes, unroll), "ms": t, "candidates": [((form, lanes, unroll), ms), ...]}.
    """
    results = []
    W.setApplyForm("crs")
    for shape in SPMV_SHAPES:
        W.setApplyShape(*shape)
        results.append((("crs",) + shape, _time(lambda: W.apply(x, y, values=vals), reps)))
    if W.on_handle_graph:
        W.setApplyForm("entity")
        for shape in ENTITY_SHAPES:
            W.setEntityApplyShape(*shape)
            results.append((("entity",) + shape, _time(lambda: W.apply(x, y, values=vals), reps)))
    best = min(results, key=lambda r: r[1])
    best_crs = min((r for r in results if r[0][0] == "crs"), key=lambda r: r[1])
    W.setApplyShape(*best_crs[0][1:])
    if best[0][0] == "entity":
        W.setEntityApplyShape(*best[0][1:])
    W.setApplyForm(best[0][0])
    return {"form": best[0][0], "shape": best[0][1:], "ms": best[1], "candidates": results}
