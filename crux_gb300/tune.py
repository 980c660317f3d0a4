"""Autotuner of the plan walker's launch shape.

The walker's shape is five numbers, set process-wide by ``cxgTune`` and
``cxgTuneLanes`` (include/cxlik_gpu.h) and read when a plan, batch, MC3 run
or server request is translated:

* ``tile``: patterns per CTA (32, 64 or 128);
* ``tpp``: threads per pattern (1, 2 or 4). The FP32 form splits a
  pattern's components over that many consecutive threads when the count
  divides them;
* ``ppt``: patterns per thread (1 or 2). The FP32 form with one thread per
  pattern and at most five components can give each thread two patterns,
  half a tile apart, for twice the independent arithmetic per thread;
* ``budget``: shared-memory bytes for the CL stack of a tile. This caps the
  number of stack slots; results that find no slot go through HBM;
* ``lanes``: op lanes of single plans (1 or 2). With 2, the FP32 form with
  one thread and one pattern per thread, at most five components and staged
  leaves runs two independent node updates per step on two thread groups
  over the same patterns. Batches, MC3 and the server keep one lane.

Every shape gives bit-identical results, so the choice is speed alone.
``tune_plan`` and ``tune_batch`` time each candidate on the caller's own
workload with CUDA events (the walker launch, after warm-up), set the
fastest with ``cxgTune`` and return the whole table.
"""
import ctypes
import itertools

TILES = (32, 64, 128)
TPPS = (1, 2, 4)
PPTS = (1, 2)
BUDGETS = (0, 12 << 10, 24 << 10, 48 << 10, 96 << 10)
LANES = (1, 2)
MAX_THREADS = 256


def get(lib):
    """The current shape as (tile, tpp, ppt, budget, lanes)."""
    t, g, p = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_uint()
    b = ctypes.c_size_t()
    lanes = ctypes.c_uint()
    lib.cxgTuneGet(ctypes.byref(t), ctypes.byref(g), ctypes.byref(p),
                   ctypes.byref(b))
    lib.cxgTuneLanesGet(ctypes.byref(lanes))
    return t.value, g.value, p.value, b.value, lanes.value


def set_shape(lib, tile, tpp, ppt, budget, lanes=1):
    if lib.cxgTune(tile, tpp, ppt, budget) != 0:
        raise ValueError("cxgTune: %s" % lib.cxgLastError().decode())
    if lib.cxgTuneLanes(lanes) != 0:
        raise ValueError("cxgTuneLanes: %s" % lib.cxgLastError().decode())


def shape_ok(precision, kact, tile, tpp, ppt=1, lanes=1):
    """Whether the library has a walker for this shape (the C rules of
    walker_shape_ok, lanes_shape_ok and tuned_ppt,
    crux_gb300/csrc/cxg_internal.h)."""
    if tile * tpp * lanes > MAX_THREADS or kact < 1:
        return False
    if lanes == 2:
        return (precision == "fp32" and tpp == 1 and ppt == 1 and
                1 <= kact <= 5 and tile <= 64)
    if lanes != 1:
        return False
    if ppt == 2:
        return (precision == "fp32" and tpp == 1 and 1 <= kact <= 5
                and tile >= 64)
    if ppt != 1:
        return False
    if tpp == 1:
        return 1 <= kact <= 8
    if precision != "fp32" or kact % tpp:
        return False
    return kact // tpp <= (4 if tpp == 2 else 2)


def candidates(precision, kact, tiles=TILES, tpps=TPPS, budgets=BUDGETS,
               ppts=PPTS, lanes=LANES):
    """(tile, tpp, ppt, budget, lanes) shapes the library has a walker for.
    Lanes apply to single plans only: pass lanes=(1,) for batches, MC3 and
    the server."""
    return [(t, g, p, b, n) for t, g, p, b, n in
            itertools.product(tiles, tpps, ppts, budgets, lanes)
            if shape_ok(precision, kact, t, g, p, n)]


def active_components(lik):
    """Mixture components with non-zero weight (the walker's kact)."""
    L = lik.lik
    return sum(1 for c in range(L.compsLen) if L.comps[c].weightScaled != 0.0)


def _sweep(lib, shapes, measure):
    saved = get(lib)
    table = []
    try:
        for shape in shapes:
            set_shape(lib, *shape)
            row = {"tile": shape[0], "tpp": shape[1], "ppt": shape[2],
                   "budget": shape[3],
                   "lanes": shape[4] if len(shape) > 4 else 1}
            try:
                row["ms"] = measure()
            except RuntimeError as e:
                # A shape the device cannot launch is skipped, with why.
                row["ms"] = float("inf")
                row["error"] = str(e)
            table.append(row)
    finally:
        set_shape(lib, *saved)
    best = min(table, key=lambda r: r["ms"])
    if best["ms"] == float("inf"):
        raise RuntimeError("no walker shape ran: %s" % table[0].get("error"))
    set_shape(lib, best["tile"], best["tpp"], best["ppt"], best["budget"],
              best["lanes"])
    return {"best": best, "table": table}


def tune_plan(lik, precision="fp32", iters=20, shapes=None):
    """Tune on one Lik's current full plan (``lik._prep`` done); the time is
    the walker kernel's mean over `iters` back-to-back runs."""
    from .plan import Plan
    shapes = shapes or candidates(precision, active_components(lik))

    def measure():
        plan = Plan(lik, precision)
        try:
            plan.time(3)
            return plan.time(iters)["kernel_ms"]
        finally:
            plan.close()

    return _sweep(lik.lib, shapes, measure)


def tune_mc3(lib, make, precision="fp32", kact=4, gens=32, warm=16, shapes=None):
    """Tune on an MC3 run.  ``make()`` builds an ``Mc3`` with the shape
    that is set; each candidate runs `warm` generations, then `gens` more,
    and its time is their device time (``cxgMc3Run``) per generation.  MC3
    walks short dirty paths over many (chain, tile) items, so per-tile
    costs weigh more there than on a full plan, and the two can prefer
    different tiles."""
    shapes = shapes or candidates(precision, kact, tpps=(1,), ppts=(1,),
                                  budgets=(0, 24 << 10), lanes=(1,))

    def measure():
        m = make()
        try:
            m.run(warm)
            return 1e3 * m.run(gens) / gens
        finally:
            m.close()

    return _sweep(lib, shapes, measure)


def tune_batch(liks, precision="fp32", iters=5, shapes=None):
    """Tune on a batch of planned Liks (one persistent launch); the time is
    the walker's mean over `iters` graph replays."""
    from .batch import Batch
    lk = liks[0]
    shapes = shapes or candidates(precision, active_components(lk),
                                  lanes=(1,))

    def measure():
        b = Batch(liks, precision)
        try:
            b.time(2)
            return b.time(iters)["walk_ms"]
        finally:
            b.close()

    return _sweep(lk.lib, shapes, measure)
