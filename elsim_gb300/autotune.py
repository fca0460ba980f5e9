"""Launch-shape autotuner of the mixed-precision solver.

For one context (one grid size) it times complete solves of a representative
problem under each candidate setting and keeps the fastest:

* zc32   -- z planes per CTA of the FP32 stencil (TMA tile depth, or planes
            per thread of the register-tiled kernel),
* chunk  -- CG iterations per captured graph chunk (per two-iteration unit
            in the mixed solver),
* no_tma -- register-tiled instead of TMA-staged stencil.

Each candidate is timed with the solver's own CUDA-event clock after one
warm-up solve (which also captures its graph).  Results are cached in memory
per grid shape, so every context of a batch with the same shape reuses them.
"""
from __future__ import annotations

import itertools

from . import sbm

DEFAULT_SPACE = {"zc32": (8, 16, 32), "chunk": (8, 16), "no_tma": (False, True)}
_cache: dict[tuple, dict] = {}


def tune(ctx: "sbm.Context", load, tol: float = 1e-8, precond: int = sbm.PC_JACOBI,
         space: dict | None = None, reps: int = 1) -> dict:
    """Tunes `ctx`; `load()` re-uploads the problem's fields (x is overwritten
    by every solve).  Returns {"best": {...}, "trials": [...]} and leaves the
    best setting active on the context."""
    key = tuple(ctx.shape)
    if key in _cache:
        best = _cache[key]["best"]
        ctx.set_tuning(zc32=best["zc32"], chunk=best["chunk"], no_tma=best["no_tma"])
        return _cache[key]
    space = space or DEFAULT_SPACE
    trials = []
    names = list(space)
    for values in itertools.product(*(space[n] for n in names)):
        cfg = dict(zip(names, values))
        ctx.set_tuning(zc32=cfg["zc32"], chunk=cfg["chunk"], no_tma=cfg["no_tma"])
        times = []
        for r in range(reps + 1):
            load()
            info = ctx.cg_solve(op=sbm.OP_GENERIC, bc_x0=sbm.BC_ZERO, bc_x1=sbm.BC_ZERO,
                                scale=1.0, tol=tol, max_it=200000, stop_rule=sbm.STOP_REL_RES,
                                precision=sbm.PREC_MIXED, precond=precond)
            if r:
                times.append(info["ms"])
        trials.append({**cfg, "ms": min(times), "iters": info["iters"]})
    best = min(trials, key=lambda t: t["ms"])
    ctx.set_tuning(zc32=best["zc32"], chunk=best["chunk"], no_tma=best["no_tma"])
    out = {"best": best, "trials": trials}
    _cache[key] = out
    return out


def apply_cached(ctx: "sbm.Context") -> bool:
    """Applies a cached result for this context's shape, if any."""
    res = _cache.get(tuple(ctx.shape))
    if not res:
        return False
    b = res["best"]
    ctx.set_tuning(zc32=b["zc32"], chunk=b["chunk"], no_tma=b["no_tma"])
    return True
