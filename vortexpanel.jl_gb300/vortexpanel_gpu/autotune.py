"""Autotuner of the far tier's tile: how many test triangles one CTA of the far kernel holds in shared memory against
each 128-source tile (vp_set_far_tile). Fewer test triangles per tile give more CTAs and less shared memory per
CTA; more give more reuse of each source tile loaded into registers. The best choice depends on the mesh size and the
precision, so it is measured.

sweep() times the far phase (CUDA events on the library's stream, ctx.phase_times) of a family of meshes for every
tile a precision has, and table() turns the measurements into a choice per precision and size class. Running this
module on a GPU writes both to a JSON file:

    python -m vortexpanel_gpu.autotune --out tuning.json [--quick]

The package reads `tuning.json` beside this module (the committed sweep); assemble() and assemble_batch() set the
tile of the mesh's size class before each call. Without the file the library's defaults hold (4 in FP64, 8 mixed).
"""
from __future__ import annotations

import json
import math
import os
import time

import numpy as np

TILES = {"fp64": (1, 2, 4), "mixed": (2, 4, 8)}
TABLE_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning.json")
_table = None


def load_table(path: str = TABLE_FILE):
    """the committed choice per precision: {"fp64": [{"max_ntri": n, "tile": t}, ...], "mixed": [...]}, or None"""
    global _table
    if _table is None or path != TABLE_FILE:
        t = None
        if os.path.exists(path):
            with open(path) as f:
                t = json.load(f).get("table")
        if path != TABLE_FILE:
            return t
        _table = t if t is not None else {}
    return _table or None


def far_tile(precision: str, ntri: int, table=None):
    """the tuned tile of a mesh of ntri triangles (None: keep the library's default)"""
    table = table if table is not None else load_table()
    if not table or precision not in table:
        return None
    for e in sorted(table[precision], key=lambda e: e["max_ntri"]):
        if ntri <= e["max_ntri"]:
            return int(e["tile"])
    rows = table[precision]
    return int(max(rows, key=lambda e: e["max_ntri"])["tile"]) if rows else None


def apply(ctx, precision: str, ntri: int) -> None:
    """set the context's far tile for a mesh of ntri triangles from the committed table"""
    from . import _lib
    t = far_tile(precision, ntri)
    if t is not None:
        prec = _lib.VP_MIXED if precision == "mixed" else _lib.VP_FP64
        _lib.check(ctx.h, _lib.load().vp_set_far_tile(ctx.h, prec, int(t)))


def wing_family(quick: bool = False):
    """the sizes the sweep measures: the AR 4-12 wing family of the batch, ~2k to ~25k triangles"""
    from . import meshes
    sizes = [(28, 18, 4.0), (44, 28, 6.0), (64, 40, 8.0), (80, 44, 9.0), (112, 56, 12.0)]
    if quick:
        sizes = sizes[:2]
    out = []
    a = math.radians(5.0)
    V = np.array([math.cos(a), 0.0, math.sin(a)])
    for nc, ns, ar in sizes:
        w = meshes.wing(nc, ns, aspect=ar)
        wake = meshes.build_wake(w.g, w.dm, (1.0, 0.0, 0.0), length=2.5)
        out.append((f"wing {nc}x{ns} AR{ar:g}", w.g, w.dm, V, wake))
    return out


def sweep(cases, precisions=("mixed", "fp64"), reps: int = 3, ctx=None):
    """far-phase milliseconds (the minimum of reps, after one warm-up) per case, precision and tile"""
    from . import _lib, api
    ctx = ctx or api.default_context()
    L = _lib.load()
    recs = []
    for name, g, dm, V, wake in cases:
        els = api.build_elements(g)
        sig = api.source_strengths(els, V)
        for prec in precisions:
            code = _lib.VP_MIXED if prec == "mixed" else _lib.VP_FP64
            default = L.vp_get_far_tile(ctx.h, code)
            opts = api.AssemblyOptions(precision=prec)
            for tile in TILES[prec]:
                _lib.check(ctx.h, L.vp_set_far_tile(ctx.h, code, tile))
                times = []
                for k in range(reps + 1):
                    ctx.phase_times(reset=True)
                    A, b, _ = api.assemble(g, dm, els, sig, V, opts=opts, wake=wake, ctx=ctx, tune=False)
                    del A
                    ph, _ = ctx.phase_times(reset=True)
                    if k:
                        times.append(ph["far"])
                recs.append({"case": name, "ntri": int(g.ntri), "precision": prec, "tile": tile,
                             "far_ms": float(min(times)), "far_ms_all": [float(t) for t in times]})
            _lib.check(ctx.h, L.vp_set_far_tile(ctx.h, code, default))
    return recs


def table(recs):
    """the fastest tile per precision and case; a case's class reaches halfway (geometrically) to the next size"""
    out = {}
    for prec in sorted({r["precision"] for r in recs}):
        best = {}
        for r in recs:
            if r["precision"] != prec:
                continue
            b = best.get(r["ntri"])
            if b is None or r["far_ms"] < b["far_ms"]:
                best[r["ntri"]] = r
        ns = sorted(best)
        rows = []
        for i, n in enumerate(ns):
            hi = int(math.sqrt(n * ns[i + 1])) if i + 1 < len(ns) else 2**31 - 1
            rows.append({"max_ntri": hi, "tile": best[n]["tile"]})
        out[prec] = rows
    return out


def main(argv=None):
    import argparse
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--out", default=TABLE_FILE)
    ap.add_argument("--quick", action="store_true")
    ap.add_argument("--reps", type=int, default=3)
    args = ap.parse_args(argv)
    t0 = time.time()
    recs = sweep(wing_family(args.quick), reps=args.reps)
    res = {"what": "far-tier tile sweep: far phase ms per mesh, precision and test triangles per tile",
           "table": table(recs), "sweep": recs, "seconds": time.time() - t0}
    with open(args.out, "w") as f:
        json.dump(res, f, indent=1)
    for r in recs:
        print(f"{r['case']:24s} {r['ntri']:6d} {r['precision']:5s} tile {r['tile']}  far {r['far_ms']:8.2f} ms")
    print(json.dumps(res["table"]))


if __name__ == "__main__":
    main()
