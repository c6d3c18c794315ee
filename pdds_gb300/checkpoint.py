"""Checkpoint and resume of an estimation, one knot range at a time.

The reference snapshots its Output/ directory after every outer iteration
(PDDAlgorithms/PDDSparseGM.cpp:997, 3863) and reads the solution back to
resume (Read_Solution, :3451-3502).  Here the unit is finer: the knots with
paths are split into `parts` ranges of hand-out positions, each range is
estimated on its own (pdds_estimate's knot range) and its rows are written
to `directory/part_NNNN.npz` as soon as they are back; a later call with the
same arguments loads the parts on disk and runs only the missing ones.

Every knot draws its own Philox streams (seed, instance, knot, path, step),
so a knot's results do not depend on which other knots ran with it: a run
assembled from parts equals one whole run bit for bit in the replay mode,
and up to summation order in the FP64 and MIXED modes.

`directory/manifest.json` records what the parts belong to (layout, problem,
paths, step, seed, mode and options); a call whose arguments differ raises
instead of mixing two runs.  Parts are written to a temporary name and
renamed, so an interrupted write leaves no partial part behind.
"""
from __future__ import annotations

import json
import os
import zlib

import numpy as np


def _crc(a) -> int:
    return zlib.crc32(np.ascontiguousarray(a).tobytes())


def _jsonable(v):
    if isinstance(v, np.ndarray):
        return {"crc32": _crc(v), "shape": list(v.shape)}
    if isinstance(v, (np.integer, np.floating)):
        return v.item()
    if isinstance(v, (list, tuple)):
        return [_jsonable(x) for x in v]
    return v


def signature(pd, bvp, npaths: int, h: float, parts: int, opts: dict) -> dict:
    """What a set of parts belongs to."""
    tables = None
    if getattr(bvp, "tables", None) is not None:
        coef, g, bounds = bvp.tables
        tables = [_crc(coef), _crc(g), [float(b) for b in bounds]]
    return {
        "K": int(pd.K), "nnz": int(pd.nnz), "n_mc": int(pd.n_mc),
        "layout_crc": [_crc(pd.row_ptr), _crc(pd.col), _crc(pd.x), _crc(pd.y), _crc(pd.order)],
        "problem": [int(bvp.kind), [float(p) for p in bvp.params], bool(bvp.use_cv), tables],
        "npaths": int(npaths), "h": float(h), "parts": int(parts),
        "opts": {k: _jsonable(v) for k, v in sorted(opts.items())},
    }


def part_ranges(n_mc: int, parts: int):
    """[first, count) of each part over the hand-out positions."""
    b = [(p * n_mc) // parts for p in range(parts + 1)]
    return [(b[p], b[p + 1] - b[p]) for p in range(parts)]


def _save(path: str, **arrays):
    tmp = path + ".tmp.npz"  # np.savez keeps a name that ends in .npz
    np.savez(tmp, **arrays)
    os.replace(tmp, path)


def estimate_resumable(pd, directory: str, bvp, npaths: int, h: float, parts: int = 8,
                       max_new_parts: int | None = None, **opts):
    """PDDSparseGM.estimate of every knot, written part by part under
    directory and resumed from the parts found there.  Returns the assembled
    Estimate, or None when max_new_parts parts were run and others remain
    (the caller stopped early: call again to continue).  opts are
    PDDSparseGM.estimate's keyword options (mode, seed, richardson, ...);
    adaptive_n is not allowed (a knot range runs a fixed number of paths)."""
    from .api import Estimate

    if opts.get("adaptive_n"):
        raise ValueError("checkpointed estimates run a fixed number of paths per knot")
    for k in ("knot_first", "knot_count"):
        if k in opts:
            raise ValueError(k + " is set per part")
    parts = max(1, min(int(parts), max(pd.n_mc, 1)))
    os.makedirs(directory, exist_ok=True)
    sig = signature(pd, bvp, npaths, h, parts, opts)
    man = os.path.join(directory, "manifest.json")
    if os.path.exists(man):
        with open(man) as f:
            old = json.load(f)
        if old != json.loads(json.dumps(sig)):
            raise ValueError("checkpoint directory %s holds parts of another run" % directory)
    else:
        with open(man + ".tmp", "w") as f:
            json.dump(sig, f)
        os.replace(man + ".tmp", man)

    rows = np.repeat(np.arange(pd.K), np.diff(pd.row_ptr))
    new = 0
    loaded = []
    for p, (first, count) in enumerate(part_ranges(pd.n_mc, parts)):
        path = os.path.join(directory, "part_%04d.npz" % p)
        if not os.path.exists(path):
            if max_new_parts is not None and new >= max_new_parts:
                return None
            est = pd.estimate(bvp, npaths, h, knot_first=first, knot_count=count, **opts)
            knots = np.flatnonzero(est.npaths > 0)
            ent = np.flatnonzero(np.isin(rows, knots))
            arrays = dict(knots=knots, entries=ent, val=est.val[ent], var=est.var[ent], B=est.B[knots],
                          BB=est.BB[knots], npaths=est.npaths[knots], B_all=est.B, BB_all=est.BB,
                          path_steps=np.int64(est.info.get("path_steps", 0)),
                          ms_paths=np.float64(est.info.get("ms_paths", 0.0)))
            if est.diag is not None:
                arrays["diag"] = est.diag[knots]
            _save(path, **arrays)
            new += 1
        with np.load(path) as z:
            loaded.append({k: z[k] for k in z.files})

    val = np.zeros(pd.nnz)
    var = np.zeros(pd.nnz)
    B = np.zeros(pd.K)
    BB = np.zeros(pd.K)
    kn = np.zeros(pd.K, np.int32)
    diag = None
    # the boundary knots (no paths in any part) take B = g, BB = g^2 from the
    # first part; every other knot is overwritten by the part that ran it
    B[:] = loaded[0]["B_all"]
    BB[:] = loaded[0]["BB_all"]
    for z in loaded:
        k = z["knots"]
        val[z["entries"]] = z["val"]
        var[z["entries"]] = z["var"]
        B[k] = z["B"]
        BB[k] = z["BB"]
        kn[k] = z["npaths"]
        if "diag" in z:
            if diag is None:
                from . import _capi as capi
                diag = np.zeros((pd.K, capi.DIAG_N))
            diag[k] = z["diag"]
    info = {"parts": parts, "parts_run": new, "path_steps": int(sum(int(z["path_steps"]) for z in loaded)),
            "ms_paths": float(sum(float(z["ms_paths"]) for z in loaded)), "paths": int(kn.sum())}
    return Estimate(pd.row_ptr, pd.col, val, var, B, BB, info, kn, diag)
