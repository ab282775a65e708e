"""Autotuner of the NUFFT plans (bin size and points per subproblem) and of the tensor-core
distance kernel (reference tile and TMA ring depth).

The bin size sets the shared-memory subgrid of a subproblem ((bin_size + w)^3 cells, so the
CTAs per SM) and, with the point density, how many points share a window; the points per
subproblem set the CTA count and how often a bin's subgrid is flushed.  The best pair
depends on the point distribution, the grid size and the GPU, so it is measured: for each
candidate a scratch plan gets the caller's points, and ``reuse`` executes after one sort
are timed with CUDA events (the sort counts once; a CG solve that spreads once per sort
has reuse 1, a plan applied to many mode sets more).  Results are cached in memory and in
a JSON file (``CMT_TUNE_CACHE``, default ``~/.cache/cmtip_gb300/tune.json``) keyed by GPU,
library version and problem signature.  The reference has no counterpart: finufft chooses
its own bins.

The distance kernel's tile (``TILES``: references per tile 128 / 256, ring stages) trades
per-unit epilogue work and the unit count (how evenly the persistent CTAs share the work)
against shared memory for the TMA ring; ``autotune_match`` times each on the caller's
matchers (one grouped launch), results being independent of the tile.
"""
from __future__ import annotations

import json
import os
import threading

import torch

from . import _lib
from .nufft import DEFAULT_EPS, Plan

BIN_SIZES = (4, 5, 8, 16)
TILES = ((256, 4), (256, 3), (128, 6), (128, 4))
MAXSUBS = (2048, 4096, 8192, 16384)

_mem = {}
_lock = threading.Lock()


def _cache_path():
    return os.environ.get("CMT_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "cmtip_gb300",
                                                         "tune.json"))


def _load_file():
    try:
        with open(_cache_path()) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _store_file(key, val):
    path = _cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        d = _load_file()
        d[key] = val
        tmp = path + ".tmp"
        with open(tmp, "w") as fh:
            json.dump(d, fh, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass  # a read-only home only loses the persistence


def signature(nufft_type, M, prec, eps, n_points, tag=""):
    """Cache key: GPU, library version, transform and a power-of-two bucket of the point count."""
    dev = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
    bucket = max(0, int(n_points).bit_length() - 1)
    return f"{dev}|{_lib.version()}|t{nufft_type}|M{M}|p{prec}|eps{eps:g}|N2^{bucket}|{tag}"


def candidates(plan: Plan, bin_sizes=BIN_SIZES, maxsubs=MAXSUBS):
    """The (bin_size, maxsub) pairs the plan accepts (shared memory permitting)."""
    out = []
    for bs in bin_sizes:
        for ms in maxsubs:
            try:
                plan.set_tuning(bs, ms)
            except (ValueError, _lib.CmtError):
                continue
            out.append((bs, ms))
    return out


def _time_ms(fn, reps):
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    fn()  # warm-up (allocations, kernel attributes)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def autotune(nufft_type, M, set_points, data, prec=32, eps=DEFAULT_EPS, isign=None, reuse=1, real_out=True,
             tag="", n_points=None, bin_sizes=BIN_SIZES, maxsubs=MAXSUBS, cache=True, reps=2):
    """Best (bin_size, maxsub) for a transform on the caller's points.

    set_points(plan) gives a plan its points (e.g. ``lambda p: p.set_pts_quat(inv, ppr, rext)``);
    data is the execute input (None: unit strengths, type 1).  Returns
    ``dict(bin_size, maxsub, ms, table)`` with ms = sort + reuse x execute."""
    plan = Plan(nufft_type, M, eps=eps, isign=isign, prec=prec)
    try:
        set_points(plan)
        key = signature(nufft_type, M, prec, eps, n_points or plan.N, tag)
        if cache:
            with _lock:
                hit = _mem.get(key) or _load_file().get(key)
            if hit:
                _mem[key] = hit
                return dict(hit, cached=True)
        table = []
        for bs, ms in candidates(plan, bin_sizes, maxsubs):
            plan.set_tuning(bs, ms)
            t_sort = _time_ms(lambda: set_points(plan), reps)
            t_exec = _time_ms(lambda: plan.execute(data, real_out=real_out), reps)
            table.append(dict(bin_size=bs, maxsub=ms, sort_ms=t_sort, exec_ms=t_exec, ms=t_sort + reuse * t_exec))
        best = min(table, key=lambda r: r["ms"])
        res = dict(bin_size=best["bin_size"], maxsub=best["maxsub"], ms=best["ms"], table=table)
        if cache:
            with _lock:
                _mem[key] = res
            _store_file(key, res)
        return dict(res, cached=False)
    finally:
        plan.close()


def apply(plan: Plan, cfg) -> Plan:
    """Set a tuned configuration on a plan (before set_pts)."""
    return plan.set_tuning(int(cfg["bin_size"]), int(cfg["maxsub"]))


def match_signature(matchers):
    """Cache key of a distance problem: GPU, library version, form and power-of-two buckets of
    the image and reference counts and of the pixel count of every matcher."""
    dev = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
    b = lambda v: max(0, int(v).bit_length() - 1)
    shapes = ",".join(f"{b(m.n_img)}/{b(m.n_ref)}/{b(m.n_pix)}" for m in matchers)
    return f"{dev}|{_lib.version()}|match|m{matchers[0].mode}|{shapes}"


def autotune_match(matchers, tiles=TILES, cache=True, reps=2):
    """Best tile for one grouped tensor-core launch over ``matchers`` (data and references
    set): each candidate is timed by CUDA events over ``reps`` runs after a warm-up, and the
    winner is left set on the matchers.  Returns dict(bn, stages, ms, table)."""
    from .alignment import Matcher
    matchers = list(matchers)
    key = match_signature(matchers)
    if cache:
        with _lock:
            hit = _mem.get(key) or _load_file().get(key)
        if hit:
            _mem[key] = hit
            for m in matchers:
                m.set_tile(hit["bn"], hit["stages"])
            return dict(hit, cached=True)
    table = []
    for bn, st in tiles:
        for m in matchers:
            m.set_tile(bn, st)
        ms = _time_ms(lambda: Matcher.run_many(matchers), reps)
        table.append(dict(bn=bn, stages=st, ms=ms))
    best = min(table, key=lambda r: r["ms"])
    for m in matchers:
        m.set_tile(best["bn"], best["stages"])
    res = dict(bn=best["bn"], stages=best["stages"], ms=best["ms"], table=table)
    if cache:
        with _lock:
            _mem[key] = res
        _store_file(key, res)
    return dict(res, cached=False)
