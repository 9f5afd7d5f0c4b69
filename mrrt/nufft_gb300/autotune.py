"""Autotuner for the tile shapes of a plan: picks the gather tile and the
spread tile for one geometry, trajectory and coil count by timing the two
interpolation kernels on the GPU.

The gather tile only affects the forward interpolation and the spread tile
only the adjoint, so the two are tuned independently: every candidate is a
real plan (sorted lists for that tiling) and is timed with CUDA events on
the current stream after a warm-up launch, median of ``reps`` launches.
Results are cached in memory, and in a JSON file when ``cache_path`` (or the
``GBNUFFT_TUNE_CACHE`` environment variable) names one, keyed by geometry,
per-frame sample counts, a SHA-256 digest of the trajectory itself, coil
count and precision.

The reference has no tile shapes to tune (its CPU kernels loop over samples,
its CuPy kernels launch one thread per sample).
"""
import hashlib
import json
import os
import threading

import numpy as np
import torch

__all__ = ["candidate_tiles", "tune_series", "tune_operator"]

_cache = {}
_lock = threading.Lock()


def candidate_tiles(ndim):
    """(gather tiles, spread tiles) tried for a dimensionality, in the
    reference's axis order.  Spread tiles are whole 4 x 4 (x 1) register
    blocks, at most 8 per tile (one warp each); the planner shrinks gather
    tiles whose halo does not fit shared memory."""
    if ndim == 1:
        return [(128,), (256,), (512,)], [(128,), (64,), (32,)]
    if ndim == 2:
        return ([(16, 8), (16, 16), (32, 8), (32, 16), (32, 32), (64, 16)],
                [(16, 8), (8, 16), (32, 4), (8, 8), (16, 4)])
    return ([(8, 8, 4), (8, 8, 8), (16, 8, 4), (16, 16, 2), (8, 8, 2)],
            [(8, 8, 2), (16, 8, 1), (8, 4, 4), (16, 4, 2), (4, 4, 8)])


def trajectory_digest(omegas):
    """SHA-256 of every frame's coordinates (as float64, row-major), so that
    two trajectories with the same sample counts get different cache keys."""
    h = hashlib.sha256()
    for om in omegas:
        a = om.detach().cpu().numpy() if isinstance(om, torch.Tensor) else np.asarray(om)
        a = np.ascontiguousarray(a, dtype=np.float64)
        h.update(np.asarray(a.shape, dtype=np.int64).tobytes())
        h.update(a.tobytes())
    return h.hexdigest()[:32]


def _key(kind, Nd, Kd, Jd, counts, coils, precision, digest):
    return "%s|%s|%s|%s|%s|%d|%s|%s" % (kind, tuple(Nd), tuple(Kd), tuple(Jd),
                                       ",".join(str(int(c)) for c in counts), int(coils), precision,
                                       digest)


def _load(path):
    if path and os.path.exists(path):
        try:
            with open(path) as f:
                return json.load(f)
        except (OSError, ValueError):
            return {}
    return {}


def _store(path, key, value):
    if not path:
        return
    data = _load(path)
    data[key] = value
    tmp = "%s.%d.tmp" % (path, os.getpid())
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def _time(fn, reps):
    fn()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    torch.cuda.synchronize()
    for a, b in ev:
        a.record()
        fn()
        b.record()
    torch.cuda.synchronize()
    return float(np.median([a.elapsed_time(b) for a, b in ev]))


def _sweep(make, Kd, coils, frames, gathers, spreads, reps):
    Kp = int(np.prod(Kd))
    report = {"gather": [], "spread": []}
    grid = None
    for t in gathers:
        s = make(tile=t, stile=None)
        P = s.plan
        if grid is None:
            grid = torch.randn((frames * coils * Kp,), dtype=P.ctype, device=P.device)
        y = torch.empty((coils * P.M_total,), dtype=P.ctype, device=P.device)
        report["gather"].append((list(t), _time(lambda: P.interp_forward(grid, y, coils), reps)))
        del s, P
    for t in spreads:
        s = make(tile=None, stile=t)
        P = s.plan
        y = torch.randn((coils * P.M_total,), dtype=P.ctype, device=P.device)
        g = torch.empty((frames * coils * Kp,), dtype=P.ctype, device=P.device)
        report["spread"].append((list(t), _time(lambda: P.interp_adjoint(y, g, coils), reps)))
        del s, P
    best_g = min(report["gather"], key=lambda r: r[1])[0]
    best_s = min(report["spread"], key=lambda r: r[1])[0]
    return tuple(best_g), tuple(best_s), report


def tune_series(Nd, omegas, Jd=6, Kd=None, Ld=1024, coils=1, precision="single", reps=5,
                cache_path=None, candidates=None):
    """Best (tile, stile) for a ``NufftSeries`` of these frames; returns
    ``(tile, stile, report)`` where report lists (tile, ms) per candidate."""
    from .series import NufftSeries

    ndim = len(Nd)
    Jd = (Jd,) * ndim if np.isscalar(Jd) else tuple(Jd)
    Kd = tuple(Kd) if Kd is not None else tuple(int(1.5 * n) for n in Nd)
    counts = [int(np.asarray(o).shape[0]) for o in omegas]
    key = _key("series", Nd, Kd, Jd, counts, coils, precision, trajectory_digest(omegas))
    path = cache_path or os.environ.get("GBNUFFT_TUNE_CACHE")
    with _lock:
        if key in _cache:
            return _cache[key]
        stored = _load(path).get(key)
    if stored is not None:
        res = (tuple(stored["tile"]), tuple(stored["stile"]), stored["report"])
        with _lock:
            _cache[key] = res
        return res
    gathers, spreads = candidates or candidate_tiles(ndim)

    def make(tile, stile):
        return NufftSeries(Nd, omegas, Jd=Jd, Kd=Kd, Ld=Ld, precision=precision, coils=coils,
                           tile=tile, stile=stile)

    tile, stile, report = _sweep(make, Kd, coils, len(counts), gathers, spreads, reps)
    res = (tile, stile, report)
    with _lock:
        _cache[key] = res
    _store(path, key, {"tile": list(tile), "stile": list(stile), "report": report})
    return res


def tune_operator(Nd, omega, Jd=6, Kd=None, Ld=1024, coils=1, precision="single", reps=5,
                  cache_path=None, candidates=None):
    """Best (tile, stile) for a single-frame operator (``NufftBase(...,
    tile=..., stile=...)``); same return value as ``tune_series``."""
    return tune_series(Nd, [omega], Jd=Jd, Kd=Kd, Ld=Ld, coils=coils, precision=precision,
                       reps=reps, cache_path=cache_path, candidates=candidates)
