"""Launch-shape autotuner for the fused evolve step.

The knobs are the block sizes of the three kernels of a step (flux,
update, distribute), the persistent double-buffered mixed flux, and the
number of steps captured per CUDA graph (``swgpu_set_launch_config``).
Results do not depend on them, so tuning is pure measurement: each
candidate shape runs whole steps through the device-resident loop (CUDA
graphs, programmatic dependent launches, exactly as evolve issues them),
timed with CUDA events on the handle's stream (``swgpu_evolve_run_timed``),
one knob at a time from the current best; a candidate is kept when its step
is at least 1% faster.  Timing kernels one by one instead would miss what the
graph overlaps (a persistent flux that looks faster alone holds the SMs
against the next kernel's early blocks).  The steps the measurement runs
advance the model: tune a throwaway copy of a domain (``tune_domain``
does), or tune before setting the initial state.

Chosen shapes are cached in a JSON file keyed by device, precision, method
and mesh size (rounded to a power of two), at ``$ANUGA_CUDA_TUNE_CACHE`` or
``~/.cache/anuga_cuda/autotune.json``.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os

from . import _lib
from ._lib import check, lib

__all__ = ["get_config", "set_config", "tune_handle", "tune_domain", "cache_path",
           "cached_config", "DEFAULT_CANDIDATES", "STEPS_PER_GRAPH"]

DEFAULT_CANDIDATES = {"flux": (64, 128, 256), "update": (128, 256, 512),
                      "distribute": (128, 256, 512)}
_FIELD = {"flux": "flux_block", "update": "update_block", "distribute": "distribute_block"}


def get_config(h) -> dict:
    c = _lib.LaunchConfig_t()
    check(lib().swgpu_get_launch_config(h, C.byref(c)), h)
    return {"flux_block": c.flux_block, "update_block": c.update_block,
            "distribute_block": c.distribute_block, "steps_per_graph": c.steps_per_graph,
            "flux_pipelined": c.flux_pipelined, "dependent_launch": c.dependent_launch}


def set_config(h, cfg: dict) -> None:
    c = _lib.LaunchConfig_t(int(cfg["flux_block"]), int(cfg["update_block"]),
                            int(cfg["distribute_block"]), int(cfg.get("steps_per_graph", 16)),
                            int(cfg.get("flux_pipelined", 0)),
                            int(cfg.get("dependent_launch", get_config(h)["dependent_launch"])))
    check(lib().swgpu_set_launch_config(h, C.byref(c)), h)


STEPS_PER_GRAPH = (8, 16, 32)
KEEP = 0.99   # a candidate replaces the best when its step time is below KEEP x best


def _step_ms(h, steps):
    """Device milliseconds per step of ``steps`` steps of the evolve loop."""
    st, ms = _lib.State_t(), C.c_double()
    check(lib().swgpu_evolve_run_timed(h, int(steps), C.byref(st), C.byref(ms)), h)
    return ms.value / max(int(steps), 1)


def _time_shape(h, cfg, steps):
    """Best of two timed runs of ``steps`` steps with shape ``cfg``, after one
    untimed graph (capture and first launch)."""
    set_config(h, cfg)
    _step_ms(h, cfg.get("steps_per_graph", 16))
    return min(_step_ms(h, steps), _step_ms(h, steps))


def tune_handle(h, steps=64, candidates=None, ensemble=False) -> dict:
    """Tune the launch shape of handle ``h`` in place (its evolve must have
    been started, with no yield or final time within the steps tuning
    runs); returns {"config", "default_ms", "tuned_ms"}: the chosen shape and
    the device milliseconds per whole step of the starting and the chosen
    shape.  ``ensemble`` limits update/distribute blocks to 256."""
    cand = dict(DEFAULT_CANDIDATES)
    cand.update(candidates or {})
    if ensemble:
        cand["update"] = tuple(b for b in cand["update"] if b <= 256)
        cand["distribute"] = tuple(b for b in cand["distribute"] if b <= 256)
    best = get_config(h)
    best_ms = start_ms = _time_shape(h, best, steps)
    trials = []
    for kernel, values in cand.items():
        trials += [{_FIELD[kernel]: v} for v in values]
        if kernel == "flux":
            # persistent double-buffered flux (mixed precision, tiles <= 128)
            trials += [{"flux_block": v, "flux_pipelined": 1} for v in values if v <= 128]
    trials += [{"steps_per_graph": n} for n in STEPS_PER_GRAPH]
    for change in trials:
        trial = dict(best, **change)
        if "flux_block" in change and "flux_pipelined" not in change:
            trial["flux_pipelined"] = 0
        if trial == best:
            continue
        try:
            t = _time_shape(h, trial, steps)
        except _lib.SwgpuError:
            set_config(h, best)
            continue
        if t < KEEP * best_ms:
            best, best_ms = trial, t
    set_config(h, best)
    return {"config": best, "default_ms": start_ms, "tuned_ms": best_ms}


def cache_path() -> str:
    return os.environ.get("ANUGA_CUDA_TUNE_CACHE") or os.path.join(
        os.path.expanduser("~"), ".cache", "anuga_cuda", "autotune.json")


def _device_name() -> str:
    buf = C.create_string_buffer(256)
    check(lib().swgpu_device_info(buf, 256), None)
    return buf.value.decode()


def _key(precision, n, method="euler", ensemble=False) -> str:
    bucket = 1 << max(int(math.log2(max(n, 1))), 0)
    return f"{_device_name()}|{precision}|{method}|{'ensemble' if ensemble else 'single'}|{bucket}"


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def cached_config(precision, n, method="euler", ensemble=False):
    return _load().get(_key(precision, n, method, ensemble))


def _store(key, cfg):
    data = _load()
    data[key] = cfg
    path = cache_path()
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def tune_domain(domain, steps=64, use_cache=True) -> dict:
    """Choose the launch shape of a GPU_domain: from the cache when it holds
    one for this device, precision, timestepping method and size; otherwise
    by tuning a copy of the domain (same mesh, parameters, state and
    boundaries) and caching the result.  The shape is applied to
    ``domain``; returns the tuning record (or {"config", "cached": True})."""
    from .gpu_domain import GPU_domain
    key = _key(domain.precision, domain.number_of_elements, domain.get_timestepping_method())
    if use_cache:
        cfg = _load().get(key)
        if cfg:
            set_config(domain._h, cfg)
            return {"config": cfg, "cached": True}
    twin = GPU_domain(mesh=domain.mesh, parameters=domain.parameters,
                      precision=domain.precision)
    for name in ("elevation", "friction", "stage", "xmomentum", "ymomentum"):
        q = domain.quantities[name]
        twin._upload(name, domain._to_internal(q.centroid_values),
                     domain._to_internal(q.vertex_values), domain._to_internal(q.edge_values))
    twin.set_boundary(dict(domain.boundary_map))
    twin.set_timestepping_method(domain.get_timestepping_method())
    twin.evolve_steps(0)
    rec = tune_handle(twin._h, steps)
    set_config(domain._h, rec["config"])
    if use_cache:
        _store(key, rec["config"])
    return rec
