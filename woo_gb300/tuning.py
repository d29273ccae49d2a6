"""Launch shapes picked by the engine's autotuner (wdem_autotune), cached per GPU and workload.

The key is the device name with a coarse description of the workload (particle count to the nearest
power of two, contact law, periodic cell, ellipsoids, number of batched scenes); the cache is a JSON file
(WOO_GB300_TUNING, default ~/.cache/woo_gb300/launch_shapes.json).  A cached shape is applied as is; a
missing one is tuned on a probe handle holding a copy of the state (the tuning runs steps, which must not
advance the caller's simulation), or on the handle itself when no probe is given (its run then advances
by the tuning steps; results do not depend on the shape), and stored.
"""
import json
import math
import os

from . import abi


def cache_path():
    return os.environ.get("WOO_GB300_TUNING",
                          os.path.join(os.path.expanduser("~"), ".cache", "woo_gb300", "launch_shapes.json"))


def device_name(device=0):
    try:
        import torch
        return torch.cuda.get_device_name(device)
    except Exception:
        return f"cuda:{device}"


def workload_key(n, law, periodic=False, ellipsoids=False, scenes=1):
    law_name = {abi.LAW_IDEALELPL: "IdealElPl", abi.LAW_HERTZ_DMT: "HertzDMT"}.get(law, str(law))
    return (f"n~2^{int(round(math.log2(max(n, 1))))}|{law_name}|{'peri' if periodic else 'box'}|"
            f"{'ell' if ellipsoids else 'sph'}|scenes~2^{int(round(math.log2(max(scenes, 1))))}")


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def lookup(device, key, path=None):
    return _load(path or cache_path()).get(f"{device_name(device)}|{key}")


def store(device, key, entry, path=None):
    path = path or cache_path()
    data = _load(path)
    data[f"{device_name(device)}|{key}"] = entry
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def tuned(handle, device, key, steps_per_candidate=10, path=None, probe=None):
    """Apply the cached launch shape for (device, key), or tune it and cache it: on probe() (a callable
    returning a handle with a copy of the state, closed afterwards) when given, else on `handle`.  Returns
    the entry: dict(shape=..., ms=..., ms_start=..., cached=bool)."""
    hit = lookup(device, key, path)
    if hit is not None:
        handle.set_launch_shape(**hit["shape"])
        return dict(hit, cached=True)
    if probe is not None:
        t = probe()
        try:
            res = t.autotune(steps_per_candidate)
        finally:
            t.close()
        handle.set_launch_shape(**res["shape"])
    else:
        res = handle.autotune(steps_per_candidate)
    store(device, key, res, path)
    return dict(res, cached=False)
