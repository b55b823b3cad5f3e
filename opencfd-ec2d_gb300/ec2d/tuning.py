"""Autotuner cache: the launch choices of ec2d_autotune kept in a JSON file,
keyed by the context's launch signature (ec2d_launch_signature), so that a
later run of the same cases on the same kind of device applies them at once
instead of timing every candidate again.

The signature names everything the timings depend on: the device (name,
compute capability, SM count), the library version and a digest of its
sources, the method flags and precisions, the number of cases and every
level's block shapes with their variables.  A run whose signature is in the
file gets the stored choices (ec2d_set_launch_config); any other runs the
autotuner and adds its result.  None of the choices changes the
discretisation, so a stale entry can only cost speed, never the answer.

File layout (one file may hold many signatures):

    {"format": "ec2d-launch-cache-1",
     "entries": {"<sha256 of the signature, 20 hex>":
                 {"signature": "...", "config": {"lusgs_cs": 0, "rows": 12,
                  "lanes": 0, "concurrent": 1, "tile_residual": 0},
                  "ms_per_step": 0.89, "trial_steps": 5}}}

The file is replaced atomically (written beside it, then renamed), so
processes sharing it never read a torn file; of two that tune the same
signature at once, the last writer's entry stays.

    from ec2d import tuning
    result = tuning.autotune_cached(solver, "tuning.json")
"""
from __future__ import annotations

import hashlib
import json
import os
import tempfile
import warnings

FORMAT = "ec2d-launch-cache-1"
ENV = "EC2D_TUNING_CACHE"


def signature_key(signature: str) -> str:
    return hashlib.sha256(signature.encode()).hexdigest()[:20]


def load(path: str) -> dict:
    """The cache's entries; an absent file is empty, an unreadable or foreign
    one is treated as empty (with a warning) and replaced on the next store."""
    if not os.path.exists(path):
        return {}
    try:
        with open(path) as fh:
            doc = json.load(fh)
    except (OSError, ValueError) as e:
        warnings.warn(f"ec2d tuning cache {path} unreadable ({e}); starting a new one")
        return {}
    if not isinstance(doc, dict) or doc.get("format") != FORMAT or not isinstance(doc.get("entries"), dict):
        warnings.warn(f"ec2d tuning cache {path} has another format; starting a new one")
        return {}
    return doc["entries"]


def store(path: str, signature: str, config: dict, ms_per_step: float, trial_steps: int) -> None:
    entries = load(path)
    entries[signature_key(signature)] = {"signature": signature, "config": dict(config),
                                         "ms_per_step": float(ms_per_step), "trial_steps": int(trial_steps)}
    d = os.path.dirname(os.path.abspath(path))
    os.makedirs(d, exist_ok=True)
    fd, tmp = tempfile.mkstemp(prefix=".ec2d_tuning_", suffix=".json", dir=d)
    try:
        with os.fdopen(fd, "w") as fh:
            json.dump({"format": FORMAT, "entries": entries}, fh, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except BaseException:
        if os.path.exists(tmp):
            os.unlink(tmp)
        raise


def lookup(path: str, signature: str):
    """The stored entry of this exact signature, or None."""
    e = load(path).get(signature_key(signature))
    if e is None or e.get("signature") != signature:
        return None
    cfg = e.get("config")
    if not isinstance(cfg, dict):
        return None
    return e


def autotune_cached(solver, path: str | None = None, trial_steps: int = 5, refresh: bool = False) -> dict:
    """The solver's launch choices from the cache at `path` (default: the
    EC2D_TUNING_CACHE environment variable) when its signature is stored
    there, else from ec2d_autotune, whose result is then stored.  With no
    path the autotuner runs and nothing is stored; refresh=True times the
    candidates even when the signature is stored and replaces the entry.

    Returns {"source": "cache" | "autotune", "config": {...},
    "ms_per_step": ms (the autotuner's, or the stored one)}."""
    path = path or os.environ.get(ENV) or None
    sig = solver.launch_signature() if path else None
    if path and not refresh:
        e = lookup(path, sig)
        if e is not None:
            try:
                solver.set_launch_config(e["config"])
            except (KeyError, TypeError, ValueError, RuntimeError) as err:
                warnings.warn(f"ec2d tuning cache entry rejected ({err}); autotuning")
            else:
                return {"source": "cache", "config": solver.launch_config(), "ms_per_step": e.get("ms_per_step")}
    ms = solver.autotune(trial_steps)[3]
    cfg = solver.launch_config()
    if path:
        store(path, sig, cfg, ms, trial_steps)
    return {"source": "autotune", "config": cfg, "ms_per_step": ms}
