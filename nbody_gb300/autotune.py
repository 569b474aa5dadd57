"""Autotuner front end with a persistent cache.

The timing itself is native (nbg_autotune / nbg_ensemble_autotune time every
candidate configuration on the device with CUDA events and keep the fastest).
This module remembers the winners per GPU model, force path and problem size,
so a later run on the same kind of GPU applies them without timing again:

    from nbody_gb300.autotune import tune
    report = tune(engine)          # engine: NbodyEngineGB300 or Ensemble

Cache file: $NBG_TUNE_CACHE, else ~/.cache/nbody_gb300/tune.json.  Entries are
keyed "<gpu name>|<SM count>|<path variant>|<size bucket>", the size bucket
being N rounded up to a power of two (total bodies for an ensemble).
"""
from __future__ import annotations

import json
import os
import tempfile
from pathlib import Path
from typing import Callable, Optional


def default_cache_path() -> Path:
    env = os.environ.get("NBG_TUNE_CACHE")
    if env:
        return Path(env)
    return Path.home() / ".cache" / "nbody_gb300" / "tune.json"


def size_bucket(n: int) -> int:
    """N rounded up to a power of two (1 for N <= 1)."""
    n = int(n)
    return 1 if n <= 1 else 1 << (n - 1).bit_length()


def cache_key(gpu: str, sm_count: int, variant: str, n: int) -> str:
    return f"{gpu}|{int(sm_count)}|{variant}|{size_bucket(n)}"


class TuneCache:
    """A JSON dictionary key -> {"best": {...}, "report": {...}} on disk."""

    def __init__(self, path: Optional[Path] = None):
        self.path = Path(path) if path is not None else default_cache_path()
        self._data: dict = {}
        if self.path.exists():
            try:
                self._data = json.loads(self.path.read_text())
            except (OSError, ValueError):
                self._data = {}  # unreadable cache: start over

    def get(self, key: str) -> Optional[dict]:
        ent = self._data.get(key)
        return dict(ent["best"]) if ent and isinstance(ent.get("best"), dict) else None

    def put(self, key: str, best: dict, report: dict) -> None:
        self._data[key] = {"best": dict(best), "report": report}
        self.path.parent.mkdir(parents=True, exist_ok=True)
        fd, tmp = tempfile.mkstemp(dir=self.path.parent, prefix=".tune-", suffix=".json")
        with os.fdopen(fd, "w") as fh:
            json.dump(self._data, fh, indent=1, sort_keys=True)
        os.replace(tmp, self.path)  # atomic on POSIX: readers never see half a file

    def __len__(self) -> int:
        return len(self._data)


def _gpu_identity(device: int) -> tuple:
    import torch  # plumbing only: the device name and SM count
    props = torch.cuda.get_device_properties(device)
    return props.name, props.multi_processor_count


def tune(target, reps: int = 3, cache: Optional[TuneCache] = None, force: bool = False,
         identity: Optional[Callable[[int], tuple]] = None) -> dict:
    """Apply cached winners for `target` (an engine or an ensemble that is
    initialised), or run its native autotuner and cache the result.

    Returns {"source": "cache" | "measured", "best": {...}, "report": {...} | None}.
    """
    cache = cache if cache is not None else TuneCache()
    gpu, sms = (identity or _gpu_identity)(target.device)
    n = int(target.counts.sum()) if hasattr(target, "counts") else target.problem_size() // 6
    key = cache_key(gpu, sms, target.tune_variant(), n)
    best = None if force else cache.get(key)
    if best is not None:
        for k, v in best.items():
            target.tune_set(k, int(v))
        return {"source": "cache", "key": key, "best": best, "report": None}
    report = target.autotune(reps)
    best = {k: int(v) for k, v in report["best"].items()}
    cache.put(key, best, report)
    return {"source": "measured", "key": key, "best": best, "report": report}
