"""Launch-schedule autotuner control (nca_tune_*): ``set_mode(0 | 1 | 2)``
(heuristics only / cached choices / search on a miss), ``get(key)`` and
``entries()`` (the cached choices), ``clear()``."""
from __future__ import annotations

import ctypes
from pathlib import Path

from . import _lib


def set_mode(mode: int) -> None:
    _lib.call("nca_tune_set_mode", int(mode))


def get(key: str):
    vals = (ctypes.c_int32 * 8)()
    n = ctypes.c_int32(0)
    _lib.call("nca_tune_get", key.encode(), vals, 8, ctypes.byref(n))
    return list(vals[: min(n.value, 8)]) if n.value else None


def clear() -> None:
    _lib.call("nca_tune_clear")


def entries(cache_dir: str | None = None) -> dict:
    """Parses tune.txt of the JIT cache directory: {key: [values]}."""
    import os
    d = cache_dir or os.environ.get("NCA_GB300_CACHE_DIR") or str(
        Path(os.environ.get("XDG_CACHE_HOME", str(Path.home() / ".cache"))) / "ncarray_gb300")
    f = Path(d) / "tune.txt"
    out = {}
    if f.exists():
        for line in f.read_text().splitlines():
            parts = line.split()
            if len(parts) >= 2:
                out[parts[0]] = [int(v) for v in parts[1:]]
    return out
