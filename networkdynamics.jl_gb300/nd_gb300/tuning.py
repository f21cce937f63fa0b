"""Autotuner cache: the block size that the ensemble autotuner picked for a workload, kept
in a JSON file so that later processes skip the probe solves.

The file is ``$ND_GB300_CACHE_DIR/autotune.json`` (default ``$XDG_CACHE_HOME/nd_gb300`` or
``~/.cache/nd_gb300``).  Each entry is keyed by the device name, the library version, the
component kinds, the precision, the instance count and sizes and the tolerances of the
probe; a missing or unreadable file is an empty cache, and writes replace the file
atomically.
"""
from __future__ import annotations

import json
import os
import tempfile
from pathlib import Path
from typing import Optional


def cache_path() -> Path:
    env = os.environ.get("ND_GB300_CACHE_DIR")
    if env:
        return Path(env) / "autotune.json"
    base = os.environ.get("XDG_CACHE_HOME") or str(Path.home() / ".cache")
    return Path(base) / "nd_gb300" / "autotune.json"


def workload_key(device: str, version: int, vertex_kind: int, edge_kind: int, dtype_code: int, n_instances: int,
                 n_vertices: int, n_edges: int, reltol: float, abstol: float, t_probe: float) -> str:
    return (f"{device}|v{version}|vk{vertex_kind}|ek{edge_kind}|dt{dtype_code}|n{n_instances}|nv{n_vertices}"
            f"|ne{n_edges}|rt{reltol:.3e}|at{abstol:.3e}|tp{t_probe:.3e}")


class AutotuneCache:
    def __init__(self, path: Optional[os.PathLike] = None):
        self.path = Path(path) if path is not None else cache_path()

    def _load(self) -> dict:
        try:
            data = json.loads(self.path.read_text())
        except (OSError, ValueError):
            return {}
        return data if isinstance(data, dict) else {}

    def get(self, key: str) -> Optional[int]:
        entry = self._load().get(key)
        if isinstance(entry, dict) and isinstance(entry.get("threads"), int) and entry["threads"] > 0:
            return entry["threads"]
        return None

    def put(self, key: str, threads: int) -> None:
        data = self._load()
        data[key] = {"threads": int(threads)}
        self.path.parent.mkdir(parents=True, exist_ok=True)
        fd, tmp = tempfile.mkstemp(dir=self.path.parent, prefix=".autotune.", suffix=".json")
        try:
            with os.fdopen(fd, "w") as f:
                json.dump(data, f, indent=1, sort_keys=True)
            os.replace(tmp, self.path)
        except BaseException:
            try:
                os.unlink(tmp)
            except OSError:
                pass
            raise
