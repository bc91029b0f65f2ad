"""Autotuner of the batched FEM solves.

A batch of designs solved together (``BatchFEM.solve_all``: the 8-design evaluation batch,
``VoxelFEMEvaluator.evaluate_batch``, ``BatchSIMP``'s rounds) has three free parameters that
the library exposes through ``gbsimp_solve_opts``:

- the form: designs sharing persistent cooperative launches (``fused`` = 1) or each design in
  its own device-driven graph loop (``fused`` = 0);
- the SM share of each design in a persistent launch (``batch_share``): in proportion to its
  element count, or to element count x longest extent (Jacobi-PCG iteration counts grow about
  with the longest extent, so the designs of a launch then finish together instead of small
  ones leaving their SMs idle while a large one converges);
- the designs per launch (``batch_group``): all that are resident together, or launches of a
  few designs run one after the other.

The element form and threads per element are not free: two elements per thread is what the
packed FP32x2 arithmetic of the modal kernel needs, and its tile (a 512-element flat chunk per
CTA) is fixed by the register and shared-memory budget of two CTAs per SM.

On the first solve of a grid class (the multiset of grid shapes of the batch) the tuner runs the
batch once per candidate on copies of the designs (same densities, loads and warm starts, fresh
displacements and workspaces), times each with the device synchronised on both sides, and keeps
the fastest. The choice is cached per grid class for the life of the process and, when a path
is given (argument or the GBSIMP_TUNE_CACHE environment variable), in a JSON file. The
reference has no counterpart: it solves each design with its own thread (voxel_fem.py:559-611).
"""
from __future__ import annotations

import json
import os
import threading
import time
from dataclasses import asdict, dataclass
from typing import Callable, Dict, List, Optional, Sequence, Tuple


@dataclass(frozen=True)
class BatchConfig:
    fused: int = 1        # 1: persistent launches shared by designs; 0: one graph loop per design
    batch_share: int = 0  # 0: SMs by element count; 1: by element count x longest extent
    batch_group: int = 0  # designs per persistent launch (0: as many as are resident together)

    def label(self) -> str:
        if not self.fused:
            return "graph loop per design"
        share = "elements" if self.batch_share == 0 else "elements x extent"
        group = "all resident" if self.batch_group == 0 else f"<= {self.batch_group}"
        return f"persistent, share by {share}, {group} per launch"


CANDIDATES: Tuple[BatchConfig, ...] = (
    BatchConfig(1, 0, 0),
    BatchConfig(1, 1, 0),
    BatchConfig(1, 1, 4),
    BatchConfig(1, 0, 1),
    BatchConfig(0, 0, 0),
)
DEFAULT = CANDIDATES[0]

GridClass = Tuple[Tuple[Tuple[int, int, int], int], ...]


def grid_class(grids: Sequence[Sequence[int]]) -> GridClass:
    """The multiset of grid shapes, as a sorted tuple of (shape, count)."""
    counts: Dict[Tuple[int, int, int], int] = {}
    for g in grids:
        key = tuple(int(v) for v in g)
        counts[key] = counts.get(key, 0) + 1
    return tuple(sorted(counts.items()))


def _class_key(gc: GridClass) -> str:
    return ";".join(f"{s[0]}x{s[1]}x{s[2]}*{n}" for s, n in gc)


class BatchTuner:
    """Picks a BatchConfig per grid class by timing the candidates (see the module docstring).
    ``trial(config) -> seconds`` runs the batch once with a configuration; the tuner calls it
    once per candidate the first time a grid class is seen."""

    def __init__(self, candidates: Sequence[BatchConfig] = CANDIDATES, cache_path: Optional[str] = None,
                 clock: Callable[[], float] = time.perf_counter):
        self.candidates = tuple(candidates)
        self.cache_path = cache_path if cache_path is not None else os.environ.get("GBSIMP_TUNE_CACHE")
        self.clock = clock
        self._lock = threading.Lock()
        self.cache: Dict[str, BatchConfig] = {}
        self.timings: Dict[str, Dict[str, float]] = {}
        self._load()

    def _load(self):
        if not self.cache_path or not os.path.exists(self.cache_path):
            return
        try:
            with open(self.cache_path) as fh:
                raw = json.load(fh)
            for k, v in raw.get("choices", {}).items():
                self.cache[k] = BatchConfig(**v)
        except (OSError, ValueError, TypeError):
            pass  # an unreadable cache is retuned, not fatal

    def _save(self):
        if not self.cache_path:
            return
        tmp = self.cache_path + ".tmp"
        with open(tmp, "w") as fh:
            json.dump({"choices": {k: asdict(v) for k, v in self.cache.items()}, "timings": self.timings}, fh,
                      indent=1, sort_keys=True)
        os.replace(tmp, self.cache_path)

    def choice(self, grids: Sequence[Sequence[int]]) -> Optional[BatchConfig]:
        """The cached configuration of this grid class, or None."""
        with self._lock:
            return self.cache.get(_class_key(grid_class(grids)))

    def tune(self, grids: Sequence[Sequence[int]], trial: Callable[[BatchConfig], float]) -> BatchConfig:
        """The configuration of this grid class, timing every candidate first if it is new.
        A candidate whose trial raises is skipped; if all fail, DEFAULT is kept."""
        key = _class_key(grid_class(grids))
        with self._lock:
            if key in self.cache:
                return self.cache[key]
        times: Dict[str, float] = {}
        best, best_t = DEFAULT, float("inf")
        for cfg in self.candidates:
            try:
                t = float(trial(cfg))
            except Exception:  # noqa: BLE001 - a candidate the library refuses is not chosen
                continue
            times[cfg.label()] = t
            if t < best_t:
                best, best_t = cfg, t
        with self._lock:
            self.cache[key] = best
            self.timings[key] = times
            self._save()
        return best


_TUNER: Optional[BatchTuner] = None
_TUNER_LOCK = threading.Lock()


def default_tuner() -> BatchTuner:
    """The process-wide tuner (cache shared by every BatchFEM)."""
    global _TUNER
    with _TUNER_LOCK:
        if _TUNER is None:
            _TUNER = BatchTuner()
        return _TUNER


def timed(run: Callable[[], object], sync: Callable[[], None], clock: Callable[[], float] = time.perf_counter) -> float:
    """Seconds of run() with sync() on both sides."""
    sync()
    t0 = clock()
    run()
    sync()
    return clock() - t0


def summary(tuner: BatchTuner, grids: Sequence[Sequence[int]]) -> dict:
    """The choice and the candidates' trial times of a grid class (for reports)."""
    key = _class_key(grid_class(grids))
    cfg = tuner.cache.get(key)
    return {"grid_class": key, "choice": None if cfg is None else cfg.label(),
            "trial_seconds": dict(tuner.timings.get(key, {}))}


__all__: List[str] = ["BatchConfig", "BatchTuner", "CANDIDATES", "DEFAULT", "default_tuner", "grid_class", "summary",
                      "timed"]
