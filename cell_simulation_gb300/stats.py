"""Statistics stream helpers mirroring the reference's example host code
(examples/no_window.rs:16-62): a bounded per-species container of
(iteration, value) samples with mean/last, and CSV output with ';' as the
delimiter and one "iteration;value" record per sample, values written the way
Rust prints an f32."""
from __future__ import annotations

from collections import deque
from pathlib import Path

import numpy as np


def rust_f32(v) -> str:
    """Display of an f32 in Rust: shortest round-trip digits, no exponent, no
    trailing ".0" for integral values."""
    f = np.float32(v)
    if not np.isfinite(f):
        return "NaN" if np.isnan(f) else ("inf" if f > 0 else "-inf")
    if f == np.floor(f) and abs(f) < 1e16:
        return str(int(f))
    s = np.format_float_positional(f, unique=True, trim="-")
    return s


class StatisticContainer:
    """Last `capacity` samples of one species (StatisticContainer, no_window.rs:16-52)."""

    def __init__(self, capacity: int = 500):
        self.x: deque[int] = deque(maxlen=capacity)
        self.y: deque[float] = deque(maxlen=capacity)

    def add(self, x: int, y: float) -> None:
        self.x.append(int(x))
        self.y.append(float(np.float32(y)))

    def mean(self) -> float:
        return float(np.float32(sum(np.float32(v) for v in self.y) / np.float32(len(self.y)))) if self.y else float("nan")

    def last(self) -> float:
        return self.y[-1] if self.y else 0.0

    def to_csv(self, path) -> None:
        """Writes and drains the samples (to_csv, no_window.rs:53-62)."""
        with open(Path(path), "w", newline="") as f:
            while self.x and self.y:
                f.write(f"{self.x.popleft()};{rust_f32(self.y.popleft())}\n")


def make_all_stats(names, capacity: int = 500) -> dict[str, StatisticContainer]:
    return {n: StatisticContainer(capacity) for n in names}


def drain(sim, all_stats: dict[str, StatisticContainer]) -> int:
    """Moves the simulation's pending SolverStatisticSamples into the containers
    of the species being tracked (no_window.rs:76-80); returns the count."""
    n = 0
    while sim.stats:
        s = sim.stats.popleft()
        if s.name in all_stats:
            all_stats[s.name].add(s.iteration_count, s.value)
        n += 1
    return n
