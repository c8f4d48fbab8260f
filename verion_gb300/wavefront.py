"""Wavefront buffer sizes and stage order: crates/verion-gpu/src/wavefront.rs (the reference's
bookkeeping, which `Sizes` restates), and the sizes this backend actually allocates."""
from __future__ import annotations

from dataclasses import dataclass
from enum import Enum

from .pack import MAX_DEPTH

BASE_WORDS = 16   # wavefront.rs:7
SPLIT_WORDS = 17  # wavefront.rs:9
GROUP = 64        # wavefront.rs:11


@dataclass(frozen=True)
class Sizes:
    """wavefront.rs:15-44"""
    state: int
    hits: int
    queue: int
    counts: int
    args: int

    @staticmethod
    def new(paths: int, lighting: bool, depth: int = MAX_DEPTH) -> "Sizes":
        words = BASE_WORDS + (SPLIT_WORDS if lighting else 0)
        return Sizes(paths * words * 4, paths * 16, paths * 4, (depth + 1) * 4, depth * 12)

    def total(self) -> int:
        return self.state + self.hits + 2 * self.queue + self.counts + self.args


class Stage(Enum):
    """wavefront.rs:48-72"""
    SELECT = 0
    ARGS = 1
    EXTEND = 2
    SHADE = 3

    @staticmethod
    def of_depth(depth: int, adaptive: bool):
        out = [Stage.SELECT] if depth == 0 and adaptive else []
        return out + [Stage.ARGS, Stage.EXTEND, Stage.SHADE]

    def timing_slot(self) -> int:
        return 1 if self is Stage.SHADE else 0


def cuda_bytes(paths: int, lighting: bool, depth_alloc: int = 64) -> int:
    """Bytes this backend allocates for one accumulation's wavefront: 16-byte state planes (4, or 9
    with the lighting split), 16-byte hit records, two queues, and counters for up to
    `depth_alloc` depths (queue lengths plus extend/shade work counters). Depth 0 needs no
    dispatch arguments: queue lengths are read on the device."""
    planes = 4 + (5 if lighting else 0)
    return paths * planes * 16 + paths * 16 + 2 * paths * 4 + (depth_alloc + 1) * 4 + 2 * (depth_alloc + 1) * 4
