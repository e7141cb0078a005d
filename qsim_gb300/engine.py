"""Host-side engine objects exposed through the C ABI: random numbers now,
circuits, fusion plans and runners as they are added."""
from __future__ import annotations

import numpy as np

from . import _native as N


class Rng:
    """std::mt19937(seed) with uniform_real_distribution<double> draws, the
    generator the reference passes to Measure (lib/statespace.h:97-140)."""

    def __init__(self, seed: int):
        self.h = N.lib.qsg_rng_create(seed & 0xFFFFFFFF)

    def next_u32(self) -> int:
        return int(N.lib.qsg_rng_next_u32(self.h))

    def uniform(self, max_value: float) -> float:
        return float(N.lib.qsg_rng_uniform(self.h, max_value))

    def __del__(self):
        try:
            N.lib.qsg_rng_destroy(self.h)
        except Exception:
            pass


def generate_random_values(num: int, seed: int, max_value: float) -> np.ndarray:
    """GenerateRandomValues (lib/util.h:67-85) without the sentinel."""
    out = np.empty(max(1, num), dtype=np.float64)
    N.lib.qsg_generate_random_values(num, seed & 0xFFFFFFFF, max_value,
                                     out.ctypes.data_as(N.P_f64))
    return out[:num]
