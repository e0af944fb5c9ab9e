"""BF16 helpers on the host: round-to-nearest-even conversion of float32 arrays
to bf16 bit patterns (uint16) and back."""
from __future__ import annotations

import numpy as np


def to_bf16_bits(x) -> np.ndarray:
    a = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    rounding = ((a >> 16) & 1) + np.uint32(0x7FFF)
    return ((a + rounding) >> 16).astype(np.uint16)


def from_bf16_bits(b) -> np.ndarray:
    return (np.asarray(b, dtype=np.uint16).astype(np.uint32) << 16).view(np.float32)


def round_bf16(x) -> np.ndarray:
    return from_bf16_bits(to_bf16_bits(x))
