"""The integer-pipe binary64 routines (csrc/emu64.cuh, csrc/exact_div.cuh)
that the split precision form and the FP64 form use: every result must
have the bits of the device's own instruction (the exact FP32 -> FP64
conversion, the round-to-nearest-even FP64 -> FP32 conversion and the
double-float split, FP64 add, subtract and multiply, and the FP64 form's
division from a shared reciprocal with its rounding decided by integer
arithmetic), over seeded operands in six classes -- everyday
magnitudes, the full exponent range, sparse significands (rounding ties),
zeros / subnormals / infinities / NaN / the range ends, values around the
binary32 range, and near cancellation -- with every binary32 bit pattern
for the widening conversion."""
from __future__ import annotations

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 20261204])
def test_emulated_binary64_matches_the_instructions(ctx, seed):
    bad = ctx.probe_emu64(n_per_class=1 << 24, seed=seed)
    assert bad == (0, 0, 0, 0, 0), f"mismatches f2d/d2f/add/mul/div: {bad}"
