"""multiply_using_layout: layout validation on the host (no GPU needed).

Malformed descriptions are rejected before any device work, with the status
the C interface documents: a missing or duplicated block, a block of another
rank, splits that do not start at 0, and operand shapes that do not chain.
"""
import numpy as np
import pytest


def _layout(rows, cols, rb, cb, skip=None, dup=False, owner=0):
    from cosma_gb300 import BlockLayout
    rs = [int(x) for x in np.linspace(0, rows, rb + 1)]
    cs = [int(x) for x in np.linspace(0, cols, cb + 1)]
    blocks = {}
    for r in range(rb):
        for c in range(cb):
            if (r, c) == skip:
                continue
            h = np.zeros((max(rs[r + 1] - rs[r], 1), max(cs[c + 1] - cs[c], 1)), order="F")
            blocks[(r, c)] = (h, h.shape[0])
    lay = BlockLayout(rs, cs, blocks, owners=[owner] * (rb * cb))
    if dup:
        lay.c.localblocks[1] = lay.c.localblocks[0]
    return lay


def test_rejects_malformed_layouts(native_lib):
    from cosma_gb300 import CosmaGpuError, multiply_using_layout
    good_a, good_b, good_c = _layout(6, 5, 2, 2), _layout(5, 4, 2, 2), _layout(6, 4, 2, 2)
    cases = [
        (_layout(6, 5, 2, 2, skip=(1, 1)), good_b, good_c, 1),   # a block missing
        (_layout(6, 5, 2, 2, dup=True), good_b, good_c, 1),      # a block listed twice
        (_layout(6, 5, 2, 2, owner=1), good_b, good_c, 4),       # another rank's block
        (good_a, _layout(7, 4, 2, 2), good_c, 1),                # k of op(A) != k of op(B)
        (good_a, good_b, _layout(6, 5, 2, 2), 1),                # C is not m x n
    ]
    for a, b, c, code in cases:
        with pytest.raises(CosmaGpuError) as e:
            multiply_using_layout("N", "N", 1.0, a, b, 0.0, c)
        assert e.value.code == code, e.value


def test_tiles_for_memory_fit_and_grow(native_lib):
    """The memory-limited tiling (sequential-split counterpart): tiles are
    multiples of 256, grow with the budget, shrink for methods with more
    scratch, and an impossible budget is an OUT_OF_MEMORY error."""
    from cosma_gb300 import CosmaGpuError, tiles_for_memory
    budgets = [2 ** 28, 2 ** 30, 2 ** 33, 2 ** 36]
    for scalar in "sdcz":
        for method in ("native", "ozaki", "bf16x3", "auto"):
            t = [tiles_for_memory(scalar, method, b)[0] for b in budgets]
            assert all(x % 256 == 0 and x > 0 for x in t)
            assert t == sorted(t)
            es = {"s": 4, "d": 8, "c": 8, "z": 16}[scalar]
            for x, b in zip(t, budgets):
                assert 6 * x * x * es <= b  # the A, B, C tile slots alone fit
    assert tiles_for_memory("d", "ozaki", 2 ** 30)[0] < tiles_for_memory("d", "native", 2 ** 30)[0]
    with pytest.raises(CosmaGpuError) as e:
        tiles_for_memory("d", "native", 1 << 20)
    assert e.value.code == 3
