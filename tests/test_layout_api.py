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
