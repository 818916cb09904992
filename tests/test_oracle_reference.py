"""Pins the oracle against the reference build in oracle/_ref directly (runs
only where the reference compiles; skipped elsewhere, e.g. on aarch64)."""
import os
import tempfile

import numpy as np
import pytest

import oracle
import refbind
import synth

pytestmark = pytest.mark.skipif(not refbind.available(), reason="reference build absent")


@pytest.mark.parametrize("d", [4, 5, 7, 9, 15, 17, 19, 31, 33, 47, 63, 65, 100, 102, 127, 129])
def test_rotation_rule_matches_reference(d):
    tmp = tempfile.mkdtemp()
    spec = dict(seed=d, n=64, dim=d, ncomp=4, nlist=2, nq=24, rotation="random")
    p = os.path.join(tmp, "x")
    q, _ = synth.materialize(spec, p)
    ref = refbind.RefIndex(p).rotate_rows(q)
    mine = oracle.OracleIndex(p).rotate(q)
    assert np.array_equal(ref, mine)


def test_sq16_kernel_grid_matches_reference():
    """tests/test_kernels.cpp:151-154 grid: bytes 0/255 with probability 1/4
    each, else uniform; the oracle's distance equals the reference's kernel."""
    rng = np.random.default_rng(7)
    step_sq = 1.0 / (65535.0 * 65535.0)
    for dc in (64, 128, 1024):
        for m in (1, 5, 16):
            for n in (1, 15, 17, 70, 256):
                def draw(shape):
                    c = rng.integers(0, 4, shape)
                    return np.where(c == 0, 0, np.where(c == 1, 255, rng.integers(0, 256, shape))).astype(np.uint8)
                qh, ql, xh, xl = draw((m, dc)), draw((m, dc)), draw((n, dc)), draw((n, dc))
                code = lambda h, l: h.astype(np.int64) * 256 + l
                qn = (code(qh, ql) ** 2).sum(1)
                xn = (code(xh, xl) ** 2).sum(1)
                a = refbind.sq16_l2(qh, ql, xh, xl, qn, xn, step_sq)
                b = oracle.sq16_l2(qh, ql, xh, xl, qn, xn, step_sq)
                assert np.array_equal(a, b), (dc, m, n)
