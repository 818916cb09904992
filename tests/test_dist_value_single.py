"""The device's single-precision path of dist_value (csrc/dist_value.h,
dist_value_single), restated operation for operation in numpy float32 (every
float32 operation is correctly rounded; an fma's exact product error is formed
in float64, which holds the product of two floats exactly). Whatever value
the path accepts must equal the reference's float(double(l2) * step_sq)
(src/kernels.cpp:166-168): on random values, and on values placed a few units
from a float rounding midpoint, where the double rounding decides. The GPU
test of katoann_gpu_dist_values runs the device code on the same kinds of
values."""
import numpy as np
import pytest

F32 = np.float32


def split_scale(step_sq: float):
    s1 = F32(step_sq)
    s2 = F32(step_sq - np.float64(s1))
    return s1, s2, F32(np.ldexp(s1, 23)), F32(np.ldexp(s2, 23))


def bits_f32(u):
    return np.asarray(u, np.uint32).view(np.float32)


def single_path(l2: np.ndarray, step_sq: float):
    """(value, accepted) as the device computes them."""
    s1, s2, a1, a2 = split_scale(step_sq)
    ok = (l2 > 0) & (l2 < (1 << 46))
    x = np.where(ok, l2, 1)
    fh = (x >> 23).astype(np.float32)
    fl = (x & 0x7FFFFF).astype(np.float32)

    def two_prod(a, b):
        p = a * b
        e = (a.astype(np.float64) * np.float64(b) - p.astype(np.float64)).astype(np.float32)
        return p, e

    p1, e1 = two_prod(fh, a1)
    p3, e3 = two_prod(fl, s1)
    p2, p4 = fh * a2, fl * s2
    s0 = p1 + p3
    e0 = p3 - (s0 - p1)
    tail = (((e0 + e1) + e3) + p2) + p4
    r = s0 + tail
    d = (s0 - r) + tail
    rb = r.view(np.uint32)
    E = (rb >> 23).astype(np.int64)
    ok &= (E >= 64) & (E <= 253)
    Ec = np.clip(E, 64, 253).astype(np.uint32)
    hup = bits_f32((Ec - 24) << 23)
    hdn = np.where(rb & 0x7FFFFF, hup, bits_f32((Ec - 25) << 23))
    m2 = bits_f32((Ec - 38) << 23)
    ok &= (d < hup - m2) & (-d < hdn - m2)
    return r, ok


def exact(l2: np.ndarray, step_sq: float) -> np.ndarray:
    return (l2.astype(np.float64) * step_sq).astype(np.float32)


def near_midpoints(rng, step_sq: float, n: int, lo: float, hi: float) -> np.ndarray:
    """l2 values whose product lies within a few step_sq of the midpoint
    between two neighbouring floats (a quarter of them at powers of two)."""
    f = rng.uniform(lo, hi, n).astype(np.float32)
    pw = F32(2.0) ** np.floor(np.log2(f)).astype(np.float32)
    f = np.where(rng.random(n) < 0.25, pw, f)
    up = np.nextafter(f, F32(np.inf)).astype(np.float64)
    dn = np.nextafter(f, F32(0)).astype(np.float64)
    mid = np.where(rng.random(n) < 0.5, (f.astype(np.float64) + up) / 2, (f.astype(np.float64) + dn) / 2)
    c = np.floor(mid / step_sq).astype(np.int64)
    return np.concatenate([c + o for o in range(-3, 4)])


SCALES = [1.76061467e-08, 2.98203776e-09, 1.0 / 65535.0 ** 2, 1.3e-10, 0.37, 123.4, 2.0 ** -30,
          7.7e-20]


@pytest.mark.parametrize("step_sq", SCALES)
def test_accepted_values_are_the_references(step_sq):
    rng = np.random.default_rng(int(step_sq * 1e9) % 1000 + 1)
    top = (1 << 46) - 1
    parts = [
        np.arange(0, 5000, dtype=np.int64),
        rng.integers(1, top, 400000, dtype=np.int64),
        np.exp2(rng.uniform(0, 46, 400000)).astype(np.int64),
        np.array([1 << 23, (1 << 23) - 1, (1 << 23) + 1, top, top - 1, 1 << 45], np.int64),
    ]
    smax = float(top) * step_sq
    parts.append(near_midpoints(rng, step_sq, 100000, max(step_sq * 64, 1e-30), min(smax, 3e38)))
    l2 = np.concatenate(parts)
    l2 = l2[(l2 >= 0) & (l2 <= top)]
    r, ok = single_path(l2, step_sq)
    want = exact(l2, step_sq)
    bad = ok & (r.view(np.uint32) != want.view(np.uint32))
    assert not bad.any(), (step_sq, l2[bad][:5], r[bad][:5], want[bad][:5])
    # the path settles almost every value of the size searches give (the rest
    # take the integer path: exact ties, which a float-exact or decimal scale
    # makes common among small l2, and products below 2^-63)
    rand = rng.integers(1 << 30, top, 400000, dtype=np.int64)
    _, ok_rand = single_path(rand, step_sq)
    assert ok_rand.mean() > 0.999, ok_rand.mean()


def test_near_midpoints_do_fall_back():
    """Values within a unit of a midpoint are refused (so the exact integer
    path decides them), and every refusal is near a midpoint or out of range."""
    step_sq = 1.76061467e-08
    rng = np.random.default_rng(5)
    l2 = near_midpoints(rng, step_sq, 20000, 1e-3, 1e5)
    _, ok = single_path(l2, step_sq)
    assert (~ok).sum() > 0
    rand = rng.integers(1 << 30, 1 << 46, 200000, dtype=np.int64)
    r, ok = single_path(rand, step_sq)
    assert ok.mean() > 0.9995
