"""The variance gate's reciprocal square root (cascade.cuh inv_sqrt_as_reference)
against the reference's rounding, float(1 / sqrt(x)) through a double square
root and a double division (face_vision_engine.cu:463-492).

The device function takes one double Newton step from rsqrtf and keeps the
result only when the bits below float precision are far from the halfway
pattern; otherwise it falls back to the double square root and division.  This
CPU test replays that arithmetic in IEEE double (numpy rounds each operation
the same way) with the float starting value anywhere within rsqrtf's documented
2-ulp error, and checks that every kept result equals the reference's float."""
import numpy as np

HALF = 1 << 28
KEEP = 1 << 16


def reference(x):
    return (np.float64(1.0) / np.sqrt(x)).astype(np.float32)


def fast_path(x, y0):
    """(kept, value) of the Newton step from the float start y0."""
    y = y0.astype(np.float64)
    y1 = y * (1.5 - (0.5 * x) * (y * y))
    low = (y1.view(np.uint64) & np.uint64(0x1FFFFFFF)).astype(np.int64)
    kept = np.abs(low - HALF) > KEEP
    return kept, y1.astype(np.float32)


def starts(x):
    """rsqrtf's possible results: the float nearest 1/sqrt(float(x)) and the
    floats up to 2 ulp either side."""
    xf = x.astype(np.float32).astype(np.float64)
    r = (1.0 / np.sqrt(xf)).astype(np.float32)
    out = [r]
    up, dn = r.copy(), r.copy()
    for _ in range(2):
        up = np.nextafter(up, np.float32(np.inf))
        dn = np.nextafter(dn, np.float32(0))
        out += [up.copy(), dn.copy()]
    return out


def check(x):
    ref = reference(x)
    kept_any = np.zeros(len(x), bool)
    for y0 in starts(x):
        kept, val = fast_path(x, y0)
        bad = kept & (val.view(np.uint32) != ref.view(np.uint32))
        assert not bad.any(), (x[bad][:5], val[bad][:5], ref[bad][:5])
        kept_any |= kept
    return kept_any


def test_small_integers_exhaustive():
    x = np.arange(1, 1 << 20, dtype=np.float64)
    kept = check(x)
    assert kept.mean() > 0.999


def test_random_integers_up_to_2_pow_42():
    rng = np.random.default_rng(7)
    x = np.floor(rng.random(1 << 20) * 2.0 ** 42) + 1
    kept = check(x)
    assert kept.mean() > 0.999


def test_values_next_to_float_rounding_boundaries():
    """Integers whose 1/sqrt lies close to a halfway point between floats:
    the step either reproduces the reference's rounding or falls back."""
    rng = np.random.default_rng(11)
    x = np.floor(rng.random(1 << 22) * 2.0 ** 40) + 1
    r = 1.0 / np.sqrt(x)
    low = (r.view(np.uint64) & np.uint64(0x1FFFFFFF)).astype(np.int64)
    near = x[np.abs(low - HALF) < (1 << 20)]
    assert len(near) > 100
    kept = check(near)
    # the closest ones must take the double path
    r = 1.0 / np.sqrt(near)
    low = (r.view(np.uint64) & np.uint64(0x1FFFFFFF)).astype(np.int64)
    assert not kept[np.abs(low - HALF) < (1 << 12)].any()
