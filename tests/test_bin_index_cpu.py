"""The time-bin index identity the gathers use in place of a float -> int
conversion, emulated exactly on the CPU.

For a path ratio x >= 0 (float32) and a window starting at bin a, the
kernels (csrc/bp_gather.cuh: PATH_FAST, PATH_2D and the voxel-scattering
walk) take

    idx = min(bits(x +rz float(2^23 - a)) - 0x4B000000, slot_w)   (uint32)

and the reference takes static_cast<int>(x) - a, clamped to the same slot
(transient_reconstruction.cuh:112-126 and :93-136).  A round-toward-zero add
of 2^23 - a lands in [2^23, 2^24), where float32 values are the integers, so
its bits are 0x4B000000 + floor(x) - a; below the window it lands under 2^23
and the unsigned difference wraps past slot_w; far above it the exponent grows
and the difference again exceeds slot_w.  This checks that claim over random
and edge-case x, a and window widths."""
import numpy as np

TWO23 = 8388608


def _add_rz_f32(x: np.ndarray, c: np.ndarray) -> np.ndarray:
    """float32 x + c rounded toward zero (x, c >= 0): the float64 sum is exact
    for float32 operands this close in exponent, then stepped down to the
    float32 at or below it."""
    exact = x.astype(np.float64) + c.astype(np.float64)
    r = exact.astype(np.float32)  # round to nearest
    over = r.astype(np.float64) > exact
    r[over] = np.nextafter(r[over], np.float32(0))
    return r


def _trick(x, a, slot_w):
    c = (TWO23 - a).astype(np.float32)  # exact: a < 2^23
    bits = _add_rz_f32(x, c).view(np.uint32)
    return np.minimum((bits - np.uint32(0x4B000000)).astype(np.uint32), np.uint32(slot_w))


def _reference(x, a, slot_w):
    b = np.where(x >= 2.0 ** 31, np.float64(2 ** 31 - 1), np.trunc(x.astype(np.float64))).astype(np.int64)
    d = (b - a.astype(np.int64)) & 0xFFFFFFFF  # (uint32)(b - a)
    return np.minimum(d, slot_w).astype(np.uint32)


def test_bin_index_trick_equals_truncation():
    rng = np.random.default_rng(7)
    n = 400_000
    a = rng.integers(0, 1 << 16, n).astype(np.int64)
    slot_w = 1 << 12
    # Ratios around the window, across bin edges, and far outside it.
    parts = [
        (a + rng.uniform(-3.0, slot_w + 3.0, n)).clip(0),
        a + rng.integers(-2, slot_w + 2, n) + rng.choice([0.0, 1e-7, 0.5, 1 - 6e-8], n),
        rng.uniform(0, 2.0 ** 24, n),
        np.exp(rng.uniform(0, np.log(3e38), n)),
    ]
    for x64 in parts:
        x = np.asarray(x64, dtype=np.float64).astype(np.float32)
        x = np.where(np.isfinite(x), x, np.float32(3e38))
        np.testing.assert_array_equal(_trick(x, a, slot_w), _reference(x, a, slot_w))


def test_bin_index_trick_edges():
    slot_w = 64
    for a in (0, 1, 7, 1000, TWO23 - slot_w - 1):
        base = np.float32(a)
        xs = [0.0, base - 1, base - 1e-3, base, base + 1e-3, base + 1 - 1e-4, base + slot_w - 1,
              base + slot_w, base + slot_w + 0.5, float(TWO23), float(2 * TWO23), 2.0 ** 31, 3.0e38]
        x = np.array([v for v in xs if v >= 0], dtype=np.float32)
        x = np.nextafter(x, np.float32(0)).astype(np.float32).tolist() + x.tolist()
        x = np.array(x, dtype=np.float32)
        av = np.full(x.shape, a, dtype=np.int64)
        np.testing.assert_array_equal(_trick(x, av, slot_w), _reference(x, av, slot_w))
    inf = np.array([np.inf], dtype=np.float32)
    assert _trick(inf, np.array([5]), slot_w)[0] == slot_w
