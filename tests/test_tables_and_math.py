"""Tag family tables (reference test_family_tables, test_detector.cpp:70-102)
and the accuracy of the deterministic math helpers (detmath.h)."""
import re
from pathlib import Path

import numpy as np

import oracle

INC = Path(__file__).resolve().parent.parent / "bd-cudatag_gb300" / "csrc" / "families_data.inc"


def load_tables():
    text = INC.read_text()
    out = {}
    for name in ("BD_CODEWORDS_36H11", "BD_CODEWORDS_16H5"):
        count = int(re.search(r"#define %s_COUNT (\d+)" % name, text).group(1))
        body = text.split("#define %s \\" % name, 1)[1].split("#define", 1)[0]
        vals = [int(v, 16) for v in re.findall(r"0x([0-9a-f]+)ull", body)]
        assert len(vals) == count
        out[name] = vals
    return out["BD_CODEWORDS_36H11"], out["BD_CODEWORDS_16H5"]


def rotate(codes: np.ndarray, bits: int) -> np.ndarray:
    n = bits * bits
    out = np.zeros_like(codes)
    for r in range(bits):
        for c in range(bits):
            bit = (codes >> np.uint64(n - 1 - (r * bits + c))) & np.uint64(1)
            out |= bit << np.uint64(n - 1 - (c * bits + (bits - 1 - r)))
    return out


def popcount(x: np.ndarray) -> np.ndarray:
    return np.unpackbits(x.view(np.uint8).reshape(*x.shape, 8), axis=-1).sum(-1)


def min_distance(codes, bits):
    a = np.array(codes, dtype=np.uint64)
    best = 1000
    rot = a.copy()
    for k in range(4):
        d = popcount(a[:, None] ^ rot[None, :])
        if k == 0:
            np.fill_diagonal(d, 1000)
        best = min(best, int(d.min()))
        rot = rotate(rot, bits)
    return best


def test_family_tables():
    t36, t16 = load_tables()
    assert len(t36) == 587 and len(t16) == 30
    assert max(t36) < 1 << 36 and max(t16) < 1 << 16
    assert min_distance(t36, 6) == 11
    assert min_distance(t16, 4) == 5


def test_detmath_accuracy():
    L = oracle.lib()
    rng = np.random.default_rng(1)
    xs = np.concatenate([rng.uniform(-7.0, 7.0, 4000), np.linspace(-3.2, 3.2, 257)]).astype(np.float32)
    for x in xs:
        s, c = L.bdo_sinf(float(x)), L.bdo_cosf(float(x))
        assert abs(s - np.sin(np.float64(x))) <= 3e-7
        assert abs(c - np.cos(np.float64(x))) <= 3e-7
    ys = rng.uniform(-50, 50, (3000, 2)).astype(np.float32)
    for y, x in ys:
        a = L.bdo_atan2f(float(y), float(x))
        ref = np.arctan2(np.float64(y), np.float64(x))
        assert abs(a - ref) <= 4e-7 * max(1.0, abs(ref))
    # signed zeros as C99 Annex F
    assert L.bdo_atan2f(0.0, -0.0) == np.float32(np.pi)
    assert L.bdo_atan2f(-0.0, -0.0) == -np.float32(np.pi)
    assert np.signbit(L.bdo_atan2f(-0.0, 0.0))


def test_otsu_prefix_exact_below_2_24():
    """k_stats replaces the reference's sequential FP32 Otsu prefix sums
    (gpu_detector.cu:200-229) by an integer scan converted to float while the
    weighted sum sum_i i * hist[i] is below 2^24: every partial sum is then an
    integer that FP32 holds exactly, so both give the same bits.  Checked on
    random histograms up to the bound, with the sequential loop in float32."""
    rng = np.random.default_rng(11)
    for trial in range(300):
        tiles = int(rng.integers(1, 266305))
        hist = rng.multinomial(tiles, rng.dirichlet(np.full(64, 0.3))).astype(np.int64)
        if int(np.dot(np.arange(64), hist)) >= (1 << 24):
            continue
        total = np.float32(0.0)
        s = np.float32(0.0)
        for i in range(64):
            total = np.float32(total + np.float32(hist[i]))
            s = np.float32(s + np.float32(i) * np.float32(hist[i]))
            assert total == np.float32(np.sum(hist[:i + 1]))
            assert s == np.float32(np.dot(np.arange(i + 1), hist[:i + 1]))


def _valley_reference(mags, best, best_mag):
    """The reference's first-pass test (gpu_detector.cu fit_edge_line_warp):
    the first i in [1, best - 2] that is a local peak of at least 0.70 *
    best_mag with min(mags[i + 1 .. best - 1]) below half of it."""
    accept = np.float32(0.70) * best_mag
    for i in range(1, best - 1):
        if mags[i] < accept or mags[i] < mags[i - 1] or mags[i] < mags[i + 1]:
            continue
        valley = np.float32(np.finfo(np.float32).max)
        for k in range(i + 1, best):
            valley = min(valley, mags[k])
        if valley < np.float32(0.5) * mags[i]:
            return i, mags[i]
    return best, best_mag


def _valley_one_pass(mags, best, best_mag):
    """The kernels' form (stage_quad.cuh, fit_edges_warp and
    fit_edge_line_warp): one pass from the right with a running minimum; the
    last index recorded is the first qualifying one."""
    accept = np.float32(0.70) * best_mag
    valley = np.float32(np.finfo(np.float32).max)
    first = -1
    for i in range(best - 2, 0, -1):
        valley = min(valley, mags[i + 1])
        if mags[i] < accept or mags[i] < mags[i - 1] or mags[i] < mags[i + 1]:
            continue
        if valley < np.float32(0.5) * mags[i]:
            first = i
    return (first, mags[first]) if first >= 0 else (best, best_mag)


def test_valley_one_pass_matches_reference_loop():
    """The one-pass valley test picks the same probe as the reference's
    quadratic loop, on random rise profiles with ties, plateaus and zeros."""
    rng = np.random.default_rng(5)
    for trial in range(4000):
        probes = int(rng.integers(5, 50))
        kind = trial % 3
        if kind == 0:
            mags = rng.uniform(0, 60, probes)
        elif kind == 1:
            mags = rng.integers(0, 6, probes) * 10.0  # many ties
        else:
            mags = np.abs(np.sin(np.arange(probes) * rng.uniform(0.2, 1.5))) * rng.uniform(5, 80)
        mags = mags.astype(np.float32)
        best, best_mag = -1, np.float32(0.0)
        for i, m in enumerate(mags):  # in-order peak scan, strict >
            if m > best_mag:
                best, best_mag = i, m
        if best <= 2:
            continue
        assert _valley_one_pass(mags, best, best_mag) == _valley_reference(mags, best, best_mag)
