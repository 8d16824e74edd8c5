"""Generates tests/golden/convex_hull_fixtures.npz from the parry repository's own convex-hull tests
(crates/parry3d/tests/geometry/convex_hull.rs: `test_complex_convex_hull`, a 4,000-point cloud, and
`test_planar_convex_hull`, 8 coplanar points). Each test builds `transformation::convex_hull` of
its cloud and requires `transformation::check_convex_hull` to accept the result.

    python tests/golden/make_hull_fixtures.py [path to the parry repository]

The point literals are read from the test file and rounded to f32 exactly as Rust rounds an f32
literal (correctly rounded, ties to even), via exact rational arithmetic rather than through f64.
"""
import re
import sys
from fractions import Fraction
from pathlib import Path

import numpy as np

TEST_FILE = "crates/parry3d/tests/geometry/convex_hull.rs"
POINT = re.compile(r"Point3::new\(\s*([-+0-9.eE]+)\s*,\s*([-+0-9.eE]+)\s*,\s*([-+0-9.eE]+)\s*\)")


def f32_of_literal(s: str) -> np.float32:
    """The f32 nearest to the decimal literal `s` (ties to even)."""
    x = Fraction(s)
    c = np.float32(float(x))
    best = c
    for cand in (np.nextafter(c, np.float32(-np.inf)), np.nextafter(c, np.float32(np.inf))):
        d_best, d_cand = abs(Fraction(float(best)) - x), abs(Fraction(float(cand)) - x)
        if d_cand < d_best or (d_cand == d_best and (int(cand.view(np.uint32)) & 1) == 0):
            best = cand
    return best


def clouds(text: str) -> dict:
    """Point clouds of the test functions, by test name."""
    out = {}
    for m in re.finditer(r"fn\s+(\w+)\s*\(\s*\)\s*\{(.*?)\n\}", text, re.S):
        pts = [[f32_of_literal(v) for v in p] for p in POINT.findall(m.group(2))]
        if pts:
            out[m.group(1)] = np.array(pts, np.float32)
    return out


def main():
    ref = Path(sys.argv[1]) if len(sys.argv) > 1 else Path("/root/reference")
    found = clouds((ref / TEST_FILE).read_text())
    assert set(found) == {"test_complex_convex_hull", "test_planar_convex_hull"}, sorted(found)
    out = Path(__file__).resolve().parent / "convex_hull_fixtures.npz"
    np.savez_compressed(out, complex=found["test_complex_convex_hull"], planar=found["test_planar_convex_hull"],
                        source=np.array(TEST_FILE))
    print(out, {k: v.shape for k, v in found.items()})


if __name__ == "__main__":
    main()
