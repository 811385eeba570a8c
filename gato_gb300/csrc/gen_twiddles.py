"""Regenerate twiddles.cuh: cos and sin of 2 pi e / R for the register DFT radices."""
import math
import os

RADICES = [4, 6, 8, 10, 12, 14, 16, 20, 24]


def _exact(x):
    """Snap values that are exactly 0, +-1/2, +-1 mathematically (roundoff of pi)."""
    for v in (0.0, 0.5, -0.5, 1.0, -1.0):
        if abs(x - v) < 1e-15:
            return v
    return x


def cos_sin(e, R):
    """Correctly rounded cos/sin(2 pi e / R), evaluated with 50 significant digits."""
    import mpmath
    mpmath.mp.dps = 50
    a = 2 * mpmath.pi * e / R
    return _exact(float(mpmath.cos(a))), _exact(float(mpmath.sin(a)))


def main():
    lines = ["// cos / sin (2 pi e / R) for the in-register DFT twiddles, e < R, as switch",
             "// functions that fold to immediates once e is a compile-time constant.",
             "// Generated (correctly rounded) by gato_gb300/csrc/gen_twiddles.py.",
             "#pragma once", "", "namespace gato {", "", "template <int R> struct TwC;"]
    for R in RADICES:
        cs = [cos_sin(e, R) for e in range(R)]
        lines.append(f"template <> struct TwC<{R}> {{")
        for name, idx in (("c", 0), ("s", 1)):
            lines.append(f"  __host__ __device__ static constexpr double {name}(int e) {{")
            lines.append("    switch (e) {")
            for e in range(R):
                lines.append(f"      case {e}: return {cs[e][idx]!r};")
            lines.append("      default: return 0.0;")
            lines.append("    }")
            lines.append("  }")
        lines.append("};")
    lines += ["", "}  // namespace gato", ""]
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "twiddles.cuh"), "w") as f:
        f.write("\n".join(lines))


if __name__ == "__main__":
    main()
