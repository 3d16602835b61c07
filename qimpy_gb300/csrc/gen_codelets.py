"""Generate ``codelets.cuh``: straight-line complex DFTs of small sizes for CUDA.

Each codelet computes X[k] = sum_n x[n] exp(SIGN * 2 pi i n k / R) in registers
for R in CODELET_SIZES and SIGN in {-1, +1}.  Prime sizes use the classic
symmetric butterflies (radix 2, 3, 4, 5 and 7); composite sizes are built at
generation time by the Cooley-Tukey split R = R1 * R2 with constant twiddles,
folding trivial ones (1, -1, +-i, eighth turns).  Constants are printed with
17 significant digits from Python's float64 trigonometry.

Usage: python gen_codelets.py > codelets.cuh   (the build does this when the
header is missing or older than this script).
"""
from __future__ import annotations

import math
import sys

CODELET_SIZES = (1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 12, 14, 15, 16)


class Emitter:
    def __init__(self):
        self.lines: list[str] = []
        self.n = 0

    def tmp(self, expr: str) -> str:
        name = f"t{self.n}"
        self.n += 1
        self.lines.append(f"  const T {name} = {expr};")
        return name


def lit(v: float) -> str:
    return f"T({v!r})"


def cadd(e, a, b):
    return (e.tmp(f"{a[0]} + {b[0]}"), e.tmp(f"{a[1]} + {b[1]}"))


def csub(e, a, b):
    return (e.tmp(f"{a[0]} - {b[0]}"), e.tmp(f"{a[1]} - {b[1]}"))


def cmul_i(e, a, s):
    """s * i * a for s = +-1: i(x + iy) = -y + ix."""
    if s > 0:
        return (e.tmp(f"-{a[1]}"), a[0])
    return (a[1], e.tmp(f"-{a[0]}"))


def cscale(e, a, c):
    return (e.tmp(f"{lit(c)} * {a[0]}"), e.tmp(f"{lit(c)} * {a[1]}"))


def twiddle(e, a, num: int, den: int, s: int):
    """a * exp(s * 2 pi i num / den), folding the exact cases."""
    num %= den
    if num == 0:
        return a
    g = math.gcd(num, den)
    num, den = num // g, den // g
    if den == 2:
        return (e.tmp(f"-{a[0]}"), e.tmp(f"-{a[1]}"))
    if den == 4:
        return cmul_i(e, a, s if num == 1 else -s)
    if den == 8:
        # exp(s*i*pi*num/4) = (cx + i s sx) with |cx| = |sx| = 1/sqrt(2)
        h = math.sqrt(0.5)
        c = math.cos(math.pi * num / 4.0)
        sn = s * math.sin(math.pi * num / 4.0)
        cs, ss = (1 if c > 0 else -1), (1 if sn > 0 else -1)
        # (x + iy)(cs + i ss) h = h[(cs x - ss y) + i(ss x + cs y)]
        re = f"{lit(h)} * ({'' if cs > 0 else '-'}{a[0]} {'-' if ss > 0 else '+'} {a[1]})"
        im = f"{lit(h)} * ({'' if ss > 0 else '-'}{a[0]} {'+' if cs > 0 else '-'} {a[1]})"
        return (e.tmp(re), e.tmp(im))
    ang = 2.0 * math.pi * num / den
    c, sn = math.cos(ang), s * math.sin(ang)
    re = e.tmp(f"{lit(c)} * {a[0]} - {lit(sn)} * {a[1]}")
    im = e.tmp(f"{lit(c)} * {a[1]} + {lit(sn)} * {a[0]}")
    return (re, im)


def dft2(e, x, s):
    return [cadd(e, x[0], x[1]), csub(e, x[0], x[1])]


def dft3(e, x, s):
    c = math.sqrt(3.0) / 2.0
    t1 = cadd(e, x[1], x[2])
    t2 = (e.tmp(f"{x[0][0]} - {lit(0.5)} * {t1[0]}"), e.tmp(f"{x[0][1]} - {lit(0.5)} * {t1[1]}"))
    d = csub(e, x[1], x[2])
    t3 = cmul_i(e, cscale(e, d, c), s)
    return [cadd(e, x[0], t1), cadd(e, t2, t3), csub(e, t2, t3)]


def dft4(e, x, s):
    a = cadd(e, x[0], x[2])
    b = cadd(e, x[1], x[3])
    c = csub(e, x[0], x[2])
    d = cmul_i(e, csub(e, x[1], x[3]), s)
    return [cadd(e, a, b), cadd(e, c, d), csub(e, a, b), csub(e, c, d)]


def dft_odd_prime(e, x, s, R):
    """Symmetric real/imaginary split for an odd prime R (used for 5 and 7)."""
    h = (R - 1) // 2
    a = [cadd(e, x[j], x[R - j]) for j in range(1, h + 1)]
    b = [csub(e, x[j], x[R - j]) for j in range(1, h + 1)]
    out = [None] * R
    s0 = x[0]
    for aj in a:
        s0 = cadd(e, s0, aj)
    out[0] = s0
    for k in range(1, h + 1):
        re_terms = [x[0][0]] + [f"{lit(math.cos(2 * math.pi * j * k / R))} * {a[j - 1][0]}" for j in range(1, h + 1)]
        im_terms = [x[0][1]] + [f"{lit(math.cos(2 * math.pi * j * k / R))} * {a[j - 1][1]}" for j in range(1, h + 1)]
        P = (e.tmp(" + ".join(re_terms)), e.tmp(" + ".join(im_terms)))
        # Q = sum_j sin(2 pi j k / R) * b_j ; contribution s * i * Q
        q_re = " + ".join(f"{lit(math.sin(2 * math.pi * j * k / R))} * {b[j - 1][0]}" for j in range(1, h + 1))
        q_im = " + ".join(f"{lit(math.sin(2 * math.pi * j * k / R))} * {b[j - 1][1]}" for j in range(1, h + 1))
        Q = (e.tmp(q_re), e.tmp(q_im))
        iQ = cmul_i(e, Q, s)
        out[k] = cadd(e, P, iQ)
        out[R - k] = csub(e, P, iQ)
    return out


def smallest_factor(R):
    for p in (4, 2, 3, 5, 7):
        if R % p == 0:
            return p
    raise ValueError(R)


def dft(e, x, s):
    R = len(x)
    if R == 1:
        return list(x)
    if R == 2:
        return dft2(e, x, s)
    if R == 3:
        return dft3(e, x, s)
    if R == 4:
        return dft4(e, x, s)
    if R in (5, 7):
        return dft_odd_prime(e, x, s, R)
    # Cooley-Tukey R = R1 * R2: n = n1 + R1 n2, k = k2 + R2 k1
    R1 = smallest_factor(R)
    if R1 == R:
        R1 = 2
    R2 = R // R1
    Y = {}
    for n1 in range(R1):
        col = dft(e, [x[n1 + R1 * n2] for n2 in range(R2)], s)
        for k2 in range(R2):
            Y[(n1, k2)] = twiddle(e, col[k2], n1 * k2, R, s)
    X = [None] * R
    for k2 in range(R2):
        row = dft(e, [Y[(n1, k2)] for n1 in range(R1)], s)
        for k1 in range(R1):
            X[k2 + R2 * k1] = row[k1]
    return X


def emit_codelet(R: int, s: int) -> str:
    e = Emitter()
    x = [(f"re[{j}]", f"im[{j}]") for j in range(R)]
    X = dft(e, x, s)
    body = list(e.lines)
    # Copy outputs into temporaries first (inputs may still be referenced).
    outs = []
    for j, (a, b) in enumerate(X):
        outs.append(f"  const T o{j}r = {a};\n  const T o{j}i = {b};")
    stores = [f"  re[{j}] = o{j}r; im[{j}] = o{j}i;" for j in range(R)]
    name = "fwd" if s < 0 else "inv"
    return (
        f"template <typename T>\n__device__ __forceinline__ void dft{R}_{name}(T* __restrict__ re, T* __restrict__ im) {{\n"
        + "\n".join(body + outs + stores)
        + "\n}\n"
    )


def main() -> None:
    out = [
        "// Generated by gen_codelets.py -- do not edit.",
        "// Straight-line complex DFTs X[k] = sum_n x[n] exp(SIGN 2 pi i n k / R);",
        "// *_fwd uses SIGN = -1, *_inv uses SIGN = +1.",
        "#pragma once",
        "",
        "namespace qgb {",
        "",
    ]
    for R in CODELET_SIZES:
        for s in (-1, +1):
            out.append(emit_codelet(R, s))
    out.append("// Codelet<R, SIGN>::run dispatches to dft{R}_{fwd,inv} at compile time.")
    out.append("template <int R, int SIGN> struct Codelet;")
    for R in CODELET_SIZES:
        for s, name in ((-1, "fwd"), (1, "inv")):
            out.append(
                f"template <> struct Codelet<{R}, {s}> {{ template <typename T> "
                f"__device__ __forceinline__ static void run(T* re, T* im) {{ dft{R}_{name}(re, im); }} }};"
            )
    out.append("")
    out.append("#define QGB_CODELET_SIZES " + ", ".join(str(r) for r in CODELET_SIZES))
    out.append("}  // namespace qgb")
    sys.stdout.write("\n".join(out) + "\n")


if __name__ == "__main__":
    main()
