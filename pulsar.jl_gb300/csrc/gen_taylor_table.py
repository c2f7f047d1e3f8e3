"""Generate ``taylor_table.h``: the largest 1-norm theta_m for which the
truncated Taylor series of exp of degree m has a tail below the unit roundoff.

For ||B||_1 <= theta the remainder of T_m(B) = sum_{k<=m} B^k/k! obeys
    ||exp(B) - T_m(B)|| <= sum_{k>m} theta^k / k!  =: tail_m(theta),
and theta_m is the largest theta with tail_m(theta) <= u (bisection).  The
scaling-and-squaring drivers pick, per slice, the degree m and squarings s
with ||A||_1 / 2^s <= theta_m that minimise the matrix products: degrees
{4,8,12,16,20} (3 + m/4 - 1 products, + s) in FP64 and FP32, and every degree
m = q L with block size q in {2, 3, 4} in df (costed by the products it
executes).  This is the standard
forward-error bound of a truncated exponential series; the constants below are
computed here, not taken from any library.

Run:  python gen_taylor_table.py > taylor_table.h
"""
import math
import sys

DEGREES = (4, 8, 12, 16, 20)


def tail(theta: float, m: int) -> float:
    s, term, k = 0.0, theta ** (m + 1) / math.factorial(m + 1), m + 1
    while term > 1e-40 * max(s, 1e-300) and k < 200:
        s += term
        k += 1
        term *= theta / k
    return s


def theta_for(m: int, u: float) -> float:
    lo, hi = 0.0, 64.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if tail(mid, m) <= u:
            lo = mid
        else:
            hi = mid
    return lo


def main(out=sys.stdout):
    # df32 (hi + lo float pairs) carries ~48 significant bits; its table keeps
    # the truncation below 2^-47, under the df rounding of one product.
    u64, u32, udf = 2.0 ** -53, 2.0 ** -24, 2.0 ** -47
    print("// Generated by gen_taylor_table.py -- do not edit.", file=out)
    print("#pragma once", file=out)
    assert DEGREES == tuple(4 * (i + 1) for i in range(len(DEGREES)))
    print(f"#define PGX_N_DEGREES {len(DEGREES)}  /* degrees 4, 8, ..., 4*N */", file=out)
    for name, u in (("PGX_THETA64_INIT", u64), ("PGX_THETA32_INIT", u32), ("PGX_THETADF_INIT", udf)):
        vals = ", ".join(f"{theta_for(m, u):.17g}" for m in DEGREES)
        print(f"#define {name} {{{vals}}}", file=out)
    # every degree 1..20 in df, for the df expm's choice of Paterson-Stockmeyer
    # block size q in {2, 3, 4} (degrees m = q L)
    vals = ", ".join(f"{theta_for(m, udf):.17g}" for m in range(1, max(DEGREES) + 1))
    print(f"#define PGX_THETADF_ALL_INIT {{{vals}}}  /* index m - 1 */", file=out)
    inv = ", ".join(f"{1.0 / math.factorial(k):.17g}" for k in range(max(DEGREES) + 1))
    print(f"#define PGX_N_INVFACT {max(DEGREES) + 1}", file=out)
    print(f"#define PGX_INVFACT_INIT {{{inv}}}", file=out)
    # 1/k! as a float (FP32 Taylor) and as a double-float pair hi + lo (df Taylor)
    import numpy as np
    his, pairs = [], []
    for k in range(max(DEGREES) + 1):
        x = 1.0 / math.factorial(k)
        hi = np.float32(x)
        lo = np.float32(x - float(hi))
        his.append(f"{float(hi):.9e}f")
        pairs.append(f"{{{float(hi):.9e}f, {float(lo):.9e}f}}")
    print(f"#define PGX_INVFACT32_INIT {{{', '.join(his)}}}", file=out)
    print(f"#define PGX_INVFACT_DF_INIT {{{', '.join(pairs)}}}", file=out)


if __name__ == "__main__":
    main()
