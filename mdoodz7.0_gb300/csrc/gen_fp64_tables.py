"""Generate fp64_tables.inc: the tables of fp64_math.cuh and dd_math.cuh, correctly
rounded from 60-digit decimal arithmetic (python decimal), plus the split constants.
A double-float entry is the pair (hi, lo) of FP32 numbers with hi the value rounded to
FP32 and lo the remainder rounded to FP32.

    python gen_fp64_tables.py > fp64_tables.inc
"""
from decimal import Decimal, getcontext

import numpy as np

getcontext().prec = 60
LN2 = Decimal(2).ln()


def d(x: Decimal) -> str:
    return float(x).hex()  # float() rounds a Decimal to nearest


def f(x: Decimal) -> str:
    return float(np.float32(float(x))).hex() + "f"  # the value rounded to FP32


def pair(x: Decimal) -> str:
    hi = Decimal(float(np.float32(float(x))))
    return "{" + f(x) + ", " + f(x - hi) + "}"


def main():
    print("// generated by gen_fp64_tables.py -- do not edit")
    print("#define MDZ_EXP2J_TABLE { \\")
    print(", \\\n".join(", ".join(d((LN2 * j / 256).exp()) for j in range(r, r + 4)) for r in range(0, 256, 4)) + " }")
    print("#define MDZ_INVF_TABLE { \\")
    vals = [d(Decimal(256) / j) for j in range(192, 385)]
    print(", \\\n".join(", ".join(vals[i:i + 4]) for i in range(0, len(vals), 4)) + " }")
    print("#define MDZ_LOGF_TABLE { \\")
    vals = [d((Decimal(j) / 256).ln()) for j in range(192, 385)]
    print(", \\\n".join(", ".join(vals[i:i + 4]) for i in range(0, len(vals), 4)) + " }")
    c = LN2 / 256
    c_hi = Decimal(float(c))
    print(f"#define MDZ_LN2_256_HI {d(c)}")
    print(f"#define MDZ_LN2_256_LO {d(c - c_hi)}")
    print(f"#define MDZ_INV_LN2_256 {d(256 / LN2)}")
    l_hi = Decimal(float(LN2))
    print(f"#define MDZ_LN2_HI {d(LN2)}")
    print(f"#define MDZ_LN2_LO {d(LN2 - l_hi)}")
    # double-float tables: 2^(j/256), log(j/256) and 256/j as in the FP64 tables
    print("#define MDZ_EXP2J_DD_TABLE { \\")
    print(", \\\n".join(", ".join(pair((LN2 * j / 256).exp()) for j in range(r, r + 4)) for r in range(0, 256, 4)) + " }")
    print("#define MDZ_LOGF_DD_TABLE { \\")
    vals = [pair((Decimal(j) / 256).ln()) for j in range(192, 385)]
    print(", \\\n".join(", ".join(vals[i:i + 4]) for i in range(0, len(vals), 4)) + " }")
    print("#define MDZ_INVF_F32_TABLE { \\")
    vals = [f(Decimal(256) / j) for j in range(192, 385)]
    print(", \\\n".join(", ".join(vals[i:i + 8]) for i in range(0, len(vals), 8)) + " }")
    # ln2/256 in three FP32 parts for the argument reduction of exp: the first with 8
    # significant bits (177 / 2^16), so k * part is exact for |k| < 2^15
    c1 = Decimal(int((c * 2 ** 16).to_integral_value(rounding="ROUND_FLOOR"))) / Decimal(2) ** 16
    c2 = Decimal(float(np.float32(float(c - c1))))
    c3 = Decimal(float(np.float32(float(c - c1 - c2))))
    print(f"#define MDZ_LN2_256_F1 {f(c1)}")
    print(f"#define MDZ_LN2_256_F2 {f(c2)}")
    print(f"#define MDZ_LN2_256_F3 {f(c3)}")
    print(f"#define MDZ_INV_LN2_256_F {f(256 / LN2)}")
    # ln2 in three FP32 parts: the first with 16 significant bits, so m * part is exact
    # for |m| < 2^7
    l1 = Decimal(int((LN2 * 2 ** 16).to_integral_value(rounding="ROUND_FLOOR"))) / Decimal(2) ** 16
    l2 = Decimal(float(np.float32(float(LN2 - l1))))
    l3 = Decimal(float(np.float32(float(LN2 - l1 - l2))))
    print(f"#define MDZ_LN2_F1 {f(l1)}")
    print(f"#define MDZ_LN2_F2 {f(l2)}")
    print(f"#define MDZ_LN2_F3 {f(l3)}")


if __name__ == "__main__":
    main()
