"""Generate fp64_tables.inc: the tables of fp64_math.cuh, correctly rounded from
50-digit decimal arithmetic (python decimal), plus the split constants.

    python gen_fp64_tables.py > fp64_tables.inc
"""
from decimal import Decimal, getcontext

getcontext().prec = 60
LN2 = Decimal(2).ln()


def d(x: Decimal) -> str:
    return float(x).hex()  # float() rounds a Decimal to nearest


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


if __name__ == "__main__":
    main()
