"""Generate exp_table.h: the constants of the FP64 exponential of the rate
kernels (Tang's table-driven method, ACM TOMS 15(2), 1989).

2^(j/256) for j = 0..255 as an unevaluated sum hi + lo of two doubles (hi the
nearest double, lo the nearest double to the remainder), and ln2/256 split
into a head with 32 significant bits (so that k * head is exact for
|k| < 2^21) and a tail. Computed with Python's decimal module at 60 digits.

Usage: python metallic_glasses_gb300/csrc/exp_table.py > metallic_glasses_gb300/csrc/exp_table.h
"""
import math
from decimal import Decimal, getcontext

getcontext().prec = 60


def nearest_double(d):
    return float(d)  # Decimal -> float rounds to nearest


def split(d):
    hi = nearest_double(d)
    lo = nearest_double(d - Decimal(hi))
    return hi, lo


def main():
    ln2 = Decimal(2).ln()
    step = ln2 / 256
    # head of ln2/256: 32 significant bits
    f, ex = math.frexp(float(step))
    head = math.ldexp(math.floor(f * 2.0 ** 32) / 2.0 ** 32, ex)
    tail = nearest_double(step - Decimal(head))
    inv = nearest_double(256 / ln2)
    out = ["// Generated by exp_table.py (Tang's table-driven exponential): do not edit.",
           "// The includer defines STZ_EXP_TABLE_STORAGE (for example __device__ const).",
           "#pragma once",
           "#ifndef STZ_EXP_TABLE_STORAGE",
           "#define STZ_EXP_TABLE_STORAGE static const",
           "#endif",
           "#define STZ_EXP_INV_STEP %s   /* 256 / ln 2 */" % float(inv).hex(),
           "#define STZ_EXP_STEP_HEAD %s  /* ln 2 / 256, 32 significant bits */" % float(head).hex(),
           "#define STZ_EXP_STEP_TAIL %s  /* ln 2 / 256 - head */" % float(tail).hex(),
           "/* 2^(j/256) = kExp2Hi[j] + kExp2Lo[j] */",
           "STZ_EXP_TABLE_STORAGE double kExp2Hi[256] = {"]
    his, los = [], []
    for j in range(256):
        hi, lo = split(Decimal(2) ** (Decimal(j) / 256))
        his.append(hi)
        los.append(lo)
    for i in range(0, 256, 4):
        out.append("    " + ", ".join(float(v).hex() for v in his[i:i + 4]) + ",")
    out.append("};")
    out.append("STZ_EXP_TABLE_STORAGE double kExp2Lo[256] = {")
    for i in range(0, 256, 4):
        out.append("    " + ", ".join(float(v).hex() for v in los[i:i + 4]) + ",")
    out.append("};")
    print("\n".join(out))


if __name__ == "__main__":
    main()
