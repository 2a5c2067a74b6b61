"""Writes pc_exp_tables.h: the tables of pc_exp.h, computed with 60-digit
decimal arithmetic and rounded to double (hex literals).

  exp: T[j] = 2^(j/64) = hi + lo, j = 0..63
  log: F_j = 1 + j/128, j = 0..128: 1/F_j rounded, log(F_j) = hi + lo with hi
       a multiple of 2^-42, like ln2_hi (so m ln2_hi + hi is exact for
       |m| < 2^11)
  ln2/64 = hi + lo with hi of 31 significant bits (kd hi exact for |kd| < 2^22).

Run: python gen_exp_tables.py > pc_exp_tables.h
"""
from decimal import Decimal, getcontext

getcontext().prec = 60


def hexd(d: Decimal) -> str:
    return float(d).hex()


def on_grid(d: Decimal, ulp_exp: int):
    """(hi, lo): hi = d rounded to a multiple of 2^ulp_exp, lo = d - hi rounded."""
    scale = Decimal(2) ** (-ulp_exp)
    hi = (d * scale).to_integral_value() / scale
    return float(hi), float(d - hi)


def split(d: Decimal, bits: int):
    """(hi, lo): hi = d rounded to `bits` significant bits, lo = d - hi rounded."""
    f = float(d)
    if f == 0.0:
        return 0.0, float(d)
    import math

    e = math.frexp(f)[1]
    scale = Decimal(2) ** (bits - e)
    hi = (d * scale).to_integral_value() / scale
    return float(hi), float(d - hi)


LN2 = Decimal(2).ln()
lines = ["// Generated by gen_exp_tables.py; do not edit.", "#pragma once", ""]
l1, l2 = split(LN2 / 64, 31)
lines.append(f"#define PC_EXP_LN2_64_HI {l1.hex()}  // ln2/64, 31 significant bits")
lines.append(f"#define PC_EXP_LN2_64_LO {l2.hex()}")
lines.append(f"#define PC_EXP_64_LN2 {hexd(64 / LN2)}")
h1, h2 = on_grid(LN2, -42)
lines.append(f"#define PC_LOG_LN2_HI {h1.hex()}  // ln2 on the 2^-42 grid")
lines.append(f"#define PC_LOG_LN2_LO {h2.hex()}")
lines.append("")
lines.append("#define PC_EXP_TABLE_HI { \\")
his, los = [], []
for j in range(64):
    v = Decimal(2) ** (Decimal(j) / 64)
    hi = float(v)
    his.append(hi.hex())
    los.append(float(v - Decimal(hi)).hex())
for i in range(0, 64, 4):
    lines.append("  " + ", ".join(his[i:i + 4]) + ", \\")
lines.append("}")
lines.append("#define PC_EXP_TABLE_LO { \\")
for i in range(0, 64, 4):
    lines.append("  " + ", ".join(los[i:i + 4]) + ", \\")
lines.append("}")
inv, lh, ll = [], [], []
for j in range(129):
    F = 1 + Decimal(j) / 128
    inv.append(float(1 / F).hex())
    a, b = on_grid(F.ln(), -42)
    lh.append(a.hex())
    ll.append(b.hex())
for name, arr in (("PC_LOG_TABLE_INV", inv), ("PC_LOG_TABLE_HI", lh), ("PC_LOG_TABLE_LO", ll)):
    lines.append(f"#define {name} {{ \\")
    for i in range(0, 129, 4):
        lines.append("  " + ", ".join(arr[i:i + 4]) + ", \\")
    lines.append("}")
print("\n".join(lines))
