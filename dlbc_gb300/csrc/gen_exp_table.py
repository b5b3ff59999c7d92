"""Write lb_exp_table.h: the constants of the integer exp (lbmath::lb_exp in
lb_math.h), computed with 80-digit decimal arithmetic.

  kExp256[j] = round(2^(j/256) * 2^127), j = 0..255, as (high, low) words
  kExpK      = round(256/ln2 * 2^55)
  kExpL136   = round(ln2/256 * 2^136) as (high, low) words
  kExpP0..5  = round(2^63 / (i+3)!), i = 0..5

Run: python gen_exp_table.py > lb_exp_table.h
"""
import decimal
import math

D = decimal.Decimal
decimal.getcontext().prec = 80
LN2 = D(2).ln()


def rnd(v):
    return int(v.to_integral_value(rounding=decimal.ROUND_HALF_EVEN))


def words(v):
    return v >> 64, v & ((1 << 64) - 1)


def main():
    out = ["// Generated by gen_exp_table.py (80-digit decimal arithmetic); do not edit.",
           "// Constants of the integer exp in lb_math.h.", "#pragma once", "", "#include <stdint.h>", "",
           "namespace lbmath {", ""]
    out.append(f"constexpr uint64_t kExpK = 0x{rnd(D(256) / LN2 * D(2) ** 55):016x}ull;  // 256/ln2 * 2^55")
    hi, lo = words(rnd(LN2 / D(256) * D(2) ** 136))
    out.append(f"constexpr uint64_t kExpL136Hi = 0x{hi:016x}ull, kExpL136Lo = 0x{lo:016x}ull;  // ln2/256 * 2^136")
    ps = [rnd(D(2) ** 63 / D(math.factorial(i + 3))) for i in range(6)]
    out.append("// 2^63/(i+3)!, i = 0..5")
    out.append("constexpr int64_t " + ", ".join(f"kExpP{i} = 0x{p:016x}ll" for i, p in enumerate(ps)) + ";")
    out.append("")
    out.append("// 2^(j/256) * 2^127 as {high, low} words")
    out.append("LB_EXP256_QUAL uint64_t kExp256[256][2] = {")
    for j in range(256):
        hi, lo = words(rnd(D(2) ** (D(j) / D(256)) * D(2) ** 127))
        out.append(f"    {{0x{hi:016x}ull, 0x{lo:016x}ull}},")
    out.append("};")
    out.append("")
    out.append("}  // namespace lbmath")
    print("\n".join(out))


if __name__ == "__main__":
    main()
