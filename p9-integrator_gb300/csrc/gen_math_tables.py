"""Generate merc_math_tables.h: the constants of merc_math.h, rounded from
50-digit mpmath values (run: python gen_math_tables.py > merc_math_tables.h)."""
import mpmath as mp

mp.mp.dps = 60


def d(x):
    return float(x)


def split(x, n=3):
    """x as a sum of n doubles (each the rounding of the remainder)."""
    parts = []
    r = mp.mpf(x)
    for _ in range(n):
        p = d(r)
        parts.append(p)
        r = r - mp.mpf(p)
    return parts


def lit(v):
    return float(v).hex()


out = []
out.append("// Generated by gen_math_tables.py from 60-digit mpmath values. Do not edit.")
out.append("#pragma once")
p1, p2, p3 = split(mp.pi / 2, 3)
out.append(f"#define MERC_PIO2_1 {lit(p1)}")
out.append(f"#define MERC_PIO2_2 {lit(p2)}")
out.append(f"#define MERC_PIO2_3 {lit(p3)}")
h, l = split(mp.pi / 2, 2)
out.append(f"#define MERC_PIO2_HI {lit(h)}")
out.append(f"#define MERC_PIO2_LO {lit(l)}")
h, l = split(mp.pi, 2)
out.append(f"#define MERC_PI_HI {lit(h)}")
out.append(f"#define MERC_PI_LO {lit(l)}")
out.append(f"#define MERC_2_OVER_PI {lit(d(2 / mp.pi))}")
h, l = split(mp.log(2), 2)
out.append(f"#define MERC_LN2_HI {lit(h)}")
out.append(f"#define MERC_LN2_LO {lit(l)}")
out.append(f"#define MERC_INV_LN2 {lit(d(1 / mp.log(2)))}")
hi, lo = [], []
for k in range(17):
    a, b = split(mp.atan(mp.mpf(k) / 16), 2)
    hi.append(lit(a))
    lo.append(lit(b))
out.append("// atan(k/16), k = 0..16, as hi + lo")
out.append("#define MERC_ATAN_TABLE_HI {" + ", ".join(hi) + "}")
out.append("#define MERC_ATAN_TABLE_LO {" + ", ".join(lo) + "}")
print("\n".join(out))
