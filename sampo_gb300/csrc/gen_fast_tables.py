"""Generate sampo_fast_tables.h: the breakpoint tables of the binary32 fast
paths in sampo_math_fast.h (log on (0, 1], sin on [0, 2*pi]).

Every entry is computed with mpmath at 300 bits and rounded once to binary32
(round to nearest even), so the header is the same wherever it is made.

  log table, 128 entries, indexed by the 7 mantissa bits that follow the
  reduction offset 0x3F340000 (m in [0.703125, 1.40625)):
      c  = 1 / (centre of the entry's m interval), rounded to binary32;
           exactly 1 for the two entries that touch m = 1
      Th + Tl = -log(c) as an unevaluated binary32 pair
  sin table, 513 entries for k = 0..512, x_k = k * pi / 256:
      Ph + Pm + Pl = x_k as an unevaluated binary32 triple
      Sh + Sl = sin(x_k),  Ch + Cl = cos(x_k)  (exact 0 and +-1 where they are)
  constants: ln 2 = LN2_A + LN2_B + LN2_C with A and B of 16 significant
      bits (k * A and k * B are exact for |k| < 256); 256/pi.

Run: python sampo_gb300/csrc/gen_fast_tables.py  (rewrites the header beside it)
"""
import os
import struct

import mpmath as mp

mp.mp.prec = 300
LOG_OFF = 0x3F340000
LOG_ONE_ENTRIES = (75, 76)   # [1 - 2^-8, 1) and [1, 1 + 2^-7)


def f32(x):
    """Round an mpf to the nearest binary32 (ties to even), as a Python float."""
    if x == 0:
        return 0.0
    with mp.workprec(24):
        y = +mp.mpf(x)
    v = float(y)
    assert struct.unpack("<f", struct.pack("<f", v))[0] == v
    return v


def bits_to_f32(u):
    return struct.unpack("<f", struct.pack("<I", u))[0]


def lit(v):
    if v == 0.0:
        return "0.0f" if struct.pack("<d", v)[0:8] == struct.pack("<d", 0.0) else "-0.0f"
    return float(v).hex() + "f"


def split2(x):
    h = f32(x)
    return h, f32(x - h)


def split3(x):
    h = f32(x)
    m = f32(x - h)
    return h, m, f32(x - h - m)


def bits_round(x, nb):
    """Round an mpf to nb significant bits."""
    with mp.workprec(nb):
        return float(+mp.mpf(x))


def constants():
    ln2 = mp.log(2)
    a = bits_round(ln2, 16)
    b = bits_round(ln2 - a, 16)
    c = f32(ln2 - a - b)
    return [("SAMPO_FAST_LN2_A", a), ("SAMPO_FAST_LN2_B", b), ("SAMPO_FAST_LN2_C", c),
            ("SAMPO_FAST_256_OVER_PI", f32(256 / mp.pi))]


def log_table():
    rows = []
    for i in range(128):
        lo = mp.mpf(bits_to_f32(LOG_OFF + (i << 16)))
        hi = mp.mpf(bits_to_f32(LOG_OFF + ((i + 1) << 16)))
        if i in LOG_ONE_ENTRIES:
            rows.append((1.0, 0.0, 0.0, 0.0))
            continue
        c = f32(1 / ((lo + hi) / 2))
        th, tl = split2(-mp.log(mp.mpf(c)))
        rows.append((c, th, tl, 0.0))
    return rows


def sin_table():
    rows = []
    for k in range(513):
        x = k * mp.pi / 256
        ph, pm, pl = split3(x)
        if k % 128 == 0:
            q = k // 128
            s = (0.0, 1.0, 0.0, -1.0, 0.0)[q]
            c = (1.0, 0.0, -1.0, 0.0, 1.0)[q]
            sh, sl, ch, cl = s, 0.0, c, 0.0
        else:
            sh, sl = split2(mp.sin(x))
            ch, cl = split2(mp.cos(x))
        rows.append(((ph, pm, pl, 0.0), (sh, sl, ch, cl)))
    return rows


def main():
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "sampo_fast_tables.h")
    lines = [
        "/* sampo_fast_tables.h - generated by gen_fast_tables.py; do not edit. */",
        "#ifndef SAMPO_FAST_TABLES_H",
        "#define SAMPO_FAST_TABLES_H",
        "",
    ]
    lines += ["#define %s %s" % (n, lit(v)) for n, v in constants()]
    lines += [
        "",
        "/* {c, Th, Tl, 0}: m in [0.703125, 1.40625) split at the 7 bits after 0x3F340000 */",
        "#define SAMPO_LOG_TABLE_INIT { \\",
    ]
    for r in log_table():
        lines.append("  {" + ", ".join(lit(v) for v in r) + "}, \\")
    lines += ["}", "", "/* {Ph, Pm, Pl, 0}, {Sh, Sl, Ch, Cl} for x_k = k*pi/256, k = 0..512 */",
              "#define SAMPO_SIN_TABLE_INIT { \\"]
    for a, b in sin_table():
        lines.append("  {{" + ", ".join(lit(v) for v in a) + "}, {" + ", ".join(lit(v) for v in b) + "}}, \\")
    lines += ["}", "", "#endif", ""]
    with open(out, "w") as f:
        f.write("\n".join(lines))
    print("wrote", out)


if __name__ == "__main__":
    main()
