"""
Generator of ff_tables.h, the float-float tables of ff.h:

    kFfExp2Tab[2j], [2j+1] = hi, lo of 2^(j/256),        j = 0..255
    kFfSinTab / kFfCosTab [2j], [2j+1] = hi, lo of sin / cos(j pi / 256),
                                                          j = 0..256

hi is the value rounded to the nearest FP32 number (ties to even) and lo the
remainder, again rounded to the nearest FP32 number (a zero of the value's
sign when the remainder is exact), so hi + lo carries about 48 significant
bits.  sin(pi) and cos(pi/2), tiny in 60 digits, round to zeros of their
computed signs.  The values are computed in 60-digit arithmetic (mpmath,
shipped with sympy) and rounded here with integer arithmetic, never through
a binary64 intermediate, so no value is rounded twice.

    python atomistica_gb300/csrc/gen_ff_tables.py > atomistica_gb300/csrc/ff_tables.h
"""

import sys

import mpmath

mpmath.mp.dps = 60


def round_f32(x):
    """x (mpf) rounded to the nearest FP32 value, ties to even, as a Python
    float (exact: every FP32 value is a binary64 value)."""
    if x == 0:
        return 0.0
    sign = -1.0 if x < 0 else 1.0
    m, e = mpmath.frexp(abs(x))  # abs(x) = m 2^e, 1/2 <= m < 1
    # quantum: 2^(e-24) for normal numbers (24 significant bits), 2^-149
    # below the normal range (subnormals; values under 2^-150 become zeros)
    qe = max(e - 24, -149)
    scaled = abs(x) / mpmath.mpf(2) ** qe
    q = int(mpmath.floor(scaled))
    rem = scaled - q
    if rem > 0.5 or (rem == 0.5 and q % 2 == 1):
        q += 1
    return sign * float(mpmath.ldexp(q, qe))


def ff_pair(x):
    hi = round_f32(x)
    r = x - mpmath.mpf(hi)
    # an exact remainder is a zero of the value's sign
    lo = round_f32(r) if r != 0 else (-0.0 if x < 0 else 0.0)
    return hi, lo


def literal(v):
    s = float(v).hex()
    if s in ("0x0.0p+0", "-0x0.0p+0"):
        return s + "f"
    mant, exp = s.split("p")
    head, frac = mant.split(".")
    return "%s.%sp%sf" % (head, frac.ljust(13, "0"), exp)


def table(name, values):
    flat = []
    for v in values:
        flat.extend(ff_pair(v))
    out = ["static __device__ const float %s[%d] = {" % (name, len(flat))]
    for q in range(0, len(flat), 6):
        out.append("    " + " ".join(literal(x) + "," for x in flat[q:q + 6]))
    out.append("};")
    return "\n".join(out)


def main(stream=sys.stdout):
    exp2 = [mpmath.mpf(2) ** (mpmath.mpf(j) / 256) for j in range(256)]
    ang = [mpmath.pi * j / 256 for j in range(257)]
    sin = [mpmath.sin(a) for a in ang]
    cos = [mpmath.cos(a) for a in ang]
    parts = [
        "// Float-float tables (hi, lo pairs, correctly rounded parts) for ff.h:",
        "// kFfExp2Tab[2j..2j+1] = 2^(j/256), j = 0..255;",
        "// kFfSinTab / kFfCosTab [2j..2j+1] = sin / cos (j pi / 256), j = 0..256.",
        "// Generated by gen_ff_tables.py (60-digit arithmetic); do not edit.",
        "#pragma once",
        "",
        "namespace gb {",
        "",
        table("kFfExp2Tab", exp2),
        "",
        table("kFfSinTab", sin),
        "",
        table("kFfCosTab", cos),
        "",
        "}  // namespace gb",
    ]
    stream.write("\n".join(parts) + "\n")


if __name__ == "__main__":
    main()
