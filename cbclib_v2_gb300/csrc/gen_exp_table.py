"""Generate exp_table.inc: C * exp(-j/256), j = 0..CBC_EXP_TABLE_N-1, with C the
gaussian profile's constant 0.3989422804014327 (the double the reference writes for
1/sqrt(2 pi)), as float pairs (hi, lo): hi = float(v), lo = float(v - hi), v evaluated
with 60 significant digits; and C * exp(-j/64), j = 0..CBC_EXP_TABLE64_N-1, as double
pairs for the float64 profile.  Used by the table-driven gaussian profiles in
exact.cuh (Tang's table method: exp(-t) = exp(-j/256) * exp(-(t - j/256)))."""
import os
import struct

import mpmath

N = 1154  # covers t = (3x)^2 / 2 <= 4.5 for x <= 1 (j <= 1152)
N64 = 290  # the same range in steps of 1/64 (j <= 288)
C = 0.3989422804014327


def f32(v) -> float:
    return struct.unpack('f', struct.pack('f', float(v)))[0]


def main() -> None:
    mpmath.mp.dps = 60
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'exp_table.inc')
    rows = []
    c = mpmath.mpf(C)            # the double's exact value
    for j in range(N):
        v = c * mpmath.exp(-mpmath.mpf(j) / 256)
        hi = f32(v)
        lo = f32(v - mpmath.mpf(hi))         # hi + lo within 2^-48 of v
        rows.append(f"    {{{hi.hex()}f, {lo.hex()}f}},")
    rows64 = []
    for j in range(N64):
        v = c * mpmath.exp(-mpmath.mpf(j) / 64)
        hi = float(v)
        lo = float(v - mpmath.mpf(hi))       # hi + lo within 2^-106 of v
        rows64.append(f"    {{{hi.hex()}, {lo.hex()}}},")
    with open(out, 'w') as fh:
        fh.write("/* generated by gen_exp_table.py: {C exp(-j/256) hi, lo}, C = 0.3989422804014327 */\n")
        fh.write(f"#define CBC_EXP_TABLE_N {N}\n")
        fh.write("CBC_EXP_TABLE_QUALIFIER float cbc_gauss_table[CBC_EXP_TABLE_N][2] = {\n")
        fh.write("\n".join(rows) + "\n};\n")
        fh.write("/* {C exp(-j/64) hi, lo} as doubles, for the float64 gaussian */\n")
        fh.write(f"#define CBC_EXP_TABLE64_N {N64}\n")
        fh.write("CBC_EXP_TABLE_QUALIFIER double cbc_gauss_table64[CBC_EXP_TABLE64_N][2] = {\n")
        fh.write("\n".join(rows64) + "\n};\n")


if __name__ == '__main__':
    main()
