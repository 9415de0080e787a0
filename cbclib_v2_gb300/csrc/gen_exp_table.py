"""Generate exp_table.inc: exp(-j/256), j = 0..CBC_EXP_TABLE_N-1, as float pairs
(hi, lo) with hi = float(e) and lo = float(e - hi), for the table-driven gaussian
profile in exact.cuh (Tang's table method: exp(-t) = exp(-j/256) * exp(-(t - j/256)))."""
import math
import os
import struct

N = 1154  # covers t = (3x)^2 / 2 <= 4.5 for x <= 1 (j <= 1152)


def f32(v: float) -> float:
    return struct.unpack('f', struct.pack('f', v))[0]


def main() -> None:
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'exp_table.inc')
    rows = []
    for j in range(N):
        e = math.exp(-j / 256.0)
        hi = f32(e)
        lo = f32(e - hi)
        rows.append(f"    {{{hi.hex()}f, {lo.hex()}f}},")
    with open(out, 'w') as fh:
        fh.write("/* generated by gen_exp_table.py: {exp(-j/256) hi, lo} */\n")
        fh.write(f"#define CBC_EXP_TABLE_N {N}\n")
        fh.write("CBC_EXP_TABLE_QUALIFIER float cbc_exp_table[CBC_EXP_TABLE_N][2] = {\n")
        fh.write("\n".join(rows) + "\n};\n")


if __name__ == '__main__':
    main()
