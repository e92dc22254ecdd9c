"""Generate pow5_table.h: 128-bit approximations of 5^q, q in [-342, 308].

Build step for the Eisel-Lemire decimal-to-double conversion in decimal.cuh
(D. Lemire, "Number Parsing at a Gigabyte per Second", Software: Practice and
Experience 51(8), 2021; N. Mushtak and D. Lemire, "Fast number parsing without
fallback", 2023). For q >= 0 the entry is 5^q normalised so its top bit is
bit 127 and truncated; for q < 0 it is ceil(2^b / 5^-q) for the smallest b
that puts the top bit at 127. Run: python gen_pow5.py > pow5_table.h
"""


def entries():
    out = []
    for q in range(-342, 0):
        p5 = 5 ** (-q)
        z = p5.bit_length()
        if q >= -27:
            # 5^-q < 2^64: round the reciprocal up.
            out.append((1 << (z + 127)) // p5 + 1)
        else:
            # wider quotient, then truncate to 128 bits
            c = (1 << (2 * z + 128)) // p5 + 1
            while c >= (1 << 128):
                c >>= 1
            out.append(c)
    for q in range(0, 309):
        v = 5 ** q
        while v < (1 << 127):
            v <<= 1
        while v >= (1 << 128):
            v >>= 1
        out.append(v)
    return out


def main():
    es = entries()
    print("// Generated by gen_pow5.py: 128-bit powers of five for q in [-342, 308].")
    print("// Entry (q + 342) holds {high 64 bits, low 64 bits}.")
    print("#pragma once")
    print("#define FALX_POW5_COUNT %d" % len(es))
    print("#define FALX_POW5_ENTRIES \\")
    print("    { \\")
    for v in es:
        print("        {0x%016xull, 0x%016xull}, \\" % (v >> 64, v & ((1 << 64) - 1)))
    print("    }")


if __name__ == "__main__":
    main()
