// Word-at-a-time (SWAR) decoding of the two commonest cell shapes, as plain
// integer functions on little-endian words (the first byte is the low
// byte). Host and device: the columns kernel feeds them words it loads
// from shared memory; the CPU tests feed them words built from byte
// strings and compare with str::parse semantics.
//
//   u32:     1-10 plain digits (str::parse::<u32> of such a cell; a value
//            above u32::MAX is left to the general decoder).
//   fixed6:  [+-]?d{1,3}.d{6}: the mantissa m (integer and fraction digits)
//            and the f64 bits of m / 1e6, correctly rounded
//            (csv_geo.rs:1414-1475 divides in IEEE arithmetic; Eisel-Lemire
//            gives the same correctly rounded quotient with integer
//            operations).
// A cell they reject goes to the general decoders, which give the same
// value for every cell these accept.
#pragma once
#include <cstdint>

#include "decimal.cuh"

namespace falx {
namespace swar {

// Every byte of x that `keep` selects (0xFF per byte) is an ASCII digit.
// Per byte b < 0x80: b + 0x46 reaches bit 7 iff b > '9'; (b | 0x80) - 0x30
// keeps bit 7 iff b >= '0' and never borrows. Only a byte >= 0xBA carries
// into the byte above it; such a byte fails the test itself when kept, and
// the callers' unkept bytes are zero, or a digit and '.' checked elsewhere.
FALX_HD bool digits_ok(uint64_t x, uint64_t keep) {
    const uint64_t H = 0x8080808080808080ull;
    const uint64_t bad = (x | (x + 0x4646464646464646ull) | ~((x | H) - 0x3030303030303030ull)) & H & keep;
    return bad == 0;
}

// Four digits, the most significant in byte 0 (bytes '0'-'9' or 0):
// pairs 10 a + b in bytes 0 and 2 (each at most 99: no carries), then
// 100 x pair0 + pair1.
FALX_HD uint32_t four_digits(uint32_t w) {
    w &= 0x0F0F0F0Fu;
    w = w * 10u + (w >> 8);
    return (w & 0xFFu) * 100u + ((w >> 16) & 0xFFu);
}
FALX_HD uint32_t eight_digits(uint64_t x) {
    return four_digits((uint32_t)x) * 10000u + four_digits((uint32_t)(x >> 32));
}

// x = the 8 bytes from the cell's start, n = its length in [1, 8].
FALX_HD bool u32_word(uint64_t x, uint32_t n, uint32_t &v) {
    const uint32_t sh = 8u * (8u - n);
    x <<= sh;  // the n bytes at the top, zeros below
    if (!digits_ok(x, ~0ull << sh)) return false;
    v = eight_digits(x);
    return true;
}

// n in [9, 10]: h = the 4 bytes from the cell's start (its n - 8 leading
// digits first), t = the 8 bytes that end the cell (its last 8 digits).
// Values above u32::MAX are rejected (the general decoder reports them).
FALX_HD bool u32_word10(uint32_t h, uint64_t t, uint32_t n, uint32_t &v) {
    const uint32_t hs = 8u * (12u - n);  // the n - 8 leading digits at the top of h
    h <<= hs;
    if (!digits_ok(t, ~0ull) || !digits_ok(h, (uint64_t)(0xFFFFFFFFu << hs))) return false;
    const uint64_t x = (uint64_t)four_digits(h) * 100000000ull + eight_digits(t);
    if (x > 0xFFFFFFFFull) return false;
    v = (uint32_t)x;
    return true;
}

// n in [8, 11], c0 its first byte, sg = 1 after a sign, k = n - 7 - sg in
// [1, 3] integer digits; t = the 8 bytes that end the cell (last integer
// digit, '.', six fraction digits), u = the 4 bytes after the sign.
FALX_HD bool fixed6_words(uint32_t c0, uint32_t k, uint64_t t, uint32_t u, uint64_t &bits, uint32_t &m, bool &neg) {
    const uint32_t ish = 8u * (4u - k);
    u <<= ish;  // the k integer digits at the top
    if (((uint32_t)(t >> 8) & 0xFFu) != '.' || !digits_ok(t, 0xFFFFFFFFFFFF0000ull) ||
        !digits_ok(u, (uint64_t)(0xFFFFFFFFu << ish)))
        return false;
    m = four_digits(u) * 1000000u + eight_digits(t & 0xFFFFFFFFFFFF0000ull);
    neg = c0 == '-';
    bits = dec::eisel_lemire(m, -6) | ((uint64_t)neg << 63);
    return true;
}

}  // namespace swar
}  // namespace falx
