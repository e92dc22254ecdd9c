// Cell decoders with Rust `str::parse` semantics, for device code (also
// compiles as host C++ so the CPU tests can exercise it).
//
//  parse_f64: the str::parse::<f64> grammar (optional sign; digits with an
//    optional '.', at least one mantissa digit; optional e/E exponent with at
//    least one digit; or inf / infinity / nan, ASCII case-insensitive) and the
//    correctly rounded IEEE binary64 value. Paths:
//      - Clinger's exact fast path (w <= 2^53, |q| <= 22): one IEEE op;
//      - Eisel-Lemire with 128-bit powers of five (Lemire 2021; the
//        no-fallback analysis of Mushtak & Lemire 2023) for up to 19
//        significant digits, and for longer mantissas when the truncated and
//        incremented mantissas agree;
//      - otherwise a big-decimal conversion (the "simple decimal" method:
//        repeated exact shifts of a decimal digit string by powers of two,
//        then round-half-even), as used by Go's strconv and Rust's dec2flt.
//  parse_i64 / parse_u32: str::parse::<i64> / ::<u32>.
//  exact_e6: value * 1e6 as an exact integer for [+-]?d*(.d{0,6})? cells.
//
// The reference's f64 cell path (csv_geo.rs:1313-1486) is a fixed-shape
// SWAR decoder and a Clinger scanner that defer to str::parse; every path
// there and here is correctly rounded, so the bits agree.
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define FALX_HD __host__ __device__ __forceinline__
#define FALX_HD_NOINLINE static __host__ __device__ __noinline__
#else
#define FALX_HD static inline
#define FALX_HD_NOINLINE static
#endif

#include "pow5_table.h"

namespace falx {
namespace dec {

#ifdef __CUDACC__
static __device__ const uint64_t kPow5Dev[FALX_POW5_COUNT][2] = FALX_POW5_ENTRIES;
#endif
static const uint64_t kPow5Host[FALX_POW5_COUNT][2] = FALX_POW5_ENTRIES;
#ifdef __CUDA_ARCH__
#define FALX_POW5 kPow5Dev
#else
#define FALX_POW5 kPow5Host
#endif

FALX_HD bool is_digit(uint8_t c) { return (uint8_t)(c - '0') < 10; }

FALX_HD uint64_t d2u(double d) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(d);
#else
    union { double d; uint64_t u; } x;
    x.d = d;
    return x.u;
#endif
}
FALX_HD double u2d(uint64_t u) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    union { double d; uint64_t u; } x;
    x.u = u;
    return x.d;
#endif
}

FALX_HD int clz64(uint64_t x) {
#ifdef __CUDA_ARCH__
    return __clzll((long long)x);
#else
    return __builtin_clzll(x);
#endif
}

FALX_HD void mul128(uint64_t a, uint64_t b, uint64_t &hi, uint64_t &lo) {
#ifdef __CUDA_ARCH__
    lo = a * b;
    hi = __umul64hi(a, b);
#else
    unsigned __int128 p = (unsigned __int128)a * b;
    lo = (uint64_t)p;
    hi = (uint64_t)(p >> 64);
#endif
}

// Eisel-Lemire: w != 0, returns the biased binary64 bits (sign excluded).
FALX_HD uint64_t eisel_lemire(uint64_t w, int32_t q) {
    if (w == 0 || q < -342) return 0;
    if (q > 308) return 0x7FF0000000000000ull;
    int lz = clz64(w);
    w <<= lz;
    const int idx = q + 342;
    uint64_t hi, lo;
    mul128(w, FALX_POW5[idx][0], hi, lo);
    if ((hi & 0x1FF) == 0x1FF) {
        uint64_t hi2, lo2;
        mul128(w, FALX_POW5[idx][1], hi2, lo2);
        lo += hi2;
        if (hi2 > lo) hi++;
    }
    int upper = (int)(hi >> 63);
    int shift = upper + 9;
    uint64_t mant = hi >> shift;
    // floor(log2(10^q)) + 63 = ((217706 * q) >> 16) + 63
    int32_t power2 = (int32_t)((((int64_t)(152170 + 65536) * q) >> 16) + 63) + upper - lz + 1023;
    if (power2 <= 0) {
        if (-power2 + 1 >= 64) return 0;
        mant >>= -power2 + 1;
        mant += mant & 1;
        mant >>= 1;
        power2 = mant < (1ull << 52) ? 0 : 1;
        return ((uint64_t)power2 << 52) | (mant & ((1ull << 52) - 1));
    }
    // Exactly halfway between two doubles only when 5^q fits the product.
    if (lo <= 1 && q >= -4 && q <= 23 && (mant & 3) == 1) {
        if ((mant << shift) == hi) mant &= ~1ull;
    }
    mant += mant & 1;
    mant >>= 1;
    if (mant >= (2ull << 52)) {
        mant = 1ull << 52;
        power2++;
    }
    mant &= ~(1ull << 52);
    if (power2 >= 0x7FF) return 0x7FF0000000000000ull;
    return ((uint64_t)power2 << 52) | mant;
}

// --------------------------------------------------------------------------
// Big-decimal slow path.
// --------------------------------------------------------------------------
constexpr int kMaxDigits = 768;
constexpr int kDpRange = 2047;

struct BigDec {
    int32_t nd;      // number of digits
    int32_t dp;      // decimal point position
    bool truncated;  // nonzero digits were dropped
    uint8_t d[kMaxDigits + 20];
};

FALX_HD void bd_trim(BigDec &b) {
    while (b.nd > 0 && b.d[b.nd - 1] == 0) b.nd--;
}

// Multiply by 2^shift (shift <= 60), in place.
FALX_HD void bd_lshift(BigDec &b, int shift) {
    if (b.nd == 0) return;
    const int kExtra = 19;
    int r = b.nd - 1, wpos = b.nd - 1 + kExtra;
    uint64_t acc = 0;
    for (; r >= 0; r--, wpos--) {
        acc += (uint64_t)b.d[r] << shift;
        b.d[wpos] = (uint8_t)(acc % 10);
        acc /= 10;
    }
    while (acc > 0) {
        b.d[wpos--] = (uint8_t)(acc % 10);
        acc /= 10;
    }
    int first = wpos + 1;
    int n = b.nd + kExtra - first;
    for (int i = 0; i < n; i++) b.d[i] = b.d[first + i];
    b.dp += n - b.nd;
    if (n > kMaxDigits) {
        for (int i = kMaxDigits; i < n; i++)
            if (b.d[i]) b.truncated = true;
        n = kMaxDigits;
    }
    b.nd = n;
    bd_trim(b);
}

// Divide by 2^shift (shift <= 60), in place.
FALX_HD void bd_rshift(BigDec &b, int shift) {
    int rd = 0, wr = 0;
    uint64_t n = 0;
    while ((n >> shift) == 0) {
        if (rd < b.nd) {
            n = 10 * n + b.d[rd++];
        } else if (n == 0) {
            return;
        } else {
            while ((n >> shift) == 0) {
                n *= 10;
                rd++;
            }
            break;
        }
    }
    b.dp -= rd - 1;
    if (b.dp < -kDpRange) {
        b.nd = 0;
        b.dp = 0;
        b.truncated = false;
        return;
    }
    uint64_t mask = (1ull << shift) - 1;
    while (rd < b.nd) {
        uint8_t nd = (uint8_t)(n >> shift);
        n = 10 * (n & mask) + b.d[rd++];
        b.d[wr++] = nd;
    }
    while (n > 0) {
        uint8_t nd = (uint8_t)(n >> shift);
        n = 10 * (n & mask);
        if (wr < kMaxDigits) b.d[wr++] = nd;
        else if (nd > 0) b.truncated = true;
    }
    b.nd = wr;
    bd_trim(b);
}

FALX_HD uint64_t bd_round(const BigDec &b) {
    if (b.nd == 0 || b.dp < 0) return 0;
    if (b.dp > 18) return ~0ull;
    int dp = b.dp;
    uint64_t n = 0;
    for (int i = 0; i < dp; i++) {
        n *= 10;
        if (i < b.nd) n += b.d[i];
    }
    bool up = false;
    if (dp < b.nd) {
        up = b.d[dp] >= 5;
        if (b.d[dp] == 5 && dp + 1 == b.nd) up = b.truncated || (dp != 0 && (b.d[dp - 1] & 1));
    }
    return n + (up ? 1 : 0);
}

FALX_HD int bd_shift_for(int n) {
    const uint8_t kP[19] = {0, 3, 6, 9, 13, 16, 19, 23, 26, 29, 33, 36, 39, 43, 46, 49, 53, 56, 59};
    return n < 19 ? kP[n] : 60;
}

// Digits of a validated decimal (sign already removed) -> biased bits.
FALX_HD_NOINLINE uint64_t slow_decimal(const uint8_t *s, uint32_t len) {
    BigDec b;
    b.nd = 0;
    b.dp = 0;
    b.truncated = false;
    uint32_t i = 0;
    while (i < len && s[i] == '0') i++;
    while (i < len && is_digit(s[i])) {
        if (b.nd < kMaxDigits) b.d[b.nd] = (uint8_t)(s[i] - '0');
        else if (s[i] != '0') b.truncated = true;
        b.nd++;
        i++;
    }
    b.dp = b.nd;
    if (i < len && s[i] == '.') {
        i++;
        if (b.nd == 0) {
            while (i < len && s[i] == '0') {
                b.dp--;
                i++;
            }
        }
        while (i < len && is_digit(s[i])) {
            if (b.nd < kMaxDigits) b.d[b.nd] = (uint8_t)(s[i] - '0');
            else if (s[i] != '0') b.truncated = true;
            b.nd++;
            i++;
        }
    }
    if (b.nd > kMaxDigits) b.nd = kMaxDigits;
    if (i < len && (s[i] | 0x20) == 'e') {
        i++;
        bool eneg = false;
        if (i < len && (s[i] == '+' || s[i] == '-')) {
            eneg = s[i] == '-';
            i++;
        }
        int32_t e = 0;
        while (i < len && is_digit(s[i])) {
            if (e < 0x10000) e = 10 * e + (s[i] - '0');
            i++;
        }
        b.dp += eneg ? -e : e;
    }
    bd_trim(b);
    if (b.nd == 0 || b.dp < -324) return 0;
    if (b.dp >= 310) return 0x7FF0000000000000ull;
    int32_t exp2 = 0;
    while (b.dp > 0) {
        int sh = bd_shift_for(b.dp);
        bd_rshift(b, sh);
        if (b.dp < -kDpRange) return 0;
        exp2 += sh;
    }
    while (b.dp <= 0) {
        int sh;
        if (b.dp == 0) {
            if (b.d[0] >= 5) break;
            sh = (b.d[0] == 0 || b.d[0] == 1) ? 2 : 1;
        } else {
            sh = bd_shift_for(-b.dp);
        }
        bd_lshift(b, sh);
        if (b.dp > kDpRange) return 0x7FF0000000000000ull;
        exp2 -= sh;
    }
    exp2 -= 1;
    while (-1022 > exp2) {
        int n = -1022 - exp2;
        if (n > 60) n = 60;
        bd_rshift(b, n);
        exp2 += n;
    }
    if (exp2 + 1023 >= 0x7FF) return 0x7FF0000000000000ull;
    bd_lshift(b, 53);
    uint64_t mant = bd_round(b);
    if (mant >= (1ull << 53)) {
        bd_rshift(b, 1);
        exp2 += 1;
        mant = bd_round(b);
        if (exp2 + 1023 >= 0x7FF) return 0x7FF0000000000000ull;
    }
    int32_t power2 = exp2 + 1023;
    if (mant < (1ull << 52)) power2 -= 1;
    mant &= (1ull << 52) - 1;
    return ((uint64_t)power2 << 52) | mant;
}

FALX_HD bool ieq_lit(const uint8_t *s, uint32_t len, const char *lit, uint32_t ll) {
    if (len != ll) return false;
    for (uint32_t i = 0; i < ll; i++)
        if ((s[i] | 0x20) != (uint8_t)lit[i]) return false;
    return true;
}

FALX_HD bool parse_f64(const uint8_t *s, uint32_t len, double &out) {
    if (len == 0) return false;
    uint32_t i = 0;
    bool neg = false;
    if (s[0] == '-' || s[0] == '+') {
        neg = s[0] == '-';
        i = 1;
        if (len == 1) return false;
    }
    const uint32_t body = i;
    // Fixed shape d{1,3}.d{6}: the overwhelmingly common cell.
    uint32_t bl = len - body;
    if (bl >= 8 && bl <= 10 && s[len - 7] == '.') {
        uint64_t m = 0;
        bool ok = true;
        for (uint32_t k = body; k < len; k++) {
            if (k == len - 7) continue;
            uint8_t c = (uint8_t)(s[k] - '0');
            ok &= c < 10;
            m = m * 10 + c;
        }
        if (ok) {
            // m / 1e6 correctly rounded, as the reference's IEEE division
            // gives it; Eisel-Lemire is exact for decimal exponents in
            // [-27, 55] and needs no floating-point unit
            out = u2d(eisel_lemire(m, -6) | ((uint64_t)neg << 63));
            return true;
        }
    }
    uint64_t w = 0;
    int nsig = 0, nd = 0;
    int32_t e10 = 0;
    bool trunc = false;
    while (i < len && is_digit(s[i])) {
        uint32_t d = s[i] - '0';
        if (nsig == 0 && d == 0) {
        } else if (nsig < 19) {
            w = w * 10 + d;
            nsig++;
        } else {
            e10++;
            if (d) trunc = true;
        }
        i++;
        nd++;
    }
    if (i < len && s[i] == '.') {
        i++;
        while (i < len && is_digit(s[i])) {
            uint32_t d = s[i] - '0';
            if (nsig == 0 && d == 0) {
                e10--;
            } else if (nsig < 19) {
                w = w * 10 + d;
                nsig++;
                e10--;
            } else if (d) {
                trunc = true;
            }
            i++;
            nd++;
        }
    }
    if (nd == 0) {
        const uint8_t *r = s + body;
        uint32_t rl = len - body;
        uint64_t bits;
        if (ieq_lit(r, rl, "inf", 3) || ieq_lit(r, rl, "infinity", 8)) bits = 0x7FF0000000000000ull;
        else if (ieq_lit(r, rl, "nan", 3)) bits = 0x7FF8000000000000ull;
        else return false;
        out = u2d(bits | ((uint64_t)neg << 63));
        return true;
    }
    if (i < len && (s[i] | 0x20) == 'e') {
        i++;
        bool eneg = false;
        if (i < len && (s[i] == '+' || s[i] == '-')) {
            eneg = s[i] == '-';
            i++;
        }
        if (i >= len || !is_digit(s[i])) return false;
        int32_t e = 0;
        while (i < len && is_digit(s[i])) {
            if (e < 0x10000) e = 10 * e + (s[i] - '0');
            i++;
        }
        e10 += eneg ? -e : e;
    }
    if (i != len) return false;
    uint64_t bits;
    if (w == 0) {
        bits = 0;
    } else if (!trunc && e10 >= -27 && e10 <= 55) {
        // exact 128-bit product range (covers Clinger's exact doubles too)
        bits = eisel_lemire(w, e10);
    } else if (!trunc) {
        bits = eisel_lemire(w, e10);
    } else {
        uint64_t a = eisel_lemire(w, e10), b = eisel_lemire(w + 1, e10);
        bits = a == b ? a : slow_decimal(s + body, len - body);
    }
    out = u2d(bits | ((uint64_t)neg << 63));
    return true;
}

FALX_HD bool parse_i64(const uint8_t *s, uint32_t len, int64_t &out) {
    if (len == 0) return false;
    uint32_t i = 0;
    bool neg = false;
    if (s[0] == '+' || s[0] == '-') {
        if (len == 1) return false;
        neg = s[0] == '-';
        i = 1;
    }
    uint64_t v = 0;
    const uint64_t lim = neg ? (1ull << 63) : (1ull << 63) - 1;
    for (; i < len; i++) {
        uint32_t d = (uint8_t)(s[i] - '0');
        if (d >= 10) return false;
        if (v > (lim - d) / 10) return false;
        v = v * 10 + d;
    }
    out = neg ? (int64_t)(0 - v) : (int64_t)v;
    return true;
}

FALX_HD bool parse_u32(const uint8_t *s, uint32_t len, uint32_t &out) {
    if (len == 0) return false;
    uint32_t i = 0;
    if (s[0] == '+') {
        if (len == 1) return false;
        i = 1;
    }
    // nine digits fit 32 bits; a tenth is checked in 64
    uint32_t v = 0;
    const uint32_t end9 = len - i > 9 ? i + 9 : len;
    for (; i < end9; i++) {
        const uint32_t d = (uint8_t)(s[i] - '0');
        if (d >= 10) return false;
        v = v * 10 + d;
    }
    uint64_t w = v;
    for (; i < len; i++) {
        const uint32_t d = (uint8_t)(s[i] - '0');
        if (d >= 10) return false;
        w = w * 10 + d;
        if (w > 0xFFFFFFFFull) return false;
    }
    out = (uint32_t)w;
    return true;
}

// value * 1e6 exactly, for cells of the form [+-]?d*(.d{0,6})? with at least
// one digit and |value * 1e6| < 2^63.
FALX_HD bool exact_e6(const uint8_t *s, uint32_t len, int64_t &out) {
    uint32_t i = 0;
    bool neg = false;
    if (len && (s[0] == '+' || s[0] == '-')) {
        neg = s[0] == '-';
        i = 1;
    }
    uint64_t ip = 0;
    uint32_t nd = 0;
    bool over = false;
    while (i < len && is_digit(s[i])) {
        if (ip > 922337203684ull) over = true;
        ip = ip * 10 + (s[i] - '0');
        i++;
        nd++;
    }
    uint64_t fr = 0;
    uint32_t nf = 0;
    if (i < len && s[i] == '.') {
        i++;
        while (i < len && is_digit(s[i])) {
            if (nf == 6) return false;
            fr = fr * 10 + (s[i] - '0');
            i++;
            nf++;
            nd++;
        }
    }
    if (nd == 0 || i != len || over) return false;
    for (; nf < 6; nf++) fr *= 10;
    if (ip > 9223372036853ull) return false;
    uint64_t m = ip * 1000000ull + fr;
    if (m > 0x7FFFFFFFFFFFFFFFull) return false;
    out = neg ? -(int64_t)m : (int64_t)m;
    return true;
}

// Numeric view of a raw cell: quoted cells ("...") parse their inner bytes;
// an inner quote (or an unbalanced leading quote) can never be numeric.
// Returns false if the cell cannot be numeric at all.
FALX_HD bool numeric_view(const uint8_t *&s, uint32_t &len) {
    if (len == 0 || s[0] != '"') return true;
    if (len < 2 || s[len - 1] != '"') return false;
    for (uint32_t k = 1; k + 1 < len; k++)
        if (s[k] == '"') return false;
    s += 1;
    len -= 2;
    return true;
}

}  // namespace dec
}  // namespace falx
