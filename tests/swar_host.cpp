// Host build of the word-at-a-time cell decoders (falx_gb300/csrc/swar.cuh)
// for the CPU tests: the same functions the columns kernel calls, fed with
// words built from byte strings.
#include <cstdint>
#include <cstring>

#include "swar.cuh"

static uint64_t le64(const uint8_t *b) {
    uint64_t x = 0;
    for (int i = 7; i >= 0; i--) x = (x << 8) | b[i];
    return x;
}
static uint32_t le32(const uint8_t *b) { return (uint32_t)b[0] | (uint32_t)b[1] << 8 | (uint32_t)b[2] << 16 | (uint32_t)b[3] << 24; }

// `buf` holds the cell at offset 0 followed by at least 8 bytes of padding
// (whatever follows a cell in the staged window).
extern "C" int swar_u32_cell(const uint8_t *buf, uint32_t n, uint32_t *v) {
    if (n - 1u <= 7u) return falx::swar::u32_word(le64(buf), n, *v) ? 1 : 0;
    if (n - 9u <= 1u) return falx::swar::u32_word10(le32(buf), le64(buf + n - 8), n, *v) ? 1 : 0;
    return 0;
}

extern "C" int swar_fixed6_cell(const uint8_t *buf, uint32_t n, uint64_t *bits, uint32_t *m, int *neg) {
    if (n - 8u > 3u) return 0;
    const uint32_t c0 = buf[0];
    const uint32_t sg = (c0 == '-' || c0 == '+') ? 1u : 0u;
    const uint32_t k = n - 7u - sg;
    if (k - 1u > 2u) return 0;
    bool ng = false;
    if (!falx::swar::fixed6_words(c0, k, le64(buf + n - 8), le32(buf + sg), *bits, *m, ng)) return 0;
    *neg = ng ? 1 : 0;
    return 1;
}
