// Host build of the GPU inflate decoder's shared core (inflate_core.h) for
// the tests: the same decoding, bounds checks and statuses, with a serial
// sink in place of the warp.
#include <cstdint>
#include <cstring>

#include "inflate_core.h"

using namespace falx::gz;

namespace {
struct HostSink {
    uint8_t *out;
    void sync() {}
    void flush() {}
    void literal(uint32_t pos, uint32_t c) { out[pos] = (uint8_t)c; }
    void match(uint32_t pos, uint32_t dist, uint32_t len) {
        for (uint32_t k = 0; k < len; k++) out[pos + k] = out[pos - dist + (dist >= len ? k : k % dist)];
    }
    void stored(const uint8_t *s, uint32_t pos, uint32_t len) { memcpy(out + pos, s, len); }
    void fill_fast(uint16_t *fast, int F, const uint16_t *count, const uint16_t *sym) {
        for (uint32_t i = 0; i < (1u << F); i++) fast[i] = fast_entry(i, F, count, sym);
    }
};
}  // namespace

extern "C" int gz_core_inflate(const uint8_t *in, uint32_t n, uint8_t *out, uint32_t out_len) {
    static Consts K;
    static bool ready = false;
    if (!ready) {
        make_consts(K);
        ready = true;
    }
    Tables T;
    memset(&T, 0xA5, sizeof T);  // garbage, as shared memory would hold
    Bits b{in, n, 0u, 0ull, 0, false};
    HostSink s{out};
    return inflate_stream(b, T, K, s, out_len);
}

#ifdef GZ_FUZZ_MAIN
// Standalone driver for the sanitizer run: reads records
// [u32 payload bytes][u32 output bytes][payload] from argv[1] and prints,
// per record, the status and an FNV-1a hash of the output. Every payload
// and output sits in its own allocation of exactly its size.
#include <cstdio>
#include <cstdlib>
#include <vector>

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 2;
    uint32_t hdr[2];
    while (fread(hdr, 4, 2, f) == 2) {
        uint8_t *in = static_cast<uint8_t *>(malloc(hdr[0] ? hdr[0] : 1));
        if (hdr[0] && fread(in, 1, hdr[0], f) != hdr[0]) return 3;
        uint8_t *out = static_cast<uint8_t *>(malloc(hdr[1] ? hdr[1] : 1));
        memset(out, 0, hdr[1]);
        const int rc = gz_core_inflate(in, hdr[0], out, hdr[1]);
        uint64_t h = 1469598103934665603ull;
        for (uint32_t i = 0; i < hdr[1]; i++) h = (h ^ out[i]) * 1099511628211ull;
        printf("%d %016llx\n", rc, (unsigned long long)h);
        free(in);
        free(out);
    }
    fclose(f);
    return 0;
}
#endif
