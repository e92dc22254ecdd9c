import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


class Rng:
    """xorshift64* (the reference's tests/common/mod.rs:6-16)."""

    def __init__(self, seed):
        self.s = seed & 0xFFFFFFFFFFFFFFFF

    def next(self):
        s = self.s
        s ^= s >> 12
        s ^= (s << 25) & 0xFFFFFFFFFFFFFFFF
        s ^= s >> 27
        self.s = s
        return (s * 0x2545F4914F6CDD1D) & 0xFFFFFFFFFFFFFFFF


@pytest.fixture(scope="session")
def engine():
    import falx_gb300 as fx

    e = fx.Engine(0)
    yield e
    e.close()


# Dialect alphabets of the reference's generated-kernel differential test
# (tests/codegen.rs:392-468): structural bytes, quote twice, escape three
# times, comment twice, then "xy".
DIALECT_ALPHABETS = {
    0: b',\n""xy',
    1: b',\n""##xy',
    2: b"\t\nxy",
    3: b' =\n""\\\\\\xy',
    4: b'\n""\\\\\\xy',
}


def random_doc(rng, alphabet, length):
    return bytes(alphabet[rng.next() % len(alphabet)] for _ in range(length))


def reference_shape_ndjson(rng, lines):
    """NDJSON in the shape of the reference's id + score fixture
    (tests/ndjson_id_score.rs:5-19): each line starts `{"id":<int>`, then
    a name string, a tags array and `"nested":{"score":<int>,...}`, then a
    note. Names and notes carry escaped quotes and backslashes, braces and
    decoy keys ("id", "score") inside strings; blank and CR-ended lines are
    mixed in. The reference's literal sink accepts every such line, so its
    records and sum are the known answer for a JSON-aware sink."""
    decoys = [b'plain', b'quoted \\" id\\":999', b'slash \\\\ nested score\\":123', b'brace } inside',
              b'{\\"id\\":5}', b'],\\"nested\\":{\\"score\\":1}', b'tab\\tand\\nnewline', b'']
    out = bytearray()
    for _ in range(lines):
        if rng.next() % 17 == 0:
            out += b"\n" if rng.next() % 2 else b"\r\n"
        ident = rng.next() % 2_000_000_000 - 1_000_000_000
        score = rng.next() % 200_001 - 100_000
        name = decoys[rng.next() % len(decoys)]
        note = decoys[rng.next() % len(decoys)]
        ntags = rng.next() % 4
        tags = b",".join(b'"t%d"' % (rng.next() % 100) for _ in range(ntags))
        ok = b"true" if rng.next() % 2 else b"false"
        out += (b'{"id":%d,"name":"%s","tags":[%s],"nested":{"score":%d,"ok":%s},"note":"%s"}'
                % (ident, name, tags, score, ok, note))
        out += b"\r\n" if rng.next() % 11 == 0 else b"\n"
    return bytes(out)
