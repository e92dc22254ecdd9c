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
