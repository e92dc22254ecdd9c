"""Incremental parsing of unbounded input (csv_geo.rs:688-807 StreamParser;
csv_hash.rs:739-830 with comment records skipped).

Feed chunks of any size; each completed record is handed to a callback.
The parser keeps the bytes of the record that is still open. A feed runs
the seeded tape pass (falx_parse_tape_seeded) over those bytes plus the
new chunk, starting at the open record: a record starts right after a
structural newline, where every dialect's automaton is outside any region
(no quote, comment or pending escape) and a new line begins, so the pass
resumes exactly where the previous feed left the stream. Bytes after the
last terminator stay buffered for the next feed; `finish` ends the stream
and emits a trailing record without a terminator.

Records are views over the parser's buffer (Record.data), with positions
relative to it as in the reference; `Record.stream_offset` gives the
buffer's position in the stream. A record must fit in memory and be
shorter than 4 GiB. Each feed re-reads the open record, so a record that
spans many feeds is read once per feed."""

from ctypes import byref, c_uint64, c_void_p

import numpy as np

from . import _lib
from ._lib import CSV, CSV_HASH, check


class StreamRecord:
    """A record of a stream: `record` (a Record over the buffer of its feed)
    and `stream_offset`, the buffer's position in the stream."""

    __slots__ = ("record", "stream_offset")

    def __init__(self, record, stream_offset):
        self.record, self.stream_offset = record, stream_offset

    def __getattr__(self, name):
        return getattr(self.record, name)

    def span(self):
        """The record's [start, end) in the stream."""
        return (self.stream_offset + self.record.start, self.stream_offset + self.record.end)


class StreamParser:
    """Feed chunks, receive complete records (StreamParser::feed / finish)."""

    def __init__(self, dialect=CSV, engine=None):
        from . import engine as default_engine

        self.eng = engine or default_engine()
        self.dialect = dialect
        self.buf = bytearray()
        self.offset = 0       # stream position of buf[0]
        self.at_start = True  # buf[0] is the stream's first byte
        self.done = False

    def feed(self, chunk, on_record):
        """Append `chunk`; call on_record(record) for every record it completes."""
        if self.done:
            raise RuntimeError("the stream is finished")
        self.buf += bytes(chunk)
        self._emit(on_record, final=False)

    def finish(self, on_record):
        """End of input: records completed by the last bytes, then a
        trailing record without a terminator."""
        if not self.done:
            self._emit(on_record, final=True)
            self.done = True

    def _tape(self, data):
        e = self.eng
        torch = e.torch
        d = e.to_device(np.frombuffer(data, dtype=np.uint8))
        n = d.numel()
        e._sync_stream()
        prev = -1 if self.at_start else 0x0A
        cap_s, cap_e = n // 2 + 64, n // 4 + 64
        while True:
            seps = e.empty(cap_s, torch.int32)
            ends = e.empty(cap_e, torch.int64)
            ni, ns, ne = c_uint64(), c_uint64(), c_uint64()
            rc = e.lib.falx_parse_tape_seeded(e.ctx, self.dialect, c_void_p(d.data_ptr()), n, prev, 0, 0, 0, None, 0,
                                              c_void_p(seps.data_ptr()), cap_s, c_void_p(ends.data_ptr()), cap_e,
                                              byref(ni), byref(ns), byref(ne))
            if rc == _lib.FALX_ERR_CAPACITY:
                cap_s, cap_e = max(cap_s, ns.value), max(cap_e, ne.value)
                continue
            check(rc, "falx_parse_tape_seeded")
            return (seps[: ns.value].cpu().numpy().view(np.uint32),
                    ends[: ne.value].cpu().numpy().view(np.uint64))

    def _emit(self, on_record, final):
        from . import Record

        if not self.buf:
            return
        data = bytes(self.buf)
        seps, ends = self._tape(data)
        start, sep_pos = 0, 0
        for e in ends:
            e = int(e)
            end, cum = e & 0xFFFFFFFF, e >> 32
            if not self._comment(data, start, end):
                on_record(StreamRecord(Record(data, start, end, seps[sep_pos:cum]), self.offset))
            start, sep_pos = end + 1, cum
        if final:
            if start < len(data) and not self._comment(data, start, len(data)):
                on_record(StreamRecord(Record(data, start, len(data), seps[sep_pos:]), self.offset))
            start = len(data)
        if start:
            del self.buf[:start]
            self.offset += start
            self.at_start = False

    def _comment(self, data, start, end):
        # csv_hash comment records: first byte '#' (csv_hash.rs:1381)
        return self.dialect == CSV_HASH and end > start and data[start] == 0x23


def stream(dialect=CSV, engine=None):
    """A new StreamParser (csv_geo.rs:705 stream())."""
    return StreamParser(dialect, engine)
