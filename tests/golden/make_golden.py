"""Build tests/golden/reference_vectors.json.

The inputs are the known-answer and hand-picked vectors held in the
reference's own tests (Mapika/falx tests/ndjson_id_score.rs:5-19,
tests/comments.rs:13-56, tests/csv_hash_fused_par.rs:60-120,
tests/columns.rs:408-451 and :623-639). The reference is a Rust crate and
cannot run here, so the expected outputs are the reference tests' own
assertions where they state them (records, keys, amounts, sums) and
otherwise come from the pure-Python restatement below: a byte-serial
automaton (src/scalar.rs:23-59), the record/field rules of the generated
sinks, and str::parse rules checked with Python's exact float/int
conversion. This script shares no code with oracle/ (the C oracle), so the
fixtures pin the oracle independently.

Run: python tests/golden/make_golden.py
"""

import base64
import json
import math
import os
import re
import struct

HERE = os.path.dirname(os.path.abspath(__file__))

DIALECTS = {
    0: dict(structural=b",\n", quote=b'"', escape=None, comment=None),
    1: dict(structural=b",\n", quote=b'"', escape=None, comment=b"#"),
    2: dict(structural=b"\t\n", quote=None, escape=None, comment=None),
    3: dict(structural=b" =\n", quote=b'"', escape=b"\\", comment=None),
    4: dict(structural=b"\n", quote=b'"', escape=b"\\", comment=None),
}


def index_spec(data, d):
    dl = DIALECTS[d]
    out = []
    in_q = in_c = False
    run = 0
    ls = True
    for i, b in enumerate(data):
        c = bytes([b])
        escaped = run % 2 == 1
        run = run + 1 if dl["escape"] == c else 0
        if in_c:
            if c == b"\n":
                in_c = False
                if b"\n" in dl["structural"]:
                    out.append(i)
        elif dl["quote"] == c:
            if not escaped:
                in_q = not in_q
        elif not in_q and dl["comment"] == c and ls:
            in_c = True
        elif not in_q and c in dl["structural"]:
            out.append(i)
        ls = c == b"\n"
    return out


def records(data, d):
    """(record_start, end, [(from, to), ...]) per record, comments included."""
    idx = index_spec(data, d)
    recs = []
    rs = fs = 0
    spans = []
    for p in idx + [None]:
        last = p is None
        if last:
            if rs >= len(data):
                break
            p = len(data)
        if last or data[p] == 0x0A:
            to = p - 1 if (p > rs and data[p - 1] == 0x0D) else p
            spans.append((fs, to))
            recs.append((rs, p, spans))
            rs = fs = p + 1
            spans = []
        else:
            spans.append((fs, p))
            fs = p + 1
    return recs


def is_comment(data, d, rs, end):
    return d == 1 and end > rs and data[rs] == 0x23


def clean(raw):
    if len(raw) >= 2 and raw[0] == 0x22 and raw[-1] == 0x22:
        inner = raw[1:-1]
        out = bytearray()
        i = 0
        while i < len(inner):
            out.append(inner[i])
            i += 2 if (inner[i] == 0x22 and i + 1 < len(inner) and inner[i + 1] == 0x22) else 1
        return bytes(out)
    return raw


def numeric(raw):
    return clean(raw) if raw[:1] == b'"' else raw


F64_RE = re.compile(rb"[+-]?(?:[0-9]+\.?[0-9]*|\.[0-9]+)(?:[eE][+-]?[0-9]+)?\Z")


def parse_f64(s):
    """str::parse::<f64>: returns the IEEE bits or None."""
    body = s[1:] if s[:1] in (b"+", b"-") else s
    neg = s[:1] == b"-"
    low = body.lower()
    if low in (b"inf", b"infinity"):
        return (0xFFF0000000000000 if neg else 0x7FF0000000000000)
    if low == b"nan":
        return (0xFFF8000000000000 if neg else 0x7FF8000000000000)
    if not F64_RE.match(s) or not body or body[:1] in (b"+", b"-"):
        return None
    v = float(s.decode())  # correctly rounded
    return struct.unpack("<Q", struct.pack("<d", v))[0]


def parse_i64(s):
    if not re.fullmatch(rb"[+-]?[0-9]+", s):
        return None
    v = int(s)
    return v if -(2 ** 63) <= v < 2 ** 63 else None


def columns(data, d, cols):
    rows = []
    for rs, end, spans in records(data, d):
        if is_comment(data, d, rs, end):
            continue
        row = []
        for f, t in cols:
            if f >= len(spans):
                row.append(None)
                continue
            a, b = spans[f]
            raw = data[a:b]
            if t == "i64":
                row.append(parse_i64(numeric(raw)))
            elif t == "f64":
                row.append(parse_f64(numeric(raw)))
            elif t == "str":
                row.append(base64.b64encode(clean(raw)).decode())
            elif t == "bytes":
                row.append([a, b] if b > a else None)
        rows.append(row)
    return rows


def field_bytes(data, d):
    f = b = 0
    for rs, end, spans in records(data, d):
        if is_comment(data, d, rs, end):
            continue
        for a, e in spans:
            f += 1
            b += len(clean(data[a:e]))
    return [f, b]


def tape(data, d):
    seps, ends = [], []
    for p in index_spec(data, d):
        if data[p] == 0x0A:
            ends.append((len(seps) << 32) | p)
        else:
            seps.append(p)
    return seps, ends


def case(name, source, dialect, data, **extra):
    seps, ends = tape(data, dialect)
    c = {"name": name, "source": source, "dialect": dialect, "data": base64.b64encode(data).decode(),
         "index": index_spec(data, dialect), "seps": seps, "ends": ends,
         "field_bytes": field_bytes(data, dialect) if dialect in (0, 1, 2) else None}
    c.update(extra)
    return c


def main():
    cases = []
    # tests/comments.rs:13-56
    hp = (b"# header comment, with \"quotes\" and, commas\nfoo,42\n#mid, comment\nbar,7\n"
          b"\"#not,a comment\",9\n# trailing comment")
    key_amount = [[0, "str"], [1, "i64"]]
    got = columns(hp, 1, key_amount)
    assert [base64.b64decode(r[0]) for r in got] == [b"foo", b"bar", b"#not,a comment"]
    assert [r[1] for r in got] == [42, 7, 9]
    cases.append(case("comments_hand_picked", "tests/comments.rs:13-43", 1, hp,
                      records=[base64.b64encode(x).decode() for x in (b"foo,42", b"bar,7", b"\"#not,a comment\",9")],
                      columns={"schema": key_amount, "rows": got}))
    tricky = b"#comment with one \" quote\na,\"multi\nline\"\n#another \" stray\nb,2\n"
    cases.append(case("comments_tricky", "tests/comments.rs:45-55", 1, tricky,
                      records=[base64.b64encode(x).decode() for x in (b"a,\"multi\nline\"", b"b,2")]))
    # tests/csv_hash_fused_par.rs:60-88 (14 region hazards)
    hazards = [
        ("plain", b"a,1\nb,2\nc,3\n"), ("leading comment", b"# header\na,1\nb,2\n"),
        ("trailing comment", b"a,1\n# tail\n"), ("comment only", b"# just a comment\n"),
        ("quoted newline", b"\"a\nb\",1\nc,2\n"), ("hash inside quotes", b"\"a#b\",1\n\"#\",2\n"),
        ("quote inside comment", b"# a \" b\na,1\n"), ("unbalanced quote in comment", b"# \"\na,1\nb,2\n"),
        ("quoted comma", b"\"a,b\",1\n"), ("doubled quotes", b"\"a\"\"b\",1\n"), ("empty cells", b",\n,\n"),
        ("no trailing newline", b"a,1\nb,2"), ("crlf", b"a,1\r\nb,2\r\n"), ("comment mid stream", b"a,1\n# mid\nb,2\n"),
    ]
    for label, data in hazards:
        cases.append(case("hazard: " + label, "tests/csv_hash_fused_par.rs:60-88", 1, data,
                          columns={"schema": key_amount, "rows": columns(data, 1, key_amount)}))
    # tests/csv_hash_fused_par.rs:91-120: hazards padded across 64-byte seams
    for hz in (b"\"x\ny\",7\n", b"# c \" c\n", b"\"#\",7\n", b"\"a\"\"b\",7\n"):
        for pad in (0, 1, 5, 13, 39):
            data = b"".join(b"k%d,%d\n" % (i, i) for i in range(pad)) + hz + b"tail,99\n"
            cases.append(case("padded hazard %r pad %d" % (hz, pad), "tests/csv_hash_fused_par.rs:91-120", 1, data,
                              columns={"schema": key_amount, "rows": columns(data, 1, key_amount)}))
    # tests/columns.rs:408-451: hand-picked typed cells (csv_typed schema)
    typed = [[0, "i64"], [1, "str"], [2, "f64"], [4, "bytes"]]
    hand = (b"9223372036854775807,hello,1.5,x,label0\n"
            b"-9223372036854775808,,-0.0,x,\"lab,el1\"\n"
            b"9223372036854775808,\"a,\"\"b\"\",0.1,x,\"\"\n"
            b"+5,\"quo\nted\",0.0,x,lab3\n"
            b"-0,\"\",1_000,x,lab4\n"
            b"0007,world,1.5e308,x,\"123\"\n"
            b",,,5e-324,x,\"abc\"\n"
            b"17\n"
            b"18,test,NaN,x,label8\n"
            b"19,\"a\"\"b\",inf,x,label9\n"
            b"20,simple,-inf,x,label10\n")
    rows = columns(hand, 0, typed)
    # Checks a reader can make by hand against Rust's str::parse. The title
    # cell of row 2, "a,""b"", leaves a quote open, so the rest of the input
    # is one quoted span and the document has four records.
    assert len(rows) == 4
    assert rows[0][:3] == [2 ** 63 - 1, base64.b64encode(b"hello").decode(), 0x3FF8000000000000]
    assert rows[1][:3] == [-(2 ** 63), "", 0x8000000000000000]
    cases.append(case("columns_hand_picked_cells", "tests/columns.rs:408-451", 0, hand,
                      columns={"schema": typed, "rows": rows}))
    # tests/columns.rs:623-639: records positioned across 64-byte seams
    for pad in range(55, 71):
        data = (b"a" * pad + b"x,10,20.5,x,label\n") * 5
        cases.append(case("block boundary pad %d" % pad, "tests/columns.rs:623-639", 0, data,
                          columns={"schema": typed, "rows": columns(data, 0, typed)}))
    # tests/ndjson_id_score.rs:5-19
    nd = (b'{"id":10,"name":"a","tags":["x","y"],"nested":{"score":7,"ok":true},"note":"plain"}\n'
          b'{"id":-3,"name":"quoted \\" id\\":999","tags":["n","m"],"nested":{"score":11,"ok":true},'
          b'"note":"brace } inside"}\n'
          b'{"id":42,"name":"slash \\\\ nested score\\":123","tags":["p","q"],"nested":{"score":-5,"ok":true},'
          b'"note":"end"}\n')
    cases.append(case("ndjson_id_score", "tests/ndjson_id_score.rs:5-19", 4, nd, ndjson={"records": 3, "sum": 62}))
    with open(os.path.join(HERE, "reference_vectors.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": cases}, f, indent=0)
    print("wrote %d cases" % len(cases))


if __name__ == "__main__":
    main()
