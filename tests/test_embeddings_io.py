"""NodeEmbeddings text files (EmbeddingWriter::stream, src/io.rs:44-76, and
EmbeddingReader::load / line_to_embedding, src/io.rs:134-262) through the
native formatter and parser.

Values are written as the shortest decimal that reads back to the same f32,
so a save/load round trip is bit-exact; files in the reference's own
spelling (ryu's "1.0", "1e-5", "NaN", spaces after commas) read to the same
f32 values as Python's float() rounded to f32.  No GPU is used."""
import gzip

import numpy as np
import pytest

import cloverleaf_gb300 as cl
from cloverleaf_gb300 import _native
from cloverleaf_gb300.graph import RangeVocab, Vocab


def _special_rows():
    f = np.finfo(np.float32)
    return np.array([[0.0, -0.0, 1.0, -1.0],
                     [f.max, -f.max, f.tiny, -f.tiny],
                     [f.smallest_subnormal, 1e-40, 3.0e-39, 0.1],
                     [np.inf, -np.inf, 123456789.0, 1e-7]], np.float32)


def _same_bits(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_round_trip_bit_exact(tmp_path):
    rng = np.random.default_rng(3)
    t = np.concatenate([_special_rows(),
                        (rng.standard_normal((997, 4)) * 10.0 ** rng.integers(-30, 30, (997, 4))).astype(np.float32)])
    v = Vocab()
    for i in range(len(t)):
        v.get_or_insert(["user", "item", "tag"][i % 3], f"n{i * 7919 % 100003}")
    e = cl.NodeEmbeddings(v, t)
    for name in ("e.emb", "e.emb.gz"):
        p = str(tmp_path / name)
        e.save(p)
        back = cl.NodeEmbeddings.load(p)
        assert _same_bits(back.table, t)
        assert list(back.vocab_) == list(v)


def test_nan_round_trip_and_python_reader_agrees(tmp_path):
    t = np.array([[np.nan, 2.5, -0.3333333]], np.float32)
    e = cl.NodeEmbeddings(Vocab(), t)
    e.vocab_.get_or_insert("a", "b")
    p = str(tmp_path / "n.emb")
    e.save(p)
    line = open(p).read()
    assert line.endswith("\n") and line.count("\n") == 1
    typ, name, vec = line.rstrip("\n").split("\t")
    assert (typ, name) == ("a", "b") and vec[0] == "[" and vec[-1] == "]"
    py = np.array([float(x) for x in vec[1:-1].split(",")], np.float32)
    assert np.isnan(py[0]) and _same_bits(py[1:], t[0, 1:])
    back = cl.NodeEmbeddings.load(p).table
    assert np.isnan(back[0, 0]) and _same_bits(back[0, 1:], t[0, 1:])


def test_reference_spelling(tmp_path):
    # ryu-style spellings, spaces around values, CRLF endings, a blank line,
    # a leading '+', and values beyond f32's range (saturating)
    text = ("user\tu1\t[1.0,1e-5,-3.4028235e38,NaN]\r\n"
            "user\tu2\t[ 0.1 , -0.0,inf,-inf ]\r\n"
            "\n"
            "item\ti9\t[+2.5,1E2,1e39,1e-50]\n")
    p = str(tmp_path / "ref.emb.gz")
    with gzip.open(p, "wt", newline="") as f:
        f.write(text)
    e = cl.NodeEmbeddings.load(p)
    want = np.array([[1.0, 1e-5, -3.4028235e38, np.nan], [0.1, -0.0, np.inf, -np.inf], [2.5, 100.0, np.inf, 0.0]],
                    np.float32)
    got = e.table
    assert np.array_equal(np.isnan(got), np.isnan(want))
    ok = ~np.isnan(want)
    assert _same_bits(got[ok], want[ok])
    assert list(e.vocab_) == [("user", "u1"), ("user", "u2"), ("item", "i9")]


def test_filter_type_and_skip_rows(tmp_path):
    p = str(tmp_path / "f.emb")
    with open(p, "w") as f:
        f.write("header line that is not an embedding\n")
        for i in range(10):
            f.write(f"{'ab'[i % 2]}\t{i}\t[{i}.0,{-i}.5]\n")
    e = cl.NodeEmbeddings.load(p, skip_rows=1, filter_type="b")
    assert list(e.vocab_) == [("b", str(i)) for i in range(1, 10, 2)]
    assert np.array_equal(e.table[:, 0], np.arange(1, 10, 2, dtype=np.float32))
    e2 = cl.NodeEmbeddings.load(p, skip_rows=1, filter_type=["a", "b"])
    assert len(e2.vocab_) == 10 and e2.dims() == 2
    with pytest.raises(ValueError):
        cl.NodeEmbeddings.load(p)                          # the header line is not an embedding


def test_anonymous_vocab_round_trips_as_range(tmp_path):
    t = np.random.default_rng(5).standard_normal((3000, 8)).astype(np.float32)
    e = cl.NodeEmbeddings(Vocab.anonymous(3000), t)
    p = str(tmp_path / "anon.emb")
    e.save(p)
    with open(p) as f:
        first = f.readline()
    assert first.startswith("node\t0\t[")
    back = cl.NodeEmbeddings.load(p)
    assert isinstance(back.vocab_, RangeVocab) and len(back.vocab_) == 3000
    assert back.vocab_.get_node_id("node", "2999") == 2999 and _same_bits(back.table, t)
    # names out of order, a leading zero, or a second type: an ordinary vocabulary
    lines = open(p).read().splitlines(True)
    for bad in (lines[1:] + lines[:1], [lines[0].replace("\t0\t", "\t00\t")] + lines[1:],
                lines[:-1] + [lines[-1].replace("node", "other", 1)]):
        with open(p, "w") as f:
            f.writelines(bad)
        b = cl.NodeEmbeddings.load(p)
        assert not isinstance(b.vocab_, RangeVocab) and len(b.vocab_) == 3000


@pytest.mark.parametrize("line,why", [
    ("a\tb[1.0]", "two fields"),
    ("a\tb\tc\t[1.0]", "four fields"),
    ("a\tb\t[]", "no values"),
    ("a\tb\t[1.0,,2.0]", "an empty value"),
    ("a\tb\t[1.0,x]", "not a number"),
    ("a\tb\t[1.0 2.0]", "space-separated"),
    ("a\tb\t[", "one byte"),
])
def test_malformed_lines_raise(tmp_path, line, why):
    p = str(tmp_path / "bad.emb")
    with open(p, "w") as f:
        f.write("a\tok\t[1.0]\n" + line + "\n")
    with pytest.raises(ValueError, match="Error parsing line"):
        cl.NodeEmbeddings.load(p)


def test_widths_and_duplicates(tmp_path):
    p = str(tmp_path / "w.emb")
    with open(p, "w") as f:
        f.write("a\t1\t[1.0,2.0]\na\t2\t[1.0,2.0,3.0]\n")
    with pytest.raises(ValueError, match="different sizes"):
        cl.NodeEmbeddings.load(p)
    with open(p, "w") as f:
        f.write("a\t1\t[1.0]\na\t2\t[2.0]\na\t1\t[3.0]\n")
    with pytest.raises(KeyError, match="duplicate"):
        cl.NodeEmbeddings.load(p)
    # a width fixed by an earlier block
    with pytest.raises(ValueError, match="different sizes"):
        _native.parse_embeddings(b"a\tb\t[1,2,3]\n", dims=2)


def test_parse_offsets_and_empty():
    buf = b"typ\tname\t[1]\nx\ty\t[2]"
    vals, tok = _native.parse_embeddings(buf)
    assert vals.tolist() == [[1.0], [2.0]]
    assert [buf[int(a):int(b)] for a, b, _, _ in tok] == [b"typ", b"x"]
    assert [buf[int(c):int(d)] for _, _, c, d in tok] == [b"name", b"y"]
    v, t = _native.parse_embeddings(b"")
    assert len(v) == 0 and len(t) == 0
    assert _native.format_embeddings(np.zeros((0, 3), np.float32), "node") == b""


def test_large_block_parallel_round_trip():
    # several formatter threads and parser chunks; names given explicitly
    rng = np.random.default_rng(11)
    t = rng.standard_normal((60000, 24)).astype(np.float32)
    names = [f"n{i}" for i in range(len(t))]
    buf = _native.format_embeddings(t, "node", names)
    assert buf.count(b"\n") == len(t)
    vals, tok = _native.parse_embeddings(buf)
    assert _same_bits(vals, t)
    assert buf[int(tok[-1, 2]):int(tok[-1, 3])] == b"n59999"
    dec = _native.format_embeddings(t[:5000], "node", None, 123)
    assert dec.split(b"\n")[0].startswith(b"node\t123\t[")
