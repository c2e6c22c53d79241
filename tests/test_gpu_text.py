"""Device parse of edge-list text (read_edges, src/convert.cpp:74-138) against the
oracle's parser and the reference's line rules, and text -> graph end to end."""
import os
import tempfile

import numpy as np
import pytest

import golden_data as G
import oracle as O
import scd_gb300 as S
import scdgen

pytestmark = pytest.mark.gpu

# the hand-written inputs of the golden fixtures
TEXTS = {
    "triangle_pendant": "0 1\n1 2\n2 0\n2 3\n",
    "readme_example": "1 2\n2 3\n3 5\n1 5\n",
    "messy_text": ("# comment line\n\n   7000000 12\n12 7000000\n12 12\n  99 12\n99 7000000\n"
                   "\t5 99\n5 12\n5 5\n5 7000000\n# trailing comment\n8 9\n9 10\n10 8\n10 8\n11 10\n"),
}


@pytest.fixture(scope="module")
def engine():
    e = S.Engine(0)
    yield e
    e.close()


def oracle_pairs(text):
    with tempfile.NamedTemporaryFile("w", suffix=".txt", delete=False) as f:
        f.write(text)
        path = f.name
    try:
        return O.read_text(path)
    finally:
        os.unlink(path)


@pytest.mark.parametrize("name", sorted(TEXTS))
def test_fixture_texts(engine, name):
    got = engine.parse_text(TEXTS[name].encode())
    assert np.array_equal(got, oracle_pairs(TEXTS[name]))
    assert np.array_equal(got, G.pairs(name))
    engine.convert_text(TEXTS[name].encode())
    assert engine.graph_bytes() == G.graph_bytes(name)


@pytest.mark.parametrize("make", [lambda: scdgen.rmat(12, 16, seed=5), lambda: scdgen.planted(5000, 12.0, 0.2, 20, 100, 3)])
def test_generated_text(engine, make):
    pairs = make()
    with tempfile.NamedTemporaryFile(suffix=".txt", delete=False) as f:
        path = f.name
    try:
        scdgen.write_text(path, pairs)
        text = open(path, "rb").read()
        assert np.array_equal(engine.parse_text(text), O.read_text(path))
    finally:
        os.unlink(path)
    engine.convert_text(text)
    ref, _ = O.convert(pairs)
    assert engine.graph_bytes() == ref.to_bytes()


def test_line_rules(engine):
    text = ("\r\n  \t\n#x 1 2\n 4294967297 3\r\n7\t8 trailing words\n9 10" )   # no final newline
    assert engine.parse_text(text.encode()).tolist() == [[1, 3], [7, 8], [9, 10]]
    assert engine.parse_text(b"").shape == (0, 2)
    assert engine.parse_text(b"\n\n# only comments\n").shape == (0, 2)
    assert engine.parse_text(b"5 6\x00 7 8\n\x00 1 2\n").tolist() == [[5, 6]]   # NUL ends a line
    ok = ("1 2" + " " * 1020)[:1023] + "\n3 4\n"                                # 1023 characters: fine
    assert engine.parse_text(ok.encode()).tolist() == [[1, 2], [3, 4]]


@pytest.mark.parametrize("text,message", [
    ("1 2\n3 x\n4 5\n", "line 2 is corrupt"),
    ("1 2\n\n# c\n  5\n", "line 4 is corrupt"),
    ("a 1\n", "line 1 is corrupt"),
    ("1 2\n" + "3 4" + " " * 1100 + "\n5 x\n", "an error occured while reading input file"),
    ("1 2\n" + "x" * 1100 + "\n", "line 2 is corrupt"),                       # corrupt first 1023 characters
    ("1 2\n3 y\n" + "4 5" + " " * 1100 + "\n", "line 2 is corrupt"),          # the first failing line wins
])
def test_errors(engine, text, message):
    with pytest.raises(S.ScdError) as ex:
        engine.parse_text(text.encode())
    assert ex.value.status == -5 and message in str(ex.value)
    with pytest.raises(S.ScdError):
        engine.convert_text(text.encode())
