"""Binary-format fast path (Graph::read, src/graph.cpp:273-321, with
cuda_transfer_graph): a .graph file, or its bytes in host memory, straight to the
device; the same resident graph and run as the host-array transfer, and the
reader's errors."""
import os
import tempfile

import numpy as np
import pytest

import golden_data as G
import scd_gb300 as S
import scdgen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def engine():
    e = S.Engine(0)
    yield e
    e.close()


def _file(data):
    f = tempfile.NamedTemporaryFile(suffix=".graph", delete=False)
    f.write(data)
    f.close()
    return f.name


@pytest.mark.parametrize("name", ["planted_10k", "rmat_12", "triangle_pendant"])
def test_file_and_bytes_match_transfer(engine, name):
    data = G.graph_bytes(name)
    path = _file(data)
    try:
        engine.load_graph_file(path)
        assert engine.graph_bytes() == data
        info = engine.graph_info()
        r1 = engine.run(0.01, 50)
        l1 = engine.labels_from_device()
        engine.transfer_graph_bytes(data)
        assert engine.graph_bytes() == data and engine.graph_info() == info
        r2 = engine.run(0.01, 50)
        assert np.array_equal(np.asarray(r1["wcc"]), np.asarray(r2["wcc"]))
        assert np.array_equal(l1, engine.labels_from_device())
    finally:
        os.unlink(path)


def test_empty_graph_file(engine):
    data = G.graph_bytes("readme_example")   # no edge of it lies on a triangle: n = m = 0
    path = _file(data)
    try:
        engine.load_graph_file(path)
        assert engine.graph_info()[:2] == (0, 0) and engine.graph_bytes() == data
    finally:
        os.unlink(path)


def test_large_file_in_pieces(engine):
    # more than two 64 MB pieces (the pinned buffers are reused)
    engine.convert_edges(scdgen.rmat(21, 16, seed=4))
    data = engine.graph_bytes()
    assert len(data) > 2 * (64 << 20)
    path = _file(data)
    try:
        engine.load_graph_file(path)
        assert engine.graph_bytes() == data
    finally:
        os.unlink(path)


def test_reader_errors(engine):
    data = G.graph_bytes("planted_10k")
    with pytest.raises(S.ScdError) as ex:
        engine.load_graph_file("/nonexistent/dir/x.graph")
    assert ex.value.status == -1 and "failed to open" in str(ex.value)
    bad = [data[:-4], data + b"\0", data[:6]]
    wrong = bytearray(data)
    wrong[8:12] = (1).to_bytes(4, "little")   # indices[0] != 0
    bad.append(bytes(wrong))
    for b in bad:
        path = _file(b)
        try:
            with pytest.raises(S.ScdError) as ex:
                engine.load_graph_file(path)
            assert ex.value.status == -5
        finally:
            os.unlink(path)
        with pytest.raises(S.ScdError):
            engine.transfer_graph_bytes(b)
