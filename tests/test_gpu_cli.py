"""The command-line drop-ins: `convert`, `main-gpu` and `main` (het-scd_gb300/_build,
on the engine through the C ABI) print what the reference's tools print.

For every golden case, the stdout lines of the reference's own `convert` and
`main` (timer lines dropped; recorded by tests/golden/make_golden.py --cli) are
the expectation: nodes, edges, avg. cc, initial WCC, every iteration's WCC,
num. communities, the final WCC and the iteration count, formatted by the same
default ostream conversion.  `main-gpu` prints "work group size" where `main`
prints "num. threads" (src/main-gpu.cpp:63-69).  The file `convert` writes must
equal the reference's byte for byte."""
import os
import subprocess

import numpy as np
import pytest

import golden_data as G
import scd_gb300 as S
import scdgen

pytestmark = pytest.mark.gpu
BUILD = os.path.join(os.path.dirname(S.LIB_PATH))
CASES = [c for c in G.partition_cases() if "ref_convert_lines" in G.manifest()[c]]


def _lines(out):
    """Non-empty stdout lines without the timer lines ("<name>: <t> ms")."""
    return [l for l in out.splitlines() if l and not l.endswith(" ms")]


def _run(args, **kw):
    r = subprocess.run(args, capture_output=True, text=True, timeout=300, **kw)
    assert r.returncode == 0, r.stderr
    return r.stdout


@pytest.mark.parametrize("name", CASES)
def test_convert_cli_matches_reference(tmp_path, name):
    txt, out = str(tmp_path / "in.txt"), str(tmp_path / "out.graph")
    scdgen.write_text(txt, G.pairs(name))
    got = _lines(_run([os.path.join(BUILD, "convert"), txt, out]).replace(txt, "<input>").replace(out, "<output>"))
    want = [l for l in G.manifest()[name]["ref_convert_lines"] if not l.startswith("removed ")]
    assert got == want
    assert open(out, "rb").read() == G.graph_bytes(name)


@pytest.mark.parametrize("tool", ["main-gpu", "main"])
@pytest.mark.parametrize("name", [c for c in CASES if "ref_main_lines" in G.manifest()[c]])
def test_main_clis_match_reference(tmp_path, name, tool):
    gpath = str(tmp_path / "g.graph")
    with open(gpath, "wb") as f:
        f.write(G.graph_bytes(name))
    args = [os.path.join(BUILD, tool), gpath] + (["0"] if tool == "main-gpu" else [])
    got = [l for l in _lines(_run(args)) if not l.startswith("selected device")]
    want = G.manifest()[name]["ref_main_lines"]
    if tool == "main-gpu":
        want = ["work group size: 256" if l.startswith("num. threads") else l for l in want]
    assert got == want


def test_main_gpu_labels_file(tmp_path):
    """SCD_LABELS_OUT: the best labels the reference keeps in memory
    (src/main-gpu.cpp:99-103) written as a file."""
    name = "planted_2k_mu03"
    gpath, lpath = str(tmp_path / "g.graph"), str(tmp_path / "labels.bin")
    with open(gpath, "wb") as f:
        f.write(G.graph_bytes(name))
    _run([os.path.join(BUILD, "main-gpu"), gpath, "0"], env=dict(os.environ, SCD_LABELS_OUT=lpath))
    assert np.array_equal(np.fromfile(lpath, np.uint32), G.trace(name)["best_labels"])
