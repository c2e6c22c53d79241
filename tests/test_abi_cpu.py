"""CPU-side checks of the C ABI library and the generators (no GPU calls)."""
import ctypes
import re

import numpy as np

import scd_gb300 as S
import scdgen


def test_library_loads_and_exports_every_declared_symbol():
    lib = S.lib()
    declared = S.header_symbols()
    assert len(declared) >= 18
    missing = [name for name in declared if not hasattr(lib, name)]
    assert not missing, missing


def test_header_declares_extern_c_and_status_codes():
    text = open(S.HEADER_PATH).read()
    assert 'extern "C"' in text
    for code, name in S.ERRORS.items():
        assert re.search(r"#define %s \(%d\)" % (name, code), text), name


def test_create_without_gpu_fails_cleanly():
    # no GPU in this container: scd_create must return an error, not crash
    import torch
    if torch.cuda.is_available():
        return
    ctx = ctypes.c_void_p()
    rc = S.lib().scd_create(ctypes.byref(ctx), 0, 256, 0)
    assert rc != 0 and not ctx.value


def test_generators_are_deterministic_and_canonical():
    for fn in (lambda: scdgen.planted(3000, 12.0, 0.2, 20, 100, seed=3),
               lambda: scdgen.rmat(11, 16, seed=4),
               lambda: scdgen.chunglu(5000, 2.1, 5.0, 500.0, 0.2, 10, 100, seed=5)):
        a, b = fn(), fn()
        assert np.array_equal(a, b)
        assert (a[:, 0] < a[:, 1]).all()
        key = a[:, 0].astype(np.uint64) << 32 | a[:, 1]
        assert (np.diff(key.astype(np.int64)) > 0).all()   # sorted, unique


def test_planted_partition_shape():
    e = scdgen.planted(10000, 18.0, 0.1, 20, 100, seed=1)
    deg = np.bincount(e.ravel(), minlength=10000)
    assert abs(deg.mean() - 20.0) < 1.0   # 18 internal + 2 external on average


def test_autotune_report_gives_the_chosen_in_list_split():
    report = ["small<=32 warp<=64 cta<=512 in-list>0: 3.210 ms",
              "small<=32 warp<=64 cta<=512 in-list>16: 2.950 ms",
              "small<=32 warp<=64 cta<=512 in-list>32: 3.001 ms",
              "small<=16 warp<=64 cta<=512 in-list>16: 1.000 ms"]   # another split, not chosen
    assert S.chosen_in_list_min(report, 32, 64, 512) == 16
    assert S.chosen_in_list_min(report, 0, 16, 256) is None
