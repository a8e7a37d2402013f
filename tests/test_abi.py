"""The C-ABI library without a GPU: it loads, exports every function that
include/*.h declares, and its host-side tables reproduce the reference."""
import ctypes
import os
import re

import numpy as np

from conftest import ROOT, cases


def declared_functions(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*[A-Za-z_][\w\s\*]*?\b(\w+)\s*\(", text, flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "while", "sizeof")))


def test_library_exports_every_declared_symbol(native_lib):
    from genpk_gb300 import native
    names = declared_functions("genpk_gb300.h")
    assert len(names) >= 18
    for n in names:
        assert hasattr(native_lib, n), n
    assert set(names) == set(native.ABI), set(names) ^ set(native.ABI)


def test_compat_library_exports_reference_signatures(native_lib):
    from genpk_gb300 import native
    lib = native.load_compat()
    for n in declared_functions("genpk_compat.h"):
        sym = native.COMPAT_FIELDIZE if n == "fieldize" else n
        assert hasattr(lib, sym), n
    # fieldize keeps the reference's C++ linkage (gen-pk.h:93): same mangled name.
    assert native.COMPAT_FIELDIZE == "_Z8fieldizediPdlPfS0_di"


def test_invwindow_known_answers(native_lib):
    """test.cpp:52-57 through the ABI."""
    from genpk_gb300 import invwindow
    assert abs(invwindow(0, 3, 4, 5) - 71.8177719) <= 71.8177719e-5
    assert abs(invwindow(4, 4, 4, 5) - 6111.20801) <= 6111.20801e-5
    assert invwindow(1, 1, 1, 0) == 0


def test_invwindow_matches_oracle(native_lib, oracle_port):
    from genpk_gb300 import invwindow
    for n in (4, 5, 64, 127, 1024):
        for k in [(1, 2, 3), (n // 2, n // 2, n // 2), (-3, 7 % n, 0), (n - 1, 1, n // 3)]:
            assert invwindow(*k, n) == oracle_port.invwindow(*k, n)


def test_geometry_counts_bit_exact_vs_reference(native_lib, golden):
    """Mode counts of the library's host bin tables equal the reference's."""
    from genpk_gb300 import geometry
    for key, c in cases(golden["counts"]).items():
        dims, nrbins = map(int, key.split("_"))
        cnt, k = geometry(dims, nrbins)
        assert np.array_equal(cnt, c["count"]), key
        np.testing.assert_allclose(k, c["keffs"], rtol=1e-12, err_msg=key)


def test_geometry_counts_match_port_large(native_lib, oracle_port):
    """Larger grids than the fixtures: library tables vs the oracle port."""
    from genpk_gb300 import geometry
    for dims, nrbins in ((384, 64), (300, 300)):
        cnt, k = geometry(dims, nrbins)
        zero = np.zeros((dims, dims, dims // 2 + 1), dtype=np.complex128)
        _, c_ref, k_ref = oracle_port.powerspectrum(dims, zero, zero, nrbins, 1.0, 1.0)
        assert np.array_equal(cnt, c_ref)
        np.testing.assert_allclose(k, k_ref, rtol=1e-12)
    for dims in (512, 1024):
        cnt, _ = geometry(dims, 64)
        assert int(cnt.astype(np.int64).sum()) == dims ** 3 - 1


def test_geometry_rejects_bad_arguments(native_lib):
    c = np.zeros(4, dtype=np.int32)
    k = np.zeros(4)
    from genpk_gb300 import native
    assert native_lib.genpk_geometry(1, 4, c.ctypes.data_as(native.c_i32p),
                                     k.ctypes.data_as(native.c_f64p)) != 0
    assert native_lib.genpk_geometry(8, 0, c.ctypes.data_as(native.c_i32p),
                                     k.ctypes.data_as(native.c_f64p)) != 0


def test_context_creation_fails_cleanly_without_gpu_or_bad_args(native_lib):
    from genpk_gb300 import native
    h = ctypes.c_void_p()
    assert native_lib.genpk_ctx_create(1, 8, 1, 0, ctypes.byref(h)) != 0
    assert native_lib.genpk_ctx_create(64, 8, 99, 0, ctypes.byref(h)) != 0
    assert native_lib.genpk_status_string(5) == b"bad particle data"
    assert native_lib.genpk_last_error(None) == b"null context"
    assert native.ABI["genpk_deposit"][0] is ctypes.c_int


def test_batch_entry_points_reject_null_and_bad_arguments(native_lib):
    """The batch calls on a null batch or with bad arguments return their
    error values without touching a GPU."""
    h = ctypes.c_void_p()
    dims = (ctypes.c_int64 * 2)(64, 128)
    assert native_lib.genpk_batch_create(0, dims, 8, 0, ctypes.byref(h)) != 0
    assert native_lib.genpk_batch_create(2, dims, 0, 0, ctypes.byref(h)) != 0
    assert native_lib.genpk_batch_set_mode(None, 1) != 0
    assert native_lib.genpk_batch_last_mode(None) == -1
    assert native_lib.genpk_batch_groups(None) == -1
    assert native_lib.genpk_batch_group(None, 0, None, None) is None
    assert native_lib.genpk_batch_auto_times(None, None, None) == -1
    assert native_lib.genpk_batch_graph_replays(None) == -1
    assert native_lib.genpk_batch_launches(None) == -1
    assert native_lib.genpk_batch_last_error(None) == b"null batch"
