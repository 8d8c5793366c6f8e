"""Host-side checks of the restated reference GPU baseline library
(baseline/_build/librefgpu.so): it loads, exports its entry points, and
rejects bad arguments before touching a GPU."""
import ctypes as C
import sys

from conftest import ROOT

sys.path.insert(0, str(ROOT / "baseline"))
import refgpu  # noqa: E402


def test_library_exports():
    from pdgb import build as B

    B.build_refgpu()
    L = refgpu.lib()
    for name in ("rg_create", "rg_step", "rg_upload", "rg_read", "rg_system_nnz", "rg_destroy", "rg_last_error"):
        assert hasattr(L, name), name


def test_bad_arguments_rejected_on_host():
    L = refgpu.lib()
    h = C.c_void_p()
    rc = L.rg_create(0, 0, None, None, None, None, None, 1 / 120, 9.8, 10, 0.0, 0.9995, 1e6, 1, C.byref(h))
    assert rc != 0 and not h.value
    assert b"bad arguments" in L.rg_last_error()
    assert L.rg_step(None, 1, None, None) != 0
