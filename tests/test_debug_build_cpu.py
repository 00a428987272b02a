"""The debug build's host-side switches, without a GPU: the release library reports
itself as such and refuses the debug-only capacity override; the debug library
(PROLAND_GB300_DEBUG=1, built with TP_DEBUG) loads, exports every declared entry
point and reports itself as the debug build."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BOOK = 2


def test_release_build_flags(product):
    tp = product
    assert tp.lib().tp_build_is_debug() == 0
    s = tp.TileStorage(101, 3, 4, on_device=BOOK)
    assert tp.lib().tp_storage_check_guards(s.handle) == tp.TP_OK
    assert tp.lib().tp_debug_check_capacity(s.handle, 2) == tp.TP_E_BAD_ARG


def test_debug_library_loads_and_exports(product):
    import importlib.util
    spec = importlib.util.spec_from_file_location("pb", os.path.join(ROOT, "proland-4.0_gb300", "build.py"))
    pb = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(pb)
    pb.build(debug=True)
    code = ("import sys; sys.path.insert(0, %r); sys.path.insert(0, %r)\n"
            "from tests.test_capi_host import declared_symbols\n"
            "import proland_gb300 as tp\n"
            "L = tp.lib()\n"
            "missing = [n for n in declared_symbols() if not hasattr(L, n)]\n"
            "assert not missing, missing\n"
            "assert L.tp_build_is_debug() == 1\n"
            "s = tp.TileStorage(101, 3, 4, on_device=2)\n"
            "assert L.tp_debug_check_capacity(s.handle, 2) == 0\n"
            "print('debug ok', tp._lib.LIB_PATH)\n" % (os.path.join(ROOT, "proland-4.0_gb300"), ROOT))
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=dict(os.environ, PROLAND_GB300_DEBUG="1"),
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    assert "libproland_gb300_debug.so" in out.stdout
