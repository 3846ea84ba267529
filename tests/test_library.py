"""The C-ABI library builds, loads and exports every function include/cfdgpu.h declares."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    text = open(os.path.join(ROOT, "include", "cfdgpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cfdg_[a-z0-9_]+)\s*\(", text)) - {"cfdg_poll_fn"})


def test_header_symbols_exported(engine_lib, pkg):
    names = declared()
    assert len(names) >= 14
    for name in names:
        assert hasattr(engine_lib, name), name
    assert sorted(pkg.engine.EXPORTS) == names


def test_no_device_is_an_error_not_a_fallback(engine_lib, pkg):
    # Without a GPU the context cannot be created; the engine never computes on the CPU.
    import ctypes as C

    h = C.c_void_p()
    rc = engine_lib.cfdg_context_create(0, 0, C.byref(h))
    if rc != 0:
        assert rc == pkg.engine.CFDG_ERR_CUDA
        assert pkg.engine.last_error()
    else:
        engine_lib.cfdg_context_destroy(h)
