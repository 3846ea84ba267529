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


def _cc(tmp_path, compiler, std, name, source, link=False, lib=None):
    import shutil
    import subprocess

    import pytest

    if shutil.which(compiler) is None:
        pytest.skip(f"no {compiler}")
    src = tmp_path / name
    src.write_text(source)
    cmd = [compiler, f"-std={std}", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), str(src)]
    if link:
        out = tmp_path / (name + ".bin")
        cmd += ["-o", str(out), "-L", os.path.dirname(lib), "-lcfdgpu", f"-Wl,-rpath,{os.path.dirname(lib)}"]
    else:
        cmd += ["-fsyntax-only"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out if link else None


def test_header_is_plain_c_and_cpp(tmp_path):
    """cfdgpu.h is a C header (the boundary a cgo, JNI or Rust -sys binding reads) that also
    compiles as C++, without warnings."""
    src = '#include "cfdgpu.h"\nint main(void) { return cfdg_last_error() == 0; }\n'
    _cc(tmp_path, "gcc", "c11", "h.c", src)
    _cc(tmp_path, "g++", "c++17", "h.cpp", src)


def test_plain_c_caller_links_and_gets_an_error_without_a_gpu(tmp_path, engine_lib, pkg):
    """A C program links against libcfdgpu.so through the header alone; without a GPU,
    cfdg_context_create returns CFDG_ERR_CUDA with a message (never a CPU fallback), and
    with one it creates and destroys a context."""
    import subprocess

    src = r'''#include <stdio.h>
#include "cfdgpu.h"
int main(void) {
  cfdg_context *ctx = NULL;
  int rc = cfdg_context_create(0, 0, &ctx);
  if (rc == 0) { cfdg_context_destroy(ctx); printf("ok\n"); return 0; }
  printf("%d %s\n", rc, cfdg_last_error());
  return rc == CFDG_ERR_CUDA && cfdg_last_error()[0] != 0 ? 0 : 1;
}
'''
    exe = _cc(tmp_path, "gcc", "c11", "caller.c", src, link=True, lib=pkg.engine.LIB_PATH)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr


def test_integration_binds_every_production_entry_point():
    """The Rust extern block a maintainer adds (the -sys crate of the integration notes)
    declares every entry point of the header except the test and measurement hooks."""
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    bound = set(re.findall(r"\bfn (cfdg_[a-z0-9_]+)\(", text))
    hooks = {n for n in declared() if n.startswith("cfdg_debug_")} | {
        "cfdg_batch_time_kernel", "cfdg_batch_debug_rhs", "cfdg_launch_count"}
    missing = sorted(set(declared()) - hooks - bound)
    assert not missing, missing
    assert not sorted(bound - set(declared()))
