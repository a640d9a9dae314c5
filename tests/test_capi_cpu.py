"""CPU tests of the boundary: the C-ABI library loads, exports every symbol
include/tebd_capi.h declares, and rejects bad arguments without a GPU."""
import ctypes
import os
import re

import pytest

from conftest import ROOT, gpu_present


def _header_symbols():
    txt = open(os.path.join(ROOT, "include", "tebd_capi.h")).read()
    return sorted(set(re.findall(r"\b(tebd_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(pkg):
    lib = pkg.load_library()
    declared = _header_symbols()
    assert declared, "no declarations parsed"
    for name in declared:
        assert hasattr(lib, name), name
    assert sorted(pkg.EXPORTED_SYMBOLS) == declared


def test_library_is_built_for_sm103a(pkg):
    from opentebd_extended_gb300 import tebd as T

    assert os.path.exists(T.LIB_PATH)
    blob = open(T.LIB_PATH, "rb").read()
    assert b"sm_103a" in blob or b"sm_103" in blob


def test_invalid_arguments_rejected_before_cuda(pkg):
    lib = pkg.load_library()
    from opentebd_extended_gb300.tebd import Opts, TEBD_ERR_ARG

    o = Opts()
    lib.tebd_default_opts(ctypes.byref(o))
    h = ctypes.c_void_p()
    assert lib.tebd_create(1, 2, 4, 0, ctypes.byref(o), ctypes.byref(h)) == TEBD_ERR_ARG
    assert lib.tebd_create(4, 0, 4, 0, ctypes.byref(o), ctypes.byref(h)) == TEBD_ERR_ARG
    assert lib.tebd_create(4, 2, 4, 7, ctypes.byref(o), ctypes.byref(h)) == TEBD_ERR_ARG
    o.version = 99
    assert lib.tebd_create(4, 2, 4, 0, ctypes.byref(o), ctypes.byref(h)) == TEBD_ERR_ARG
    assert b"version" in lib.tebd_last_error(None)
    # null handles are rejected, never dereferenced
    assert lib.tebd_destroy(None) == TEBD_ERR_ARG
    assert lib.tebd_sync(None) == TEBD_ERR_ARG
    assert lib.tebd_kernel_launches(None) == -1


@pytest.mark.skipif(gpu_present(), reason="checks the no-GPU error path")
def test_create_without_gpu_fails_cleanly(pkg):
    with pytest.raises(pkg.TebdError) as e:
        pkg.Chain(4, 2, 4)
    assert e.value.code == 2  # TEBD_ERR_CUDA


def test_fortran_binding_mentions_every_entry_point():
    """include/tebd_cuda_iface.f90 declares a BIND(C) interface for every function
    of include/tebd_capi.h, and nothing else."""
    import re

    hdr = open(os.path.join(ROOT, "include", "tebd_capi.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    declared = set(re.findall(r"\b(tebd_[a-z0-9_]+)\s*\(", hdr))
    f90 = open(os.path.join(ROOT, "include", "tebd_cuda_iface.f90")).read()
    bound = set(re.findall(r"NAME='(tebd_[a-z0-9_]+)'", f90))
    assert declared and declared == bound, (sorted(declared - bound), sorted(bound - declared))
    assert "MODULE tebd_cuda_iface" in f90 and "END MODULE tebd_cuda_iface" in f90
    assert max(len(line) for line in f90.splitlines()) <= 132  # free-form line limit


def test_header_is_plain_c(tmp_path):
    """tebd_capi.h compiles as C99 (the language a Fortran or C host binds to):
    a translation unit that takes the address of every entry point."""
    import re
    import shutil
    import subprocess

    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    hdr = open(os.path.join(ROOT, "include", "tebd_capi.h")).read()
    names = sorted(set(re.findall(r"\b(tebd_[a-z0-9_]+)\s*\(", re.sub(r"/\*.*?\*/", "", hdr, flags=re.S))))
    src = tmp_path / "use_capi.c"
    src.write_text('#include "tebd_capi.h"\n#include <stddef.h>\n'
                   "typedef void (*entry_fn)(void);\n"
                   "const entry_fn entry_points[] = {\n"
                   + ",\n".join("  (entry_fn)&%s" % n for n in names) + "\n};\n"
                   "size_t n_entry_points = sizeof(entry_points) / sizeof(entry_points[0]);\n")
    r = subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-c", str(src),
                        "-I", os.path.join(ROOT, "include"), "-o", str(tmp_path / "use_capi.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
