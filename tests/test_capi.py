"""The C ABI library builds, loads without a GPU and exports every symbol that
include/gvom_gb300.h declares (no compute calls: there may be no GPU here)."""
import ctypes
import os
import re

from conftest import REPO


def _declared_symbols():
    hdr = open(os.path.join(REPO, "include", "gvom_gb300.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    return sorted(set(re.findall(r"\b(gvom_[a-z0-9_]+)\s*\(", hdr)))


def test_header_declares_expected_entry_points():
    names = _declared_symbols()
    for must in ("gvom_create", "gvom_destroy", "gvom_process", "gvom_combine", "gvom_debug_voxel_map",
                 "gvom_process_batch", "gvom_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(gpu_lib):
    lib = ctypes.CDLL(os.path.join(REPO, "gvom_gb300", "_build", "libgvom_gb300.so"))
    missing = [n for n in _declared_symbols() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_python_binding_covers_header():
    from gvom_gb300 import _lib
    assert set(_lib.EXPORTS) == set(_declared_symbols())


def test_version_and_error_strings_without_gpu(gpu_lib):
    assert b"sm_103a" in gpu_lib.gvom_version()
    assert gpu_lib.gvom_last_error() == b""


def test_bad_params_rejected_before_any_device_call(gpu_lib):
    from gvom_gb300._lib import GVOM_ERR_ARG, GvomParams
    p = GvomParams(0.2, 0.2, 0, 32, 2, 1.0, 0.5, 0.5, 0.3, 2.0, 4.0, 1.0, 1, 1)
    h = ctypes.c_void_p()
    assert gpu_lib.gvom_create(ctypes.byref(p), ctypes.byref(h)) == GVOM_ERR_ARG
    assert b"positive" in gpu_lib.gvom_last_error()
    p = GvomParams(0.2, 0.2, 64, 32, 40, 1.0, 0.5, 0.5, 0.3, 2.0, 4.0, 1.0, 1, 1)
    assert gpu_lib.gvom_create(ctypes.byref(p), ctypes.byref(h)) == GVOM_ERR_ARG
    assert gpu_lib.gvom_process(None, None, 0, 0, 3, None, None, -1) == GVOM_ERR_ARG


def test_ctypes_structures_match_the_header_layout(tmp_path):
    """Every struct of include/gvom_gb300.h has the same field names, offsets
    and size in the ctypes binding (the C compiler reports its own layout)."""
    import shutil
    import subprocess

    import pytest

    from gvom_gb300 import _lib
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    hdr = open(os.path.join(REPO, "include", "gvom_gb300.h")).read()
    structs = {"GvomParams": _lib.GvomParams, "GvomScan": _lib.GvomScan, "GvomTuning": _lib.GvomTuning,
               "GvomRosParams": _lib.GvomRosParams}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gvom_gb300.h"', "int main(void) {"]
    for name, cls in structs.items():
        body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), hdr, re.S).group(1)
        body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
        fields = re.findall(r"(\w+)(?:\[\d+\])?;", body)
        assert fields == [f[0] for f in cls._fields_], (name, fields)
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (name, name))
        for f in fields:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (name, f, name, f))
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = str(tmp_path / "layout")
    subprocess.run([gcc, "-I", os.path.join(REPO, "include"), "-o", exe, str(src)], check=True)
    out = dict(line.split() for line in subprocess.run([exe], capture_output=True, text=True).stdout.splitlines())
    for name, cls in structs.items():
        assert int(out[name]) == ctypes.sizeof(cls), name
        for f, _ in cls._fields_:
            assert int(out[f"{name}.{f}"]) == getattr(cls, f).offset, (name, f)
