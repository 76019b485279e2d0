"""The Python bindings' ctypes structures against the C header's structs: a C program built from
include/vedo_gpu.h prints every struct's size and each mirrored field's offset, and the ctypes
layout must match (a field added to the header and not to the binding, or the reverse, shifts the
offsets after it).  CPU only: gcc and the header, no GPU and no library."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

from vedo_gb300 import _abi
from vedo_gb300.serve import JobInfo

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

MIRRORS = {
    "vedo_do_model": _abi.DOModelDesc,
    "vedo_iact_model": _abi.IactModelDesc,
    "vedo_scene_desc": _abi.SceneDesc,
    "vedo_engine_opts": _abi.EngineOpts,
    "vedo_state_view": _abi.StateView,
    "vedo_contact_view": _abi.ContactView,
    "vedo_job_info": JobInfo,
}


def test_ctypes_mirrors_match_the_c_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "vedo_gpu.h"', "int main(void) {"]
    for cname, py in MIRRORS.items():
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'    printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    c_layout = {}
    for line in out:
        if line:
            name, field, value = line.split()
            c_layout[(name, field)] = int(value)
    for cname, py in MIRRORS.items():
        assert C.sizeof(py) == c_layout[(cname, "size")], cname
        for fname, _ in py._fields_:
            assert getattr(py, fname).offset == c_layout[(cname, fname)], (cname, fname)
