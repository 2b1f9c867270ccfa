"""The C-ABI library loads and exports every entry point include/rdsim.h
declares (no compute calls: runs without a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions(header=None):
    names = set()
    inc = os.path.join(ROOT, "include")
    for h in sorted(os.listdir(inc)) if header is None else [header]:
        if not h.endswith(".h"):
            continue
        with open(os.path.join(inc, h)) as f:
            text = re.sub(r"/\*.*?\*/", "", f.read(), flags=re.S)
        names |= set(re.findall(r"\b(rdsim_[a-z_]+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from pyrdsim_gb300 import build
    try:
        build.build()
    except Exception as exc:  # nvcc must exist wherever the tests run
        pytest.fail(f"engine build failed: {exc}")
    return ctypes.CDLL(build.LIB)


def test_header_declares_the_engine_api():
    names = declared_functions()
    for n in ["rdsim_create", "rdsim_step", "rdsim_destroy", "rdsim_get_state",
              "rdsim_get_drift", "rdsim_get_pairs", "rdsim_get_cell_ids"]:
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_declares_every_export():
    from pyrdsim_gb300 import adjoint, engine
    assert sorted(engine.EXPORTS) == declared_functions("rdsim.h")
    assert sorted(adjoint.EXPORTS) == declared_functions("rdsim_adjoint.h")


def test_struct_sizes_match_header(lib):
    """Field layout of the ctypes mirrors, checked through offsets that the
    C compiler would produce for the same declarations."""
    from pyrdsim_gb300 import abi
    assert ctypes.sizeof(abi.Interaction) == 4 * 4 + 5 * 8
    assert ctypes.sizeof(abi.Reaction) == 6 * 4 + 3 * 8
    assert ctypes.sizeof(abi.Term) == 4 * 4 + 2 * 8
    assert ctypes.sizeof(abi.Template) == 16
    assert abi.System.seed.offset % 8 == 0
    assert ctypes.sizeof(abi.Observables) == 6 * 8 + 2 * 8 + abi.MAX_TYPES * 8
    from pyrdsim_gb300.adjoint import AdjointSystemStruct
    assert AdjointSystemStruct.mobility.offset == 16 + 3 * 8 + 8
    assert ctypes.sizeof(AdjointSystemStruct) == 16 + 4 * 8 + 3 * 8 + 8


def test_last_error_is_callable_without_gpu(lib):
    lib.rdsim_last_error.restype = ctypes.c_char_p
    assert isinstance(lib.rdsim_last_error(), bytes)


def test_option_and_info_layout_match_the_c_compiler(tmp_path):
    """rdsim_options and rdsim_info as the C compiler lays them out (sizes and
    the offsets of every field) equal their ctypes mirrors."""
    import shutil
    import subprocess
    from pyrdsim_gb300 import abi
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    fields = {"rdsim_options": abi.Options, "rdsim_info": abi.Info}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "rdsim.h"', "int main(void) {"]
    for cname, cls in fields.items():
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.check_call([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    out = subprocess.check_output([str(exe)], text=True).split("\n")
    got = {}
    for line in out:
        if line.strip():
            cname, f, v = line.split()
            got[(cname, f)] = int(v)
    for cname, cls in fields.items():
        assert got[(cname, "sizeof")] == ctypes.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert got[(cname, f)] == getattr(cls, f).offset, (cname, f)
