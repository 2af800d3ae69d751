"""The C-ABI library loads and exports every entry point include/lh.h declares, and
the ctypes mirror of lh_config / lh_scalars has the C layout (no compute calls)."""
import ctypes
import os
import re
import subprocess

import pytest

from rnl_multiblock_nofft_gb300 import abi, build_native, native

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
HDR = os.path.join(ROOT, "include", "lh.h")


def declared():
    txt = open(HDR).read()
    return sorted(set(re.findall(r"\b(lh_[a-z0-9_]+)\s*\(", txt)))


def test_header_matches_binding_list():
    assert declared() == sorted(native.EXPORTS)


def test_library_exports_every_symbol():
    lib = build_native.build()
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True, check=True).stdout
    syms = {l.split()[-1] for l in out.splitlines() if " T " in l}
    missing = [s for s in declared() if s not in syms]
    assert not missing, missing
    L = ctypes.CDLL(lib)
    for s in declared():
        assert hasattr(L, s)


def test_struct_layout_matches_c(tmp_path):
    src = tmp_path / "lay.c"
    fields_c = [f for f, _ in abi.LhConfig._fields_]
    body = "\n".join(f'printf("{f} %zu\\n", offsetof(lh_config, {f}));' for f in fields_c)
    body2 = "\n".join(f'printf("S{f} %zu\\n", offsetof(lh_scalars, {f}));' for f, _ in abi.LhScalars._fields_)
    src.write_text(f'#include <stdio.h>\n#include <stddef.h>\n#include "{HDR}"\nint main(void){{\n'
                   f'printf("size %zu\\n", sizeof(lh_config));\nprintf("ssize %zu\\n", sizeof(lh_scalars));\n'
                   f'{body}\n{body2}\nreturn 0;}}\n')
    exe = tmp_path / "lay"
    subprocess.run(["gcc", "-o", str(exe), str(src)], check=True)
    got = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True).stdout.splitlines())
    assert int(got["size"]) == ctypes.sizeof(abi.LhConfig)
    assert int(got["ssize"]) == ctypes.sizeof(abi.LhScalars)
    for f in fields_c:
        assert int(got[f]) == getattr(abi.LhConfig, f).offset, f
    for f, _ in abi.LhScalars._fields_:
        assert int(got["S" + f]) == getattr(abi.LhScalars, f).offset, f


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(RuntimeError):
        native._lib = None
        native.load(str(tmp_path / "nope.so"))
    native._lib = None
