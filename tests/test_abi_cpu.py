"""The C-ABI library loads and exports every entry point the header declares,
and the ctypes struct mirrors have the C layout.  No device calls."""
import ctypes as C
import os
import re
import subprocess

import pytest

from diffusecode_gb300 import _abi, _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "discus_gpu.h")


def header_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(dgpu_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def built_lib():
    if not os.path.exists(_lib.LIB_PATH):
        from diffusecode_gb300 import build
        build.build()
    return _lib.load()


def test_every_declared_symbol_is_exported(built_lib):
    names = header_functions()
    assert len(names) >= 14
    for n in names:
        assert hasattr(built_lib, n), n
    assert sorted(_lib.EXPORTS) == names


def test_struct_layouts_match_c(tmp_path):
    prog = tmp_path / "sz.c"
    prog.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "discus_gpu.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n\", sizeof(dgpu_crystal),"
        " sizeof(dgpu_grid), sizeof(dgpu_opts), sizeof(dgpu_info), offsetof(dgpu_opts, cancel),"
        " offsetof(dgpu_info, res), offsetof(dgpu_crystal, delfi), offsetof(dgpu_crystal, isym),"
        " offsetof(dgpu_opts, discamb), sizeof(dgpu_discamb), offsetof(dgpu_discamb, form_tsc)); return 0;}\n")
    exe = tmp_path / "sz"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(prog), "-o", str(exe)])
    vals = [int(x) for x in subprocess.check_output([str(exe)]).split()]
    assert vals == [C.sizeof(_abi.Crystal), C.sizeof(_abi.Grid), C.sizeof(_abi.Opts), C.sizeof(_abi.Info),
                    _abi.Opts.cancel.offset, _abi.Info.res.offset, _abi.Crystal.delfi.offset,
                    _abi.Crystal.isym.offset, _abi.Opts.discamb.offset, C.sizeof(_abi.Discamb),
                    _abi.Discamb.form_tsc.offset]


def test_output_struct_layouts_match_c(tmp_path):
    fields = [("dgpu_output", _abi.Output, f) for f, _ in _abi.Output._fields_]
    fields += [("dgpu_nipl", _abi.Nipl, f) for f, _ in _abi.Nipl._fields_]
    cname = {"lambda_": "lambda"}
    expr = ", ".join(f"offsetof({s}, {cname.get(f, f)})" for s, _, f in fields)
    prog = tmp_path / "so.c"
    prog.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "discus_gpu.h"\n'
        "int main(void){size_t v[] = {sizeof(dgpu_output), sizeof(dgpu_nipl), " + expr + "};"
        " for (size_t k = 0; k < sizeof v / sizeof v[0]; k++) printf(\"%zu \", v[k]); return 0;}\n")
    exe = tmp_path / "so"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(prog), "-o", str(exe)])
    vals = [int(x) for x in subprocess.check_output([str(exe)]).split()]
    want = [C.sizeof(_abi.Output), C.sizeof(_abi.Nipl)] + [getattr(t, f).offset for _, t, f in fields]
    assert vals == want


def test_lmn_host_entry_needs_no_device(built_lib):
    """dgpu_fourier_lmn is host code (quad precision) and runs without a GPU."""
    import kat_cases as K
    import numpy as np
    for case in K.LMN_CASES:
        e = np.zeros(12)
        e[:3] = case["eck"]
        v = np.asarray(case["vi"], dtype=np.float64).reshape(-1).copy()
        inc = np.asarray(case["inc"], dtype=np.int32)
        lmn = np.zeros(6, np.int32)
        off = np.zeros(9)
        rc = built_lib.dgpu_fourier_lmn(_abi.dptr(e), _abi.dptr(v), _abi.iptr(inc), _abi.iptr(lmn),
                                        _abi.dptr(off))
        assert rc == case["rc"]
        if rc == 0:
            assert list(lmn) == case["lmn"]
            np.testing.assert_allclose(off.reshape(3, 3), np.asarray(case["off"]), atol=1e-15)


def test_context_creation_fails_loudly_without_gpu(built_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    with pytest.raises(_lib.DiscusGpuError):
        _lib.Context(0)
