"""C-ABI checks that need no GPU: the library loads and exports every
function declared in include/fringe_gb300.h; the ctypes mirrors of the public
structs have the C layout."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fringe_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fpl_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from fringe_gb300 import build, _lib
    build.build()
    return _lib.load()


def test_exports_every_declared_function(lib):
    names = declared_functions()
    assert "fpl_run" in names and "fpl_process" in names
    for n in names:
        assert hasattr(lib, n), n


def test_struct_layout_matches_header(lib, tmp_path):
    import ctypes
    from fringe_gb300 import _lib
    src = tmp_path / "sz.c"
    src.write_text('#include "fringe_gb300.h"\n#include <stdio.h>\n#include <stddef.h>\n'
                   'int main(){printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(fpl_job), sizeof(fpl_options),'
                   ' sizeof(fpl_stats), offsetof(fpl_job, stack), offsetof(fpl_options, method),'
                   ' sizeof(fpl_ps_job), offsetof(fpl_ps_job, tcorr_out), sizeof(fpl_nmap_job),'
                   ' offsetof(fpl_nmap_job, count), offsetof(fpl_nmap_job, method));}\n')
    exe = tmp_path / "sz"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    out = subprocess.check_output([str(exe)]).decode().split()
    want = [ctypes.sizeof(_lib.FplJob), ctypes.sizeof(_lib.FplOptions), ctypes.sizeof(_lib.FplStats),
            _lib.FplJob.stack.offset, _lib.FplOptions.method.offset,
            ctypes.sizeof(_lib.FplPsJob), _lib.FplPsJob.tcorr_out.offset, ctypes.sizeof(_lib.FplNmapJob),
            _lib.FplNmapJob.count.offset, _lib.FplNmapJob.method.offset]
    assert [int(x) for x in out] == want


def test_error_strings_and_defaults(lib):
    import ctypes
    from fringe_gb300 import _lib
    assert lib.fpl_error_string(0) == b"ok"
    assert b"options" in lib.fpl_error_string(101)
    # every status code the header defines has its own message
    codes = {k: v for k, v in _lib.header_defines().items() if k == "FPL_OK" or k.startswith("FPL_ERR_")}
    assert codes["FPL_ERR_HOST"] == 208
    for name, code in codes.items():
        assert lib.fpl_error_string(code) != b"unknown error", name
    o = _lib.FplOptions()
    lib.fpl_options_default(ctypes.byref(o))
    # evdOptions defaults, src/evd/evd.hpp:58-68
    assert (o.blocksize, o.memsize, o.Nx, o.Ny, o.minNeighbors, o.miniStackCount,
            o.method, o.bandWidth) == (64, 2048, 5, 5, 2, 1, b"MLE", -1)
