"""CPU checks of the C ABI: the library loads and exports every entry point
include/cxlik_gpu.h declares; the ctypes mirror has the header's layout."""
import ctypes
import os
import re
import subprocess

from crux_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "cxlik_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{]*\)\s*;", text)
    return sorted(set(n for n in names if n.startswith(("Cx", "cxg"))))


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("CxLikQDecomp", "CxLikPt", "CxLikExecute", "cxgLikExecuteLnL",
              "cxgPlanCreate"):
        assert n in names


def test_library_exports_every_declared_symbol():
    from crux_gb300 import _native
    lib = _native.load()
    for n in declared_functions():
        assert hasattr(lib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", _native.LIB_PATH],
                         capture_output=True, text=True, check=True).stdout
    exported = set(line.split()[-1] for line in out.splitlines() if line)
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing


def test_struct_layout_matches_header():
    """Compile a probe against the header and compare offsets/sizes."""
    src = r'''
#include <stddef.h>
#include <stdio.h>
#include "cxlik_gpu.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu\n", sizeof(CxtLik), sizeof(CxtLikCL),
         sizeof(CxtLikComp), sizeof(struct CxsLikModel), sizeof(CxtLikStep));
  printf("%zu %zu %zu %zu %zu %zu\n", offsetof(CxtLik, charFreqs),
         offsetof(CxtLik, wNorm), offsetof(CxtLik, comps),
         offsetof(CxtLik, rootCLC), offsetof(CxtLik, steps),
         offsetof(CxtLik, stepsMax));
  printf("%zu %zu %zu\n", offsetof(struct CxsLikModel, qEigVals),
         offsetof(struct CxsLikModel, comp0), offsetof(CxtLikStep, edgeLen));
  return 0;
}
'''
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "p.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "p")
        subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"),
                        c, "-o", exe], check=True)
        got = subprocess.run([exe], capture_output=True, text=True,
                             check=True).stdout.split()
    want = [ctypes.sizeof(_abi.CxtLik), ctypes.sizeof(_abi.CxtLikCL),
            ctypes.sizeof(_abi.CxtLikComp), ctypes.sizeof(_abi.CxtLikModel),
            ctypes.sizeof(_abi.CxtLikStep),
            _abi.CxtLik.charFreqs.offset, _abi.CxtLik.wNorm.offset,
            _abi.CxtLik.comps.offset, _abi.CxtLik.rootCLC.offset,
            _abi.CxtLik.steps.offset, _abi.CxtLik.stepsMax.offset,
            _abi.CxtLikModel.qEigVals.offset, _abi.CxtLikModel.comp0.offset,
            _abi.CxtLikStep.edgeLen.offset]
    assert [int(x) for x in got] == want


def test_load_without_gpu_reports_no_device():
    from crux_gb300 import _native
    lib = _native.load()
    buf = ctypes.create_string_buffer(256)
    assert lib.cxgInfo(buf, 256) == 0
    assert buf.value.startswith(b"cxlik_gpu")


def test_extension_struct_layouts_match_header():
    """The ctypes mirrors of the MC3, server and native-planner structs
    (crux_gb300.mc3, crux_gb300.serve, crux_gb300._abi) have the header's
    field offsets and sizes."""
    from crux_gb300 import mc3, serve
    pairs = [("cxgMc3Config", mc3.Mc3Config),
             ("cxgMc3ModelState", mc3.Mc3ModelState),
             ("cxgRequest", serve.Request),
             ("cxgServerConfig", serve.ServerConfig),
             ("cxgServerStatsT", serve.ServerStats),
             ("cxgPlanSnap", _abi.CxgPlanSnap)]
    lines = []
    want = []
    for cname, py in pairs:
        lines.append('printf("%%zu\\n", sizeof(%s));' % cname)
        want.append(ctypes.sizeof(py))
        for f in py._fields_:
            lines.append('printf("%%zu\\n", offsetof(%s, %s));' % (cname, f[0]))
            want.append(getattr(py, f[0]).offset)
    src = ("#include <stddef.h>\n#include <stdio.h>\n#include \"cxlik_gpu.h\"\n"
           "int main(void) {\n" + "\n".join(lines) + "\nreturn 0;\n}\n")
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "p.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "p")
        subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"),
                        c, "-o", exe], check=True)
        got = subprocess.run([exe], capture_output=True, text=True,
                             check=True).stdout.split()
    assert [int(x) for x in got] == want
