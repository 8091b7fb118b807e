"""The host-code emitter of the --backend cuda path (codegen_cuda.py), on CPU:
it reproduces the golden host programs of tests/golden/cuda_host byte for
byte, and every golden program compiles as C99 against include/hyd_cuda.h
alone and, where the reference source tree is present, against the
reference's own runtime/hydrangea_runtime.h included first (the array types
then come from that header: the ABI check)."""
import os
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "hydrangea-compiler_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden", "cuda_host")
sys.path.insert(0, PKG)
import codegen_cuda  # noqa: E402

NAMES = sorted(codegen_cuda.PROGRAMS)


@pytest.mark.parametrize("name", NAMES)
def test_emitter_reproduces_golden(name):
    prog = codegen_cuda.PROGRAMS[name]()
    with open(os.path.join(GOLDEN, name + ".c")) as f:
        assert codegen_cuda.emit(prog) == f.read()
    if prog.export:
        with open(os.path.join(GOLDEN, name + ".h")) as f:
            assert codegen_cuda.emit_header(prog) == f.read()


def test_name_rules():
    # CodegenC.hs:1983-1993: reserved names get hyd_, export names do not
    assert codegen_cuda.c_name("main") == "hyd_main"
    assert codegen_cuda.c_name("row-of'") == "row_of_"
    assert codegen_cuda.export_name("main") == "main"
    hdr = codegen_cuda.emit_header(codegen_cuda.PROGRAMS["coo_csr_build"]())
    assert "#ifndef HYDRANGEA_EXPORT_IMOD_H" in hdr and "int64_t hyd_export_imod(int64_t x, int64_t m);" in hdr


@pytest.mark.parametrize("name", NAMES)
def test_golden_compiles_against_the_runtime_header(name):
    cc = shutil.which("cc") or shutil.which("gcc")
    if cc is None:
        pytest.skip("no C compiler")
    src = os.path.join(GOLDEN, name + ".c")
    p = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-Wno-unused-function", "-fsyntax-only",
                        "-I", os.path.join(ROOT, "include"), src], capture_output=True, text=True)
    assert p.returncode == 0, p.stderr


@pytest.mark.parametrize("name", NAMES)
def test_golden_abi_matches_reference_header(name):
    from oracle import build as ob
    ref = ob.DEFAULT_REFERENCE_ROOT
    hdr = os.path.join(ref, "runtime", "hydrangea_runtime.h")
    cc = shutil.which("cc") or shutil.which("gcc")
    if not os.path.exists(hdr) or cc is None:
        pytest.skip("reference runtime header not present")
    # the reference header needs SIMDe; the oracle's scalar shim stands in
    p = subprocess.run([cc, "-std=c99", "-fsyntax-only", "-D_POSIX_C_SOURCE=200809L",
                        "-I", os.path.join(ref, "runtime"), "-I", os.path.join(ROOT, "oracle"),
                        "-include", "hydrangea_runtime.h", "-I", os.path.join(ROOT, "include"),
                        os.path.join(GOLDEN, name + ".c")], capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
