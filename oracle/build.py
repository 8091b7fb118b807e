"""Build recipe for the oracle (test infrastructure only).

* ``libhyd_oracle.so`` -- the C restatement in ``hyd_oracle.c``, compiled with
  the reference C backend's flags minus ``-march=native`` (the library must
  give identical results on the x86 and Arm hosts): ``-O3 -std=c99 -fopenmp``.
* ``_ref/libhyd_refwitness.so`` -- the reference's own kernels compiled from
  the reference source tree where it lies (``witness/*.c`` include them), only
  when that tree is present.  Output goes to ``_ref/`` and stays out of git.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libhyd_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_SO = os.path.join(REF_DIR, "libhyd_refwitness.so")
# The reference source tree, read in place: $HYD_REFERENCE_ROOT, else a
# checkout named ``reference`` beside this repository.
DEFAULT_REFERENCE_ROOT = os.environ.get(
    "HYD_REFERENCE_ROOT", os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))

CFLAGS = ["-O3", "-std=c99", "-fopenmp", "-fPIC", "-shared", "-Wall", "-Wno-unused-function"]


def _run(cmd):
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + proc.stdout + proc.stderr)


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_oracle(force=False):
    src = os.path.join(HERE, "hyd_oracle.c")
    hdr = os.path.join(HERE, "hyd_oracle.h")
    if force or _stale(ORACLE_SO, [src, hdr, __file__]):
        _run(["gcc", *CFLAGS, "-o", ORACLE_SO, src, "-lm"])
    return ORACLE_SO


def build_reference_witness(reference_root=None, force=False):
    """Compile the witness library; returns its path or None without the tree."""
    root = reference_root or os.environ.get("HYD_REFERENCE_ROOT", DEFAULT_REFERENCE_ROOT)
    if not os.path.isdir(os.path.join(root, "runtime")):
        return None
    wdir = os.path.join(HERE, "witness")
    srcs = sorted(os.path.join(wdir, f) for f in os.listdir(wdir) if f.endswith(".c"))
    shim = [os.path.join(HERE, "simde", "x86", f) for f in ("sse2.h", "avx.h")]
    if force or _stale(REF_SO, srcs + shim + [__file__]):
        os.makedirs(REF_DIR, exist_ok=True)
        # the reference's timing.h uses clock_gettime/CLOCK_MONOTONIC, which
        # ISO C99 mode hides without a POSIX feature macro.
        flags = CFLAGS + ["-D_POSIX_C_SOURCE=199309L", "-w"]
        _run(["gcc", *flags, "-I", root, "-I", HERE, "-o", REF_SO, *srcs, "-lm"])
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_reference_witness(force="--force" in sys.argv))
