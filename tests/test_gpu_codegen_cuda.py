"""GPU end-to-end test of the generated host code of --backend cuda: each
golden host program (tests/golden/cuda_host, emitted by codegen_cuda.py) is
compiled with `cc -std=c99`, linked against libhyd_cuda.so, run on the GPU,
and its printed results (the C backend's main: every zero-argument procedure,
in the reference's print format) and files are checked against the oracle."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "hydrangea-compiler_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden", "cuda_host")


def _build_and_run(hc, name, tmp_path, env=None):
    hc.lib()
    cc = shutil.which("cc") or shutil.which("gcc")
    exe = str(tmp_path / name)
    p = subprocess.run([cc, "-std=c99", "-O2", "-I", os.path.join(ROOT, "include"),
                        os.path.join(GOLDEN, name + ".c"), "-L", PKG, "-lhyd_cuda", "-Wl,-rpath," + PKG,
                        "-o", exe], capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    e = dict(os.environ)
    e.update(env or {})
    r = subprocess.run([exe], cwd=str(tmp_path), capture_output=True, text=True, env=e, timeout=300)
    assert r.returncode == 0, r.stderr
    return r.stdout.splitlines()


def _ints(line):
    body = line[1:line.index("] (shape:")]
    return [int(v) for v in body.split(", ")] if body else []


def _floats(line):
    body = line[1:line.index("] (shape:")]
    return np.array([float(v) for v in body.split(", ")] if body else [], dtype=np.float64)


def _shape(line):
    return [int(v) for v in re.search(r"\(shape: \[(.*)\]\)$", line).group(1).split(", ") if v]


def test_weighted_histogram_program(hc, orc, tmp_path):
    out = _build_and_run(hc, "weighted_histogram", tmp_path)
    data = np.arange(1024, dtype=np.int64)
    assert _ints(out[0]) == data.tolist() and _shape(out[0]) == [1024]
    expect = orc.weighted_hist(data, 64)
    assert _ints(out[1]) == expect.tolist() and _shape(out[1]) == [64]
    # the program's comment: bin[k] = sum_{j=0}^{15} (k + 64 j)^2
    assert _ints(out[1]) == [sum((k + 64 * j) ** 2 for j in range(16)) for k in range(64)]
    assert out[1] == "[" + ", ".join(str(v) for v in expect) + "] (shape: [64])"


def test_dot_csv_program(hc, orc, tmp_path):
    a = np.array([0.1, -2.5, 3.75])
    b = np.array([1.0 / 3.0, 4.0, -0.2])
    (tmp_path / "examples").mkdir()
    for nm, v in (("dotA_f.csv", a), ("dotB_f.csv", b)):
        (tmp_path / "examples" / nm).write_text(", ".join("%.17g" % x for x in v) + "\n")
    out = _build_and_run(hc, "dot_csv_f", tmp_path)
    assert np.array_equal(_floats(out[0]), a) and np.array_equal(_floats(out[1]), b)
    truth = orc.dot_compensated(a, b)
    res = _floats(out[2])
    assert _shape(out[2]) == [] and len(res) == 1
    assert abs(res[0] - truth) <= 1e-12 * max(1.0, float(np.abs(a * b).sum()))
    assert float(out[3]) == res[0]
    assert out[3] == "%.17g" % res[0]


def test_heat_2d_program(hc, orc, tmp_path):
    out = _build_and_run(hc, "heat_2d", tmp_path)
    assert out[0] == "8" and out[1] == "4"
    idx = np.arange(64)
    init = ((idx // 8) * 8 + idx % 8).astype(np.float64) * 0.01
    got_init = _floats(out[2])
    assert np.array_equal(got_init.view(np.int64), init.view(np.int64)) and _shape(out[2]) == [8, 8]
    ref = orc.iterate_stencil2d(orc.HEAT_EXAMPLE, init.reshape(8, 8), 4)
    got = _floats(out[3]).reshape(8, 8)
    assert np.array_equal(got.view(np.int64), ref.view(np.int64))  # bit-exact after 4 steps
    assert out[4] == "0"  # write_array_float's result
    text = (tmp_path / "heat_2d_out.csv").read_text()
    vals = np.array([float(v) for v in re.split(r"[,\s]+", text.strip())])
    assert np.array_equal(vals.view(np.int64), ref.reshape(-1).view(np.int64))


@pytest.mark.parametrize("nrows,ncols,nnz,dup", [(1000, 800, 20000, 4), (37, 53, 5001, 1), (4096, 4096, 300000, 7)])
def test_coo_csr_build_program(hc, orc, tmp_path, nrows, ncols, nnz, dup):
    env = {"COO_NROWS": str(nrows), "COO_NCOLS": str(ncols), "COO_NNZ": str(nnz), "COO_DUP_PERIOD": str(dup)}
    out = _build_and_run(hc, "coo_csr_build", tmp_path, env)
    assert out[:4] == [str(nrows), str(ncols), str(nnz), str(dup)]
    rows, cols, vals = (np.zeros(nnz, dtype=np.int64) for _ in range(3))
    orc.lib().orc_coo_csr_bench_inputs(nrows, ncols, nnz, dup, rows, cols, vals)
    perm = orc.sort_indices(rows * ncols + cols)
    cr, cc, cv, k = orc.coo_sum_duplicates(rows[perm], cols[perm], vals[perm])
    rp, ci, ov = orc.csr_from_sorted_coo(nrows, k, cr, cc, cv)
    expect = int(rp.sum()) + int(ci[:k].sum()) + int(ov[:k].sum()) + int(k)
    assert int(out[4]) == expect


def test_missing_environment_variable_exits_like_the_reference(hc, tmp_path):
    hc.lib()
    cc = shutil.which("cc") or shutil.which("gcc")
    exe = str(tmp_path / "coo")
    subprocess.run([cc, "-std=c99", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(GOLDEN, "coo_csr_build.c"), "-L", PKG, "-lhyd_cuda", "-Wl,-rpath," + PKG,
                    "-o", exe], check=True)
    e = {k: v for k, v in os.environ.items() if not k.startswith("COO_")}
    r = subprocess.run([exe], cwd=str(tmp_path), capture_output=True, text=True, env=e, timeout=120)
    assert r.returncode == 1
    assert "get_env_int: environment variable 'COO_NROWS' not set" in r.stderr
