"""Host-code emitter of the `--backend cuda` path.

The reference compiler lowers a .hyd program to a CFG of fused loop nests and
hands it to a backend that renders C: ``genProgram`` in
src/Language/Hydrangea/CodegenC.hs:290-370 (one C function per top-level
binding, an export wrapper ``RET hyd_export_<name>(PARAMS)`` with its header,
:372-460, and a ``main`` that calls every zero-argument procedure and prints
its result, :492-640); the Metal backend does the same around its kernels
(CodegenMSL.hs:157-205 for codegenMSL, :1120-1230 for the host side).  GHC is
not available to build a ``CodegenCUDA.hs``, so this module restates that
backend's host side in Python.  Its input is the fused loop nests of a
program, one node per loop template the GB300 runtime serves (the same
templates the C backend renders as OpenMP loops), and its output is the C host
program: each loop nest becomes one call into libhyd_cuda.so (include/hyd_cuda.h),
device buffers hold the intermediate arrays, and procedures return the
reference's host ``hyd_array_t`` so that printing, CSV output and embedding
hosts see the same ABI.

Name rules follow the C backend: a binding whose name is a C reserved name
(``main``) is emitted as ``hyd_<name>`` (CodegenC.hs:1983-1988); export
wrappers use the unsanitised name (:1990-1993) and header guards
``HYDRANGEA_EXPORT_<NAME>_H`` (:458-460).

``PROGRAMS`` holds the fused CFG of the four programs the runtime's benches
come from; ``emit(program)`` renders one, and ``tests/golden/cuda_host/``
keeps the rendered files.
"""
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

C_RESERVED = {"main", "int", "double", "float", "char", "long", "return", "if", "else", "for", "while", "static",
              "void", "struct", "union", "switch", "case", "default", "break", "continue"}


def c_name(name):
    """CodegenC.hs sanitize: reserved names get a ``hyd_`` prefix, other
    characters than [A-Za-z0-9_] become ``_``."""
    if name in C_RESERVED:
        return "hyd_" + name
    return "".join(ch if ch.isalnum() or ch == "_" else "_" for ch in name)


# ---- the fused loop nests (one node per runtime template) -----------------------
@dataclass
class ConstInt:           # let x = <literal>
    var: str
    value: int


@dataclass
class EnvInt:             # let x = get_env_int "NAME"
    var: str
    env: str


@dataclass
class CallInt:            # a use of a zero-argument int procedure
    var: str
    proc: str


@dataclass
class CallArray:          # a use of a zero-argument array procedure (a host hyd_array_t*)
    var: str
    proc: str


@dataclass
class Generate:           # generate / map / zipwith chain fused into one element loop
    var: str              # device buffer
    elem: str             # "i64" | "f64"
    n: str                # element count (C expression)
    body: str             # C statements over i, x0.. assigning v (a printf format when fmt_args)
    inputs: Tuple[str, ...] = ()
    fmt_args: Tuple[str, ...] = ()   # run-time values spliced into the body text


@dataclass
class ReadCsvFloat:       # read_array_float [shape] "file"
    var: str              # host array
    shape: Tuple[int, ...]
    path: str


@dataclass
class Upload:             # host array -> device buffer
    var: str
    src: str


@dataclass
class Dot:                # reduce (+) 0.0 (zipwith (*) xs ys), as a 0-D array
    var: str              # device double
    xs: str
    ys: str
    n: str


@dataclass
class SumI64:             # reduce (+) 0 xs over int64, read back
    var: str
    src: str
    n: str


@dataclass
class WeightedHistogram:  # scatter (+) (fill [bins] 0) (map (x % bins) d) (map (x * x) d)
    var: str
    data: str
    n: str
    bins: int


@dataclass
class IterateStencil2D:   # iterate k init (stencil clamp <kind>), ping-pong buffers hoisted
    var: str
    kind: str             # HYD_STENCIL_*
    src: str
    h: str
    w: str
    iters: str


@dataclass
class SortIndices:
    var: str
    keys: str
    n: str


@dataclass
class Gather:
    var: str
    perm: str
    src: str
    n: str


@dataclass
class CooSumDuplicates:   # coo_sum_duplicates: rows/cols/vals of the input's length, canonical count
    rows: str
    cols: str
    vals: str
    nnz: str              # int64 variable receiving the canonical count
    in_rows: str
    in_cols: str
    in_vals: str
    n: str


@dataclass
class CsrFromSortedCoo:
    row_ptr: str
    col_idx: str
    vals: str
    nrows: str
    nnz: str
    rows: str
    cols: str
    in_vals: str


@dataclass
class Download:           # device buffer -> new host array
    var: str
    src: str
    dims: Tuple[str, ...]
    elem: str


@dataclass
class WriteCsvFloat:      # write_array_float a "file"
    var: str
    src: str
    path: str


@dataclass
class IndexScalarF64:     # index () a of a 0-D float array
    var: str
    src: str


@dataclass
class Expr:               # a scalar C expression
    var: str
    ctype: str
    expr: str


@dataclass
class Proc:
    name: str
    ret: str              # "i64" | "f64" | "arr_i64" | "arr_f64"
    body: List[object]
    result: str
    params: Sequence[Tuple[str, str]] = ()   # (name, ctype) for scalar helper procedures
    scalar_expr: Optional[str] = None        # body of a scalar helper procedure


@dataclass
class Program:
    source: str
    procs: List[Proc]
    export: Optional[str] = None
    notes: List[str] = field(default_factory=list)


RET_CTYPE = {"i64": "int64_t", "f64": "double", "arr_i64": "hyd_array_t*", "arr_f64": "hyd_array_t*"}
ELEM_CTYPE = {"i64": "int64_t", "f64": "double"}


def _cstr(s):
    return '"' + s.replace("\\", "\\\\").replace('"', '\\"') + '"'


class _Emitter:
    def __init__(self, prog):
        self.prog = prog
        self.lines = []

    def w(self, line=""):
        self.lines.append(line)

    # one statement of a procedure body
    def stmt(self, s, dev_bufs):
        check = "hyd_cuda_gen_check"
        if isinstance(s, ConstInt):
            self.w("    int64_t %s = %dLL;" % (s.var, s.value))
        elif isinstance(s, EnvInt):
            self.w("    int64_t %s = hyd_cuda_gen_get_env_int(%s);" % (s.var, _cstr(s.env)))
        elif isinstance(s, CallInt):
            self.w("    int64_t %s = %s();" % (s.var, c_name(s.proc)))
        elif isinstance(s, CallArray):
            self.w("    hyd_array_t* %s = %s();" % (s.var, c_name(s.proc)))
        elif isinstance(s, Expr):
            self.w("    %s %s = %s;" % (s.ctype, s.var, s.expr))
        elif isinstance(s, Generate):
            ct = ELEM_CTYPE[s.elem]
            self.w("    %s* %s = (%s*)hyd_cuda_gen_alloc((%s) * (int64_t)sizeof(%s));" % (ct, s.var, ct, s.n, ct))
            dev_bufs.append(s.var)
            self.w("    {")
            if s.fmt_args:
                self.w("        char body[512];")
                self.w("        snprintf(body, sizeof body, %s, %s);" % (
                    _cstr(s.body), ", ".join("(long long)%s" % a for a in s.fmt_args)))
                body = "body"
            else:
                body = _cstr(s.body)
            if s.inputs:
                self.w("        const %s* in[%d] = {%s};" % (ct, len(s.inputs), ", ".join(s.inputs)))
                ins, nin = "in", len(s.inputs)
            else:
                ins, nin = "NULL", 0
            self.w("        %s(hyd_cuda_map_%s(%s, %s, %d, %s, %s, NULL, NULL), %s);" % (
                check, s.elem, body, ins, nin, s.n, s.var, _cstr("map_" + s.elem)))
            self.w("    }")
        elif isinstance(s, ReadCsvFloat):
            self.w("    hyd_tuple_t %s_shape;" % s.var)
            self.w("    memset(&%s_shape, 0, sizeof %s_shape);" % (s.var, s.var))
            self.w("    %s_shape.ndims = %d;" % (s.var, len(s.shape)))
            for k, e in enumerate(s.shape):
                self.w("    %s_shape.elems[%d] = %d;" % (s.var, k, e))
            self.w("    hyd_array_t* %s = hyd_cuda_read_float_array_csv(%s, %s_shape);" % (s.var, _cstr(s.path), s.var))
        elif isinstance(s, Upload):
            self.w("    void* %s = hyd_cuda_gen_upload(%s);" % (s.var, s.src))
            dev_bufs.append(s.var)
        elif isinstance(s, Dot):
            self.w("    double* %s = (double*)hyd_cuda_gen_alloc((int64_t)sizeof(double));" % s.var)
            dev_bufs.append(s.var)
            self.w("    %s(hyd_cuda_dot_f64((const double*)%s, (const double*)%s, %s, %s, NULL), %s);" % (
                check, s.xs, s.ys, s.n, s.var, _cstr("dot_f64")))
        elif isinstance(s, SumI64):
            self.w("    int64_t %s;" % s.var)
            self.w("    {")
            self.w("        int64_t* acc = (int64_t*)hyd_cuda_gen_alloc((int64_t)sizeof(int64_t));")
            self.w("        const int64_t* in[1] = {%s};" % s.src)
            self.w("        %s(hyd_cuda_map_i64(\"v = x0;\", in, 1, %s, NULL, acc, NULL), \"reduce (+)\");" % (
                check, s.n))
            self.w("        %s = hyd_cuda_gen_read_i64(acc);" % s.var)
            self.w("        hyd_cuda_gen_free(acc);")
            self.w("    }")
        elif isinstance(s, WeightedHistogram):
            self.w("    int64_t* %s = (int64_t*)hyd_cuda_gen_alloc(%dLL * (int64_t)sizeof(int64_t));" % (s.var, s.bins))
            dev_bufs.append(s.var)
            self.w("    hyd_cuda_gen_zero(%s, %dLL * (int64_t)sizeof(int64_t));" % (s.var, s.bins))
            self.w("    %s(hyd_cuda_weighted_histogram_i64(%s, %s, %dLL, %s, HYD_SCATTER_AUTO, NULL), %s);" % (
                check, s.data, s.n, s.bins, s.var, _cstr("scatter (+)")))
        elif isinstance(s, IterateStencil2D):
            self.w("    double* %s_pong = (double*)hyd_cuda_gen_alloc((%s) * (%s) * (int64_t)sizeof(double));" % (
                s.var, s.h, s.w))
            dev_bufs.append(s.var + "_pong")
            self.w("    double* %s;" % s.var)
            self.w("    {")
            self.w("        int final_buf = 0;")
            self.w("        %s(hyd_cuda_iterate_stencil2d_f64(%s, (double*)%s, %s_pong, %s, %s, %s, &final_buf, "
                   "NULL), %s);" % (check, s.kind, s.src, s.var, s.h, s.w, s.iters, _cstr("iterate")))
            self.w("        %s = final_buf ? %s_pong : (double*)%s;" % (s.var, s.var, s.src))
            self.w("    }")
        elif isinstance(s, SortIndices):
            self.w("    int64_t* %s = (int64_t*)hyd_cuda_gen_alloc((%s) * (int64_t)sizeof(int64_t));" % (s.var, s.n))
            dev_bufs.append(s.var)
            self.w("    %s(hyd_cuda_sort_indices_i64(%s, %s, %s, NULL), %s);" % (
                check, s.keys, s.n, s.var, _cstr("sort_indices")))
        elif isinstance(s, Gather):
            self.w("    int64_t* %s = (int64_t*)hyd_cuda_gen_alloc((%s) * (int64_t)sizeof(int64_t));" % (s.var, s.n))
            dev_bufs.append(s.var)
            self.w("    %s(hyd_cuda_gather_i64(%s, %s, %s, %s, %s, NULL), %s);" % (
                check, s.perm, s.n, s.src, s.n, s.var, _cstr("gather")))
        elif isinstance(s, CooSumDuplicates):
            for v in (s.rows, s.cols, s.vals):
                self.w("    int64_t* %s = (int64_t*)hyd_cuda_gen_alloc((%s) * (int64_t)sizeof(int64_t));" % (v, s.n))
                dev_bufs.append(v)
            self.w("    int64_t %s;" % s.nnz)
            self.w("    {")
            self.w("        int64_t* cnt = (int64_t*)hyd_cuda_gen_alloc((int64_t)sizeof(int64_t));")
            self.w("        %s(hyd_cuda_coo_sum_duplicates_i64(%s, %s, %s, %s, %s, %s, %s, cnt, NULL), %s);" % (
                check, s.in_rows, s.in_cols, s.in_vals, s.n, s.rows, s.cols, s.vals, _cstr("coo_sum_duplicates")))
            self.w("        %s = hyd_cuda_gen_read_i64(cnt);" % s.nnz)
            self.w("        hyd_cuda_gen_free(cnt);")
            self.w("    }")
        elif isinstance(s, CsrFromSortedCoo):
            self.w("    int64_t* %s = (int64_t*)hyd_cuda_gen_alloc((%s + 1) * (int64_t)sizeof(int64_t));" % (
                s.row_ptr, s.nrows))
            self.w("    int64_t* %s = (int64_t*)hyd_cuda_gen_alloc((%s) * (int64_t)sizeof(int64_t));" % (s.col_idx, s.nnz))
            self.w("    int64_t* %s = (int64_t*)hyd_cuda_gen_alloc((%s) * (int64_t)sizeof(int64_t));" % (s.vals, s.nnz))
            dev_bufs.extend([s.row_ptr, s.col_idx, s.vals])
            self.w("    %s(hyd_cuda_csr_from_sorted_coo_i64(%s, %s, %s, %s, %s, %s, %s, %s, NULL), %s);" % (
                check, s.nrows, s.nnz, s.rows, s.cols, s.in_vals, s.row_ptr, s.col_idx, s.vals,
                _cstr("csr_from_sorted_coo")))
        elif isinstance(s, Download):
            self.w("    hyd_tuple_t %s_shape;" % s.var)
            self.w("    memset(&%s_shape, 0, sizeof %s_shape);" % (s.var, s.var))
            self.w("    %s_shape.ndims = %d;" % (s.var, len(s.dims)))
            for k, e in enumerate(s.dims):
                self.w("    %s_shape.elems[%d] = %s;" % (s.var, k, e))
            self.w("    hyd_array_t* %s = hyd_cuda_gen_download(%s, %s_shape, sizeof(%s));" % (
                s.var, s.src, s.var, ELEM_CTYPE[s.elem]))
        elif isinstance(s, WriteCsvFloat):
            self.w("    int64_t %s = hyd_cuda_write_array_csv_float(%s, %s);" % (s.var, s.src, _cstr(s.path)))
        elif isinstance(s, IndexScalarF64):
            self.w("    double %s;" % s.var)
            self.w("    memcpy(&%s, %s->data, sizeof %s);" % (s.var, s.src, s.var))
        else:
            raise TypeError("no template for %r" % (s,))

    def proc(self, p):
        ret = RET_CTYPE[p.ret]
        name = c_name(p.name)
        if p.params:
            params = ", ".join("%s %s" % (ct, c_name(n)) for n, ct in p.params)
            self.w("static %s %s(%s) {" % (ret, name, params))
            self.w("    return %s;" % p.scalar_expr)
            self.w("}")
            return
        self.w("static %s %s(void) {" % (ret, name))
        dev_bufs = []
        host_tmp = [s.var for s in p.body if isinstance(s, (CallArray, ReadCsvFloat)) and s.var != p.result]
        for s in p.body:
            self.stmt(s, dev_bufs)
        for b in dev_bufs:
            self.w("    hyd_cuda_gen_free(%s);" % b)
        for h in host_tmp:
            self.w("    hyd_cuda_gen_array_free(%s);" % h)
        self.w("    return %s;" % p.result)
        self.w("}")

    def render(self):
        prog = self.prog
        self.w("/* Host program of the --backend cuda path for %s, emitted by codegen_cuda.py." % prog.source)
        self.w(" * Each fused loop nest is one call into the GB300 runtime (libhyd_cuda.so);")
        self.w(" * procedures return the reference runtime's host arrays. */")
        for n in prog.notes:
            self.w("/* %s */" % n)
        self.w("#include <stdint.h>")
        self.w("#include <stdio.h>")
        self.w("#include <string.h>")
        self.w("")
        self.w("#include \"hyd_cuda.h\"")
        self.w("")
        for p in prog.procs:
            self.proc(p)
            self.w("")
        if prog.export:
            p = next(q for q in prog.procs if q.name == prog.export)
            params = ", ".join("%s %s" % (ct, c_name(n)) for n, ct in p.params) or "void"
            args = ", ".join(c_name(n) for n, _ in p.params)
            self.w("%s hyd_export_%s(%s) {" % (RET_CTYPE[p.ret], export_name(p.name), params))
            self.w("    return %s(%s);" % (c_name(p.name), args))
            self.w("}")
            self.w("")
        self.w("int main(void) {")
        self.w("    hyd_cuda_gen_check(hyd_cuda_init(), \"hyd_cuda_init\");")
        for p in prog.procs:
            if p.params:
                continue
            cn = c_name(p.name)
            res = cn + "_result"
            if p.ret == "i64":
                self.w("    int64_t %s = %s();" % (res, cn))
                self.w("    hyd_cuda_gen_print_int(%s);" % res)
            elif p.ret == "f64":
                self.w("    double %s = %s();" % (res, cn))
                self.w("    hyd_cuda_gen_print_double(%s);" % res)
            else:
                self.w("    hyd_array_t* %s = %s();" % (res, cn))
                self.w("    hyd_cuda_gen_print_%s(%s);" % ("array" if p.ret == "arr_i64" else "float_array", res))
                self.w("    hyd_cuda_gen_array_free(%s);" % res)
        self.w("    hyd_cuda_cleanup();")
        self.w("    return 0;")
        self.w("}")
        return "\n".join(self.lines) + "\n"


def export_name(name):
    """CodegenC.hs sanitizeExportName: no reserved-name prefix."""
    return "".join(ch if ch.isalnum() or ch == "_" else "_" for ch in name)


def emit(prog):
    """The C host program of `prog`."""
    return _Emitter(prog).render()


def emit_header(prog):
    """The export header (CodegenC.hs:427-460 shape) of `prog`'s exported procedure."""
    p = next(q for q in prog.procs if q.name == prog.export)
    guard = "HYDRANGEA_EXPORT_%s_H" % export_name(p.name).upper()
    params = ", ".join("%s %s" % (ct, c_name(n)) for n, ct in p.params) or "void"
    return "\n".join([
        "#ifndef " + guard, "#define " + guard, "", "#include \"hyd_cuda.h\"", "",
        "#ifdef __cplusplus", "extern \"C\" {", "#endif", "",
        "%s hyd_export_%s(%s);" % (RET_CTYPE[p.ret], export_name(p.name), params), "",
        "#ifdef __cplusplus", "}", "#endif", "", "#endif", ""])


# ---- the fused CFG of the four bench programs ---------------------------------------
def weighted_histogram_program():
    """examples/weighted_histogram.hyd: scatter (+) (fill [64] 0) (map binFn data)
    (map valueFn data) over data = generate [1024] (i); the scatter_reindex fusion
    reads data once per element (the fused histogram template)."""
    return Program(
        source="examples/weighted_histogram.hyd",
        procs=[
            Proc("data", "arr_i64", [Generate("d_data", "i64", "1024", "v = i;"),
                                     Download("data", "d_data", ("1024",), "i64")], "data"),
            Proc("binFn", "i64", [], "", params=(("x", "int64_t"),), scalar_expr="x % 64"),
            Proc("valueFn", "i64", [], "", params=(("x", "int64_t"),), scalar_expr="x * x"),
            Proc("main", "arr_i64", [Generate("d_data", "i64", "1024", "v = i;"),
                                     WeightedHistogram("d_hist", "d_data", "1024", 64),
                                     Download("hist", "d_hist", ("64",), "i64")], "hist"),
        ],
        export="binFn")


def dot_program():
    """examples/dot_csv_f.hyd: reduce (+) 0.0 (zipwith (*) a b) over two float
    arrays read from CSV; fuseReduce makes it one reduce_generate (the dot)."""
    return Program(
        source="examples/dot_csv_f.hyd",
        procs=[
            Proc("add", "f64", [], "", params=(("x", "double"), ("y", "double")), scalar_expr="x + y"),
            Proc("mul", "f64", [], "", params=(("x", "double"), ("y", "double")), scalar_expr="x * y"),
            Proc("a", "arr_f64", [ReadCsvFloat("a", (3,), "examples/dotA_f.csv")], "a"),
            Proc("b", "arr_f64", [ReadCsvFloat("b", (3,), "examples/dotB_f.csv")], "b"),
            Proc("result", "arr_f64", [CallArray("ha", "a"), CallArray("hb", "b"),
                                       Upload("d_a", "ha"), Upload("d_b", "hb"),
                                       Dot("d_acc", "d_a", "d_b", "3"),
                                       Download("result", "d_acc", (), "f64")], "result"),
            Proc("main", "f64", [CallArray("r", "result"), IndexScalarF64("v", "r")], "v"),
        ],
        export="mul")


def heat_2d_program():
    """examples/heat_2d.hyd: iterate 4 steps of the clamp 5-point mean over an
    8x8 grid generated from (i * 8 + j) * 0.01, hoisted ping-pong buffers, and
    write the result as CSV."""
    return Program(
        source="examples/heat_2d.hyd",
        procs=[
            Proc("n", "i64", [ConstInt("v", 8)], "v"),
            Proc("iters", "i64", [ConstInt("v", 4)], "v"),
            Proc("init", "arr_f64", [
                CallInt("nn", "n"),
                Generate("d_init", "f64", "nn * nn",
                         "long long r = i / %lld; long long c = i %% %lld; v = (double)((r * 8) + c) * 0.01;",
                         fmt_args=("nn", "nn")),
                Download("init", "d_init", ("nn", "nn"), "f64")], "init"),
            Proc("result", "arr_f64", [
                CallInt("nn", "n"), CallInt("k", "iters"), CallArray("h0", "init"),
                Upload("d0", "h0"),
                IterateStencil2D("d_res", "HYD_STENCIL_HEAT_EXAMPLE", "d0", "nn", "nn", "k"),
                Download("result", "d_res", ("nn", "nn"), "f64")], "result"),
            Proc("main", "i64", [CallArray("r", "result"), WriteCsvFloat("written", "r", "heat_2d_out.csv")],
                 "written"),
        ],
        notes=["main's result array is released after the write, as the C backend's main does not print it"])


def coo_csr_build_program():
    """bench/coo_csr_build/coo_csr_build.hyd: generate COO triplets with
    duplicate runs, sort_indices on packed keys, gather, coo_sum_duplicates,
    csr_from_sorted_coo, and a checksum of the CSR arrays."""
    row_of = "long long g = i / %lldLL; long long a = g * 17 + 3; v = a - ((a / %lldLL) * %lldLL);"
    col_of = "long long g = i / %lldLL; long long a = g * 31 + 7; v = a - ((a / %lldLL) * %lldLL);"
    val_of = "long long g = i / %lldLL; v = (g * 13) + i + 1;"
    key_of = ("long long g = i / %lldLL; long long a = g * 17 + 3; long long b = g * 31 + 7; "
              "v = (a - ((a / %lldLL) * %lldLL)) * %lldLL + (b - ((b / %lldLL) * %lldLL));")
    return Program(
        source="bench/coo_csr_build/coo_csr_build.hyd",
        procs=[
            Proc("nrows", "i64", [EnvInt("v", "COO_NROWS")], "v"),
            Proc("ncols", "i64", [EnvInt("v", "COO_NCOLS")], "v"),
            Proc("nnz", "i64", [EnvInt("v", "COO_NNZ")], "v"),
            Proc("dup", "i64", [EnvInt("v", "COO_DUP_PERIOD")], "v"),
            Proc("imod", "i64", [], "", params=(("x", "int64_t"), ("m", "int64_t")),
                 scalar_expr="x - ((x / m) * m)"),
            Proc("main", "i64", [
                CallInt("nr", "nrows"), CallInt("nc", "ncols"), CallInt("nz", "nnz"), CallInt("dp", "dup"),
                Generate("d_rows", "i64", "nz", row_of, fmt_args=("dp", "nr", "nr")),
                Generate("d_cols", "i64", "nz", col_of, fmt_args=("dp", "nc", "nc")),
                Generate("d_vals", "i64", "nz", val_of, fmt_args=("dp",)),
                Generate("d_keys", "i64", "nz", key_of, fmt_args=("dp", "nr", "nr", "nc", "nc", "nc")),
                SortIndices("d_perm", "d_keys", "nz"),
                Gather("d_srows", "d_perm", "d_rows", "nz"),
                Gather("d_scols", "d_perm", "d_cols", "nz"),
                Gather("d_svals", "d_perm", "d_vals", "nz"),
                CooSumDuplicates("d_crows", "d_ccols", "d_cvals", "cnnz", "d_srows", "d_scols", "d_svals", "nz"),
                CsrFromSortedCoo("d_row_ptr", "d_col_idx", "d_csr_vals", "nr", "cnnz", "d_crows", "d_ccols",
                                 "d_cvals"),
                SumI64("s_row_ptr", "d_row_ptr", "nr + 1"),
                SumI64("s_col_idx", "d_col_idx", "cnnz"),
                SumI64("s_vals", "d_csr_vals", "cnnz"),
                Expr("checksum", "int64_t", "s_row_ptr + s_col_idx + s_vals + cnnz")], "checksum"),
        ],
        export="imod")


PROGRAMS = {
    "weighted_histogram": weighted_histogram_program,
    "dot_csv_f": dot_program,
    "heat_2d": heat_2d_program,
    "coo_csr_build": coo_csr_build_program,
}


def write_golden(directory):
    """Render every program (and its export header) into `directory`."""
    import os
    os.makedirs(directory, exist_ok=True)
    for name, make in PROGRAMS.items():
        prog = make()
        with open(os.path.join(directory, name + ".c"), "w") as f:
            f.write(emit(prog))
        if prog.export:
            with open(os.path.join(directory, name + ".h"), "w") as f:
                f.write(emit_header(prog))


if __name__ == "__main__":
    import sys
    write_golden(sys.argv[1] if len(sys.argv) > 1 else ".")
