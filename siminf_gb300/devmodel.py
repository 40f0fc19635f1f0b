"""Model C code compiled for the GPU: the device counterpart of R/run.R:22-98.

In the reference, a model that carries C code (mparse output,
R/C-generator.R:204-297, or a package_skeleton model file) is written to a
file, compiled with R CMD SHLIB against inst/include/SimInf.h, cached by a
digest of the code (R/run.R:93-98) and dyn.loaded; SimInf_run then calls its
trFun/ptsFun through function pointers on the host.  Here the same code is
compiled by nvcc for sm_103a as __device__ functions with their signatures
unchanged:

1. parse_model_code() splits the C file into its top-level items and finds
   the transition-rate functions and the post-time-step function by reading
   the run function's `TRFun tr_fun[] = {...}` and its
   `SimInf_run(model, options, tr_fun, &ptsFun)` call;
2. device_source() drops the R glue (the run function, the registration
   table, R_init -- everything that names SEXP or DllInfo) and the R and
   SimInf.h includes, marks every remaining function and file-scope
   variable __device__, includes siminf_model_code.h (the device stand-in
   of SimInf.h) and adds a model struct whose rate(k) calls the k-th
   tr_fun entry and whose pts() calls the post-time-step function, then
   instantiates the solver's kernel templates for it;
3. compile() builds that file into its own shared library (cached under
   _lib/models by a digest of the source, the flags and the kernel
   headers), which exports the kernels' launcher table;
4. load() hands the library to siminf_gpu_model_load and registers the
   result under the model's name, so that every entry point finds it.

The generated library is compiled with the flags of the main library
(-fmad=false among them), so rates round as in the reference's C compiled
without contraction.  Expressions that call libm (exp, pow, log ...) use
CUDA's math library, whose results can differ from glibc's in the last
bit; trajectories of such models then agree with the host build in
distribution, not bit for bit.
"""
import hashlib
import os
import re
import subprocess
import threading

from . import build

HERE = os.path.dirname(os.path.abspath(__file__))
CACHE = os.path.join(HERE, "_lib", "models")

_lock = threading.Lock()

_TOKEN = re.compile(r"""
    (?P<comment>/\*.*?\*/|//[^\n]*)
  | (?P<pp>^[ \t]*\#(?:[^\n\\]|\\.)*(?:\\\n(?:[^\n\\]|\\.)*)*)
  | (?P<string>"(?:[^"\\\n]|\\.)*"|'(?:[^'\\\n]|\\.)*')
  | (?P<ident>[A-Za-z_][A-Za-z_0-9]*)
  | (?P<number>\.?[0-9](?:[eE][+-]|[A-Za-z0-9_.])*)
  | (?P<space>\s+)
  | (?P<punct>.)
""", re.S | re.M | re.X)

R_GLUE = {"SEXP", "DllInfo", "R_CallMethodDef", "R_registerRoutines", "R_GetCCallable"}
R_HEADERS = re.compile(r'#\s*include\s*[<"](R\.h|Rinternals\.h|Rmath\.h|R_ext/[^>"]*|'
                       r'SimInf\.h)[>"]')
INTEGRAL = {"int", "long", "short", "char", "unsigned", "signed", "size_t", "ptrdiff_t"}


class ModelCode:
    """The top-level items of a model C file (kind, text), and the names of
    its rate functions (in tr_fun order) and post-time-step function."""

    def __init__(self, items, tr_names, pts_name):
        self.items = items
        self.tr_names = tr_names
        self.pts_name = pts_name


def _tokens(code):
    for m in _TOKEN.finditer(code):
        yield m.lastgroup, m.group(), m.start(), m.end()


def parse_model_code(code):
    """Split C source into top-level items: ('pp', line), ('func', text)
    for function definitions, ('decl', text) for everything ending in ';'
    at file scope, each with its leading comments dropped."""
    items = []
    start = None
    depth = 0
    last = None                 # last significant token at depth 0
    brace_is_body = []
    for kind, text, s, e in _tokens(code):
        if kind in ("comment", "space"):
            continue
        if kind == "pp" and depth == 0 and start is None:
            items.append(("pp", text.strip()))
            continue
        if start is None:
            start = s
        if text in "([{" and kind == "punct":
            if text == "{" and depth == 0:
                brace_is_body.append(last == ")")
            depth += 1
        elif text in ")]}" and kind == "punct":
            depth -= 1
            if text == "}" and depth == 0 and brace_is_body and brace_is_body.pop():
                items.append(("func", code[start:e]))
                start, last = None, None
                continue
        elif text == ";" and depth == 0:
            items.append(("decl", code[start:e]))
            start, last = None, None
            continue
        if depth == 0:
            last = text
    if start is not None and code[start:].strip():
        raise ValueError("model code ends inside a declaration")
    tr_names, pts_name = None, None
    for kind, text in items:
        m = re.search(r"TRFun\s+\w+\s*\[\s*\]\s*=\s*\{([^}]*)\}", text)
        if m:
            tr_names = [t.strip().lstrip("&").strip() for t in m.group(1).split(",")
                        if t.strip()]
        m = re.search(r"SimInf_run\s*\(\s*\w+\s*,\s*\w+\s*,\s*\w+\s*,\s*&?\s*(\w+)\s*\)", text)
        if m:
            pts_name = m.group(1)
    if not tr_names or not pts_name:
        raise ValueError("model code without a run function that passes tr_fun and the "
                         "post-time-step function to SimInf_run")
    return ModelCode(items, tr_names, pts_name)


def _idents(text):
    return {t for k, t, _, _ in _tokens(text) if k == "ident"}


def _body_idents(code, name):
    for kind, text in code.items:
        if kind == "func" and re.search(r"\b%s\s*\(" % re.escape(name), text.split("{", 1)[0]):
            return _idents(text[text.index("{"):])
    raise ValueError("function %r is not defined in the model code" % name)


def device_source(c_code, Nc, Nt, Nd, Ngd, pts_local=None):
    """The .cu file of the device model (see the module docstring).
    pts_local: whether the post-time-step function reads only its own node;
    by default it does unless its body names `node` (the offset by which
    SimInf's spatial models reach their neighbours)."""
    code = parse_model_code(c_code)
    if len(code.tr_names) != Nt:
        raise ValueError("the model code has %d transition-rate functions, the model %d"
                         % (len(code.tr_names), Nt))
    if pts_local is None:
        pts_local = "node" not in _body_idents(code, code.pts_name)
    time_invariant = all("t" not in _body_idents(code, n) for n in code.tr_names)
    out = ["/* Device model compiled from model C code by siminf_gb300.devmodel. */",
           "#define SIMINF_MODEL_RUN siminf_model_run_unused",
           "#define SIMINF_R_INIT siminf_model_r_init_unused",
           "#define SIMINF_FORCE_SYMBOLS 0",
           '#include "siminf_model_code.h"', ""]
    for kind, text in code.items:
        if _idents(text) & R_GLUE:
            continue
        if kind == "pp":
            if not R_HEADERS.search(text):
                out.append(text)
            continue
        words = _idents(text)
        if kind == "func":
            out.append("__device__ " + text)
        elif text.lstrip().startswith(("typedef", "enum", "struct", "union")):
            out.append(text)
        elif "(" in text.split("=", 1)[0] or (words & {"const"} and words & INTEGRAL and
                                              "[" not in text):
            # prototypes become device prototypes; integral constants stay
            # host-side compile-time constants device code may use
            out.append(("__device__ " + text) if "(" in text.split("=", 1)[0] else text)
        else:
            out.append("__device__ " + text)
        out.append("")
    cases = "\n".join("        case %d: return ::%s(u, v, ldata, gdata, t);" % (k, n)
                      for k, n in enumerate(code.tr_names[:-1]))
    # The model struct has internal linkage: every model library then has
    # its own kernel and launcher instantiations, which would otherwise be
    # process-wide unique symbols shared by every model library loaded.
    out.append("""namespace {
struct ModelCompiled {
    static constexpr int NC = %(nc)d, NT = %(nt)d, ND = %(nd)d, NGD = %(ngd)d;
    static constexpr bool PTS_LOCAL = %(local)s;
    static constexpr bool RATES_TIME_INVARIANT = %(tinv)s;
    template <class DC>
    __device__ __forceinline__ static double rate(int k, const int *u, const double *v,
                                                  const double *ldata, const double *gdata,
                                                  double t, DC &)
    {
        switch (k) {
%(cases)s
        default: return ::%(last)s(u, v, ldata, gdata, t);
        }
    }
    __device__ __forceinline__ static int pts(double *v_new, const int *u, const double *v,
                                              const double *ldata, const double *gdata,
                                              int node, double t)
    {
        return ::%(pts)s(v_new, u, v, ldata, gdata, node, t);
    }
};
}  // namespace

extern "C" __attribute__((visibility("default"))) int siminf_model_abi(void)
{
    return SIMINF_MODEL_ABI;
}

extern "C" __attribute__((visibility("default"))) const siminf::Launchers *
siminf_model_launchers(void)
{
    return siminf::Launch<ModelCompiled>::table();
}
""" % {"nc": Nc, "nt": Nt, "nd": Nd, "ngd": Ngd, "local": "true" if pts_local else "false",
       "tinv": "true" if time_invariant else "false", "cases": cases,
       "last": code.tr_names[-1], "pts": code.pts_name})
    return "\n".join(out)


def _headers_digest():
    h = hashlib.sha256()
    for f in sorted(os.listdir(build.CSRC)):
        if f.endswith((".h", ".cuh")):
            with open(os.path.join(build.CSRC, f), "rb") as fh:
                h.update(f.encode() + fh.read())
    return h.hexdigest()


def compile(c_code, Nc, Nt, Nd, Ngd, pts_local=None, verbose=False):
    """Path of the device model library built from c_code (cached)."""
    src = device_source(c_code, Nc, Nt, Nd, Ngd, pts_local)
    flags = build.ARCH + build.NVFLAGS
    key = hashlib.sha256((src + "\0" + " ".join(flags) + "\0" +
                          _headers_digest()).encode()).hexdigest()[:32]
    lib = os.path.join(CACHE, "model_%s.so" % key)
    with _lock:
        if os.path.exists(lib):
            return lib
        os.makedirs(CACHE, exist_ok=True)
        cu = os.path.join(CACHE, "model_%s.cu" % key)
        with open(cu, "w") as f:
            f.write(src)
        tmp = lib + ".%d.tmp" % os.getpid()
        cmd = ([build.nvcc()] + flags + ["-Xcompiler", "-fvisibility=hidden", "-shared",
                                         "-I", build.CSRC, cu, "-o", tmp, "-lcudart"])
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc could not compile the model code:\n" + r.stderr[-4000:])
        os.replace(tmp, lib)
    return lib


def load(name, c_code, Nc, Nt, Nd, Ngd, pts_local=None):
    """Compile (or find in the cache) and load the device model, registered
    under `name` for every entry point; returns its native.DeviceModel."""
    from . import native
    path = compile(c_code, Nc, Nt, Nd, Ngd, pts_local)
    return native.load_device_model(name, path)
