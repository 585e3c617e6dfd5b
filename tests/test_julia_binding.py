"""The Julia bindings (vortexpanel.jl_gb300/julia/VortexPanelGPU.jl, no Julia needed): every ccall names an entry point
the header declares, with as many arguments as its prototype and a Julia type of the matching kind for each (handles,
scalars, pointers to doubles, ints, floats or bytes, the option and result structs); the Julia structs mirror the C
structs field for field; and every entry of the header that a Julia caller of the hot path needs has a binding."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
JL = os.path.join(ROOT, "vortexpanel.jl_gb300", "julia", "VortexPanelGPU.jl")
HDR = os.path.join(ROOT, "include", "vortexpanel_gpu.h")


def _header():
    src = open(HDR).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    protos = {}
    for ret, name, params in re.findall(r"\b(int|void|const char\*)\s+(vp_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", src, flags=re.S):
        ps = [p.strip() for p in params.replace("\n", " ").split(",") if p.strip() and p.strip() != "void"]
        protos[name] = (ret, [re.sub(r"\s+\w+$", "", p).replace("const ", "").replace(" ", "") for p in ps])
    structs = {}
    for body, name in re.findall(r"typedef struct \{(.*?)\}\s*(vp_[a-z_]+)\s*;", src, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = decl.strip()
            if not decl:
                continue
            m = re.match(r"(.*?[\s*])(\w+(?:\[\d+\])?(?:\s*,\s*\w+(?:\[\d+\])?)*)$", decl, flags=re.S)
            typ = m.group(1).replace("const", "").replace(" ", "").replace("\n", "")
            for f in m.group(2).split(","):
                f = f.strip()
                arr = re.match(r"(\w+)\[(\d+)\]", f)
                fields.append((arr.group(1) if arr else f, typ, int(arr.group(2)) if arr else 0))
        structs[name] = fields
    return protos, structs


def _split_top(s):
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def _ccalls():
    src = open(JL).read()
    calls = []
    for m in re.finditer(r"ccall\(\(:(vp_[a-z0-9_]+), LIB\),\s*(\w+),\s*\(", src):
        i, depth = m.end(), 1
        while depth:
            depth += {"(": 1, ")": -1}.get(src[i], 0)
            i += 1
        calls.append((m.group(1), m.group(2), _split_top(src[m.end():i - 1])))
    return calls


# the Julia types a C parameter type may take
KINDS = {
    "int": {"Cint"}, "double": {"Cdouble"}, "double*": {"Ptr{Cdouble}", "Ref{Cdouble}"},
    "int*": {"Ptr{Cint}", "Ref{Cint}"}, "float*": {"Ptr{Cfloat}"}, "signedchar*": {"Ptr{Int8}"},
    "longlong*": {"Ptr{Clonglong}", "Ref{Clonglong}"}, "vp_ctx*": {"Ptr{Cvoid}"}, "vp_system*": {"Ptr{Cvoid}"},
    "vp_factor*": {"Ptr{Cvoid}"}, "vp_freewake*": {"Ptr{Cvoid}"}, "vp_ctx**": {"Ref{Ptr{Cvoid}}"},
    "vp_system**": {"Ref{Ptr{Cvoid}}"}, "vp_factor**": {"Ref{Ptr{Cvoid}}"}, "vp_freewake**": {"Ref{Ptr{Cvoid}}"},
    "vp_assembly_options*": {"Ref{VpOptions}"}, "vp_assembly_stats*": {"Ref{VpStats}", "Ptr{VpStats}"},
    "vp_freewake_setup*": {"Ref{VpFreeWakeSetup}"}, "vp_freewake_record*": {"Ref{VpFreeWakeRecord}"},
    "vp_freewake_counts*": {"Ref{VpFreeWakeCounts}"}, "vp_assembly_input*": {"Ptr{VpInput}"},
    "vp_system**": {"Ref{Ptr{Cvoid}}", "Ptr{Ptr{Cvoid}}"},
}
RET = {"int": "Cint", "void": "Cvoid", "constchar*": "Cstring", "const char*": "Cstring"}


def test_every_ccall_matches_the_header():
    protos, _ = _header()
    calls = _ccalls()
    assert len(calls) >= 20
    for name, ret, types in calls:
        assert name in protos, name
        cret, params = protos[name]
        assert RET[cret.replace(" ", "")] == ret, (name, ret, cret)
        assert len(types) == len(params), (name, len(types), len(params))
        for t, p in zip(types, params):
            assert t in KINDS[p], (name, p, t)


def test_bindings_cover_the_hot_path():
    names = {c[0] for c in _ccalls()}
    need = {"vp_ctx_create", "vp_ctx_destroy", "vp_last_error", "vp_assemble", "vp_system_download",
            "vp_system_download_rows", "vp_system_free", "vp_factorize", "vp_solve", "vp_solve_system",
            "vp_solve_transposed", "vp_adjoint", "vp_consistency", "vp_surface_loads", "vp_pressure_force",
            "vp_wake_loads", "vp_factor_free", "vp_freewake_create", "vp_freewake_step", "vp_freewake_get_state",
            "vp_freewake_info", "vp_freewake_free"}
    assert need <= names, sorted(need - names)


JL_TYPES = {"int": "Cint", "double": "Cdouble", "longlong": "Clonglong", "double*": "Ptr{Cdouble}",
            "int*": "Ptr{Cint}", "vp_factor*": "Ptr{Cvoid}", "vp_assembly_options": "VpOptions"}


def test_structs_mirror_the_header():
    _, structs = _header()
    src = open(JL).read()
    for cname, jname in (("vp_assembly_options", "VpOptions"), ("vp_assembly_stats", "VpStats"),
                         ("vp_freewake_setup", "VpFreeWakeSetup"), ("vp_freewake_record", "VpFreeWakeRecord"),
                         ("vp_freewake_counts", "VpFreeWakeCounts")):
        body = re.search(r"struct %s\n(.*?)\nend" % jname, src, flags=re.S).group(1)
        jf = [re.match(r"\s*(\S+)::(.+)", ln).groups() for ln in body.splitlines() if "::" in ln]
        cf = structs[cname]
        assert len(jf) == len(cf), (jname, len(jf), len(cf))
        for (jn, jt), (cn, ct, arr) in zip(jf, cf):
            want = JL_TYPES.get(ct, ct)
            if arr:
                want = f"NTuple{{{arr},{want}}}"
            assert jt.strip() == want, (jname, jn, jt, cn, ct)
