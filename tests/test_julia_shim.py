"""The Julia drop-in (julia/SSEGB300.jl) checked statically, since Julia is
not installed here or on the GPU machine: each C struct mirror has the header's
fields in the header's order with matching types, its C layout size equals
the library's own sizeof (sse_struct_sizes), and every ccall names a
function the header declares, with that function's number of arguments."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "sse_gb300.h")
SHIM = os.path.join(ROOT, "julia", "SSEGB300.jl")

# C struct name -> Julia mirror, in the order sse_struct_sizes reports them
STRUCTS = [("sse_config", "SseConfig"), ("sse_csc", "SseCsc"), ("sse_operators", "SseOperators"),
           ("sse_geometry", "SseGeometry"), ("sse_metric_operators", "SseMetricOperators"),
           ("sse_geometric_factors_out", "SseGeometricFactorsOut")]
SCALARS = {"int32_t": "Int32", "int64_t": "Int64", "double": "Float64"}
SIZE = {"Int32": 4, "Int64": 8, "Float64": 8}


def strip_c(text):
    return re.sub(r"/\*.*?\*/", "", text, flags=re.S)


def c_structs():
    text = strip_c(open(HEADER).read())
    out = {}
    for name, body in re.findall(r"typedef struct (sse_\w+) \{(.*?)\}\s*\1;", text, re.S):
        fields = []
        for decl in body.split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            m = re.match(r"(const )?(\w+)\s*(.*)", decl)
            base = m.group(2)
            for item in m.group(3).split(","):
                item = item.strip()
                stars = item.count("*")
                arr = re.search(r"\[(\d+)\]", item)
                fname = re.sub(r"\[\d+\]|[\*\s]|const", "", item)
                t = SCALARS.get(base, "Sse" + "".join(w.title() for w in base.split("_")[1:]))
                for _ in range(stars):
                    t = f"Ptr{{{t}}}"
                if arr:
                    t = f"NTuple{{{arr.group(1)}, {t}}}"
                fields.append((fname, t))
        out[name] = fields
    return out


def julia_structs():
    text = open(SHIM).read()
    out = {}
    for name, body in re.findall(r"^struct (\w+)\n(.*?)^end", text, re.S | re.M):
        out[name] = [(f, " ".join(t.split())) for f, t in re.findall(r"^\s+(\w+)::(.+)$", body, re.M)]
    return out


def c_layout(t, js):
    """(size, alignment) of a Julia field type under the C rules."""
    if t.startswith("Ptr{"):
        return 8, 8
    m = re.match(r"NTuple\{(\d+), (.+)\}$", t)
    if m:
        s, a = c_layout(m.group(2), js)
        return int(m.group(1)) * s, a
    if t in SIZE:
        return SIZE[t], SIZE[t]
    return struct_size(js[t], js)


def struct_size(fields, js):
    off, align = 0, 1
    for _, t in fields:
        s, a = c_layout(t, js)
        off = (off + a - 1) // a * a + s
        align = max(align, a)
    return (off + align - 1) // align * align, align


def test_struct_mirrors_match_the_header():
    cs, js = c_structs(), julia_structs()
    for cname, jname in STRUCTS:
        assert jname in js, jname
        assert js[jname] == cs[cname], (jname, js[jname], cs[cname])


def test_struct_sizes_match_the_library(pkg):
    pkg.build.build()
    lib = pkg.load_library()
    sizes = (C.c_int32 * 6)()
    assert lib.sse_struct_sizes(sizes) == 6
    js = julia_structs()
    assert [struct_size(js[j], js)[0] for _, j in STRUCTS] == list(sizes)


def c_arity():
    text = strip_c(open(HEADER).read())
    out = {}
    for name, args in re.findall(r"\b(sse_\w+)\s*\(([^;{]*?)\)\s*;", text, re.S):
        args = args.strip()
        out[name] = 0 if args in ("", "void") else args.count(",") + 1
    return out


def ccalls(text):
    """(function name, argument-type tuple text) of every ccall in the shim."""
    out = []
    for m in re.finditer(r"ccall\(\(:(sse_\w+), libsse\), \w+,\s*\(", text):
        depth, i = 1, m.end()
        while depth:
            depth += {"(": 1, ")": -1}.get(text[i], 0)
            i += 1
        out.append((m.group(1), text[m.end():i - 1]))
    return out


def test_every_ccall_matches_a_declared_function():
    text = open(SHIM).read()
    calls = ccalls(text)
    assert len(calls) >= 8
    arity = c_arity()
    for name, argtypes in calls:
        assert name in arity, name
        # top-level commas only (Ptr{Ptr{Cvoid}} has none, Ref{SseConfig} none)
        n = 0 if not argtypes.strip() else len([a for a in re.split(r",(?![^{]*\})", argtypes) if a.strip()])
        assert n == arity[name], (name, n, arity[name])


def test_dispatch_seam_and_rrule_are_defined():
    text = open(SHIM).read()
    assert re.search(r"struct GB300 <: AbstractParallelism", text)
    assert re.search(r"function semi_discrete_residual!\(dudt::AbstractArray\{Float64, 3\},", text)
    assert "GB300}" in text and "parallelism::GB300" in text
    assert "function ChainRulesCore.rrule(::typeof(gb300_solve)" in text
