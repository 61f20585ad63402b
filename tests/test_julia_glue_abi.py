"""The Julia glue's ccalls against the C ABI (no Julia toolchain is needed).

itensorsgpu.jl_gb300/julia/ITGBackend.jl is the drop-in for the reference's
storage layer; it cannot run here, so this test checks it mechanically: every
`ccall((:itg_..., libitg), Ret, (ArgTypes...), args...)` must name a function
include/itg.h declares, with the same number of arguments, each of a matching
C type (Cint <-> int, Int64 <-> int64_t, Cdouble <-> double, Csize_t <->
size_t, UInt64 <-> uint64_t, Ptr / CuPtr / Ref <-> any pointer), the same
return type, and exactly as many argument values as argument types.  It also
checks that the glue defines a method for every storage-level function the
reference overloads on this path (src/ITensorsGPU.jl:32-43 import list).
"""
import re
from pathlib import Path

REPO = Path(__file__).resolve().parent.parent
HEADER = REPO / "include" / "itg.h"
GLUE = REPO / "itensorsgpu.jl_gb300" / "julia" / "ITGBackend.jl"


def _c_kind(t: str) -> str:
    t = " ".join(t.replace("const", " ").split())
    if "*" in t:
        return "ptr"
    return {"int": "int32", "int64_t": "int64", "double": "double", "size_t": "size_t",
            "uint64_t": "uint64", "float": "float", "void": "void"}[t]


def header_decls():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    out = {}
    for m in re.finditer(r"ITG_API\s+((?:const\s+)?\w+\s*\**)\s*(itg_\w+)\s*\(([^)]*)\)\s*;", text):
        ret, name, args = m.group(1), m.group(2), m.group(3)
        ret_kind = "cstr" if "char" in ret else _c_kind(ret)
        kinds = []
        for a in args.split(","):
            a = a.strip()
            if not a or a == "void":
                continue
            # drop the parameter name: the last identifier not part of the type
            a = re.sub(r"\b\w+\s*$", "", a).strip() if not a.endswith("*") else a
            kinds.append(_c_kind(a))
        out[name] = (ret_kind, kinds)
    return out


def _split_top(s: str):
    """Split at commas that are not inside (), {} or []."""
    parts, depth, cur = [], 0, []
    for ch in s:
        if ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append("".join(cur).strip())
            cur = []
        else:
            cur.append(ch)
    if "".join(cur).strip():
        parts.append("".join(cur).strip())
    return parts


def _matching(s: str, i: int) -> int:
    """Index of the parenthesis closing the one at s[i]."""
    depth = 0
    for j in range(i, len(s)):
        if s[j] == "(":
            depth += 1
        elif s[j] == ")":
            depth -= 1
            if depth == 0:
                return j
    raise ValueError("unbalanced parentheses")


def _jl_kind(t: str) -> str:
    t = t.strip()
    if re.match(r"^(Ptr|CuPtr|Ref)\{", t):
        return "ptr"
    return {"Cint": "int32", "Int64": "int64", "Cdouble": "double", "Csize_t": "size_t", "UInt64": "uint64",
            "Cfloat": "float", "Cstring": "cstr", "Cvoid": "void"}[t]


def glue_ccalls():
    text = GLUE.read_text()
    text = "\n".join(line.split("#", 1)[0] for line in text.splitlines())
    calls = []
    for m in re.finditer(r"ccall\(", text):
        close = _matching(text, m.end() - 1)
        parts = _split_top(text[m.end():close])
        names = re.findall(r":(itg_\w+)", parts[0])
        assert parts[0].startswith("(") and "libitg" in parts[0], parts[0]
        ret = _jl_kind(parts[1])
        types = parts[2].strip()
        assert types.startswith("(") and types.endswith(")"), types
        tkinds = [_jl_kind(x) for x in _split_top(types[1:-1])]
        calls.append((names, ret, tkinds, len(parts) - 3))
    return calls


def test_every_glue_ccall_matches_the_header():
    decls = header_decls()
    calls = glue_ccalls()
    assert len(calls) >= 18
    seen = set()
    for names, ret, tkinds, nargs in calls:
        assert names, "ccall without an itg_ symbol"
        assert nargs == len(tkinds), (names, nargs, len(tkinds))
        for name in names:
            assert name in decls, f"{name} is not declared in include/itg.h"
            cret, ckinds = decls[name]
            assert ret == cret, (name, ret, cret)
            assert tkinds == ckinds, (name, tkinds, ckinds)
            seen.add(name)
    for must in ("itg_contract_z", "itg_permute", "itg_axpby_permuted", "itg_diag_contract", "itg_diag_diag",
                 "itg_diag_to_dense", "itg_truncate", "itg_svd_trunc", "itg_qr", "itg_eigh_trunc",
                 "itg_factorize_trunc", "itg_davidson_heff2"):
        assert must in seen, must


def test_header_parser_sees_every_declaration():
    decls = header_decls()
    text = HEADER.read_text()
    assert len(decls) == len(set(re.findall(r"ITG_API\s+[^;(]*?(itg_\w+)\s*\(", text)))
    assert decls["itg_contract"] == ("int32", ["ptr", "int32", "double", "ptr", "int32", "ptr", "ptr", "ptr",
                                               "int32", "ptr", "ptr", "double", "ptr", "int32", "ptr", "ptr",
                                               "int32"])
    assert decls["itg_last_error"] == ("cstr", ["ptr"])


def test_glue_defines_the_reference_storage_methods():
    text = GLUE.read_text()
    # storage types and converters (src/tensor/cudense.jl:1-20, src/tensor/cudiag.jl:1-4)
    for pat in (r"const CuDense\{", r"const CuDenseTensor\{", r"const CuDiag\{", r"const NonuniformCuDiagTensor\{",
                r"Dense\{T,SA\}\(x::Dense\{T,SB\}\) where \{T<:Number,SA<:CuArray", r"cpu\(x::CuDense"):
        assert re.search(pat, text), pat
    # methods the reference adds for CuDense / CuDiag storage
    for fn in ("contract!!", "outer!", "_contract_scalar!", "Base.permute!", "permutedims!!", "Base.:+",
               "Base.:-", "contract!", "dense", "truncate!", "LinearAlgebra.svd", "LinearAlgebra.qr",
               "LinearAlgebra.eigen", "contraction_output_type", "zero_contraction_output"):
        assert re.search(r"(^|\n)(function )?" + re.escape(fn) + r"\(", text), fn
    # the dmrg two-site update routed to the library
    assert "function KrylovKit.eigsolve(PH::ProjMPO" in text
    assert "function replacebond!(M::MPS" in text
