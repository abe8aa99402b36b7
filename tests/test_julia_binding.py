"""The Julia binding (hydrograd.jl_gb300/julia/HydrogradGB.jl) against the C ABI.

Julia is not installed here, so the binding is checked as text: every ccall
names an entry point that include/hydrograd_gb.h declares, with as many
argument types as the declaration has parameters and as many arguments as
types; and the binding covers the entry points the reference's call sites
need (the RHS, the time loops, the gradients)."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
JL = os.path.join(ROOT, "hydrograd.jl_gb300", "julia", "HydrogradGB.jl")
HEADER = os.path.join(ROOT, "include", "hydrograd_gb.h")


def header_arity():
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for name, params in re.findall(r"\bint\s+(hg_\w+)\s*\(([^)]*)\)\s*;", text):
        p = params.strip()
        out[name] = 0 if p in ("", "void") else p.count(",") + 1
    return out


def split_top(s):
    """Top-level comma-separated items of s (nesting by (), {} and [])."""
    items, depth, cur = [], 0, ""
    for ch in s:
        if ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
        if ch == "," and depth == 0:
            items.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        items.append(cur.strip())
    return items


def matching(s, i):
    """Index of the bracket closing the one at s[i]."""
    depth = 0
    for j in range(i, len(s)):
        if s[j] in "({[":
            depth += 1
        elif s[j] in ")}]":
            depth -= 1
            if depth == 0:
                return j
    raise ValueError("unbalanced")


def julia_ccalls():
    src = re.sub(r"#.*", "", open(JL).read())
    calls = []
    for m in re.finditer(r"ccall\(\(:(hg_\w+), lib\)", src):
        end = matching(src, m.start() + len("ccall"))
        body = split_top(src[m.start() + len("ccall("):end])
        # body: (:name, lib), Cint, (types...), args...
        assert body[1] == "Cint", (m.group(1), body[1])
        types = split_top(body[2][1:-1])
        calls.append((m.group(1), types, body[3:]))
    return calls


def test_every_ccall_matches_the_header():
    arity = header_arity()
    calls = julia_ccalls()
    assert len(calls) >= 15
    for name, types, args in calls:
        assert name in arity, name
        assert len(types) == arity[name], (name, len(types), arity[name])
        assert len(args) == len(types), (name, len(args), len(types))


def test_binding_covers_the_reference_call_sites():
    names = {c[0] for c in julia_ccalls()}
    for need in ("hg_create", "hg_destroy", "hg_rhs", "hg_integrate", "hg_integrate_tsit5", "hg_loss_and_grad",
                 "hg_final_loss_and_grad", "hg_final_vjp", "hg_set_manning_zones", "hg_set_zb_cells",
                 "hg_set_inlet_q", "hg_last_error"):
        assert need in names, need


def test_rrules_are_defined_for_both_losses():
    src = open(JL).read()
    assert re.search(r"function ChainRulesCore\.rrule\(::typeof\(probe_loss\)", src)
    assert re.search(r"function ChainRulesCore\.rrule\(::typeof\(final_loss\)", src)
    # raw pointers taken from temporaries only inside GC.@preserve blocks of named arrays
    assert "pointer(Int32." not in src
