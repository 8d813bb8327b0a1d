"""The Mojo host layer's FFI aliases against the C header (no Mojo toolchain here).

ish_gb300/mojo/ish_gpu.mojo binds every entry point of include/ish_gpu.h with an
`alias ish_gpu_<name>_fn = fn (...) -> ...` and looks it up by name with
`get_function[...]("ish_gpu_<name>")`.  A wrong type or arity there would pass
arguments in the wrong registers, so this test parses both files and requires,
for every C prototype, an alias with the same arity and the Mojo spelling of
each C type, and that every lookup names the symbol its alias describes.
"""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ish_gpu.h")
MOJO_DIR = os.path.join(ROOT, "ish_gb300", "mojo")

SCALARS = {"int": "Int32", "int32_t": "Int32", "uint32_t": "UInt32", "int64_t": "Int64", "uint64_t": "UInt64",
           "size_t": "UInt64", "float": "Float32", "double": "Float64", "uint8_t": "UInt8", "int8_t": "Int8",
           "char": "Int8"}


def c_prototypes():
    s = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"ISH_API\s+([^;]*?)\s*\(([^)]*)\)\s*;", s, flags=re.S):
        head = " ".join(m.group(1).split())
        name = re.search(r"(\w+)$", head).group(1)
        ret = head[: -len(name)].strip()
        params = " ".join(m.group(2).split())
        out[name] = (ret, [] if params == "void" else [p.strip() for p in params.split(",")])
    return out


def c_to_mojo(decl, is_return=False):
    """Mojo spelling of a C parameter declaration (name stripped) or return type."""
    d = decl.replace("const ", "").strip()
    if not is_return:
        d = re.sub(r"\s*\b\w+$", "", d) if not d.endswith("*") else d  # drop the parameter name
    stars = d.count("*")
    base = d.replace("*", "").strip()
    if base == "void" and stars == 0:
        return "None"
    if base in ("ish_ctx", "void"):
        return "OpaquePointer" if stars == 1 else "UnsafePointer[OpaquePointer]"
    t = SCALARS[base]
    for _ in range(stars):
        t = f"UnsafePointer[{t}]"
    return t


def mojo_aliases():
    s = open(os.path.join(MOJO_DIR, "ish_gpu.mojo")).read()
    out = {}
    for m in re.finditer(r"alias\s+(ish_gpu_\w+)_fn\s*=\s*fn\s*\((.*?)\)\s*->\s*([\w\[\]]+)", s, flags=re.S):
        params = [p.strip() for p in m.group(2).replace("\n", " ").split(",") if p.strip()]
        out[m.group(1)] = (m.group(3), params)
    return out


def test_every_c_entry_point_has_a_matching_mojo_alias():
    protos = c_prototypes()
    aliases = mojo_aliases()
    assert len(protos) >= 25
    assert set(protos) == set(aliases), (sorted(set(protos) ^ set(aliases)))
    for name, (ret, params) in protos.items():
        mret, mparams = aliases[name]
        assert mret == c_to_mojo(ret, is_return=True), f"{name}: return {ret!r} bound as {mret}"
        want = [c_to_mojo(p) for p in params]
        assert len(mparams) == len(want), f"{name}: {len(params)} C parameters, {len(mparams)} in the alias"
        for i, (w, g) in enumerate(zip(want, mparams)):
            assert w == g, f"{name} parameter {i} ({params[i]!r}): expected {w}, alias has {g}"


def test_lookups_name_the_symbol_of_their_alias():
    protos = c_prototypes()
    seen = 0
    for fn in sorted(os.listdir(MOJO_DIR)):
        if not fn.endswith(".mojo"):
            continue
        s = open(os.path.join(MOJO_DIR, fn)).read()
        for m in re.finditer(r"get_function\[\s*(ish_gpu_\w+)_fn\s*\]\(\s*\"(\w+)\"", s):
            assert m.group(1) == m.group(2), f"{fn}: alias {m.group(1)}_fn looked up as {m.group(2)!r}"
            assert m.group(2) in protos, f"{fn}: {m.group(2)} is not declared in include/ish_gpu.h"
            seen += 1
    assert seen >= 10


def test_drop_in_covers_the_reference_gpu_path_calls():
    """The replacement of gpu/process_batch.parallel_starts_ends goes through
    set_query, records_load, score_set and match_starts, raises on a nonzero
    status, and routes striped-local as well as semi-global."""
    s = open(os.path.join(MOJO_DIR, "gpu_process_batch.mojo")).read()
    for call in ("gpu.set_query(", "gpu.records_load(", "gpu.score_set(", "gpu.match_starts(", "gpu.records_free(",
                 "gpu.free_query("):
        assert call in s, call
    assert "fn parallel_starts_ends[" in s and "ISH_ALGO_LOCAL if local" in s
    b = open(os.path.join(MOJO_DIR, "ish_gpu.mojo")).read()
    assert "fn check(self, rc: Int32" in b and "raise Error(" in b
