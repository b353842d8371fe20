"""The LuaJIT binding (lua/hydrocuda_ffi.lua) against the C header: every
function it declares has the header's signature, its structs the header's
fields, and its name tables the indices the Python binding uses (CPU; LuaJIT
itself is not available to run it)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LUA = os.path.join(ROOT, "hydro-cl-lua_gb300", "lua", "hydrocuda_ffi.lua")
HEADER = os.path.join(ROOT, "include", "hydrocuda.h")


def _norm(decl):
    decl = re.sub(r"/\*.*?\*/", "", decl, flags=re.S)
    return re.sub(r"\s+", " ", decl).replace(" *", "*").replace("( ", "(").replace(" )", ")").strip()


def _cdef():
    text = open(LUA).read()
    return re.search(r"ffi\.cdef\[\[(.*?)\]\]", text, flags=re.S).group(1)


def _header():
    return re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)


def _functions(text):
    return {m.group(2): _norm(m.group(0)) for m in re.finditer(r"^\s*([\w\s\*]+?)\b(hc_\w+)\s*\(([^;]*)\);", text, flags=re.M)}


def _struct_fields(text, name):
    m = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), text, flags=re.S)
    assert m, name
    fields = []
    for line in m.group(1).split(";"):
        line = _norm(line)
        if not line:
            continue
        typ, rest = re.match(r"((?:unsigned long long|long long|unsigned|const char\*|\w+)\s*\**)\s*(.*)", line).groups()
        for f in rest.split(","):
            fields.append((_norm(typ), _norm(f)))
    return fields


def test_declared_functions_match_the_header():
    lua, hdr = _functions(_cdef()), _functions(_header())
    assert len(lua) >= 20
    for name, decl in lua.items():
        assert name in hdr, name
        assert decl == hdr[name], (decl, hdr[name])


@pytest.mark.parametrize("name", ["hc_solver_desc", "hc_render", "hc_init", "hc_batch_desc", "hc_done"])
def test_structs_match_the_header(name):
    assert _struct_fields(_cdef(), name) == _struct_fields(_header(), name)


def test_name_tables_match_the_python_binding():
    import hydrocuda
    text = open(LUA).read()

    def table(var):
        body = re.search(r"M\.%s = \{(.*?)\}" % var, text, flags=re.S).group(1)
        return {k.strip("'[]\" "): int(v) for k, v in re.findall(r"(\[?'?[\w\- ]+'?\]?|\w+)\s*=\s*(\d+)", body)}

    assert table("boundaryIndex") == hydrocuda.BOUNDARIES
    assert table("fluxIndex") == {k: i for i, k in enumerate(hydrocuda.FLUXES)}
    assert table("reconIndex") == {k: v for k, v in hydrocuda.RECONS.items() if isinstance(k, str)}
    assert table("renderMode") == hydrocuda.RENDER_MODES


def _lua_sources():
    base = os.path.join(ROOT, "hydro-cl-lua_gb300", "lua")
    out = []
    for d, _, files in os.walk(base):
        out += [os.path.join(d, f) for f in files if f.endswith(".lua")]
    return out


def test_every_library_call_is_declared():
    """Each hc_* entry point the Lua files call through the ffi library is
    declared by the binding's cdef (LuaJIT raises on an undeclared symbol only
    when the call runs) and exported by the header."""
    declared = set(_functions(_cdef()))
    exported = set(_functions(_header()))
    used = set()
    for path in _lua_sources():
        used |= set(re.findall(r"\blib\.(hc_\w+)", open(path).read()))
    assert len(used) >= 15
    assert used <= declared, sorted(used - declared)
    assert used <= exported, sorted(used - exported)


def test_every_ffi_struct_used_is_declared():
    """The structs the Lua files create with ffi.new are declared by a cdef."""
    cdefs = ""
    for path in _lua_sources():
        for m in re.finditer(r"ffi\.cdef\[\[(.*?)\]\]", open(path).read(), flags=re.S):
            cdefs += m.group(1)
    declared = set(re.findall(r"typedef struct (\w+)", cdefs)) | {"int", "double", "char", "float"}
    seen = 0
    for path in _lua_sources():
        for name in re.findall(r"ffi\.new\s*\(?\s*'(\w+)", open(path).read()):
            assert name in declared, (path, name)
            seen += 1
    assert seen >= 10
