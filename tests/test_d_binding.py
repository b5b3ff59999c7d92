"""The D binding (dlbc_gb300/d/lbgpu.d) and the Python ctypes structs
(dlbc_gb300/lbgpu.py) against the C header they mirror.

There is no D compiler here, so the binding is checked as text: the same
functions with the same parameter and return types, the same constants, and
struct layouts that C's rules give identically for both (offsets and sizes
of the C structs taken from gcc, the D fields laid out with C alignment, as
extern(C) D structs are).
"""
import ctypes
import os
import re
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "lbgpu.h")
DFILE = os.path.join(ROOT, "dlbc_gb300", "d", "lbgpu.d")

C_BASE = {"int32_t": "int", "int": "int", "int64_t": "long", "uint64_t": "ulong", "uint8_t": "ubyte",
          "char": "char", "double": "double", "void": "void", "size_t": "size_t"}
D_SIZE = {"int": 4, "double": 8, "ulong": 8, "long": 8}


def _strip_comments(text):
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    return re.sub(r"//[^\n]*", " ", text)


def _kind(decl, lang):
    """(base type, pointer depth) of a parameter or return type."""
    t = re.sub(r"\bconst\b", " ", decl.replace("(", " ").replace(")", " "))
    depth = t.count("*")
    words = [w for w in re.findall(r"[A-Za-z_]\w*", t)]
    base = words[0] if words else ""
    if lang == "c":
        base = C_BASE.get(base, base)
    return base, depth


def _functions(text, lang):
    out = {}
    for ret, name, args in re.findall(r"([A-Za-z_][\w\s\*\(\)]*?)\b(lbgpu_\w+)\s*\(([^;{]*?)\)\s*;", text):
        ret = ret.split(";")[-1].split("}")[-1].strip().split("\n")[-1]
        params = [a.strip() for a in args.split(",") if a.strip() and a.strip() != "void"]
        kinds = []
        for a in params:
            a = re.sub(r"\s*\b\w+\s*$", "", a) if re.search(r"[\w\)\*]\s+\w+\s*$", a) else a
            kinds.append(_kind(a, lang))
        out[name] = (_kind(ret, lang), kinds)
    return out


def _c_constants(text):
    return {k: int(v) for k, v in re.findall(r"#define\s+(LBGPU_\w+)\s+\(?(-?\d+)\)?", text)}


def _d_constants(text):
    return {k: int(v) for k, v in re.findall(r"enum\s+int\s+(LBGPU_\w+)\s*=\s*(-?\d+)\s*;", text)}


def _d_struct(text, name, consts):
    body = re.search(r"struct\s+" + name + r"\s*\{(.*?)\}", text, flags=re.S).group(1)
    fields = []
    for line in body.split(";"):
        line = line.strip()
        if not line:
            continue
        m = re.match(r"(\w+)((?:\[\w+\])*)\s+(.+)$", line)
        base, dims, names = m.group(1), m.group(2), m.group(3)
        count = 1
        for dim in re.findall(r"\[(\w+)\]", dims):
            count *= int(consts.get(dim, dim))
        for n in names.split(","):
            fields.append((n.strip(), base, count))
    # C layout rules: each field at a multiple of its alignment, the struct
    # padded to its largest alignment
    off, layout, align_max = 0, {}, 1
    for n, base, count in fields:
        size = D_SIZE[base]
        off = (off + size - 1) // size * size
        layout[n] = (off, size * count)
        off += size * count
        align_max = max(align_max, size)
    return layout, (off + align_max - 1) // align_max * align_max


def _c_layout(struct, fields):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    src = ["#include <stddef.h>", "#include <stdio.h>", f'#include "{HEADER}"', "int main(void) {"]
    for f in fields:
        src.append(f'  printf("{f} %zu %zu\\n", offsetof({struct}, {f}), sizeof((({struct}*)0)->{f}));')
    src.append(f'  printf("__size__ %zu 0\\n", sizeof({struct}));')
    src.append("  return 0; }")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "layout.c")
        exe = os.path.join(d, "layout")
        with open(c, "w") as fh:
            fh.write("\n".join(src) + "\n")
        subprocess.run([gcc, "-std=c99", "-o", exe, c], check=True, capture_output=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    res = {}
    for line in out.split("\n"):
        if line.strip():
            n, o, s = line.split()
            res[n] = (int(o), int(s))
    return res


def test_same_functions_with_the_same_types():
    c = _functions(_strip_comments(open(HEADER).read()), "c")
    d = _functions(_strip_comments(open(DFILE).read()), "d")
    assert set(c) == set(d), (sorted(set(c) - set(d)), sorted(set(d) - set(c)))
    for name in c:
        assert c[name] == d[name], (name, c[name], d[name])
    assert "lbgpu_step_host" in c and len(c) >= 30


def test_same_constants():
    c = _c_constants(_strip_comments(open(HEADER).read()))
    d = _d_constants(open(DFILE).read())
    assert c == d


@pytest.mark.parametrize("struct", ["lbgpu_config", "lbgpu_init"])
def test_struct_layouts_match(struct):
    dtext = _strip_comments(open(DFILE).read())
    consts = _d_constants(open(DFILE).read())
    d_layout, d_size = _d_struct(dtext, struct, consts)
    c_layout = _c_layout(struct, list(d_layout))
    assert c_layout.pop("__size__")[0] == d_size
    assert c_layout == d_layout


@pytest.mark.parametrize("struct,cls", [("lbgpu_config", "LbgpuConfig"), ("lbgpu_init", "LbgpuInit")])
def test_python_struct_layouts_match(struct, cls):
    """The ctypes mirrors in dlbc_gb300/lbgpu.py against the C header."""
    from dlbc_gb300 import lbgpu

    ct = getattr(lbgpu, cls)
    names = [f[0] for f in ct._fields_]
    c_layout = _c_layout(struct, names)
    assert c_layout.pop("__size__")[0] == ctypes.sizeof(ct)
    py = {n: (getattr(ct, n).offset, getattr(ct, n).size) for n in names}
    assert py == c_layout
