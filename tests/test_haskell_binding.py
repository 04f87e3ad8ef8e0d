"""The Haskell marshalling module (bling_gb300/haskell/.../GpuScene.hsc) and
the Python ctypes mirror (bling_gb300/abi.py) against the C header.

The .hsc takes every offset and size from include/bling_gpu.h through
hsc2hs directives.  There is no GHC here, so this test does what hsc2hs
does: it compiles a C program against the header that evaluates every
`#{peek/poke/ptr T, f}`, `#{size T}` and `#{const X}` the module uses (a
field that does not exist fails to compile), and checks that each record
the module writes pokes every field the header declares for it.  The same
offsets must be what the ctypes structures of abi.py give."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

from bling_gb300 import abi

ROOT = Path(__file__).resolve().parent.parent
HSC = ROOT / "bling_gb300" / "haskell" / "Graphics" / "Bling" / "IO" / "GpuScene.hsc"
HEADER = ROOT / "include" / "bling_gpu.h"

# the C structs the module writes as whole records, and their ctypes mirrors
WRITTEN = {"bling_material": abi.Material, "bling_mesh_desc": abi.MeshDesc,
           "bling_shape_desc": abi.ShapeDesc, "bling_light_desc": abi.LightDesc,
           "bling_camera_desc": abi.CameraDesc, "bling_scene_desc": abi.SceneDesc,
           "bling_render_params": abi.RenderParams, "bling_texture": abi.Texture}


def hsc_directives():
    src = HSC.read_text()
    fields = set(re.findall(r"#\{(?:peek|poke|ptr) (\w+), (\w+)\}", src))
    pokes = set(re.findall(r"#\{(?:poke|ptr) (\w+), (\w+)\}", src))
    sizes = set(re.findall(r"#\{(?:size|alignment) (\w+)\}", src))
    consts = set(re.findall(r"#\{const (\w+)\}", src))
    return fields, pokes, sizes, consts


def header_fields(struct):
    """field names of `typedef struct struct { ... } struct;` in the header"""
    src = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    m = re.search(r"typedef struct " + struct + r" \{(.*?)\} " + struct + ";", src, re.S)
    assert m, struct
    names = []
    for decl in m.group(1).split(";"):
        decl = decl.strip()
        if not decl:
            continue
        decl = re.sub(r"\[[^\]]*\]", "", decl)
        parts = decl.split(",")
        first = parts[0].split()[-1].lstrip("*")
        names.append(first)
        names += [p.strip().lstrip("*") for p in parts[1:]]
    return names


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    """offsetof/sizeof/alignof of everything the .hsc names, plus every field
    of the written structs, from a C program compiled against the header"""
    fields, _, sizes, consts = hsc_directives()
    for s in WRITTEN:
        fields |= {(s, f) for f in header_fields(s)}
        sizes.add(s)
    lines = ["#include <stdio.h>", "#include <stddef.h>", "#include <stdalign.h>",
             '#include "bling_gpu.h"', "int main(void) {"]
    for s, f in sorted(fields):
        lines.append(f'  printf("off {s} {f} %zu %zu\\n", offsetof({s}, {f}), '
                     f"sizeof((({s}*)0)->{f}));")
    for s in sorted(sizes):
        lines.append(f'  printf("size {s} %zu %zu\\n", sizeof({s}), alignof({s}));')
    for c in sorted(consts):
        lines.append(f'  printf("const {c} %lld\\n", (long long)({c}));')
    lines += ["  return 0;", "}"]
    d = tmp_path_factory.mktemp("hsc")
    (d / "layout.c").write_text("\n".join(lines))
    exe = d / "layout"
    r = subprocess.run(["gcc", "-std=c11", "-I", str(ROOT / "include"), str(d / "layout.c"), "-o",
                        str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr  # a field the module names that the header lacks
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    lay = {"off": {}, "size": {}, "const": {}}
    for ln in out.splitlines():
        t = ln.split()
        if t[0] == "off":
            lay["off"][(t[1], t[2])] = (int(t[3]), int(t[4]))
        elif t[0] == "size":
            lay["size"][t[1]] = (int(t[2]), int(t[3]))
        else:
            lay["const"][t[1]] = int(t[2])
    return lay


def test_module_names_only_header_fields(c_layout):
    fields, _, sizes, consts = hsc_directives()
    assert fields and sizes and consts
    assert all(f in c_layout["off"] for f in fields)
    assert c_layout["const"]["BLING_ABI_VERSION"] == abi.ABI_VERSION
    assert c_layout["const"]["BLING_BANDS"] == 16


@pytest.mark.parametrize("struct", sorted(WRITTEN))
def test_module_writes_every_field(struct):
    _, pokes, _, _ = hsc_directives()
    missing = [f for f in header_fields(struct) if (struct, f) not in pokes]
    assert not missing, f"{struct}: fields not written by GpuScene.hsc: {missing}"


@pytest.mark.parametrize("struct", sorted(WRITTEN))
def test_ctypes_mirror_matches_the_header(c_layout, struct):
    cls = WRITTEN[struct]
    size, align = c_layout["size"][struct]
    assert C.sizeof(cls) == size
    assert C.alignment(cls) == align
    for f in header_fields(struct):
        off, fsize = c_layout["off"][(struct, f)]
        desc = getattr(cls, f)
        assert (desc.offset, desc.size) == (off, fsize), (struct, f)
