"""The C ABI: every entry point declared in include/bonsai_gpu.h is exported by the built
libbonsai_gpu.so and declared in the ctypes mirror; struct layouts agree between the header (as
gcc lays it out) and bonsai_gb300/_abi.py.  No compute call runs here (no GPU needed)."""
import ctypes as C
import re
import subprocess
import sys

import pytest

from bonsai_gb300 import _abi as A

from .conftest import ROOT

HEADER = ROOT / "include" / "bonsai_gpu.h"
STRUCTS = ["bg_material", "bg_area_light", "bg_sphere", "bg_camera", "bg_render_opts", "bg_render_stats",
           "bg_ray", "bg_hit", "bg_device_opts", "bg_build_stats", "bg_tuning", "bg_quadric", "bg_guide_opts",
           "bg_guide_stats", "bg_batch_item", "bg_texture", "bg_obj_info", "bg_infinite_light"]


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:bg_status|void|const char\*)\s+(bg_[a-z0-9_]+)\s*\(", text, re.M)))


def _lib_path():
    p = A.LIB_PATH
    if not p.exists():
        subprocess.run([sys.executable, str(ROOT / "bonsai_gb300" / "build.py")], check=True)
    return p


def test_header_declares_the_entry_points():
    names = declared_functions()
    for required in ["bg_create", "bg_destroy", "bg_scene_commit", "bg_render", "bg_trace_closest", "bg_trace_any",
                     "bg_render_noalloc", "bg_set_tuning", "bg_guide_create", "bg_guide_forward",
                     "bg_guide_gradient", "bg_guide_train", "bg_render_guided", "bg_render_batch", "bg_obj_read",
                     "bg_scene_add_obj", "bg_write_exr", "bg_film_write_exr"]:
        assert required in names


def test_library_exports_every_declared_symbol():
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib_path())], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\sT\s(bg_[a-z0-9_]+)", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing


def test_ctypes_mirror_covers_every_declared_symbol():
    missing = [n for n in declared_functions() if n not in A.SIGNATURES]
    assert not missing, missing
    lib = A.load(_lib_path())
    for n in declared_functions():
        assert getattr(lib, n) is not None


def test_struct_layouts_match_header(tmp_path):
    src = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{HEADER}"', "int main(void) {"]
    for s in STRUCTS:
        src.append(f'  printf("{s} %zu\\n", sizeof({s}));')
        for f, _ in getattr(A, s)._fields_:
            src.append(f'  printf("{s}.{f} %zu\\n", offsetof({s}, {f}));')
    src += ["  return 0;", "}"]
    c = tmp_path / "layout.c"
    c.write_text("\n".join(src))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-o", str(exe), str(c)], check=True)
    lines = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True, check=True)
                 .stdout.splitlines())
    for s in STRUCTS:
        cls = getattr(A, s)
        assert int(lines[s]) == C.sizeof(cls), s
        for f, _ in cls._fields_:
            assert int(lines[f"{s}.{f}"]) == getattr(cls, f).offset, f"{s}.{f}"


def test_status_strings_without_device():
    lib = A.load(_lib_path())
    assert lib.bg_status_string(A.BG_OK) == b"ok"
    assert lib.bg_status_string(A.BG_ERR_NO_DEVICE) == b"no usable CUDA device"
    # null handles are rejected before any CUDA call
    assert lib.bg_render(None, None, None, None, None, None) == A.BG_ERR_INVALID
    assert lib.bg_scene_commit(None, 0, None) == A.BG_ERR_INVALID
    assert lib.bg_render_noalloc(None, None, None, None, None) == A.BG_ERR_INVALID
    assert lib.bg_set_tuning(None, None) == A.BG_ERR_INVALID


def test_guide_constants_match_header():
    text = HEADER.read_text()
    for name in ["BG_GUIDE_PARAMS", "BG_GUIDE_QUERY_FLOATS", "BG_GUIDE_OUTPUTS", "BG_GUIDE_SAMPLE_FLOATS"]:
        m = re.search(rf"#define {name} (\d+)u", text)
        assert m and int(m.group(1)) == getattr(A, name), name
    from oracle import guide as O
    assert O.PARAMS == A.BG_GUIDE_PARAMS and O.OUT == A.BG_GUIDE_OUTPUTS
