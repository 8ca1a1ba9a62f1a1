"""The C ABI without a GPU: the ctypes mirror has the C layout of include/spk.h (checked by compiling the
header), and the built library loads and exports every function the header declares."""
import ctypes as C
import os
import re
import subprocess

import pytest

from sparkle_gb300 import abi, native
from sparkle_gb300 import build as spk_build

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
HEADER = os.path.join(ROOT, "include", "spk.h")
HEADERS = [HEADER, os.path.join(ROOT, "include", "spk_denoise.h")]

STRUCTS = ["spk_mesh", "spk_instance", "spk_material", "spk_sky", "spk_camera", "spk_config", "spk_ray", "spk_hit",
           "spk_stats", "spk_tuning", "spk_scene_desc", "spk_request", "spk_texture", "spk_material_maps"]


def header_functions():
    names = set()
    for h in HEADERS:
        names |= set(re.findall(r"^\w[\w\s\*]*?\b(spk_\w+)\s*\(", open(h).read(), re.M))
    return sorted(names)


def test_header_functions_are_bound():
    assert header_functions() == sorted(native.EXPORTED)


def test_struct_layout_matches_c(tmp_path):
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "spk.h"', "int main(void) {"]
    for s in STRUCTS:
        lines.append(f'  printf("{s} %zu\\n", sizeof({s}));')
        for name, _ in getattr(abi, s)._fields_:
            lines.append(f'  printf("{s}.{name} %zu\\n", offsetof({s}, {name}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], capture_output=True, text=True).stdout.splitlines())
    for s in STRUCTS:
        cls = getattr(abi, s)
        assert int(got[s]) == C.sizeof(cls), s
        for name, _ in cls._fields_:
            assert int(got[f"{s}.{name}"]) == getattr(cls, name).offset, f"{s}.{name}"


def test_library_loads_and_exports_every_symbol():
    path = spk_build.build()
    L = C.CDLL(path)
    for name in header_functions():
        assert hasattr(L, name), name
    assert L.spk_abi_version() == abi.SPK_ABI_VERSION


def test_calls_fail_cleanly_without_a_context():
    L = native.lib()
    assert L.spk_render(None, 1) == 1
    assert L.spk_set_scene(None, None, 0, None, 0, None, 0, None) == 1
    assert L.spk_destroy(None) == 0
    out = abi.spk_camera()
    f3 = C.c_float * 3
    st = L.spk_camera_from_look(C.byref(f3(0, 0, 0)), C.byref(f3(0, 1, 0)), C.byref(f3(0, 0, 1)), 0.7, 1.0, 0.0,
                                1.0, 64, 32, C.byref(out))
    assert st == 0
    assert abs(out.front[1] - 1.0) < 1e-6 and abs(out.right[0] - 1.0) < 1e-6 and abs(out.up[2] - 1.0) < 1e-6
    assert out.max_u[0] == pytest.approx(2.0 * abs(out.max_v[2]), rel=1e-6)


def test_camera_from_look_matches_python_copy():
    a = native.camera_from_look((1, -3, 2), (0, 0, 0.5), (0, 0, 1), 0.8, 2.5, 0.01, 1.3, 320, 200)
    b = abi.camera_from_look((1, -3, 2), (0, 0, 0.5), (0, 0, 1), 0.8, 2.5, 0.01, 1.3, 320, 200)
    for name, _ in abi.spk_camera._fields_:
        va, vb = getattr(a, name), getattr(b, name)
        if isinstance(va, float):
            assert va == pytest.approx(vb, rel=1e-6, abs=1e-7), name
        else:
            assert list(va) == pytest.approx(list(vb), rel=1e-6, abs=1e-6), name


def test_tuning_defaults():
    t = abi.spk_tuning()
    native.lib().spk_tuning_defaults(C.byref(t))
    assert (t.cuda_graph, t.material_sort, t.bvh_width, t.bvh_leaf_size, t.extend_blocks_per_sm,
            t.shade_blocks_per_sm, t.batch_slots, t.ray_sort, t.bvh_collapse, t.bvh_builder,
            t.path_slots_per_pixel) == (1, 0, 8, 3, 0, 8, 0, 0, 0, 0, 64)
    assert native.lib().spk_set_tuning(None, C.byref(t)) == 1
