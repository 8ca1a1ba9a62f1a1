"""Host BVH builder invariants (no GPU): the 8-wide quantised BVH addresses every item exactly once, all
node and item indices are in range, child boxes contain their items, and leaf/inner metadata agrees with
the inner-child mask -- the facts the device walk indexes by."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from sparkle_gb300 import scenes

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    out = tmp_path_factory.mktemp("h") / "libwidecheck.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", os.path.join(HERE, "harness", "wide_bvh_check.cpp"),
                    os.path.join(ROOT, "sparkle_gb300", "csrc", "bvh_builder.cpp"), "-o", str(out), "-lpthread"],
                   check=True)
    L = C.CDLL(str(out))
    L.wide_bvh_check.argtypes = [C.c_void_p, C.c_uint32, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    return L


def tri_boxes(mesh):
    p = mesh.positions[mesh.indices]
    return np.concatenate([p.min(1), p.max(1)], 1).astype(np.float32)


def check(harness, boxes, threads=4, mode=None):
    """Checks both collapses (greedy and SAH-optimal) unless `mode` picks one; returns the greedy stats."""
    boxes = np.ascontiguousarray(boxes, np.float32)
    out = None
    for m in ((0, 1) if mode is None else (mode,)):
        stats = np.zeros(4, np.uint32)
        cost = C.c_double()
        rc = harness.wide_bvh_check(boxes.ctypes.data_as(C.c_void_p), len(boxes), threads, m,
                                    stats.ctypes.data_as(C.c_void_p), C.byref(cost))
        assert rc == 0, f"invariant {rc} violated (collapse mode {m})"
        out = stats if out is None else out
    return out


def sah_cost(harness, boxes, mode, threads=4):
    boxes = np.ascontiguousarray(boxes, np.float32)
    stats = np.zeros(4, np.uint32)
    cost = C.c_double()
    assert harness.wide_bvh_check(boxes.ctypes.data_as(C.c_void_p), len(boxes), threads, mode,
                                  stats.ctypes.data_as(C.c_void_p), C.byref(cost)) == 0
    return cost.value, stats


def test_small_meshes(harness):
    for n in (1, 2, 3, 4, 5, 9, 24, 25, 100):
        rng = np.random.default_rng(n)
        lo = rng.uniform(-5, 5, (n, 3))
        boxes = np.concatenate([lo, lo + rng.uniform(0, 1, (n, 3))], 1)
        check(harness, boxes)


def test_degenerate_boxes(harness):
    # coincident centroids, flat boxes, identical boxes
    boxes = np.tile(np.array([[0, 0, 0, 1, 1, 0]], np.float32), (50, 1))
    check(harness, boxes)
    flat = np.zeros((40, 6), np.float32)
    flat[:, 0] = np.arange(40)
    flat[:, 3] = np.arange(40) + 1
    check(harness, flat)


def test_cornell_and_icosphere(harness, cornell):
    scene, _ = cornell
    for m in scene.meshes:
        check(harness, tri_boxes(m))
    check(harness, tri_boxes(scenes.icosphere(5)))


def test_full_terrain(harness):
    mesh = scenes.heightfield(1024, 100.0, 6.0, seed=1)
    stats = check(harness, tri_boxes(mesh), threads=8, mode=0)
    check(harness, tri_boxes(mesh), threads=8, mode=1)
    assert stats[3] == 2 * 1024 * 1024
    assert stats[1] < 40


def test_sah_collapse_lowers_the_cost(harness):
    """The SAH-optimal collapse has a lower SAH cost than the greedy one on the meshes of the workloads."""
    for mesh in (scenes.heightfield(128, 40.0, 3.0, seed=2), scenes.icosphere(4)):
        g, gs = sah_cost(harness, tri_boxes(mesh), 0)
        s, ss = sah_cost(harness, tri_boxes(mesh), 1)
        assert s < g, (s, g)
        assert ss[3] == gs[3]  # every item once in both
