"""Host plan of spk_render_batch (no GPU): the groups of consecutive whole requests cover every request and
item once, in order, each at most the slot budget (a larger request alone) and as large as the budget
allows; each group's first pass queues exactly its first min(slots, items) items, each request's items in
item order, the requests walked in two-ray packets (spp >= 32) first, then one-ray packets (spp >= 8), then
the rest, with the packet counts the extend kernels split the queue by."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    out = tmp_path_factory.mktemp("h") / "libbatchplan.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", os.path.join(HERE, "harness", "batch_plan_check.cpp"),
                    "-o", str(out)], check=True)
    L = C.CDLL(str(out))
    L.batch_plan_check.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint64, C.c_uint32, C.c_uint32, C.c_void_p]
    return L


def check(harness, items, spp, slots, min1=8, min2=32):
    items = np.ascontiguousarray(items, np.uint64)
    spp = np.ascontiguousarray(spp, np.uint32)
    groups = np.zeros(1, np.uint32)
    rc = harness.batch_plan_check(items.ctypes.data_as(C.c_void_p), spp.ctypes.data_as(C.c_void_p), len(items),
                                  slots, min1, min2, groups.ctypes.data_as(C.c_void_p))
    assert rc == 0, (rc, items, spp, slots)
    return int(groups[0])


def test_one_group_when_everything_fits(harness):
    assert check(harness, [1536, 32768, 1173, 268800, 25600, 2046], [1, 8, 3, 70, 16, 2], 1 << 27) == 1


def test_requests_larger_than_the_budget_stand_alone(harness):
    # the test batch of tests/test_batch_gpu.py with a 20000-item budget: 1536 | 32768 | 1173 | 268800 | 25600 | 2046
    assert check(harness, [1536, 32768, 1173, 268800, 25600, 2046], [1, 8, 3, 70, 16, 2], 20000) == 6


def test_random_batches(harness):
    rng = np.random.default_rng(7)
    for _ in range(300):
        n = int(rng.integers(1, 40))
        spp = rng.choice([1, 2, 4, 7, 8, 9, 16, 31, 32, 33, 64, 70], n)
        pixels = rng.integers(4, 3000, n)
        slots = int(rng.integers(1, 60000))
        check(harness, pixels * spp, spp, slots)


def test_empty_batch(harness):
    assert check(harness, np.zeros(0, np.uint64), np.zeros(0, np.uint32), 1000) == 0
