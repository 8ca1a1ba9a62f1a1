"""Build of the in-tree CUDA library sparkle_gb300/_build/libspk.so (sm_103a only).

Each translation unit is compiled by its own nvcc process (in parallel), then linked with `nvcc -shared`.
Device code is built for `-gencode arch=compute_103a,code=sm_103a` with `-fmad=false`: the path tracer's
arithmetic must round every multiply and add separately, as the reference's host code does; the slab
tests that want fused multiply-adds call fmaf() explicitly.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libspk.so")

CUDA_SOURCES = ["kernels.cu", "wavefront.cu", "spk_api.cu", "conv_tc.cu", "unet.cu", "bvh_device.cu", "image_io.cu", "flip.cu", "sky.cu"]
CXX_SOURCES = ["bvh_builder.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the sparkle_gb300 CUDA library cannot be built")
    return path


def _inputs():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    files.append(os.path.abspath(__file__))
    return files


STAMP = os.path.join(OUT_DIR, "defines.txt")


def _defines() -> str:
    return os.environ.get("SPK_BUILD_DEFINES", "").strip()


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    built_with = open(STAMP).read().strip() if os.path.exists(STAMP) else ""
    if built_with != _defines():
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in _inputs())


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)
    return res.stdout + res.stderr


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    """Compiles libspk.so if missing or stale; returns its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    nv = nvcc()
    common = ["-O3", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-Xcompiler", "-fPIC,-ffp-contract=off"]
    # Tunable overrides (e.g. "-DSPK_REFILL_LANES=16"), used by the autotuner's variant builds.
    common += [d for d in os.environ.get("SPK_BUILD_DEFINES", "").split() if d.startswith("-D")]
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        obj = os.path.join(OUT_DIR, src + ".o")
        cmd = [nv, *ARCH, "-lineinfo", "-fmad=false", "--expt-relaxed-constexpr", *common, "-c",
               os.path.join(CSRC, src), "-o", obj]
        if verbose_ptxas:
            cmd.insert(1, "-Xptxas=-v")
        jobs.append(cmd)
        objs.append(obj)
    for src in CXX_SOURCES:
        obj = os.path.join(OUT_DIR, src + ".o")
        jobs.append([nv, *common, "-x", "c++", "-c", os.path.join(CSRC, src), "-o", obj])
        objs.append(obj)
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        logs = list(ex.map(_run, jobs))
    _run([nv, *ARCH, "-shared", *objs, "-o", LIB + ".tmp", "-lpthread"])
    os.replace(LIB + ".tmp", LIB)
    with open(STAMP, "w") as f:
        f.write(_defines())
    if verbose_ptxas:
        print("\n".join(l for l in logs if l.strip()))
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose_ptxas="-v" in sys.argv))
