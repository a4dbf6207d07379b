"""Build libvisor_gb300.so in-tree (no cmake; parallel nvcc/g++ invocations).

The library holds the Vulkan ICD front end (C++), the SPIR-V -> CUDA
translator, the CUDA back end with its generic kernels compiled for sm_103a,
the scene generator/driver used by tests and benchmarks, and the stage-kernel
sources that NVRTC compiles for sm_103a at pipeline creation.

    python -m visor_gb300.build
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libvisor_gb300.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

KERNEL_SOURCES = [
    ("kVgxTypes", "kernels/vgx_types.h"),
    ("kVgxDevice", "kernels/vgx_device.cuh"),
    ("kVgxTiles", "kernels/vgx_tiles.cuh"),
    ("kVgxStage", "kernels/vgx_stage.cuh"),
]

C_SOURCES = ["scene/scene.c", "scene/spirv_emit.c"]
CXX_SOURCES = ["icd/icd.cpp", "spirv/translate.cpp", "scene/driver.cpp", "runtime/serve.cpp"]
CU_SOURCES = ["runtime/vgpu.cu"]


def _embed_sources():
    """Write the stage-kernel headers as raw string literals for NVRTC."""
    os.makedirs(BUILD, exist_ok=True)
    out = ["/* generated by visor_gb300/build.py: stage kernel sources for NVRTC */"]
    for name, rel in KERNEL_SOURCES:
        text = open(os.path.join(CSRC, rel)).read()
        assert ")VGXSRC\"" not in text
        out.append(f'static const char {name}[] = R"VGXSRC({text}\n)VGXSRC";')
    path = os.path.join(BUILD, "vgx_sources.inc")
    data = "\n".join(out) + "\n"
    if not os.path.exists(path) or open(path).read() != data:
        with open(path, "w") as fh:
            fh.write(data)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stderr


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False):
    _embed_sources()
    inc = ["-I" + os.path.join(REPO, "include"), "-I" + BUILD, "-I" + CSRC]
    headers = []
    for root in (os.path.join(REPO, "include"), CSRC):
        for dp, _, fns in os.walk(root):
            headers += [os.path.join(dp, f) for f in fns if f.endswith((".h", ".cuh"))]
    jobs = []
    objs = []
    for src in C_SOURCES:
        o = os.path.join(BUILD, src.replace("/", "_") + ".o")
        objs.append(o)
        s = os.path.join(CSRC, src)
        if _newer(o, [s] + headers):
            jobs.append(["gcc", "-std=c11", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-c", s, "-o", o] + inc)
    for src in CXX_SOURCES:
        o = os.path.join(BUILD, src.replace("/", "_") + ".o")
        objs.append(o)
        s = os.path.join(CSRC, src)
        if _newer(o, [s] + headers):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fvisibility=hidden",
                         "-c", s, "-o", o, "-I" + os.path.join(CUDA, "include")] + inc)
    for src in CU_SOURCES:
        o = os.path.join(BUILD, src.replace("/", "_") + ".o")
        objs.append(o)
        s = os.path.join(CSRC, src)
        deps = [s, os.path.join(BUILD, "vgx_sources.inc")] + headers
        if _newer(o, deps):
            jobs.append([NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                                         "-Xcompiler", "-fvisibility=hidden", "-Xptxas", "-v",
                                         "-c", s, "-o", o] + inc)
    with ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 4))) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose:
        for lg in logs:
            if lg:
                print(lg)
    if jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        _run(["g++", "-shared", "-o", tmp] + objs + [
            "-L" + os.path.join(CUDA, "lib64"), "-lcudart", "-lnvrtc", "-lpthread",
            "-Wl,-rpath," + os.path.join(CUDA, "lib64"), "-Wl,-Bsymbolic", "-Wl,--no-undefined"])
        os.replace(tmp, LIB)
    return LIB


def clean():
    shutil.rmtree(BUILD, ignore_errors=True)
    if os.path.exists(LIB):
        os.remove(LIB)


if __name__ == "__main__":
    if "--clean" in sys.argv:
        clean()
    print(build(verbose="-v" in sys.argv))
