"""Builds mipt_gb300/_build/libmipt_gb300.so (CUDA for sm_103a + host C++).

    python -m mipt_gb300.build [--force]

Sources compile in parallel (one process per translation unit) and are
rebuilt only when a source or header is newer than its object.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libmipt_gb300.so")
INCLUDE = os.path.join(ROOT, "include")
APPS = os.path.join(HERE, "apps")
APP_TARGETS = [("mipt.cpp", "mipt.exe"), ("sim_tmi.cpp", "sim_tmi.exe"), ("gmn.cpp", "gmn.exe"),
               ("entropy.cpp", "entropy.exe"), ("free_energy.cpp", "free_energy.exe")]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["engine.cu", "observables.cu", "eigen.cu", "capi.cu", "fermion.cu", "noalloc.cu", "parity.cu", "gmn.cu", "mlp.cu"]
CXX_SOURCES = ["sampler.cpp"]


def _nvcc():
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    path = os.path.join(cuda, "bin", "nvcc")
    return path if os.path.exists(path) else (shutil.which("nvcc") or "nvcc")


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _stale(src, obj, headers):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + headers)


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stderr


def build(force=False, verbose=False, ptxas_info=False):
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    headers = _headers()
    jobs = []
    objs = []
    for s in CUDA_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OUT, s + ".o")
        objs.append(obj)
        if force or _stale(src, obj, headers):
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE,
                   "-I", CSRC, "--expt-relaxed-constexpr", "-c", src, "-o", obj]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for s in CXX_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OUT, s + ".o")
        objs.append(obj)
        if force or _stale(src, obj, headers):
            jobs.append(["g++", "-std=c++17", "-O3", "-fPIC", "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj])
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
            for log in ex.map(_compile, jobs):
                if verbose and log:
                    print(log)
    if jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-lpthread"]
        _compile(cmd)
        os.replace(tmp, LIB)
    build_apps(force)
    return LIB


def build_apps(force=False):
    """The drop-in executables (mipt.exe, sim_tmi.exe): host C++ over the C ABI,
    linked against the library next to them."""
    headers = [os.path.join(APPS, f) for f in os.listdir(APPS) if f.endswith(".hpp")]
    headers.append(os.path.join(INCLUDE, "mipt_gb300.h"))
    jobs = []
    for src_name, exe_name in APP_TARGETS:
        src = os.path.join(APPS, src_name)
        exe = os.path.join(OUT, exe_name)
        if force or _stale(src, exe, headers + [LIB]):
            jobs.append(["g++", "-std=c++17", "-O2", "-I", INCLUDE, src, "-o", exe, "-L", OUT, "-lmipt_gb300",
                         "-Wl,-rpath,$ORIGIN"])
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            list(ex.map(_compile, jobs))
    return [os.path.join(OUT, e) for _, e in APP_TARGETS]


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
