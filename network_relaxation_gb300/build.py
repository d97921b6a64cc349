"""Builds the in-tree native library network_relaxation_gb300/libnetrelax.so
(CUDA kernels for sm_103a + the C++ host side behind include/netrelax.h) and
the lsrelax command-line binary next to it.

Translation units compile in parallel; objects go to
network_relaxation_gb300/_build/.  FP64 kernel files are compiled with
--fmad=false and host files with -ffp-contract=off so that every fused
multiply-add is an explicit fma() (bit-reproducible arithmetic).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnetrelax.so")
CLI = os.path.join(HERE, "lsrelax")
MESH_CLI = os.path.join(HERE, "nmrelax")
SPR_CLI = os.path.join(HERE, "sp_relax")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc") if os.path.exists(os.path.join(CUDA_HOME, "bin", "nvcc")) else "nvcc"
CXX = os.environ.get("CXX", "g++")

# (source, extra flags)
CUDA_UNITS = [
    ("fire_fp64.cu", ["--fmad=false"]),
    ("fire_mixed.cu", ["--fmad=false"]),
    ("fire_dsm.cu", ["--fmad=false"]),
    ("fire_tile.cu", ["--fmad=false"]),
    ("fire_dsm64.cu", ["--fmad=false"]),
    ("api.cu", []),
    ("tuning.cu", []),
    ("noalloc.cu", ["--fmad=false"]),
    ("analysis.cu", ["--fmad=false"]),
    ("spr.cu", ["--fmad=false"]),
]
HOST_UNITS = ["host_network.cpp", "fast_io.cpp", "mesh_host.cpp", "generators.cpp", "driver.cpp"]


def _run(cmd):
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("command failed:\n  %s\n%s" % (" ".join(cmd), proc.stdout))
    return proc.stdout


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(INCLUDE, "netrelax.h"))
    return hs


def build(verbose=False, force=False):
    """Compiles every unit that is out of date and links the library + CLI."""
    os.makedirs(BUILD, exist_ok=True)
    headers = _headers()
    jobs = []
    objs = []
    for src, extra in CUDA_UNITS:
        path = os.path.join(CSRC, src)
        if not os.path.exists(path):
            continue
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if force or not _newer(obj, [path] + headers):
            jobs.append([NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                                         "-Xptxas", "-v" if verbose else "-O3", "-I", CSRC, "-I", INCLUDE] + extra
                        + ["-c", path, "-o", obj])
    for src in HOST_UNITS:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if force or not _newer(obj, [path] + headers):
            jobs.append([CXX, "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-I", CSRC, "-I", INCLUDE,
                         "-I", os.path.join(CUDA_HOME, "include"), "-c", path, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    if force or jobs or not _newer(LIB, objs):
        tmp = LIB + ".tmp"
        _run([NVCC] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs + ["-lpthread"])
        os.replace(tmp, LIB)
    for cli, main in ((CLI, "lsrelax_main.cpp"), (MESH_CLI, "nmrelax_main.cpp"), (SPR_CLI, "sp_relax_main.cpp")):
        main_src = os.path.join(CSRC, main)
        if force or not _newer(cli, [main_src, LIB]):
            _run([CXX, "-std=c++17", "-O2", "-I", INCLUDE, main_src, "-o", cli, "-L", HERE, "-lnetrelax",
                  "-Wl,-rpath,$ORIGIN"])
    return LIB


def clean():
    shutil.rmtree(BUILD, ignore_errors=True)
    for p in (LIB, CLI, MESH_CLI, SPR_CLI):
        if os.path.exists(p):
            os.remove(p)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
