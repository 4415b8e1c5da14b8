"""Build recipe of libcmm_gb300.so and the SimulationCuda2d.out CLI (sm_103a).

nvcc compiles every .cu with one -gencode (compute_103a -> sm_103a), g++ the
host .cpp files; translation units build in parallel and the results land in
cmm-turbulence_gb300/lib/ (git-ignored).  No cmake.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "lib")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libcmm_gb300.so")
CLI = os.path.join(OUT, "SimulationCuda2d.out")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"] + GENCODE
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-I" + os.path.join(CUDA_HOME, "include")]
LIBS = ["-L" + os.path.join(CUDA_HOME, "lib64"), "-lcurand", "-lcudart"]


def sources():
    cu = sorted(f for f in os.listdir(SRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(SRC) if f.endswith(".cpp") and f != "cli_main.cpp")
    return cu, cpp


def _deps():
    return [os.path.join(SRC, f) for f in os.listdir(SRC)] + [os.path.join(HERE, "..", "include", "cmm_abi.h"), __file__]


def up_to_date():
    if not (os.path.exists(LIB) and os.path.exists(CLI)):
        return False
    t = min(os.path.getmtime(LIB), os.path.getmtime(CLI))
    return all(os.path.getmtime(d) <= t for d in _deps())


def _compile(src):
    obj = os.path.join(OBJ, src + ".o")
    path = os.path.join(SRC, src)
    if src.endswith(".cu"):
        cmd = [NVCC] + CU_FLAGS + ["-c", path, "-o", obj]
    else:
        cmd = ["g++"] + CXX_FLAGS + ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    cu, cpp = sources()
    with cf.ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        objs = list(ex.map(_compile, cu + cpp + ["cli_main.cpp"]))
    lib_objs = [o for o in objs if not o.endswith("cli_main.cpp.o")]
    cmd = [NVCC] + GENCODE + ["-shared", "-o", LIB] + lib_objs + LIBS
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    cli_obj = os.path.join(OBJ, "cli_main.cpp.o")
    cmd = ["g++", "-o", CLI, cli_obj, "-L" + OUT, "-lcmm_gb300", "-Wl,-rpath,$ORIGIN"] + LIBS
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    if verbose:
        print("built", LIB, CLI)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
