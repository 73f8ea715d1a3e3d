"""Build recipe of ``libjfgpu.so``: every CUDA translation unit compiled for sm_103a with nvcc, in parallel.

The library is built in-tree (``jellyfysh_gb300/_build/libjfgpu.so``) on the machine that uses it.  FP64 code is
compiled with ``-fmad=false`` so that every multiply and add is rounded on its own, as in the reference; the FP32
screening writes its FMAs out explicitly where it wants them.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD_DIR = os.path.join(HERE, "_build")
LIBRARY = os.path.join(BUILD_DIR, "libjfgpu.so")
SOURCES = ["jf_chains.cu", "jf_engine_host.cu", "jf_potentials.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-fast-math",
         "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libjfgpu.so")
    return path


def _inputs():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(ROOT, "include", "jfgpu.h"))
    files.append(os.path.abspath(__file__))
    return files


def up_to_date() -> bool:
    if not os.path.exists(LIBRARY):
        return False
    built = os.path.getmtime(LIBRARY)
    return all(os.path.getmtime(f) <= built for f in _inputs())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIBRARY
    os.makedirs(BUILD_DIR, exist_ok=True)
    compiler = nvcc()
    extra = ["-Xptxas", "-v"] if verbose else []

    def compile_one(source):
        obj = os.path.join(BUILD_DIR, source.replace(".cu", ".o"))
        command = [compiler, *ARCH, *FLAGS, *extra, "-c", os.path.join(CSRC, source), "-o", obj]
        result = subprocess.run(command, capture_output=True, text=True)
        if result.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s%s" % (source, result.stdout, result.stderr))
        return obj, result.stderr

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as pool:
        results = list(pool.map(compile_one, SOURCES))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    temporary = LIBRARY + ".%d.tmp" % os.getpid()
    command = [compiler, *ARCH, "-shared", "-o", temporary] + [obj for obj, _ in results] + ["-lcudart"]
    subprocess.run(command, check=True)
    os.replace(temporary, LIBRARY)
    return LIBRARY


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
