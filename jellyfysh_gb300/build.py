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
SOURCES = ["jf_chains.cu", "jf_engine_host.cu", "jf_potentials.cu", "jf_observe.cu", "jf_lifting.cu", "jf_composite.cu",
           "jf_water.cu", "jf_states.cu"]
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


def build(force: bool = False, verbose: bool = False, defines=(), output: str = None) -> str:
    """Compile libjfgpu.so; ``defines`` (e.g. JF_CHAIN_MIN_BLOCKS=4) and ``output`` build a tuning variant."""
    library = output or LIBRARY
    build_dir = os.path.dirname(library)
    if not force and not defines and output is None and up_to_date():
        return LIBRARY
    os.makedirs(build_dir, exist_ok=True)
    compiler = nvcc()
    extra = ["-Xptxas", "-v"] if verbose else []

    def compile_one(source):
        obj = os.path.join(build_dir, source.replace(".cu", ".o"))
        command = [compiler, *ARCH, *FLAGS, *["-D" + d for d in defines], *extra, "-c", os.path.join(CSRC, source),
                   "-o", obj]
        result = subprocess.run(command, capture_output=True, text=True)
        if result.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s%s" % (source, result.stdout, result.stderr))
        return obj, result.stderr

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as pool:
        results = list(pool.map(compile_one, SOURCES))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    temporary = library + ".%d.tmp" % os.getpid()
    command = [compiler, *ARCH, "-shared", "-o", temporary] + [obj for obj, _ in results] + ["-lcudart"]
    subprocess.run(command, check=True)
    os.replace(temporary, library)
    return library


if __name__ == "__main__":
    import argparse
    parser = argparse.ArgumentParser()
    parser.add_argument("--force", action="store_true")
    parser.add_argument("-v", dest="verbose", action="store_true")
    parser.add_argument("-D", dest="defines", action="append", default=[])
    parser.add_argument("-o", dest="output", default=None)
    args = parser.parse_args()
    print(build(force=args.force, verbose=args.verbose, defines=args.defines, output=args.output))
