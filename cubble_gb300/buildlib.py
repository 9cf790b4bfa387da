"""Builds libcubble_gb300.so in-tree with nvcc for sm_103a.

Every translation unit compiles in parallel into cubble_gb300/_build/ and is
linked into cubble_gb300/libcubble_gb300.so (static CUDA runtime). Rebuilds
only when a source or header is newer than the library.

    python -m cubble_gb300.buildlib [--force] [--verbose]
"""
import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcubble_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-fvisibility=hidden", "--expt-relaxed-constexpr",
                     "-I", INCLUDE]


def nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h")) + [__file__]
    return any(os.path.getmtime(p) > t for p in deps)


def _compile(src, verbose):
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    cmd = [nvcc()] + NVCC_FLAGS + (["-Xptxas", "-v"] if verbose else []) + \
        ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    return obj, r.stderr


CLI_SRC = os.path.join(HERE, "cli", "cubble_cli.cpp")
CLI = os.path.join(HERE, "cubble-cli")


def build_cli(force=False):
    """Builds the cubble-cli executable (C++ over the C ABI, static cuRAND)
    next to the library. Returns its path, or None with a message on stderr
    when the toolchain lacks a part (the library does not depend on it)."""
    deps = [CLI_SRC, os.path.join(HERE, "cli", "json.hpp"), LIB,
            os.path.join(INCLUDE, "cubble_gb300.h")]
    if not force and os.path.exists(CLI) and all(
            os.path.getmtime(p) <= os.path.getmtime(CLI) for p in deps):
        return CLI
    tmp = CLI + ".tmp"
    cmd = [nvcc()] + ARCH + ["-O2", "-std=c++17", "-Xcompiler", "-ffp-contract=off",
                             "-I", INCLUDE, CLI_SRC, "-o", tmp, "-L" + HERE, "-lcubble_gb300",
                             "-lcurand_static", "-lculibos", "-Xlinker", "-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write("cubble-cli not built:\n%s%s" % (r.stdout, r.stderr))
        return None
    os.replace(tmp, CLI)
    return CLI


def build(force=False, verbose=False):
    if not force and not _stale():
        build_cli()
        return LIB
    os.makedirs(OUT, exist_ok=True)
    srcs = sources()
    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    build_cli(force=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="--verbose" in sys.argv))
