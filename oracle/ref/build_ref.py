"""TEST INFRASTRUCTURE: compiles the reference's own device code into a cubin.

Recipe: nvcc -cubin of KJLankinen/cubble's unmodified src/kernels.cu (it
builds from its own sources plus the reference's include/ tree) for sm_103a,
output only into oracle/_ref/kernels_ref.cubin (git-ignored). The cubin is
device code: tests/golden/make_golden.py loads it on the GPU through the
CUDA driver API to run the reference's kernels on seeded inputs and record
golden vectors. Nothing in the product loads it.

The reference location comes from the command line (`build_ref.py
REFERENCE_DIR`) or the CUBBLE_REFERENCE environment variable; with neither,
or where that directory holds no src/kernels.cu, it does nothing.

    python oracle/ref/build_ref.py [--force] REFERENCE_DIR
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(os.path.dirname(HERE), "_ref")
OUT = os.path.join(OUT_DIR, "kernels_ref.cubin")


def build(ref, force=False):
    if not ref:
        return None
    src = os.path.join(ref, "src", "kernels.cu")
    if not os.path.exists(src):
        return None
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= os.path.getmtime(src):
        return OUT
    os.makedirs(OUT_DIR, exist_ok=True)
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cmd = [os.path.join(cuda, "bin", "nvcc"), "-cubin",
           "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
           "-I", os.path.join(ref, "include"), "-I", os.path.join(ref, "src"),
           "-I", os.path.join(cuda, "include", "nvtx3"), src, "-o", OUT]
    subprocess.run(cmd, check=True)
    return OUT


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    ref = args[0] if args else os.environ.get("CUBBLE_REFERENCE")
    print(build(ref, force="--force" in sys.argv))
