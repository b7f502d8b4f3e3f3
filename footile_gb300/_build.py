"""Compile the CUDA library for sm_103a with nvcc, in-tree.

Each translation unit compiles in parallel into footile_gb300/_build/, which then
holds the C-ABI shared library (libfootile_gpu.so, loaded by the Python mirror) and
the same objects as a static library (libfootile_gpu.a, for a host program or a Rust
crate that links the path in: link it with the CUDA runtime, e.g. `-lcudart_static
-ldl -lpthread -lrt`, and the C++ standard library).  No torch extension machinery is
involved.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libfootile_gpu.so")
STATIC_LIB = os.path.join(OUT, "libfootile_gpu.a")

SOURCES = ["ft_kernels.cu", "ft_adjoint.cu", "ft_convert.cu", "ft_capi.cu"]
HEADERS = ["ft_device.cuh", "ft_kernels.cuh", "ft_adjoint.cuh"]
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Bit-exact float stages: no FMA contraction, IEEE division and square root.
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
           "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden", "-Xcompiler", "-ffp-contract=off",
           "--expt-relaxed-constexpr"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _inputs():
    inc = os.path.join(HERE, "..", "include")
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    deps += [os.path.join(inc, f) for f in os.listdir(inc)]
    return deps


def up_to_date():
    if not os.path.exists(LIB) or not os.path.exists(STATIC_LIB):
        return False
    t = min(os.path.getmtime(LIB), os.path.getmtime(STATIC_LIB))
    return all(os.path.getmtime(p) <= t for p in _inputs())


def build(force=False, verbose=False):
    """Compile (if stale) and return the path of the shared library."""
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    extra = os.environ.get("FT_NVCC_FLAGS", "").split()

    def compile_one(src):
        obj = os.path.join(OUT, src.replace(".cu", ".o"))
        cmd = [cc] + GENCODE + NVFLAGS + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return obj

    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [cc] + GENCODE + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc link failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    # the static library: the same objects (whole-program device code, no device link)
    tmp_a = STATIC_LIB + ".tmp"
    if os.path.exists(tmp_a):
        os.remove(tmp_a)
    r = subprocess.run(["ar", "rcs", tmp_a] + objs, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("ar failed:\n" + r.stdout + r.stderr)
    os.replace(tmp_a, STATIC_LIB)
    return LIB


def build_variant(out_dir, extra_flags):
    """Compile the library with extra nvcc flags (the bounds-check build: -DFT_CHECK=1)
    into out_dir; returns the path of its shared library."""
    os.makedirs(out_dir, exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(out_dir, src.replace(".cu", ".o"))
        cmd = [cc] + GENCODE + NVFLAGS + list(extra_flags) + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return obj

    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    lib = os.path.join(out_dir, "libfootile_gpu.so")
    r = subprocess.run([cc] + GENCODE + ["-shared", "-o", lib] + objs, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc link failed:\n" + r.stdout + r.stderr)
    return lib


if __name__ == "__main__":
    print(build(force=True, verbose=True))
