"""Build libstsgpu.so (the C-ABI CUDA library) in-tree for sm_103a.

Each translation unit is compiled by nvcc in parallel and linked into
``ceda_demonstrations_gb300/_build/libstsgpu.so``. Device code is compiled with
``--fmad=false`` (the kernels spell out every FMA with ``__fma_rn``) and host code with
``-ffp-contract=off``, which fixes the floating-point arithmetic of both sides.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libstsgpu.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libstsgpu.so")
    return cand


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


CLI_SRC = os.path.join(HERE, "cli", "diffusion_2D_gpu.cpp")
CLI = os.path.join(OUT_DIR, "diffusion_2D_gpu")


def _deps():
    return sources() + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")] + \
        [os.path.join(HERE, "..", "include", "stsgpu.h"), os.path.abspath(__file__), CLI_SRC]


# Build variants: "" is the product; "bounds" adds -DSTS_DEBUG_BOUNDS (kernels check the index
# range each thread touches and report a violation through the context's error word) into
# _build/bounds/, without the command-line driver.
VARIANTS = {"": [], "bounds": ["-DSTS_DEBUG_BOUNDS"]}


def lib_path(variant=""):
    return LIB if not variant else os.path.join(OUT_DIR, variant, "libstsgpu.so")


def up_to_date(variant=""):
    lib = lib_path(variant)
    if not os.path.exists(lib) or (not variant and not os.path.exists(CLI)):
        return False
    t = os.path.getmtime(lib) if variant else min(os.path.getmtime(lib), os.path.getmtime(CLI))
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force=False, verbose=False, extra=(), variant=""):
    if variant not in VARIANTS:
        raise ValueError("unknown build variant %r" % variant)
    lib = lib_path(variant)
    if not force and up_to_date(variant):
        return lib
    out_dir = os.path.dirname(lib)
    os.makedirs(out_dir, exist_ok=True)
    nvcc = _nvcc()
    common = [ARCH, "-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler",
              "-fPIC,-ffp-contract=off,-O2", "-I" + os.path.join(HERE, "..", "include")] + \
        VARIANTS[variant] + list(extra)
    if verbose:
        common += ["-Xptxas", "-v"]

    def compile_one(src):
        obj = os.path.join(out_dir, os.path.basename(src)[:-3] + ".o")
        cmd = [nvcc, "-c", src, "-o", obj] + common
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        results = list(ex.map(compile_one, sources()))
    if verbose:
        for _, err in results:
            sys.stderr.write(err)
    objs = [o for o, _ in results]
    tmp = lib + ".tmp"
    cmd = [nvcc, ARCH, "-shared", "-cudart", "shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, lib)
    if variant:
        return lib
    # command-line driver (reference flags and output format), linked against the library
    cmd = [nvcc, "-O2", "-std=c++17", "-x", "c++", CLI_SRC, "-o", CLI + ".tmp",
           "-I" + os.path.join(HERE, "..", "include"), "-L" + OUT_DIR, "-lstsgpu",
           "-Xlinker", "-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("driver build failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(CLI + ".tmp", CLI)
    return LIB


if __name__ == "__main__":
    v = "bounds" if "--bounds" in sys.argv else ""
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, variant=v))
