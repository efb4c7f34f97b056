"""In-tree build of libug4gb.so (CUDA, sm_103a) and its C++ adapter check.

The library is compiled straight with nvcc (one process per translation unit,
in parallel) and linked as a shared object next to this file.  No CMake, no
torch extension machinery: the product is a plain C-ABI library.
"""
import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libug4gb.so")

SOURCES = ["k_grid.cu", "k_fv1.cu", "k_fv1_rows.cu", "k_solve.cu", "k_coarse.cu", "k_sweep2.cu", "k_rap.cu", "api.cu", "api_disc.cu", "api_gmg.cu", "api_solver.cu",
           "api_noalloc.cu", "api_perm.cu", "api_io.cu", "api_newton.cu",
           "grid_unstructured.cu", "grid_refine_device.cu", "k_ilu.cu", "api_algebra.cu", "guard.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fvisibility=hidden",
              # host arithmetic identical on x86_64 and aarch64 (gcc contracts a*b+c on aarch64 by default)
              "-Xcompiler", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include")]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")] + \
           [os.path.join(ROOT, "include", "ug4gb.h")]


def build(verbose=False, extra_flags=()):
    """Compile (incrementally) and link libug4gb.so; returns its path."""
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    # objects built on another host architecture (x86_64 vs aarch64) are stale
    stamp = os.path.join(BUILD, "host_arch")
    arch = platform.machine()
    if not os.path.exists(stamp) or open(stamp).read().strip() != arch:
        for f in os.listdir(BUILD):
            if f.endswith(".o"):
                os.remove(os.path.join(BUILD, f))
        if os.path.exists(LIB):
            os.remove(LIB)
        with open(stamp, "w") as fh:
            fh.write(arch)
    hdrs = _headers()
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if _newer(o, [s] + hdrs):
            cmd = [nvcc] + ARCH + NVCC_FLAGS + list(extra_flags) + ["-c", s, "-o", o]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for cmd, r in ex.map(run, jobs):
                if verbose or r.returncode:
                    sys.stderr.write(r.stdout + r.stderr)
                if r.returncode:
                    raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if jobs or _newer(LIB, objs):
        cmd = [nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


def build_guarded(out_dir):
    """The library with guard zones around every device buffer and poisoned
    contents (UG4GB_GUARDED, csrc/guard.cu), for the tests that run the GPU
    paths against it and then call ug4gb_debug_guard_check.  Returns the path
    of the .so."""
    return _build_variant(out_dir, "libug4gb_guarded.so", ["-DUG4GB_GUARDED"], [])


def _build_variant(out_dir, name, flags_extra, link_extra, drop_o3=False):
    nvcc = _nvcc()
    os.makedirs(out_dir, exist_ok=True)
    flags = [f for f in NVCC_FLAGS if not (drop_o3 and f == "-O3")] + (["-O1"] if drop_o3 else [])
    lib = os.path.join(out_dir, name)
    hdrs = _headers()
    objs, jobs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(out_dir, src.replace(".cu", ".o"))
        objs.append(o)
        if _newer(o, [s] + hdrs):
            jobs.append([nvcc] + ARCH + flags + flags_extra + ["-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for r in ex.map(lambda cmd: subprocess.run(cmd, capture_output=True, text=True), jobs):
                if r.returncode:
                    raise RuntimeError("nvcc failed (%s): %s" % (name, r.stderr[-2000:]))
    if jobs or _newer(lib, objs):
        r = subprocess.run([nvcc] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"] + link_extra,
                           capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError("link failed (%s): %s" % (name, r.stderr[-2000:]))
    return lib


def build_sanitized(out_dir):
    """The library with AddressSanitizer and UndefinedBehaviorSanitizer in its
    host code (the file parsers, the C-ABI argument checks, the hierarchy
    set-up), for tests that load it with the sanitizer runtime preloaded;
    device code is compiled as usual.  Returns the path of the .so."""
    # one option per -Xcompiler: nvcc splits its argument at commas
    san = ["-Xcompiler", "-fsanitize=address", "-Xcompiler", "-fsanitize=undefined", "-Xcompiler",
           "-fno-omit-frame-pointer", "-Xcompiler", "-fno-sanitize-recover=undefined", "-g"]
    return _build_variant(out_dir, "libug4gb_asan.so", san,
                          ["-Xcompiler", "-fsanitize=address", "-Xcompiler", "-fsanitize=undefined"], drop_o3=True)


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
