"""Builds the CUDA library libvec_gpu.so (sm_103a) in-tree with nvcc.

Each translation unit is compiled in parallel, then linked into
fug30v0kxc_gb300/_lib/libvec_gpu.so.  Host code is compiled with
-ffp-contract=off so host-side tables come out identical on x86_64 and
aarch64.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libvec_gpu.so")
SOURCES = ["capi.cu", "lines.cu", "lines_ct.cu", "physics.cu", "split.cu", "noalloc.cu", "ensemble.cu", "closure_net.cu", "closure.cu", "peaks.cu", "netcdf_io.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def flags(extra=()):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
                   "-I" + os.path.join(HERE, "..", "include")] + list(extra)


def build(force=False, verbose=False, extra=()):
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    deps = srcs + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    deps.append(os.path.join(HERE, "..", "include", "vec.h"))
    deps.append(os.path.join(HERE, "host", "p3d_gpu.c"))
    deps.append(os.path.join(HERE, "host", "interp_gpu.c"))
    if not force and os.path.exists(LIB) and os.path.exists(HOST) and os.path.exists(INTERP):
        t = min(os.path.getmtime(LIB), os.path.getmtime(HOST), os.path.getmtime(INTERP))
        if all(os.path.getmtime(d) <= t for d in deps):
            return LIB
    objs = [os.path.join(OUT, os.path.splitext(os.path.basename(s))[0] + ".o") for s in srcs]

    def comp(pair):
        s, o = pair
        cmd = [nvcc(), "-c", s, "-o", o] + (flags(extra) if s.endswith(".cu") else
                                            ["-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-std=c++17"])
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {s}:\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        for msg in ex.map(comp, zip(srcs, objs)):
            if verbose and msg:
                print(msg)
    cmd = [nvcc(), "-shared", "-o", LIB + ".tmp"] + objs + ARCH + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(LIB + ".tmp", LIB)
    build_host(verbose)
    return LIB


HOST = os.path.join(OUT, "p3d_gpu")
INTERP = os.path.join(OUT, "interp_gpu")


def build_host(verbose=False):
    """The C host programs: p3d_gpu (src/main.F90) and interp_gpu
    (interpolate/main.F90) on the GPU library."""
    cc = shutil.which("gcc") or "cc"
    for name, exe in (("p3d_gpu.c", HOST), ("interp_gpu.c", INTERP)):
        src = os.path.join(HERE, "host", name)
        cmd = [cc, "-O2", "-std=gnu11", "-ffp-contract=off", "-I" + os.path.join(HERE, "..", "include"), src,
               "-o", exe, "-L" + OUT, "-lvec_gpu", "-lm", "-Wl,-rpath,$ORIGIN"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"host program build failed:\n{r.stdout}\n{r.stderr}")
    return HOST


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True,
          extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else ())
    print(LIB)
