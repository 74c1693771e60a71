"""Build libpimdgpu.so (the C-ABI library) in-tree with nvcc for sm_103a.

Each .cu translation unit is compiled in parallel, then linked with -shared.
Outputs go to pimd-tunneling_gb300/lib/ (git-ignored).
"""
import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "lib")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
# Host code: no floating-point contraction (-ffp-contract=off), so that host
# arithmetic gives the same bits on x86_64 and aarch64 (where GCC would
# otherwise fuse a*b + c into an FMA) and matches numpy.
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr",
         "-I" + os.path.join(HERE, "..", "include")]
SOURCES = ["pg_api.cu", "pg_ti.cu", "pg_tc.cu", "pg_instanton.cu"]
DRIVERS = ["pimd_ti", "rpi", "crossover"]  # C++ front ends (host/*.cpp), linked against libpimdgpu.so


def _compile(src, verbose=False):
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(HERE, "..", "include", "pimdgpu.h"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj, ""
    cmd = [NVCC] + ARCH + FLAGS + (["-Xptxas", "-v"] if verbose else []) + ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj, r.stderr


def build(verbose=False):
    """Compile every translation unit and link lib/libpimdgpu.so; returns its path."""
    os.makedirs(OUT, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log:
                sys.stderr.write(log)
    so = os.path.join(OUT, "libpimdgpu.so")
    if not os.path.exists(so) or os.path.getmtime(so) < max(os.path.getmtime(o) for o in objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", so] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    for d in DRIVERS:
        src = os.path.join(HERE, "host", d + ".cpp")
        exe = os.path.join(OUT, d)
        deps = [src, so] + glob.glob(os.path.join(HERE, "host", "*.hpp"))
        if os.path.exists(exe) and os.path.getmtime(exe) >= max(os.path.getmtime(p) for p in deps):
            continue
        cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe, src, "-L" + OUT,
               "-lpimdgpu",
               "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("driver build failed for %s:\n%s\n%s" % (d, r.stdout, r.stderr))
    return so


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
