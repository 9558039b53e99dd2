"""Builds the CUDA library librpm_gb300.so in-tree for sm_103a.

rpm_exact.cu and rpm_noalloc.cu are compiled with --fmad=false (no contracted
multiply-add, so the exact forms round like the CPU restatement); rpm_fast.cu and rpm_api.cu with
the default contraction.  Translation units compile in parallel.
"""
import concurrent.futures as cf
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "librpm_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]
UNITS = {"rpm_exact.cu": ["--fmad=false"], "rpm_fast.cu": ["--fmad=true"], "rpm_api.cu": [],
         "rpm_noalloc.cu": ["--fmad=false"], "rpm_server.cu": [], "rpm_io.cu": []}


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh"))]
    files.append(os.path.join(HERE, "..", "include", "rpm_gpu.h"))
    return files


def _up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def nvcc():
    cand = os.environ.get("NVCC")
    if cand:
        return cand
    for p in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(p):
            return p
    return "nvcc"


ADAPTER_DIR = os.path.join(HERE, "adapter")
ADAPTER_LIB = os.path.join(OUT_DIR, "librpm_adapter.so")


def adapter_flags():
    """Include flags for code built on the RealVectorSpaceGPU adapter (its
    StateSpace / State / Eigen stand-ins, the adapter and the C ABI)."""
    return ["-I", os.path.join(ADAPTER_DIR, "shim"), "-I", ADAPTER_DIR, "-I", os.path.join(HERE, "..", "include")]


def build_adapter(force=False):
    """The C++ RealVectorSpaceGPU adapter as librpm_adapter.so (host code on the C ABI)."""
    src = os.path.join(ADAPTER_DIR, "RealVectorSpaceGPU.cpp")
    deps = [src, os.path.join(ADAPTER_DIR, "RealVectorSpaceGPU.h"), LIB]
    for d, _, files in os.walk(os.path.join(ADAPTER_DIR, "shim")):
        deps += [os.path.join(d, f) for f in files]
    if not force and os.path.exists(ADAPTER_LIB) and all(os.path.getmtime(f) <= os.path.getmtime(ADAPTER_LIB) for f in deps):
        return ADAPTER_LIB
    tmp = ADAPTER_LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc(), "-std=c++17", "-O2", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-shared", "-x", "c++",
           src, *adapter_flags(),
           "-L", OUT_DIR, "-lrpm_gb300", "-Xlinker", "-rpath=" + OUT_DIR, "-lcudart", "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("adapter build failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, ADAPTER_LIB)
    return ADAPTER_LIB


def build(force=False, verbose=False):
    if not force and _up_to_date():
        build_adapter()
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)

    def compile_one(item):
        src, extra = item
        obj = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
        cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        results = list(ex.map(compile_one, UNITS.items()))
    if verbose:
        for _, log in results:
            print(log)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp] + [o for o, _ in results]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    build_adapter(force=True)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="-f" in sys.argv, verbose="-v" in sys.argv))
