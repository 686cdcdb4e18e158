"""Builds libshci_gpu.so (the C-ABI library) in-tree, for sm_103a only.

Translation units are compiled in parallel with nvcc (CUDA) and g++ (host C++), then linked
with the static CUDA runtime.  Output: shci_gb300/lib/libshci_gpu.so.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libshci_gpu.so")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
                  "--expt-relaxed-constexpr", "-I", CSRC]
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-pthread", "-ffp-contract=off"]


def sources():
    out = []
    for f in sorted(os.listdir(CSRC)):
        if f.endswith(".cu") or f.endswith(".cc"):
            out.append(os.path.join(CSRC, f))
    return out


def _compile(src, verbose):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC)
                    if h.endswith((".h", ".cuh"))]
    deps.append(os.path.join(HERE, "..", "include", "shci_gpu.h"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj, ""
    if src.endswith(".cu"):
        cmd = [NVCC] + NVFLAGS + ["-c", src, "-o", obj]
        if verbose:
            cmd += ["-Xptxas", "-v"]
    else:
        cmd = ["g++"] + CXXFLAGS + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj, r.stderr


def build(verbose=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log:
                sys.stderr.write(log)
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s" % (r.stdout, r.stderr))
    build_cli()
    return LIB


CLI_SRC = os.path.join(HERE, "cli", "main.cc")
CLI = os.path.join(HERE, "bin", "shci_gpu")


def build_cli():
    """The drop-in driver: links only the C ABI of libshci_gpu.so."""
    os.makedirs(os.path.dirname(CLI), exist_ok=True)
    deps = [CLI_SRC, os.path.join(HERE, "cli", "json.h"), os.path.join(HERE, "cli", "wf_file.h"),
            LIB]
    if os.path.exists(CLI) and os.path.getmtime(CLI) >= max(os.path.getmtime(d) for d in deps):
        return CLI
    cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(HERE, "..", "include"), CLI_SRC,
           "-o", CLI, "-L", LIBDIR, "-lshci_gpu", "-Wl,-rpath,$ORIGIN/../lib"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("CLI build failed: %s\n%s" % (" ".join(cmd), r.stderr))
    return CLI


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
