"""In-tree build of the engine: every .cpp / .cu under csrc/ into
lib/libsankhya_gb300.so (sm_103a only) plus the JSON-telemetry CLI lib/sankhya_cli.

Usage: python build.py [-j N] [--force]
"""
import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "lib", "obj")
LIB = os.path.join(HERE, "lib", "libsankhya_gb300.so")
CLI = os.path.join(HERE, "lib", "sankhya_cli")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
INC = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC, "-I" + os.path.join(CUDA, "include")]
CXXFLAGS = ["-O2", "-fPIC", "-std=c++17", "-Wall", "-Wno-unused-function"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                  "-Xptxas", "-warn-spills"]


def sources():
    out = []
    for d, _, files in os.walk(CSRC):
        for f in sorted(files):
            if f.endswith((".cpp", ".cu")) and "cli" not in os.path.relpath(d, CSRC).split(os.sep):
                out.append(os.path.join(d, f))
    return sorted(out)


def headers_mtime():
    t = 0.0
    for base in (CSRC, os.path.join(ROOT, "include")):
        for d, _, files in os.walk(base):
            for f in files:
                if f.endswith((".h", ".hpp", ".cuh")):
                    t = max(t, os.path.getmtime(os.path.join(d, f)))
    return t


def obj_of(src):
    rel = os.path.relpath(src, CSRC).replace(os.sep, "__")
    return os.path.join(OBJ, rel + ".o")


def compile_one(src, force, hdr_t):
    obj = obj_of(src)
    if not force and os.path.exists(obj):
        ot = os.path.getmtime(obj)
        if ot > os.path.getmtime(src) and ot > hdr_t:
            return obj, ""
    if src.endswith(".cu"):
        cmd = [NVCC] + NVFLAGS + INC + ["-c", src, "-o", obj]
    else:
        # the seeded LP generator gives the same bits on every host (no FMA contraction)
        extra = ["-ffp-contract=off"] if os.path.basename(src) == "lpgen.cpp" else []
        cmd = ["g++"] + CXXFLAGS + extra + INC + ["-c", src, "-o", obj]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), p.stdout, p.stderr))
    return obj, (p.stdout + p.stderr).strip()


def build(jobs=None, force=False, verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    if not os.path.exists(NVCC):
        raise RuntimeError("nvcc not found at %s" % NVCC)
    hdr_t = headers_mtime()
    srcs = sources()
    jobs = jobs or min(16, os.cpu_count() or 4)
    objs = []
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = {ex.submit(compile_one, s, force, hdr_t): s for s in srcs}
        for f in cf.as_completed(futs):
            obj, log = f.result()
            objs.append(obj)
            if log and verbose:
                print(log, file=sys.stderr)
    objs.sort()
    newest = max(os.path.getmtime(o) for o in objs)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [NVCC] + ARCH + ["-shared", "-cudart", "shared", "-o", LIB] + objs + \
              ["-Xlinker", "-rpath," + os.path.join(CUDA, "lib64"), "-lpthread"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("link failed: %s\n%s" % (p.stdout, p.stderr))
    cli_src = os.path.join(CSRC, "cli", "sankhya_cli.cpp")
    if os.path.exists(cli_src) and (force or not os.path.exists(CLI) or
                                    os.path.getmtime(CLI) < max(os.path.getmtime(LIB), os.path.getmtime(cli_src))):
        cmd = ["g++"] + CXXFLAGS[:-2] + ["-O2", "-std=c++17"] + INC + [cli_src, "-o", CLI,
                                                                      "-L" + os.path.dirname(LIB), "-lsankhya_gb300",
                                                                      "-Wl,-rpath,$ORIGIN"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("cli link failed: %s\n%s" % (p.stdout, p.stderr))
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("-j", type=int, default=None)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", action="store_true")
    a = ap.parse_args()
    print(build(a.j, a.force, a.v))
