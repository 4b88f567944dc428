"""Builds the CUDA engine into mbsolve_gb300/libmbsolve_gb300.so.

nvcc for sm_103a only; translation units compile in parallel, then one
shared library is linked (static CUDA runtime). Run as a script or call
build(). Set MBG_PTXAS_VERBOSE=1 for register/spill reports.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmbsolve_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith(".cu"))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
          if f.endswith((".cuh", ".hpp", ".h"))]
    hs.append(os.path.join(HERE, "..", "include", "mbsolve_gb300.h"))
    hs.append(os.path.join(HERE, "..", "include", "mbsolve_fno.h"))
    return hs


def _flags():
    f = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
         "--expt-relaxed-constexpr", "-Xcompiler", "-ffp-contract=off"] + ARCH
    if os.environ.get("MBG_PTXAS_VERBOSE"):
        f += ["-Xptxas", "-v"]
    return f


def _arch_stamp_ok():
    """Objects built on another machine type (the tree is copied between
    x86 and Arm hosts) must be rebuilt."""
    import platform
    stamp = os.path.join(BUILD, "ARCH")
    here = platform.machine()
    ok = os.path.exists(stamp) and open(stamp).read().strip() == here
    if not ok:
        with open(stamp, "w") as f:
            f.write(here + "\n")
    return ok


def build(force=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    if not _arch_stamp_ok():
        force = True
    srcs = _sources()
    hdr_time = max(os.path.getmtime(h) for h in _headers())
    objs = []
    todo = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or not os.path.exists(o) or \
                os.path.getmtime(o) < max(os.path.getmtime(s), hdr_time):
            todo.append((s, o))
    cmdbase = [nvcc()] + _flags()

    def compile_one(so):
        s, o = so
        tmp = o + ".tmp%d" % os.getpid()
        r = subprocess.run(cmdbase + ["-c", s, "-o", tmp],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" %
                               (s, r.stdout, r.stderr))
        os.replace(tmp, o)
        return s, r.stdout + r.stderr

    jobs = jobs or max(1, min(len(todo), os.cpu_count() or 4))
    logs = []
    if todo:
        with cf.ThreadPoolExecutor(jobs) as ex:
            for s, log in ex.map(compile_one, todo):
                logs.append((s, log))
    if todo or force or not os.path.exists(LIB) or \
            os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + \
            ["-Xcompiler", "-fPIC", "-lcudart_static", "-ldl", "-lrt",
             "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
        os.replace(tmp, LIB)
    if os.environ.get("MBG_PTXAS_VERBOSE"):
        for s, log in logs:
            sys.stderr.write("== %s\n%s" % (os.path.basename(s), log))
    return LIB


if __name__ == "__main__":
    print(build(force="-f" in sys.argv))
