"""ORACLE — test infrastructure only.

Builds the oracle's C++ restatement (oracle/mb_oracle.cpp) into
oracle/_build/libmb_oracle.so, and, when the reference tree is present,
oracle/_ref/libmbref.so from the reference's own sources (build_ref.sh).
Flags keep results identical across x86 and Arm: no -march, no FMA
contraction.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libmb_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libmbref.so")
REFERENCE_ROOT = os.environ.get("MBSOLVE_REFERENCE", "/root/reference")


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _arch_ok(path):
    import platform
    stamp = path + ".arch"
    ok = os.path.exists(stamp) and open(stamp).read().strip() == \
        platform.machine()
    return ok


def _write_arch(path):
    import platform
    with open(path + ".arch", "w") as f:
        f.write(platform.machine() + "\n")


def build_oracle(force=False):
    src = os.path.join(HERE, "mb_oracle.cpp")
    if not _arch_ok(ORACLE_SO):
        force = True
    hdr = os.path.join(HERE, "..", "include", "mbsolve_gb300.h")
    if not force and not _stale(ORACLE_SO, [src, hdr]):
        return ORACLE_SO
    os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
    tmp = ORACLE_SO + ".tmp%d" % os.getpid()
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fopenmp",
           "-fPIC", "-shared", "-ffp-contract=off", src, "-o", tmp]
    subprocess.check_call(cmd)
    os.replace(tmp, ORACLE_SO)
    _write_arch(ORACLE_SO)
    return ORACLE_SO


def build_reference(force=False):
    """Build oracle/_ref from the reference tree; None when it is absent."""
    if not os.path.isdir(os.path.join(REFERENCE_ROOT, "mbsolve-lib", "src")):
        return None
    srcs = [os.path.join(HERE, f) for f in
            ("ref_driver.cpp", "ref_algos.hpp", "mb_oracle.cpp")]
    if not force and _arch_ok(REF_SO) and not _stale(REF_SO, srcs):
        return REF_SO
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh"),
                           REFERENCE_ROOT])
    _write_arch(REF_SO)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="-f" in sys.argv))
    print(build_reference(force="-f" in sys.argv))
