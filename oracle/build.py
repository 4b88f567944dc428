"""ORACLE — test infrastructure only.

Builds the oracle's C++ restatement (oracle/mb_oracle.cpp) into
oracle/_build/libmb_oracle.so, and, when the reference tree is present,
oracle/_ref/libmbref.so from the reference's own sources (build_ref.sh).
Flags keep results identical across x86 and Arm: no -march, no FMA
contraction.

build_baseline() builds the same source a second time, as the CPU
baseline, with the flags of the reference's own solver-cpu build
(solver-cpu/CMakeLists.txt: -O3, OpenMP, USE_OMP_SIMD=1, the compiler's
default FP contraction) into oracle/_build/libmb_baseline.so. The
reference's -march=native is replaced by the host CPU's named target
(Arm: -mcpu of the Neoverse core the machine reports, e.g. neoverse-v2 on
Grace, with +nosve where the kernel does not report SVE; x86:
-march=x86-64-v3), kept only if a small vectorised probe built with it
runs on the host, so that the build does not depend on the machine beyond
its CPU model. Only timed, never used as the checker.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libmb_oracle.so")
BASELINE_SO = os.path.join(HERE, "_build", "libmb_baseline.so")
REF_SO = os.path.join(HERE, "_ref", "libmbref.so")
REF_BASELINE_SO = os.path.join(HERE, "_ref", "libmbref_baseline.so")
# the mbsolve source tree: $MBSOLVE_REFERENCE, else a checkout named
# "reference" beside this repository
REFERENCE_ROOT = os.environ.get("MBSOLVE_REFERENCE") or os.path.normpath(
    os.path.join(HERE, "..", "..", "reference"))


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


def _cxx_accepts(flag):
    r = subprocess.run([os.environ.get("CXX", "g++"), flag, "-x", "c++",
                        "-fsyntax-only", "-"], input="int main(){}",
                       capture_output=True, text=True)
    return r.returncode == 0


def _cxx_runs(flags):
    """A vectorised, OpenMP-SIMD loop built with `flags` runs on this host:
    a CPU model's target can use extensions (SVE on Arm) that the running
    kernel does not enable."""
    import tempfile
    src = ("#include <cstdio>\nint main() { float a[512], b[512], s = 0.f;\n"
           "for (int i = 0; i < 512; i++) { a[i] = i * 0.5f; b[i] = 2.f - i; }\n"
           "#pragma omp simd reduction(+ : s)\n"
           "for (int i = 0; i < 512; i++) s += a[i] * b[i] + a[i] / (1.f + b[i] * b[i]);\n"
           "std::printf(\"%g\\n\", s); return 0; }\n")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "probe")
        r = subprocess.run([os.environ.get("CXX", "g++"), "-O3", "-fopenmp"] +
                           flags + ["-x", "c++", "-", "-o", exe], input=src,
                           capture_output=True, text=True)
        if r.returncode != 0:
            return False
        try:
            return subprocess.run([exe], capture_output=True,
                                  timeout=20).returncode == 0
        except (OSError, subprocess.TimeoutExpired):
            return False


def _cpuinfo(key):
    """The first value of `key` in /proc/cpuinfo (lower case), or None."""
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(key):
                    return line.split(":", 1)[1].strip().lower()
    except OSError:
        pass
    return None


def cpu_target_flags():
    """The named target for this host CPU (see the module docstring), with
    SVE switched off where the kernel does not report it (virtual machines
    may hide it), and kept only if a probe built with it runs here."""
    import platform
    m = platform.machine()
    if m in ("aarch64", "arm64"):
        part = _cpuinfo("cpu part")
        # Arm Ltd. part numbers of the Neoverse cores
        names = {"0xd4f": "neoverse-v2", "0xd40": "neoverse-v1",
                 "0xd0c": "neoverse-n1", "0xd49": "neoverse-n2",
                 "0xd84": "neoverse-v3"}
        flag = "-mcpu=" + names.get(part, "neoverse-v2")
        feats = (_cpuinfo("features") or "").split()
        if "sve" not in feats and "n1" not in flag:
            flag += "+nosve"
    elif m in ("x86_64", "AMD64"):
        flag = "-march=x86-64-v3"
    else:
        return []
    return [flag] if _cxx_accepts(flag) and _cxx_runs([flag]) else []


def baseline_flags():
    return ["-O3", "-fopenmp", "-DUSE_OMP_SIMD=1"] + cpu_target_flags()


def build_baseline(force=False):
    """The CPU-baseline build of mb_oracle.cpp (reference flags)."""
    src = os.path.join(HERE, "mb_oracle.cpp")
    if not _arch_ok(BASELINE_SO):
        force = True
    hdr = os.path.join(HERE, "..", "include", "mbsolve_gb300.h")
    if not force and not _stale(BASELINE_SO, [src, hdr, __file__]):
        return BASELINE_SO
    os.makedirs(os.path.dirname(BASELINE_SO), exist_ok=True)
    tmp = BASELINE_SO + ".tmp%d" % os.getpid()
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-fPIC", "-shared"] + \
        baseline_flags() + [src, "-o", tmp]
    subprocess.check_call(cmd)
    os.replace(tmp, BASELINE_SO)
    _write_arch(BASELINE_SO)
    return BASELINE_SO


def build_reference(force=False, baseline=False):
    """Build oracle/_ref from the reference tree; None when it is absent.
    baseline=True: the same sources with the CPU baseline's flags
    (libmbref_baseline.so), to calibrate the restated baseline against the
    reference's own loops on a machine that has the reference tree."""
    if not os.path.isdir(os.path.join(REFERENCE_ROOT, "mbsolve-lib", "src")):
        return None
    out = REF_BASELINE_SO if baseline else REF_SO
    srcs = [os.path.join(HERE, f) for f in
            ("ref_driver.cpp", "ref_algos.hpp", "mb_oracle.cpp",
             "build_ref.sh")]
    if not force and _arch_ok(out) and not _stale(out, srcs):
        return out
    env = dict(os.environ)
    if baseline:
        env["REF_CXXFLAGS"] = " ".join(baseline_flags())
        env["REF_LIB"] = os.path.basename(out)
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh"),
                           REFERENCE_ROOT], env=env)
    _write_arch(out)
    return out


if __name__ == "__main__":
    print(build_oracle(force="-f" in sys.argv))
    print(build_baseline(force="-f" in sys.argv))
    print(build_reference(force="-f" in sys.argv))
