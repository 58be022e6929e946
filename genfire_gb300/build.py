"""Build libgenfire.so (sm_103a) in-tree.

The CUDA sources under ``csrc/`` are compiled to objects in parallel with
nvcc and linked into ``genfire_gb300/_build/libgenfire.so`` (static CUDA
runtime, so the library only needs the driver).  Host code is compiled with
``-ffp-contract=off``: the FP32 projection geometry feeding the bit-exact
K-point selection must round every operation as written.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libgenfire.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math", "-I", INCLUDE]


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libgenfire")
    return cand


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    return ([os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "genfire.h")]
            + [os.path.join(HERE, "harness", f) for f in os.listdir(os.path.join(HERE, "harness"))])


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra_flags=()):
    """Compile and link libgenfire.so if any source changed; return its path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = _deps()
    if not force and not _stale(LIB, deps):
        return LIB
    exe = nvcc()
    srcs = sources()
    objs = [os.path.join(OUT_DIR, os.path.basename(s)[:-3] + ".o") for s in srcs]

    def compile_one(pair):
        src, obj = pair
        cmd = [exe] + NVCC_FLAGS + list(extra_flags) + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        return r.stdout + r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        for log in ex.map(compile_one, zip(srcs, objs)):
            if verbose and log.strip():
                print(log)
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = [exe] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    build_harness()
    return LIB


HARNESS_SRC = [os.path.join(HERE, "harness", f) for f in ("genfire_run.c", "matio.c")]
HARNESS = os.path.join(OUT_DIR, "genfire_run")


def build_harness():
    """The standalone C driver (harness/genfire_run.c with the MAT-file reader and
    writer harness/matio.c), linked against libgenfire.so."""
    cmd = ["gcc", "-O2", "-std=c11", "-Wall", "-I", INCLUDE] + HARNESS_SRC + ["-o", HARNESS, "-L", OUT_DIR, "-lgenfire",
           "-Wl,-rpath,$ORIGIN", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("harness build failed:\n%s\n%s" % (r.stdout, r.stderr))
    return HARNESS


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose=True, extra_flags=sys.argv[1:]))
