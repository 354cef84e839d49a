"""Build libcomdgb.so in-tree for sm_103a (GB300).

Each translation unit is compiled by nvcc in parallel, then linked into
``comd_gb300/libcomdgb.so`` (git-ignored).  The FP64 force kernels and the
integrator/rebinning kernels are compiled with ``-fmad=false`` so their
double-precision arithmetic rounds operation by operation like the
reference; the mixed-precision force kernels and the host API keep FMA.

The C host ``comd_gb300/comdgb_run`` (``host/comdgb_run.c``: the
reference's do_compute_work loop on the drop-in boundary) is linked
against the library with gcc, as a maintainer would link the reference's
own host.

Usage: ``python -m comd_gb300.build [--force]``.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT = os.path.join(HERE, "libcomdgb.so")
HOST_SRC = os.path.join(HERE, "host", "comdgb_run.c")
HOST_OUT = os.path.join(HERE, "comdgb_run")
OBJDIR = os.path.join(HERE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                  "-I", INCLUDE, "-I", CSRC]
# extra nvcc flags (e.g. -DCOMDGB_FO_PREFETCH=4 for a parameter sweep)
NVFLAGS += os.environ.get("COMDGB_NVCC_EXTRA", "").split()
# (source, extra flags)
UNITS = [
    ("md_kernels.cu", ["-fmad=false"]),
    ("force_fp64.cu", ["-fmad=false"]),
    ("force_mixed.cu", []),
    ("api.cu", []),
    ("noalloc.cu", ["-fmad=false"]),
    ("adjoint.cu", []),
    ("virial.cu", []),
    ("clsman_io.cu", []),
    ("centro.cu", ["-fmad=false"]),
    ("autotune.cu", []),
    ("probes.cu", []),
]
CUNITS = ["host_setup.c"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [HOST_SRC]
    files += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    files.append(os.path.abspath(__file__))
    return max(os.path.getmtime(f) for f in files)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _have_zlib():
    """zlib headers and library present (gzip clsman input); probed by a test link"""
    src = os.path.join(OBJDIR, "zprobe.c")
    with open(src, "w") as f:
        f.write("#include <zlib.h>\nint main(void) { return zlibVersion() == 0; }\n")
    r = subprocess.run(["gcc", src, "-o", os.path.join(OBJDIR, "zprobe"), "-lz"],
                       capture_output=True, text=True)
    return r.returncode == 0


def build_host():
    """the C host, linked with -lcomdgb (rpath: the library beside it)"""
    tmp = HOST_OUT + ".tmp"
    _run(["gcc", "-O2", "-std=c11", "-Wall", "-I", INCLUDE, HOST_SRC, "-o", tmp, "-L", HERE,
          "-lcomdgb", "-Wl,-rpath,$ORIGIN"])
    os.replace(tmp, HOST_OUT)
    return HOST_OUT


def build(force=False, verbose=False):
    """Compile (if sources are newer than the library) and return its path."""
    if not force and all(os.path.exists(f) and os.path.getmtime(f) >= _deps()
                         for f in (OUT, HOST_OUT)):
        return OUT
    os.makedirs(OBJDIR, exist_ok=True)
    nvcc = _nvcc()
    zlib = _have_zlib()
    zdef = ["-DCOMDGB_HAVE_ZLIB"] if zlib else []
    jobs = []
    for src, extra in UNITS:
        obj = os.path.join(OBJDIR, src.replace(".cu", ".o"))
        jobs.append(([nvcc] + NVFLAGS + extra + zdef + ["-c", os.path.join(CSRC, src), "-o", obj],
                     obj))
    for src in CUNITS:
        obj = os.path.join(OBJDIR, src.replace(".c", ".o"))
        jobs.append((["gcc", "-O2", "-fPIC", "-std=c11", "-Wall", "-I", INCLUDE]
                     + zdef
                     + ["-c", os.path.join(CSRC, src), "-o", obj], obj))
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        logs = list(ex.map(lambda j: _run(j[0]), jobs))
    if verbose:
        for log in logs:
            if log.strip():
                print(log)
    tmp = OUT + ".tmp"
    _run([nvcc] + ARCH + ["-shared", "-o", tmp] + [o for _, o in jobs] + ["-lm"]
         + (["-lz"] if zlib else []))
    os.replace(tmp, OUT)
    build_host()
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
