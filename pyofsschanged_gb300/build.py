"""Build libgnlse.so in-tree with nvcc for sm_103a.

Every ``csrc/*.cu`` translation unit is compiled in parallel to an object in
``csrc/_build/`` and the objects are linked into ``pyofsschanged_gb300/libgnlse.so``.
Objects are rebuilt only when a source or header is newer than the object.

    python -m pyofsschanged_gb300.build [-j JOBS] [--force]
"""

import argparse
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
_TAG = os.environ.get("GNLSE_BUILD_TAG", "")
BUILD = os.path.join(CSRC, "_build" + (("_" + _TAG) if _TAG else ""))
LIB = os.path.join(HERE, "libgnlse%s.so" % (("_" + _TAG) if _TAG else ""))
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I" + CSRC, "-I" + INCLUDE] + \
    os.environ.get("GNLSE_NVCC_FLAGS", "").split()


def nvcc():
    exe = shutil.which("nvcc")
    if exe is None:
        cand = "/usr/local/cuda/bin/nvcc"
        if os.path.exists(cand):
            return cand
        raise RuntimeError("nvcc not found")
    return exe


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(CSRC, "*.inc")) + glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(src, obj, newest_header):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return os.path.getmtime(src) > t or newest_header > t


def _compile(src, obj):
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stderr[-4000:]}")
    return obj


def build(jobs=None, force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    units = os.environ.get("GNLSE_UNITS")  # optional regex: build a subset of units
    if units:
        import re
        srcs = [s for s in srcs if re.search(units, os.path.basename(s))]
    hdr = max([os.path.getmtime(h) for h in _headers()] + [0.0])
    todo, objs = [], []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or _stale(s, o, hdr):
            todo.append((s, o))
    jobs = jobs or max(1, os.cpu_count() or 1)
    if todo:
        if verbose:
            print(f"[gnlse build] compiling {len(todo)} units with {jobs} jobs", flush=True)
        with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
            futs = [ex.submit(_compile, s, o) for s, o in todo]
            for f in cf.as_completed(futs):
                f.result()
    lib_stale = force or not os.path.exists(LIB) or any(
        os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs)
    if lib_stale:
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr[-4000:])
    return LIB


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("-j", "--jobs", type=int, default=None)
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args(argv)
    print(build(a.jobs, a.force, verbose=True))


if __name__ == "__main__":
    sys.exit(main())
