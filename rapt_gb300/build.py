"""Build librapt_gpu.so in-tree for sm_103a.

Each translation unit under csrc/ is compiled by its own nvcc process in
parallel (one ``-gencode``), then linked into ``rapt_gb300/librapt_gpu.so``.
Objects go to ``rapt_gb300/_build/`` and are rebuilt only when a source or
header is newer than the object.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librapt_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-diag-suppress", "177"]


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _deps():
    hdrs = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
    hdrs.append(os.path.join(HERE, "..", "include", "rapt_gpu.h"))
    return max(os.path.getmtime(h) for h in hdrs)


def build(verbose=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdr_t = _deps()
    cmds, objs = [], []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if os.path.exists(o) and os.path.getmtime(o) >= max(os.path.getmtime(s), hdr_t):
            continue
        cmds.append([nvcc(), *ARCH, *FLAGS, "-c", s, "-o", o])
    jobs = jobs or min(len(cmds) or 1, os.cpu_count() or 4)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        if verbose:
            sys.stdout.write(r.stdout + r.stderr)
        return cmd[-1]

    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        list(ex.map(run, cmds))
    need_link = bool(cmds) or not os.path.exists(LIB) or any(
        os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs)
    if need_link:
        tmp = LIB + ".tmp"
        r = subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
