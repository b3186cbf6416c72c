"""Build recipe for libnsg.so (sm_103a) — plain nvcc, no cmake.

Every .cu under nscale_gb300/csrc is compiled to an object in parallel, then
linked into nscale_gb300/libnsg.so (git-ignored, built in-tree).
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libnsg.so")
OBJ = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
         "-Xcompiler", "-ffp-contract=off",  # host double math rounds like the oracle's (no fused multiply-add)
         "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stamp(srcs) -> str:
    h = hashlib.sha256()
    for p in srcs + sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))):
        h.update(p.encode())
        with open(p, "rb") as f:
            h.update(f.read())
    with open(os.path.join(HERE, "..", "include", "nsg.h"), "rb") as f:
        h.update(f.read())
    h.update(" ".join(ARCH + FLAGS).encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    srcs = _sources()
    stamp = _stamp(srcs) + ("" if not extra else "|" + " ".join(extra))
    stamp_file = os.path.join(OBJ, "stamp")
    if not force and os.path.exists(OUT) and os.path.exists(stamp_file):
        with open(stamp_file) as f:
            if f.read() == stamp:
                return OUT
    os.makedirs(OBJ, exist_ok=True)
    objs = []
    cmds = []
    for s in srcs:
        o = os.path.join(OBJ, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        cmds.append([nvcc(), *ARCH, *FLAGS, *(extra or []), "-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with cf.ThreadPoolExecutor(max_workers=min(len(cmds), os.cpu_count() or 4)) as ex:
        for cmd, r in ex.map(run, cmds):
            if verbose or r.returncode != 0:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed for {cmd[-3]}")
    tmp = OUT + ".tmp"
    link = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static" if False else "-cudart=static"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(link) + "\n" + r.stdout + r.stderr)
        raise RuntimeError("link failed")
    os.replace(tmp, OUT)
    with open(stamp_file, "w") as f:
        f.write(stamp)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
