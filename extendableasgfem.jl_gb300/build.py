"""Build libsgfem.so (the sm_103a CUDA library behind include/sgfem.h) in place.

Each translation unit under csrc/ is compiled by nvcc in parallel for
sm_103a only, then linked into a shared library next to this file.  No
CMake, no torch extension machinery: the library is plain C ABI.
"""
import concurrent.futures
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libsgfem.so")
BUILD = os.path.join(HERE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-Xcompiler", "-fvisibility=hidden"]


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _toolchain_stamp():
    """nvcc version, target architecture, flags and host machine: a change of
    any of them invalidates every object (x86 objects never link on Arm)."""
    v = subprocess.run([nvcc(), "--version"], capture_output=True, text=True).stdout.strip()
    return "\n".join([v, " ".join(ARCH), " ".join(FLAGS), platform.machine()])


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, ptxas_verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    stamp_path = os.path.join(BUILD, "toolchain.stamp")
    stamp = _toolchain_stamp()
    try:
        old = open(stamp_path).read()
    except OSError:
        old = None
    if old != stamp:
        force = True
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "sgfem.h"))
    objs = []
    jobs = []
    for src in sources():
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmd = [nvcc()] + ARCH + FLAGS + (["-Xptxas", "-v"] if ptxas_verbose else []) + ["-c", src, "-o", obj]
            jobs.append(cmd)
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        for cmd, r in zip(jobs, results):
            if verbose or ptxas_verbose or r.returncode != 0:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed for " + cmd[-3])
    linked = False
    if force or jobs or _stale(OUT, objs):
        tmp = OUT + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
        os.replace(tmp, OUT)
        linked = True
    with open(stamp_path, "w") as f:
        f.write(stamp)
    sys.stderr.write(f"libsgfem build: {len(jobs)} of {len(objs)} units compiled, "
                     f"{'linked' if linked else 'up to date'} ({platform.machine()})\n")
    return OUT


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, ptxas_verbose="--ptxas" in sys.argv, force="--force" in sys.argv)
    print(OUT)
