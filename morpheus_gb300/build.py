"""In-tree build of the CUDA C-ABI library for sm_103a.

Every ``csrc/*.cu`` is compiled by nvcc in parallel into ``_build/`` and linked
into ``libmorpheus_gb300.so``; the same objects also go into the static archive
``libmorpheus_gb300.a``.  The two library names the reference crates link
(``goldilocks_cuda_wrapper``, ``almost_goldilocks_cuda_wrapper``, see
goldilocks-cuda-rs/build.rs:157-164 and almost-goldilocks-cuda-rs/build.rs:115-117)
are provided as symlinks to each, so a crate's ``cargo:rustc-link-lib`` line (static or
dynamic) can point at this directory unchanged.
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
LIB = os.path.join(HERE, "libmorpheus_gb300.so")
ALIASES = ["libgoldilocks_cuda_wrapper.so", "libalmost_goldilocks_cuda_wrapper.so"]
# The same objects as a static archive, under the names the crates link statically
# (cargo:rustc-link-lib=static=goldilocks_cuda_wrapper beside static=cudart_static, stdc++, dl, rt,
# pthread: goldilocks-cuda-rs/build.rs:157-168, almost-goldilocks-cuda-rs/build.rs:115-121).
ARCHIVE = os.path.join(HERE, "libmorpheus_gb300.a")
ARCHIVE_ALIASES = ["libgoldilocks_cuda_wrapper.a", "libalmost_goldilocks_cuda_wrapper.a"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--default-stream", "per-thread", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build morpheus_gb300")
    return cand


def _deps():
    return sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.hpp")) +
                  glob.glob(os.path.join(HERE, "..", "include", "*.h")))


def _compile(src, extra):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    newest_dep = max([os.path.getmtime(src)] + [os.path.getmtime(d) for d in _deps()])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest_dep:
        return obj, None
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + extra + ["-c", src, "-o", obj]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        return obj, f"{' '.join(cmd)}\n{p.stdout}\n{p.stderr}"
    return obj, p.stderr.strip() or None


def build(verbose=False, extra=()):
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    objs, errors = [], []
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for obj, msg in ex.map(lambda s: _compile(s, list(extra)), srcs):
            objs.append(obj)
            if msg and ("error" in msg.lower()):
                errors.append(msg)
            elif msg and verbose:
                print(msg, file=sys.stderr)
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n\n".join(errors))
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
    if not os.path.exists(ARCHIVE) or os.path.getmtime(ARCHIVE) < newest:
        if os.path.exists(ARCHIVE):
            os.remove(ARCHIVE)
        ar = shutil.which("ar") or "ar"
        p = subprocess.run([ar, "rcs", ARCHIVE] + objs, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"ar failed: {p.stdout}\n{p.stderr}")
    for target, aliases in ((LIB, ALIASES), (ARCHIVE, ARCHIVE_ALIASES)):
        for alias in aliases:
            path = os.path.join(HERE, alias)
            if os.path.islink(path) or os.path.exists(path):
                os.remove(path)
            os.symlink(os.path.basename(target), path)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
