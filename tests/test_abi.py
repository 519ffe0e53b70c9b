"""The C-ABI library builds for sm_103a, loads without a GPU and exports every
function declared in include/*.h (CPU only: no compute calls)."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in sorted(glob.glob(os.path.join(ROOT, "include", "*.h"))):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s+\**([A-Za-z_][A-Za-z0-9_]*)\s*\(", src, re.M):
            if m.group(1) not in ("if", "return", "sizeof"):
                names.append(m.group(1))
    return sorted(set(names))


@pytest.fixture(scope="module")
def libpath():
    from morpheus_gb300 import build as B
    return B.build()


def test_headers_declare_functions():
    names = declared_functions()
    assert len(names) > 40
    assert "sumcheck_round_message_ffi" in names and "gb_sumcheck_prove_ext2" in names


def test_library_exports_every_declared_symbol(libpath):
    L = ctypes.CDLL(libpath)
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_reference_link_names_present(libpath):
    d = os.path.dirname(libpath)
    for alias in ("libgoldilocks_cuda_wrapper.so", "libalmost_goldilocks_cuda_wrapper.so"):
        assert os.path.exists(os.path.join(d, alias))


def test_python_bindings_cover_library(libpath):
    from morpheus_gb300 import _native
    L = _native.lib()
    for name in _native.SIGNATURES:
        assert hasattr(L, name), name


def test_built_for_sm103a_only():
    """Every translation unit and the link use the one sm_103a target (no PTX, no other arch)."""
    from morpheus_gb300 import build as B
    assert B.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


@pytest.mark.gpu
def test_loaded_kernels_are_sm103_binaries(gpu_lib):
    from morpheus_gb300 import _native
    assert _native.lib().gb_binary_version() == 103


def test_static_archive_links_with_the_crates_link_line(libpath, tmp_path):
    """The static archive, under the crates' library names, links a C program that takes the
    address of every declared function, with the link line the crates' build scripts emit
    (static=goldilocks_cuda_wrapper, static=cudart_static, stdc++, dl, rt, pthread).  Link only:
    the program is not run."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    cudart = "/usr/local/cuda/lib64/libcudart_static.a"
    if not cc or not os.path.exists(cudart):
        pytest.skip("no C compiler or static CUDA runtime")
    d = os.path.dirname(libpath)
    for alias in ("libgoldilocks_cuda_wrapper.a", "libalmost_goldilocks_cuda_wrapper.a"):
        assert os.path.exists(os.path.join(d, alias))
    names = declared_functions()
    src = ["#include <stdint.h>", "#include <stddef.h>",
           '#include "goldilocks_cuda_wrapper.h"', '#include "almost_goldilocks_cuda_wrapper.h"',
           "void *fns[] = {"] + [f"    (void *)&{n}," for n in names] + [
           "};", "int main(void) { return fns[0] == 0; }"]
    c = tmp_path / "link_all.c"
    c.write_text("\n".join(src) + "\n")
    for lib in ("goldilocks_cuda_wrapper", "almost_goldilocks_cuda_wrapper"):
        out = tmp_path / f"link_{lib}"
        cmd = [cc, str(c), "-I", os.path.join(ROOT, "include"), "-o", str(out), "-L", d, f"-l:lib{lib}.a",
               "-L", "/usr/local/cuda/lib64", "-lcudart_static", "-lstdc++", "-ldl", "-lrt", "-lpthread"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        assert p.returncode == 0, p.stderr[-3000:]
