"""The drop-in at link level: a plain C caller (tests/c_abi/drop_in.c) built
against the shared library and against the static archive with the static
CUDA runtime, the two ways a program that linked the reference's `mwblas`
archive would be relinked. On CPU both links must resolve every symbol the
caller uses; on the GPU both programs run their exact integer checks."""
import os
import shutil
import subprocess

import pytest

from conftest import PKG, ROOT, build_mod

SRC = os.path.join(ROOT, "tests", "c_abi", "drop_in.c")
CUDA_LIB = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64")


def _link(tmp_path, mode):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    build_mod.build()
    exe = str(tmp_path / f"drop_in_{mode}")
    cmd = [cc, "-O2", "-Wall", "-I" + os.path.join(ROOT, "include"), SRC, "-o", exe]
    if mode == "shared":
        cmd += ["-L" + PKG, "-lmwblas_gb300", "-Wl,-rpath," + PKG, "-lm"]
    else:
        cmd += [build_mod.ARCHIVE, "-L" + CUDA_LIB, "-lcudart_static", "-lstdc++", "-lpthread", "-ldl", "-lrt",
                "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    assert "warning" not in r.stderr, r.stderr[-4000:]
    return exe


@pytest.mark.parametrize("mode", ["shared", "static"])
def test_c_caller_links(tmp_path, mode):
    _link(tmp_path, mode)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["shared", "static"])
def test_c_caller_runs(tmp_path, mode):
    exe = _link(tmp_path, mode)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "drop_in ok" in r.stdout, (r.stdout[-2000:], r.stderr[-2000:])
