"""Host-side numerics and geometry of the kernels, checked on the CPU.

- df64.cuh: the integer split of a double into two floats, its common-case
  form, the integer join back to a double and the TwoProd/TwoSum dot
  products used by the complex128 kernels (tests/cpp/df64_check.cpp).
- fused_tc.cu: the tile of a tensor-core pass as a tensor-map box, and the
  staged-tile padding and row order (tests/cpp/tile_check.cpp, linked
  against the built library).
- warp_tile.cpp / batch_host.cpp: the warp tiles of the batch executor and
  the single-state dense kernels, their staged (swizzled) offsets and bank
  groups (tests/cpp/batch_tile_check.cpp, same library).
- swap_run.cu: the swap-run pass replayed on the host against the direct
  permutation (tests/cpp/swap_run_check.cpp, same library).

Both programs are compiled here with g++ and print one line of figures.
"""
import os
import shutil
import subprocess

import pytest

from q1tsim_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CPP = os.path.join(ROOT, "tests", "cpp")


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.isdir(os.path.join(c, "include")):
            return c
    nvcc = shutil.which("nvcc")
    return os.path.dirname(os.path.dirname(nvcc)) if nvcc else None


def _run(exe):
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout.strip()


@pytest.fixture(scope="module")
def gxx():
    g = shutil.which("g++")
    if g is None:
        pytest.skip("no g++")
    return g


def test_double_float_split_join_dot(gxx, tmp_path):
    exe = str(tmp_path / "df64_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe,
                    os.path.join(CPP, "df64_check.cpp")], check=True)
    out = _run(exe)
    assert out.startswith("bad 0"), out


def _link_against_library(gxx, tmp_path, name):
    cuda = _cuda_home()
    if cuda is None:
        pytest.skip("no CUDA headers")
    lib = build.build()
    libdir = os.path.dirname(lib)
    exe = str(tmp_path / name)
    cudalib = [p for p in (os.path.join(cuda, "lib64"), os.path.join(cuda, "lib")) if os.path.isdir(p)]
    cmd = [gxx, "-O2", "-std=c++17", "-I", os.path.join(cuda, "include"), "-o", exe,
           os.path.join(CPP, name + ".cpp"), "-L", libdir, "-lq1gpu", "-Wl,-rpath," + libdir]
    for d in cudalib:
        cmd += ["-L", d, "-Wl,-rpath," + d]
    cmd += ["-lcudart"]
    subprocess.run(cmd, check=True)
    return exe


def test_tile_box_and_padding(gxx, tmp_path):
    out = _run(_link_against_library(gxx, tmp_path, "tile_check"))
    assert "bad 0" in out, out


def test_batch_warp_tiles(gxx, tmp_path):
    out = _run(_link_against_library(gxx, tmp_path, "batch_tile_check"))
    assert out.startswith("bad 0"), out


def test_swap_run_pass_replays_the_permutation(gxx, tmp_path):
    out = _run(_link_against_library(gxx, tmp_path, "swap_run_check"))
    assert out.startswith("bad 0"), out
