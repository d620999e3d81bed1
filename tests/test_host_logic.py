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
- fused_tc.cu: the row layouts and register/lane swaps of shuffled
  two-block tensor-core passes, replayed on tile coordinates
  (tests/cpp/shuffle_check.cpp, same library), and the scatter of direct
  pairs into the second block's operand layout (tests/cpp/direct_check.cpp).
- f16_host.h / fused_tc.cu: binary16 rounding against numpy's float16, the
  f16 image of a block read back through its swizzle, the operand scales and
  the row-norm bound of tensor-core blocks (tests/cpp/tc_image_check.cpp).

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


def test_shuffled_pairs_redeal_the_rows(gxx, tmp_path):
    out = _run(_link_against_library(gxx, tmp_path, "shuffle_check"))
    assert out.startswith("bad 0"), out


def test_direct_pairs_scatter_into_the_operand_layout(gxx, tmp_path):
    out = _run(_link_against_library(gxx, tmp_path, "direct_check"))
    assert out.splitlines()[-1].startswith("bad 0"), out
    assert "lowest-positions pair: cost 164 of minimum 128, permuted 1" in out, out


def test_batch_warp_tiles(gxx, tmp_path):
    out = _run(_link_against_library(gxx, tmp_path, "batch_tile_check"))
    assert out.startswith("bad 0"), out


def test_swap_run_pass_replays_the_permutation(gxx, tmp_path):
    out = _run(_link_against_library(gxx, tmp_path, "swap_run_check"))
    assert out.startswith("bad 0"), out


def test_f16_rounding_and_tensor_core_images(gxx, tmp_path):
    """Binary16 rounding of the operand images equals numpy's float16
    conversion (round to nearest even) on normals, subnormals, halfway cases
    and zeros; the image reads back to 2^14 R within 2^-22."""
    import numpy as np
    rng = np.random.default_rng(5)
    vals = np.concatenate([
        rng.uniform(-2.0 ** 15, 2.0 ** 15, 20000),
        rng.standard_normal(20000) * 2.0 ** rng.integers(-30, 14, 20000),
        (rng.integers(0, 2048, 4000) + 0.5) * 2.0 ** rng.integers(-34, 4, 4000),   # ties
        (rng.integers(0, 1024, 2000) + 0.5) * 2.0 ** -24,                           # subnormal ties
        np.array([0.0, -0.0, 2.0 ** -14, 2.0 ** -25, 2.0 ** -26, 65504.0, 2047.5 * 2.0 ** -11]),
    ])
    path = tmp_path / "vals.bin"
    vals.astype(np.float64).tofile(path)
    exe = _link_against_library(gxx, tmp_path, "tc_image_check")
    r = subprocess.run([exe, str(path)], capture_output=True, text=True, timeout=600)
    lines = r.stdout.split()
    assert r.returncode == 0 and lines[:2] == ["bad", "0"], r.stdout[:200] + r.stderr
    got = np.array([int(x, 16) for x in lines[4:]], dtype=np.uint16)
    want = vals.astype(np.float16).view(np.uint16)
    assert got.shape == want.shape
    assert np.array_equal(got, want), np.flatnonzero(got != want)[:10]
