"""The drop-in claim for C++ callers: a host program written against the
reference's operator API (include/qg_ref.h; tests/ref_host/relink_driver.cpp
calls CL_RangeSelection, filterImpl, groupByImpl and parallelAggregate_init as
host/host/testFilter.cpp:197-232 and testAggAfterGB.cpp:127-193 do) is
compiled with g++ and linked with -lqg, then run on the reference generator's
records; its output files are compared with the CPU oracle."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from query_on_opencl_fpga_gb300 import build as qbuild

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]


def _write(path, rec):
    with open(path, "wb") as f:
        f.write(np.int32(rec.shape[0]).tobytes())
        f.write(np.ascontiguousarray(rec, np.int32).tobytes())


def _read(path, width):
    raw = np.fromfile(path, np.int32)
    n = int(raw[0])
    return raw[1:1 + n * width].reshape(n, width) if width > 1 else raw[1:1 + n]


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    lib = qbuild.build()
    cuda = Path(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc").resolve().parents[1]
    libdirs = [p for p in (cuda / "lib64", cuda / "lib", *cuda.glob("targets/*/lib")) if (p / "libcudart.so").exists()]
    assert libdirs, "libcudart.so not found next to nvcc"
    exe = tmp_path_factory.mktemp("relink") / "relink_driver"
    cmd = [gxx, "-O2", "-std=c++17", str(ROOT / "tests" / "ref_host" / "relink_driver.cpp"), "-o", str(exe),
           f"-I{ROOT / 'include'}", f"-I{cuda / 'include'}", f"-L{lib.parent}", "-lqg", f"-L{libdirs[0]}",
           "-lcudart", f"-Wl,-rpath,{lib.parent}", f"-Wl,-rpath,{libdirs[0]}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


@pytest.mark.parametrize("n,groups", [(100_000, 64), (1 << 18, 5000)])
def test_cpp_host_program_relinked_against_libqg(driver, orc, tmp_path, n, groups):
    rin = orc.generate_rand(100, n, 0)
    gin = orc.generate_rand(groups, n, 1)
    gin[:, 1] = np.mod(gin[:, 1], groups)  # non-negative keys, as the group-by drivers use
    small, large = 20, 60
    _write(tmp_path / "rin.bin", rin)
    _write(tmp_path / "gin.bin", gin)
    r = subprocess.run([str(driver), str(tmp_path / "rin.bin"), str(tmp_path / "gin.bin"), str(tmp_path),
                        str(small), str(large)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stderr[-2000:])
    exp_f = orc.filter_rec(rin, small, large)
    assert np.array_equal(_read(tmp_path / "sel.bin", 2), exp_f)
    assert np.array_equal(_read(tmp_path / "filt.bin", 2), exp_f)
    srt = _read(tmp_path / "sorted.bin", 2)
    exp_s = orc.sort_rec(gin)
    assert np.array_equal(srt[:, 1], exp_s[:, 1])  # keys in order; equal keys in any order, as the reference
    sp = _read(tmp_path / "startpos.bin", 1)
    assert np.array_equal(sp, orc.group_startpos(exp_s))
    for op in range(4):
        agg = _read(tmp_path / f"agg{op}.bin", 1)
        assert np.array_equal(agg, orc.aggregate_groups(srt, sp, op)), op
