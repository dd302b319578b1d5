"""The DP planner port (include/qg_plan.h) against the reference planner's own
printed plans (host/dynamic_programming.cpp run through oracle/_ref/ref_tool,
recorded in tests/golden/golden.json).  Host-only: runs without a GPU."""
import ctypes

import pytest

from query_on_opencl_fpga_gb300 import _lib


@pytest.fixture(scope="module")
def lib():
    from query_on_opencl_fpga_gb300 import build

    build.build()
    return _lib.load()


def run(lib, sub, size):
    p = _lib.Plan()
    assert lib.qg_plan_pipeline(sub, size, ctypes.byref(p)) == 0
    return p


@pytest.mark.parametrize("sub", [0, 1, 2, 3])
@pytest.mark.parametrize("size", [4, 16, 64])
def test_plan_matches_reference_printout(lib, golden, sub, size):
    meta, _ = golden
    g = meta["dp_plans"][f"{sub}_{size}"]
    p = run(lib, sub, size)
    assert "%f" % p.exec_time == g["exec_time"]
    assert p.image_num == g["image_num"]
    kernels = []
    costs = []
    reconf = []
    for i in range(p.image_num):
        im = p.images[i]
        for j in range(im.num_kernels):
            k = im.kernels[j]
            kernels.append([str(j), str(k.kernel_id), str(k.variant)])
            kernels[-1].append(lib.qg_plan_variant_name(k.kernel_id, k.variant).decode())
        costs.append(["%f" % im.total_unit_cost, "%f" % im.exec_time])
        reconf.append(["%f" % im.mem_inc, "%f" % im.reconfig_time])
    # golden kernels rows: (kernel_id, sub_id, name) per line "i: kernel_id, sub_id  name"
    assert [[k[1], k[2], k[3]] for k in kernels] == [list(x) for x in g["kernels"]]
    assert costs == [list(x) for x in g["image_costs"]]
    assert reconf == [list(x) for x in g["image_reconfig"]]


def test_headline_plans(lib):
    # The values the reference planner prints at 64 M tuples.
    assert "%f" % run(lib, 0, 64).exec_time == "0.901227"
    assert "%f" % run(lib, 1, 64).exec_time == "15.909481"
    assert "%f" % run(lib, 2, 64).exec_time == "18.674465"


def test_custom_table_and_restore(lib):
    # A GPU-style table (no resource model): one variant per primitive, cost = rows read
    rows = (_lib.PlanVariant * 9)()
    for k in range(9):
        rows[k] = _lib.PlanVariant(f"gpu_k{k}".encode(), k, 0, 0, 0, 0, 1.0 + k, 0.0, 0.0)
    assert lib.qg_plan_set_table(rows, 9, 0) == 0
    p = run(lib, 0, 64)
    assert p.image_num >= 1 and p.exec_time > 0
    assert lib.qg_plan_variant_name(3, 0) == b"gpu_k3"
    assert lib.qg_plan_set_table(None, 0, 1) == 0
    assert "%f" % run(lib, 0, 64).exec_time == "0.901227"
