"""Generate the golden fixtures that pin the CPU oracle to the reference.

Run in a checkout that has the reference sources (it builds oracle/_ref from
them with oracle/build_ref.sh).  For each case it
  1. runs the reference's own generator (host/host/generator.cpp) and checks
     that the oracle's restatement produces the same bytes,
  2. runs the oracle operator and has the reference's own validator
     (host/host/Validate.cpp) check the result, requiring its "passed" line,
  3. stores input digests, the validator output and the oracle output (or its
     digest) in tests/golden/golden.npz / golden.json,
and records the reference DP planner's printed plans
(host/dynamic_programming.cpp) for the planner port.

It also writes tests/golden/golden_refk.json, digests of the reference's own
OpenCL kernels run on host cores (oracle/_ref/libref_kernels.so) on seeded
inputs; --refk-only writes that file alone.

Usage: python tests/golden/make_golden.py [--refk-only]
"""
from __future__ import annotations

import hashlib
import json
import re
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import oracle as orc  # noqa: E402

OUT = Path(__file__).resolve().parent


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def ref_gen_rand(maxmax: int, n: int, seed: int, tmp: Path) -> tuple[np.ndarray, int]:
    p = tmp / f"gen_{maxmax}_{n}_{seed}.bin"
    out = orc.ref_tool("gen_rand", maxmax, n, seed, p)
    nxt = int(re.search(r"next_rand=(-?\d+)", out).group(1))
    return np.fromfile(p, np.int32).reshape(n, 2), nxt


def save_bin(tmp: Path, name: str, a: np.ndarray) -> Path:
    p = tmp / name
    np.ascontiguousarray(a).tofile(p)
    return p


def main() -> None:
    orc.build()
    if not orc.REF_TOOL.exists():
        raise SystemExit("reference checkout not found: oracle/_ref/ref_tool was not built")
    meta: dict = {"cases": {}}
    arrays: dict[str, np.ndarray] = {}
    with tempfile.TemporaryDirectory() as td:
        tmp = Path(td)

        # ---- filter: testFilterImpl (host/host/testFilter.cpp:197-232) ----------
        n = 1 << 16
        rin, nxt = ref_gen_rand(100, n, 0, tmp)
        mine = orc.generate_rand(100, n, 0)
        assert np.array_equal(rin, mine), "generator restatement differs from the reference"
        small = nxt % 100
        large = min(small + 6, 100)
        out = orc.filter_rec(rin, small, large)
        validator_output = orc.ref_tool("validate_filter", save_bin(tmp, "fin.bin", rin), n,
                               save_bin(tmp, "fout.bin", out), out.shape[0], small, large)
        assert "filter passed" in validator_output, validator_output
        meta["cases"]["filter"] = {"n": n, "maxmax": 100, "seed": 0, "small": int(small),
                                   "large": int(large), "out_n": int(out.shape[0]),
                                   "input_sha": sha(rin), "validator_output": validator_output.strip()}
        arrays["filter_out"] = out

        # ---- scan: testScanImpl (host/host/testScan.cpp:342-390) ----------------
        n = 1 << 16
        p = tmp / "scan_in.bin"
        orc.ref_tool("gen_rand_int", n, n, 0, p)
        sin = np.fromfile(p, np.int32)
        assert np.array_equal(sin, orc.generate_rand_int(n, n, 0))
        sout = orc.scan_excl(sin)
        validator_output = orc.ref_tool("validate_scan", p, n, save_bin(tmp, "scan_out.bin", sout))
        assert "scan test pass!" in validator_output, validator_output
        meta["cases"]["scan"] = {"n": n, "input_sha": sha(sin), "output_sha": sha(sout),
                                 "validator_output": validator_output.strip()}

        # ---- sort: testSortImpl (host/host/testSort.cpp:276-296) ----------------
        for n in (2048, 1 << 15, 100003):
            rin, _ = ref_gen_rand(200, n, 0, tmp)
            srt = orc.sort_rec(rin)
            validator_output = orc.ref_tool("validate_sort", save_bin(tmp, "sorted.bin", srt), n)
            assert "sorting passed" in validator_output, validator_output
            meta["cases"][f"sort_{n}"] = {"n": n, "maxmax": 200, "input_sha": sha(rin),
                                          "keys_sorted_sha": sha(srt[:, 1]), "validator_output": validator_output.strip()}

        # ---- group-by: testGroupByImpl (host/host/testGroupBy.cpp:156-175) -------
        # Keys are taken mod maxmax into [0, maxmax): under glibc generateRand
        # yields negative keys, and validateGroupBy sorts signed while the
        # kernels sort unsigned (the two orders then disagree).
        n = 1 << 16
        rin, _ = ref_gen_rand(64, n, 0, tmp)
        rin = rin.copy()
        rin[:, 1] = np.mod(rin[:, 1], 64)
        srt = orc.sort_rec(rin)
        sp = orc.group_startpos(srt)
        validator_output = orc.ref_tool("validate_groupby", save_bin(tmp, "gin.bin", rin), n,
                               save_bin(tmp, "gsrt.bin", srt), save_bin(tmp, "gsp.bin", sp), sp.size)
        assert "GroupBy Test passed!" in validator_output, validator_output
        meta["cases"]["groupby"] = {"n": n, "maxmax": 64, "num_groups": int(sp.size),
                                    "input_sha": sha(rin), "validator_output": validator_output.strip()}
        arrays["groupby_startpos"] = sp

        # ---- aggregation: testAggAfterGroupByImpl (host/host/testAggAfterGB.cpp:127-255)
        n = 1 << 16
        rin, _ = ref_gen_rand(50, n, 0, tmp)
        rin = rin.copy()
        rin[:, 1] = np.mod(rin[:, 1], 50)
        srt = orc.sort_rec(rin)
        sp = orc.group_startpos(srt)
        ragg = np.stack([np.arange(n, dtype=np.int32)] * 2, axis=1)  # Ragg[i].y = i
        aggcase = {"n": n, "maxmax": 50, "num_groups": int(sp.size), "input_sha": sha(rin)}
        for op, name in enumerate(["sum", "max", "min", "avg"]):
            agg = orc.aggregate_groups(srt, sp, op)
            validator_output = orc.ref_tool("validate_agg", save_bin(tmp, "asrt.bin", srt), n,
                                   save_bin(tmp, "asp.bin", sp), sp.size,
                                   save_bin(tmp, "ragg.bin", ragg), save_bin(tmp, "agg.bin", agg), op)
            assert "Test Passed!" in validator_output, (name, validator_output)
            if op == 1:
                easy = orc.ref_tool("validate_agg_easy", save_bin(tmp, "asrt.bin", srt), n,
                                    save_bin(tmp, "asp.bin", sp), sp.size,
                                    save_bin(tmp, "agg.bin", agg), op)
                assert "Agg Test Passed!" in easy, easy
            aggcase[f"{name}_validator_output"] = validator_output.strip()
            arrays[f"agg_{name}"] = agg
        meta["cases"]["aggregate"] = aggcase

        # ---- DP planner: dp_test (host/dynamic_programming.cpp:1000-1024) --------
        plans = {}
        for sub in (0, 1, 2, 3):
            for size in (4, 16, 64):
                txt = orc.ref_tool("dp", sub, size)
                m = re.search(r"total execution time: ([0-9.]+)", txt)
                images = re.findall(r"The (\d+)-th FPGA image:", txt)
                names = re.findall(r"^\d+:\s+(\d+),\s+(\d+)\s+(\S+)\s*$", txt, re.M)
                times = re.findall(r"total_unit_cost = ([0-9.]+), exec_time = ([0-9.]+)", txt)
                reconf = re.findall(r"mem_inc = ([0-9.\-]+), reconfig_time = ([0-9.\-]+)", txt)
                plans[f"{sub}_{size}"] = {
                    "exec_time": m.group(1), "image_num": len(images),
                    "kernels": [list(x) for x in names],
                    "image_costs": [list(x) for x in times],
                    "image_reconfig": [list(x) for x in reconf],
                }
        meta["dp_plans"] = plans

    np.savez_compressed(OUT / "golden.npz", **arrays)
    (OUT / "golden.json").write_text(json.dumps(meta, indent=1, sort_keys=True) + "\n")
    print("wrote", OUT / "golden.npz", OUT / "golden.json")


def refk_digests() -> None:
    """tests/golden/golden_refk.json: digests of the reference's own kernels'
    outputs (oracle/_ref/libref_kernels.so, built from kernel/filter/filter_op.cl
    and kernel/aggregation/1/group_by_cu_op_dp.cl), each checked against the
    oracle here before it is written."""
    assert orc.ref_kernels() is not None, "oracle/_ref/libref_kernels.so is not built"
    meta = {"filter": [], "sort_keys": [], "groupby": []}
    for n, maxmax, lo, hi, seed in [(1 << 17, 1000, 10, 400, 0), (1 << 18, 1 << 20, -(1 << 19), 1 << 18, 1),
                                    (1 << 18, 64, 0, 0, 2)]:
        rin = orc.generate_rand(maxmax, n, seed)
        out = orc.refk_filter_rec(rin, lo, hi)
        assert np.array_equal(out, orc.filter_rec(rin, lo, hi))
        meta["filter"].append({"n": n, "maxmax": maxmax, "lo": lo, "hi": hi, "seed": seed,
                               "count": int(out.shape[0]), "sha": sha(out)})
    for n, seed in [(2048, 0), (1 << 14, 1), (1 << 16, 2)]:
        rin = orc.generate_rand(1 << 24, n, seed)
        keys = orc.refk_sort_rec(rin)[:, 1]
        assert np.array_equal(keys, orc.sort_rec(rin)[:, 1])
        meta["sort_keys"].append({"n": n, "maxmax": 1 << 24, "seed": seed, "sha": sha(keys)})
    for n, groups, seed in [(1 << 17, 50, 3), (1 << 18, 4000, 4)]:
        rin = orc.generate_rand(1 << 20, n, seed)
        rin[:, 1] = np.mod(rin[:, 1], groups)
        srt, sp = orc.refk_groupby_rec(rin)
        assert np.array_equal(sp, orc.group_startpos(orc.sort_rec(rin)))
        aggs = [orc.refk_aggregate(srt, sp, op) for op in range(4)]
        meta["groupby"].append({"n": n, "maxmax": 1 << 20, "groups": groups, "seed": seed,
                                "startpos_sha": sha(sp), "agg_sha": [sha(a) for a in aggs]})
    (OUT / "golden_refk.json").write_text(json.dumps(meta, indent=1, sort_keys=True) + "\n")
    print("wrote", OUT / "golden_refk.json")


if __name__ == "__main__":
    if "--refk-only" not in sys.argv:
        main()
    refk_digests()
