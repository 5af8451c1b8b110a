"""bench.py's reference arm on the CPU: the JSON line it prints (keys, units, the CPU baseline and
end-to-end objects), on small cases of a single-grid and of the batched workload, and its silence on
ranks other than 0 of a multi-rank launch."""
from __future__ import annotations

import json

import pytest

import bench

CASES = [["--workload", "ldc3d_d3q19_256_fp32", "--n", "32"],
         ["--workload", "ldc3d_d3q27_256_kbc_f16c_eso", "--n", "32"],
         ["--workload", "batch2d_cylinders_512"]]


@pytest.mark.parametrize("extra", CASES, ids=[c[1] for c in CASES])
def test_reference_arm_json_line(extra, capsys, monkeypatch):
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    ret = bench.main(["--impl", "reference", "--steps", "4", "--warmup", "3", *extra])
    lines = [ln for ln in capsys.readouterr().out.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d == ret
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["unit"] == "MLUPs" and d["higher_is_better"] is True
    assert d["n_gpus"] == 1 and d["steps"] == 4 and d["warmup"] == 3 and d["value"] > 0
    assert "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "MLUPs", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    metric = "D2Q9 MLUPs (batched domains)" if "batch" in extra[1] else extra[1].split("_")[1].upper() + " MLUPs"
    assert d["metric"] == metric


def test_reference_arm_other_ranks_print_nothing(capsys, monkeypatch):
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")
    assert bench.main(["--impl", "reference", "--steps", "4", "--warmup", "3", "--n", "32"]) is None
    assert capsys.readouterr().out == ""


def test_warmup_below_three_is_rejected():
    with pytest.raises(SystemExit):
        bench.main(["--impl", "reference", "--steps", "4", "--warmup", "2", "--n", "32"])


@pytest.mark.parametrize("workload", sorted(bench.WORKLOADS))
def test_every_workload_has_a_profile_with_its_traffic(workload):
    """Each benchmark workload's roofline.traffic comes from its committed ncu summary
    (profiles/<workload>.txt): the file exists, names the workload's bench command, and holds one
    positive per-launch DRAM byte count."""
    traffic, src = bench.profiled_traffic(workload)
    assert src == f"profiles/{workload}.txt"
    assert traffic is not None and traffic > 0
    text = (bench.ROOT / src).read_text()
    assert f"--workload {workload}" in text or workload == "ldc3d_d3q19_256_fp32"
    assert "--clock-control none" in text
