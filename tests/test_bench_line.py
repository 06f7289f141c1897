"""The bench's JSON line (bench.emit) on CPU with made-up measurements: one
line on stdout, every key the line must carry, and the derived fields
(ms_per_step, roofline fraction and traffic, e2e bytes per step and the
step spread) computed from the inputs."""
import json
import os
import sys
import types

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import bench  # noqa: E402

REQUIRED = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
            "vs_baseline", "dtype", "data", "config", "e2e", "roofline", "gpu_launches", "clocks", "cpu_baseline")


PEAKS = {"fp64_tflops": 1.246, "fp32_tflops": 78.5, "int32_tops": 20.1}


def _stats(search_ms=80.0, kernel_ms=170.0):
    return types.SimpleNamespace(rays_in=563_000_000, rays_out=553_000_000, hits=560_000_000, generations=80,
                                 launches=380, search_ms=search_ms, kernel_ms=kernel_ms)


def _emit(capsys, e2e_value=9.0e8):
    args = types.SimpleNamespace(steps=10, warmup=3, workload="config2", flags="mixed")
    stats = _stats()
    krl = bench.kernel_rooflines(1, stats, 10 << 20, 6778.0, "measured", PEAKS) + \
        bench.kernel_rooflines(0, _stats(0.0, 1548.0), 10 << 20, 6778.0, "measured", PEAKS)
    e2e_steps = {"steps": 10, "min": 56.4, "median": 56.5, "max": 120.0, "all": [56.4] * 8 + [56.5, 120.0]}
    cpu = {"value": 3.3e6, "cores": 16, "kind": "reference", "sample": "16384 rays"}
    clk = {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": []}
    bench.emit(args, 1, 2.3e9, 0.2413, 0.2415, 8, 1 << 20, list(range(11)), 8, 1e-6, 5.63e7, e2e_value,
               10 * 10_592_222_680, e2e_steps, krl, PEAKS, 1, stats, clk, cpu,
               other={"value": 3.6e8}, extra={"extras": {}})
    out = capsys.readouterr().out.strip().splitlines()
    assert len(out) == 1
    return json.loads(out[0])


def test_line_carries_every_key(capsys):
    line = _emit(capsys)
    for k in REQUIRED:
        assert k in line, k
    assert line["metric"] == bench.METRIC and line["unit"] == "ray-segments/s"
    assert line["higher_is_better"] is True and line["scaling"] == "weak" and line["vs_baseline"] is None
    assert "plain_fp64" in line and "extras" in line


def test_derived_fields(capsys):
    line = _emit(capsys)
    assert abs(line["ms_per_step"] - 24.13) < 1e-9
    r = line["roofline"]
    # the mixed path's dominant kernel: the material kernel (90 of 170 ms)
    mat = bench.BYTES["material"]
    nbytes = 563_000_000 * mat["segment"] + 560_000_000 * mat["hit"] + 553_000_000 * mat["child"]
    assert r["kernel"] == "mixed_material_kernel" and r["bound"] == "hbm"
    assert abs(r["achieved"] - nbytes / 0.090 / 1e9) < 1e-6 and abs(r["frac"] - r["achieved"] / 6778.0) < 1e-12
    assert abs(r["traffic"] - bench.NCU_TRAFFIC_PER_RAY["mixed_material_kernel"] * 563_000_000 / 80) < 1e-3
    k = {e["kernel"]: e for e in line["kernel_rooflines"]}
    assert set(k) == {"mixed_search_kernel", "mixed_material_kernel", "generation_plain_kernel"}
    fp64 = bench.PLAIN_FP64_FLOPS_PER_SEGMENT * 563_000_000 / 1.548 / 1e12
    assert abs(k["generation_plain_kernel"]["pipe"]["achieved_tflops"] - fp64) < 1e-9
    assert k["generation_plain_kernel"]["bound"] == "fp64"
    assert line["measured_peaks"] == PEAKS
    e = line["e2e"]
    assert e["d2h_bytes_per_step"] == 10_592_222_680 and e["h2d_bytes_per_step"] == (1 << 20) * 188
    assert e["step_ms"] == {"min": 56.4, "median": 56.5, "max": 120.0, "all": [56.4] * 8 + [56.5, 120.0]}
    assert e["steps"] == 10
    assert line["cpu_baseline"]["cores"] == 16 and line["gpu_launches"] == 380


def test_no_e2e_leg_gives_null(capsys):
    assert _emit(capsys, e2e_value=None)["e2e"] is None
