"""bench.py's JSON contract for the reference arm (CPU only)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "dtype", "data", "config"):
        assert key in line, key
    assert line["value"] > 0 and line["steps"] == 1 and line["higher_is_better"] is True
    cpu = line["cpu_baseline"]
    assert cpu["kind"] in ("port", "reference") and cpu["cores"] >= 1 and cpu["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0
    assert e2e["d2h_bytes_per_step"] == 0 and e2e["unit"] == line["unit"]
    assert line["config"]["n"] == 2048 and line["config"]["kernels"] == 9


def test_cpu_baseline_forms_small():
    """The cpu_baseline object with its other forms (one thread, FP64, and the
    torch CPU model), on a 64^2 creature."""
    sys.path.insert(0, ROOT)
    import bench
    from cella_nova_gb300.creature import make_creature
    from oracle import oracle as O
    O.build()
    cr = make_creature(64, 2, seed=1, radius=(4, 12), seed_box=32)
    cpu = bench.cpu_baseline(cr, budget_s=1.0, nthreads=2)
    assert cpu["kind"] == "port" and cpu["cores"] == 2 and cpu["value"] > 0
    c_forms = {(f["threads"], f["dtype"]) for f in cpu["forms"] if f["impl"].startswith("C port")}
    assert c_forms == {(2, "f32"), (2, "f64"), (1, "f32"), (1, "f64")}
    torch_forms = [f for f in cpu["forms"] if f["impl"].startswith("torch")]
    assert len(torch_forms) == 1 and torch_forms[0]["threads"] >= 1
    assert all(f["cell_updates_per_s"] > 0 for f in cpu["forms"])


def test_roofline_object_reports_the_slowest_kernel():
    """bench.py's roofline object: algorithmic bytes over each kernel's time,
    the kernel with the largest device time on top, traffic from the ncu
    summary."""
    sys.path.insert(0, ROOT)
    import bench
    kms = [0.030, 0.068, 0.070, 0.040]     # ms per step: r2c, col_conv, c2r, diffusion
    traffic = {"k_row_c2r_growth_2048": {"dram_bytes_per_launch": 1.8e8}}
    r = bench.roofline_object(kms, 2048, 3, 9, 6790.0, "measured", traffic)
    assert r["kernel"] == "k_row_c2r_growth" and r["kernel_ms"] == 0.070
    px = 2048 * 2048
    assert r["algorithmic_bytes"] == (4 * 9 + 4 * 3) * px
    assert abs(r["achieved"] - r["algorithmic_bytes"] / 0.070e-3 / 1e9) < 1e-6
    assert abs(r["frac"] - r["achieved"] / 6790.0) < 1e-12 and r["traffic"] == 1.8e8
    assert [k["kernel"] for k in r["kernels"]] == list(bench.KERNEL_NAMES)
    assert sum(k["algorithmic_bytes"] for k in r["kernels"]) == bench.bytes_per_px_as_built(3, 9) * px
