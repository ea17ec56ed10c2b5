"""bench.py's reference arm (the CPU port of the reference's execute path on
the host cores) prints one JSON line with the fields a benchmark consumer
reads.  Runs on the CPU: one bounded cycle of the 512^3 workload."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["value"] > 0 and line["unit"] == "cycles/s" and line["higher_is_better"] is True
    assert line["config"]["workload"] == "c2c_c64_512x512x512_grid2x4_fwd+bwd"
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_bench_fp64_z_lines_equal_full_transforms():
    """The bench's numpy FP64 Z-line check equals the full FP64 transforms."""
    import numpy as np
    import scipy.fft as sf
    import bench
    rng = np.random.default_rng(3)
    g = rng.standard_normal((10, 12, 14)) + 1j * rng.standard_normal((10, 12, 14))
    pts = bench._z_line_points(14, 12)
    full = np.fft.fftn(g)
    np.testing.assert_allclose(bench._fp64_z_lines(g, pts), np.stack([full[:, ky, kx] for kx, ky in pts]),
                               atol=1e-10)
    r = rng.standard_normal((10, 12, 14))
    full = np.fft.rfftn(r)
    pts = bench._z_line_points(8, 12)
    np.testing.assert_allclose(bench._fp64_z_lines(r, pts, "r2c"), np.stack([full[:, ky, kx] for kx, ky in pts]),
                               atol=1e-10)
    full = sf.dctn(r, type=2, norm=None)
    pts = bench._z_line_points(14, 12)
    np.testing.assert_allclose(bench._fp64_z_lines(r, pts, "dct2"), np.stack([full[:, ky, kx] for kx, ky in pts]),
                               atol=1e-9)
