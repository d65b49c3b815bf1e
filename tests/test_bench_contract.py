"""bench.py's command-line contract on the CPU (no GPU): the reference arm's JSON line, its
rank-0-only rule under torchrun, and our arm failing loudly (no CPU fallback) when CUDA is
absent."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SMALL = ["--workload", "cfg1_2view_128x128x64"]


def _bench(args, env_extra=None, timeout=300):
    env = dict(os.environ)
    env.update(env_extra or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT, env=env,
                          capture_output=True, text=True, timeout=timeout)


def test_reference_arm_prints_the_contract_line():
    r = _bench(["--impl", "reference", "--steps", "2", "--warmup", "1", *SMALL])
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["value"] > 0 and d["unit"] == "voxel-updates/s" and d["higher_is_better"] is True
    assert d["steps"] == 2 and d["warmup"] == 1 and d["n_gpus"] == 1
    assert d["config"]["workload"] == "cfg1_2view_128x128x64"
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_runs_on_rank_zero_only():
    r = _bench(["--impl", "reference", "--steps", "1", "--warmup", "0", *SMALL],
               {"RANK": "1", "LOCAL_RANK": "1", "WORLD_SIZE": "2"})
    assert r.returncode == 0, r.stderr
    assert not [ln for ln in r.stdout.splitlines() if ln.startswith("{")]


def test_our_arm_fails_loudly_without_cuda():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = _bench(["--steps", "1", "--warmup", "3", "--no-cpu", "--no-plain", "--no-e2e", *SMALL])
    assert r.returncode != 0
    assert not [ln for ln in r.stdout.splitlines() if ln.startswith("{")]


def test_roofline_byte_contract_uses_the_reference_blocks():
    """The roofline's algorithmic bytes: per view 8 P + 64 H + 20 N over the reference's blocks
    (P, H of each block; padding of the library's tiles not credited).  Pinned to hand-computed
    figures: 128^3 blocks with a 15x15x41 PSF on 256x256x192 (3x3x3 = 27 blocks per view,
    about 202 bytes per voxel-update) and one 542x542x316 block (image + kernel - 1) for a
    31x31x61 PSF on 512x512x256 (about 75.5 bytes per voxel-update)."""
    import types

    import numpy as np

    sys.path.insert(0, ROOT)
    import bench

    n2 = 256 * 256 * 192
    p2 = types.SimpleNamespace(dims_xyz=(256, 256, 192), psfs=[np.zeros((41, 15, 15))] * 4)
    b2 = bench.reference_block_bytes(p2, (128, 128, 128))
    P, H = 128 ** 3, 65 * 128 * 128
    assert sum(b2.values()) == 4 * (27 * (8 * P + 64 * H) + 20 * n2)
    assert abs(sum(b2.values()) / (4 * n2) - 202.2) < 0.1
    n4 = 512 * 512 * 256
    p4 = types.SimpleNamespace(dims_xyz=(512, 512, 256), psfs=[np.zeros((61, 31, 31))])
    b4 = bench.reference_block_bytes(p4, None)
    P, H = 542 * 542 * 316, 272 * 542 * 316
    assert b4["plane_fwd"] == 2 * (4 * P + 8 * H)
    assert b4["zpass"] == 2 * 16 * H
    assert b4["plane_inv_quotient"] == 8 * H + 8 * n4 and b4["plane_inv_update"] == 8 * H + 12 * n4
    assert abs(sum(b4.values()) / n4 - 75.5) < 0.1
