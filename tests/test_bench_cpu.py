"""Host logic of bench.py that needs no GPU: kernel-form names and flags
against the C ABI's form constants, and the per-workload ring storage."""
import sys

import pytest

import bench
from rtm_gpu_gb300 import capi


def _args(*argv):
    old = sys.argv
    sys.argv = ["bench.py", *argv]
    try:
        return bench.parse()
    finally:
        sys.argv = old


def test_form_names_follow_the_abi_constants():
    assert bench.FORMS[capi.RTM_KERNEL_TILED] == "tiled"
    assert bench.FORMS[capi.RTM_KERNEL_PERSISTENT] == "persistent"
    assert bench.FORMS[capi.RTM_KERNEL_SPLIT] == "tiled-split"
    assert bench.FORMS[capi.RTM_KERNEL_X2] == "tiled-2col"
    assert bench.FORMS[capi.RTM_KERNEL_X2_SPLIT] == "2col-split"
    assert len(bench.FORMS) == capi.RTM_KERNEL_X2_SPLIT + 1


@pytest.mark.parametrize("argv,fwd,bwd", [
    (["--kernel", "tiled"], capi.RTM_KERNEL_TILED, capi.RTM_KERNEL_TILED),
    (["--kernel", "persistent"], capi.RTM_KERNEL_PERSISTENT, capi.RTM_KERNEL_PERSISTENT),
    (["--kernel", "split"], capi.RTM_KERNEL_SPLIT, capi.RTM_KERNEL_SPLIT),
    # the two-column forms are forward only: the backward runs tiled
    (["--kernel", "x2"], capi.RTM_KERNEL_X2, capi.RTM_KERNEL_TILED),
    (["--kernel", "x2-split"], capi.RTM_KERNEL_X2_SPLIT, capi.RTM_KERNEL_TILED),
    (["--kernel", "x2-split", "--bwd-kernel", "split"], capi.RTM_KERNEL_X2_SPLIT, capi.RTM_KERNEL_SPLIT),
    (["--kernel", "tiled", "--bwd-kernel", "persistent"], capi.RTM_KERNEL_TILED, capi.RTM_KERNEL_PERSISTENT),
])
def test_kernel_flags(argv, fwd, bwd):
    assert bench.kernel_forms(_args(*argv)) == (fwd, bwd)


@pytest.mark.parametrize("argv,ring", [
    ([], "f16"),                             # multi-shot configuration
    (["--workload", "rvsp"], "f32"),         # FP32 throughout
    (["--workload", "c5"], "i16"),
    (["--workload", "rvsp", "--ring", "f16"], "f16"),
])
def test_ring_storage_per_workload(argv, ring):
    assert bench.Config(_args(*argv)).ring == ring


def test_defaults_keep_the_contract():
    a = _args()
    assert a.gpus == 1 and a.warmup >= 3 and a.steps >= 1 and a.impl == "ours"
    assert a.kernel == "auto" and a.workload == "multishot"


class _FakeEngine:
    """Timing counters of one migration of two batches: 10 backward and 10
    forward launches per batch, 2 ms and 1 ms each, 0.5 ms per pad launch."""

    def __init__(self):
        self.on = False

    def set_timing(self, on):
        self.on = on

    def timing(self):
        return {"fwd_ms": 20 * 1.0, "bwd_ms": 20 * 2.0, "pad_ms": 40 * 0.5,
                "fwd_n": 20, "bwd_n": 20, "pad_n": 40}


def test_windowed_roofline_counts_every_shot_once_per_step(monkeypatch):
    monkeypatch.setattr(bench, "measured_peak", lambda: (1000.0, "measured"))
    NZ, nz, N2, wn = 40, 30, 5, [20, 10, 30]
    r = bench.windowed_roofline(_FakeEngine(), lambda: None, NZ, nz, N2, wn, nbl=2)
    per_step = sum(16 * (NZ * (w + 2 * N2) + nz * w) + 32 * nz * w for w in wn)
    # 2 batches of 10 backward steps: each shot 10 steps, 40 ms in all
    assert r["achieved"] == pytest.approx(per_step * 10 / 0.040 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / 1000.0)
    assert r["launch_ms"] == pytest.approx(2.0) and r["pad_kernel_ms"] == pytest.approx(0.5)
    assert r["bound"] == "hbm" and r["unit"] == "GB/s"


def test_reference_arm_runs_without_the_product_library(tmp_path):
    """--impl reference on a small grid, in a fresh process: it prints the
    product arm's config, times the reference's loop, and never maps the
    product library (its problem comes from the oracle's restatement of the
    reference's host code)."""
    import json
    import os
    import subprocess
    code = (
        "import sys, json; sys.argv = ['bench.py', '--impl', 'reference', '--small', '--nt', '16',"
        " '--steps', '1', '--warmup', '1']; import bench; bench.main();"
        " maps = open('/proc/self/maps').read();"
        " print(json.dumps({'product_mapped': 'librtm_gb300' in maps}))")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", code], cwd=root, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    line, maps = lines[0], lines[-1]
    assert maps["product_mapped"] is False
    assert line["impl"] == "reference" and line["value"] > 0 and line["steps"] == 1
    assert line["config"] == bench.Config(_args("--small", "--nt", "16")).workload()
    assert line["cpu_baseline"]["kind"] in ("reference", "port")
    assert "reference_gpu" in line  # timed, or "unavailable" without a GPU


def test_snapshot_option_config_and_bytes():
    """--snap: the config names the snapshot storage and drops the rings;
    the snapshot bytes per shot follow the engine's layout (slots 0, 1, 2,
    2+K, .. <= NT-3 of the interior at a pitch of 8 values, source field and
    its running sum; the band of 24 cells around the surface receiver line at
    every step, fp32)."""
    cfg = bench.Config(_args("--snap", "4", "--snap-storage", "f16"))
    w = cfg.workload()
    assert w["snapshots"] == {"every": 4, "storage": "f16"} and w["ring_storage"] == "none"
    assert "snapshots every 4 steps" in w["workload"]
    slots = 3 + (cfg.NT - 5) // 4
    pitch = (cfg.nx + cfg.N2 % 8 + 7) // 8 * 8
    band = (1 + 24 + 1) * (cfg.nx - 1 + 2 * 24 + 1) * (cfg.NT - 2) * 8
    assert cfg.snap_bytes() == slots * cfg.nz * pitch * (2 + 4) + band
    assert bench.Config(_args()).workload()["snapshots"] is None


def test_reference_arm_refuses_snapshots(capsys):
    """The reference stores no snapshots: its arm prints its unavailable line
    (and exits 0) instead of timing a different migration."""
    old = sys.argv
    sys.argv = ["bench.py", "--impl", "reference", "--snap", "4"]
    try:
        bench.main()
    finally:
        sys.argv = old
    line = capsys.readouterr().out.strip().splitlines()[-1]
    import json
    d = json.loads(line)
    assert d["impl"] == "reference" and "snapshots" in d["unavailable"]


@pytest.mark.parametrize("argv", [["--snap", "4", "--workload", "c1"], ["--snap", "4", "--workload", "rvsp"],
                                  ["--snap", "-1"]])
def test_snapshot_option_only_where_it_applies(argv):
    with pytest.raises(SystemExit):
        _args(*argv)
