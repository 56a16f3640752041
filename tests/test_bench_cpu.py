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
