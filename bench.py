"""Benchmark of the RTM propagate/migrate path on one GB300 (or N, one
process per GPU, shots sharded across ranks).

Workloads (--workload):
* multishot (default): the plain multi-shot configuration -- a 401x1201
  seeded layered model (12 dipping layers 1500-5500 m/s, two normal faults, a
  low-velocity lens), dx=dz=12.5 m, dt=1 ms, 4000 steps, M=8 adaptive
  least-squares coefficients, 30-cell hybrid ABC, 64 surface shots with
  full-spread receivers, FP16 boundary rings, images stacked with Kahan
  summation.  A step is the full migration of the 64 shots: forward source
  run, boundary-ring reconstruction, receiver back-propagation, imaging,
  per-shot finishing and the stack.
* c1: the plain single-shot configuration -- 201x401, dx=dz=10 m, 2000
  steps, M=6 adaptive coefficients, 20 Hz source at (2,200), 401 surface
  receivers, FP32 throughout; a step is one migration of the shot, with L2
  flushed between timed steps.
* rvsp: batched uneven aperture windows with well receivers (autotuned).
* c5: learned coefficients on the 1201x4001 model.
The observed gathers are modelled first (true model minus smoothed model,
removing the direct wave) and stay resident in HBM for `value`; `e2e` takes
them from pinned host memory every step and returns the image to the host.

Metric: grid-cell updates per second, one update = one grid point advanced
one time step; per shot NT*(2*NZ*NX + nz*nx) (forward on the padded grid,
receiver wavefield on the padded grid, source reconstruction on the interior).

--impl reference times the reference's own propagation + imaging loop
(kernel.cu kernel bodies, compiled for the host cores by oracle/build_ref.py)
on a one-shot sample of the same workload, with all host threads, on a
problem prepared by the oracle's restatement of the reference's host code
(the product library is never loaded); its line also carries the
reference's own GPU kernels timed on one full shot (`reference_gpu`).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
# time steps of the CPU baseline's one-shot sample (about 10 s of the
# reference's kernel bodies on 16 host cores for the multi-shot grid)
CPU_SAMPLE_NT = 2000
# host seconds the whole reference arm (warm-up and timed samples) may take
REF_BUDGET_S = 150.0
# stencil kernel forms by their RTM_KERNEL_* value
FORMS = ["tiled", "persistent", "tiled-split", "tiled-2col", "2col-split"]
sys.path.insert(0, ROOT)

METRIC = "Gcell-updates/s"


def cell_updates_per_shot(nz, nx, N2, NT):
    NZ, NX = nz + 2 * N2, nx + 2 * N2
    return NT * (2 * NZ * NX + nz * nx)


def kernel_forms(a):
    """(forward, backward) stencil forms of --kernel / --bwd-kernel."""
    from rtm_gpu_gb300 import capi
    v = {"tiled": capi.RTM_KERNEL_TILED, "persistent": capi.RTM_KERNEL_PERSISTENT,
         "split": capi.RTM_KERNEL_SPLIT, "x2": capi.RTM_KERNEL_X2,
         "x2-split": capi.RTM_KERNEL_X2_SPLIT}
    f = v[a.kernel]
    if a.bwd_kernel != "same":
        return f, v[a.bwd_kernel]
    return f, capi.RTM_KERNEL_TILED if f in (capi.RTM_KERNEL_X2, capi.RTM_KERNEL_X2_SPLIT) else f


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--shots", type=int, default=0, help="shots (0: the workload's own count)")
    ap.add_argument("--nt", type=int, default=0, help="time steps (0: the workload's own count)")
    ap.add_argument("--batch", type=int, default=0, help="shots per batch (0: all)")
    ap.add_argument("--coef", default="adaptive", choices=["adaptive", "taylor"])
    ap.add_argument("--ring", default=None, choices=["f32", "bf16", "f16", "i16"],
                    help="boundary-ring storage (stencil and imaging stay FP32); default f16 "
                         "for the multi-shot workload, f32 for c1 and rvsp (FP32 throughout), "
                         "i16 for c5")
    ap.add_argument("--no-plain", action="store_true",
                    help="skip timing the plain single-shot drop-in for comparison")
    ap.add_argument("--cpu-sample-nt", type=int, default=0,
                    help="time steps of the one-shot CPU sample (0: %d, about 10 s on 16 cores)"
                         % CPU_SAMPLE_NT)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--snap", type=int, default=0,
                    help="multishot: source snapshots every SNAP steps instead of boundary rings "
                         "(the backward run images at the snapshot steps; 0: the ring scheme)")
    ap.add_argument("--snap-storage", default="f16", choices=["f32", "bf16", "f16", "i16"])
    ap.add_argument("--no-fp64-check", action="store_true",
                    help="skip the one-shot image check against the FP64 oracle")
    ap.add_argument("--small", action="store_true", help="reduced grid for quick checks")
    ap.add_argument("--kernel", default="auto", choices=["auto", "tiled", "persistent", "split", "x2", "x2-split"],
                    help="stencil kernel form (auto: the autotuner picks it and shots per launch)")
    ap.add_argument("--bwd-kernel", default="same", choices=["same", "tiled", "persistent", "split"],
                    help="backward stencil form with a fixed --kernel (same: --kernel's, tiled for x2 forms)")
    ap.add_argument("--workload", default="multishot", choices=["multishot", "c1", "rvsp", "c5"],
                    help="c1: the single-shot 201x401 configuration; rvsp: batched uneven "
                         "aperture windows, well receivers, autotuned; c5: learned coefficients, "
                         "1201x4001 model, FP16 rings, uneven apertures")
    a = ap.parse_args()
    if a.snap and a.workload != "multishot":
        ap.error("--snap applies to the multishot workload")
    if a.snap < 0:
        ap.error("--snap takes a positive step count")
    return a


class Config:
    """The multi-shot (default) or single-shot (c1) configuration."""

    def __init__(self, a):
        self.name = "c1" if a.workload == "c1" else "multishot"
        self.small = a.small
        if self.name == "c1":
            self.nz, self.nx = 201, 401
            self.N2, self.M = 30, 6
            self.h, self.tao, self.f0 = 10.0, 0.001, 20.0
            self.NT = a.nt or 2000
            self.nshot = 1
        else:
            self.nz, self.nx = (101, 301) if a.small else (401, 1201)
            self.N2, self.M = 30, 8
            self.h, self.tao, self.f0 = 12.5, 0.001, 25.0
            self.NT = a.nt or 4000
            self.nshot = a.shots or 64
        self.coef = a.coef
        # c5: scaled int16 (the 16-bit storage that keeps the image within 1e-3
        # of FP64 over its 8000 steps; BF16 and FP16 rings do not, --ring bf16)
        self.ring = a.ring or {"multishot": "f16", "c1": "f32", "rvsp": "f32", "c5": "i16"}[a.workload]
        self.whitecoe = 1e-4
        # source snapshots every `snap` steps (0: the ring scheme)
        self.snap = getattr(a, "snap", 0) or 0
        self.snap_storage = getattr(a, "snap_storage", "f16")
        # optimiser settings (the reference's parameter file: nthita=1000,
        # eps=1e-5, df=1; fmax = 2*f0)
        self.fmax, self.df, self.nthita, self.eps, self.nfdmin = 2 * self.f0, 1.0, 1000, 1e-5, 2

    def true_model(self):
        from rtm_gpu_gb300 import synth
        return synth.model_c1() if self.name == "c1" else synth.model_c2(nz=self.nz, nx=self.nx)

    def shots(self, n=None):
        """Source cells (z, x) in the padded grid."""
        from rtm_gpu_gb300 import synth
        if self.name == "c1":  # 20 Hz source at (z=2, x=200), 1-based interior indices
            return [(self.N2 + 1, self.N2 + 199)]
        return synth.surface_shots(self.nx, n or self.nshot, self.N2)

    def receivers(self):
        from rtm_gpu_gb300 import synth
        return synth.full_spread(self.nx, self.N2)

    def ring_bytes(self):
        b = 4 if self.ring == "f32" else 2
        return self.NT * 2 * self.M * (self.nz + self.nx) * b

    def snap_bytes(self):
        """Snapshot bytes of one shot (source field, and its running sum in fp32)."""
        b = 4 if self.snap_storage == "f32" else 2
        pitch = (self.nx + self.N2 % 8 + 7) // 8 * 8
        rows = (self.N2 + 1 + 24) - self.N2 + 1  # surface receiver line: rows N2 .. N2+1+24
        band = rows * (self.nx - 1 + 2 * 24 + 1) * (self.NT - 2) * 8  # imaged every step, fp32
        return (3 + (self.NT - 5) // self.snap) * self.nz * pitch * (b + 4) + band

    def workload(self):
        """The `config` of both arms' bench lines (identical by construction)."""
        if self.name == "c1":
            text = ("single-shot RTM %dx%d interior, dx=dz=%g m, 30-cell hybrid ABC, M=%d %s "
                    "coefficients, %d steps, 20 Hz source at (2,200), %d surface receivers, FP32 "
                    "throughout" % (self.nz, self.nx, self.h, self.M, self.coef, self.NT, self.nx))
            l2 = "L2 flushed between timed steps (a 512 MB buffer written)"
        elif self.snap:
            text = ("multi-shot RTM %dx%d interior, 30-cell hybrid ABC, M=%d %s coefficients, "
                    "%d steps, %d surface shots, full-spread receivers, FP32 stencil/imaging, "
                    "source snapshots every %d steps in %s, their running sums in FP32 (no rings, "
                    "no source reconstruction: the "
                    "backward run images at every %dth step with end-corrected weights), Kahan "
                    "stack; Gcell-updates counted as for the ring scheme's migration of the same "
                    "shots" % (self.nz, self.nx, self.M, self.coef, self.NT, self.nshot, self.snap,
                               self.snap_storage.upper(), self.snap))
            l2 = ("inputs larger than L2 (the %d shots' snapshots are %.1f GB)"
                  % (self.nshot, self.nshot * self.snap_bytes() / 1e9))
        else:
            text = ("multi-shot RTM %dx%d interior, 30-cell hybrid ABC, M=%d %s coefficients, "
                    "%d steps, %d surface shots, full-spread receivers, FP32 stencil/imaging, %s "
                    "boundary rings, Kahan stack" % (self.nz, self.nx, self.M, self.coef, self.NT,
                                                     self.nshot, self.ring.upper()))
            l2 = ("inputs larger than L2 (the %d shots' boundary rings alone are %.1f GB)"
                  % (self.nshot, self.nshot * self.ring_bytes() / 1e9))
        return {"workload": text, "nz": self.nz, "nx": self.nx, "N2": self.N2, "M": self.M,
                "nt": self.NT, "shots": self.nshot, "dx_m": self.h, "dt_s": self.tao,
                "coefficients": self.coef, "ring_storage": "none" if self.snap else self.ring,
                "snapshots": {"every": self.snap, "storage": self.snap_storage} if self.snap else None,
                "l2": l2,
                "reference_timing": "the reference arm times one shot of this grid over a "
                                    "prefix of its time steps and reports that sample's rate"}


def build_problems(cfg, dv=1.0):
    from rtm_gpu_gb300 import synth
    from rtm_gpu_gb300.problem import build_problem
    vtrue = cfg.true_model()
    vmig = synth.smooth_model(vtrue, 10.0)
    table = None
    if cfg.coef == "adaptive":
        from rtm_gpu_gb300 import coeffs
        table = coeffs.table_source(nfdmax=cfg.M, nfdmin=cfg.nfdmin, tao=cfg.tao, h=cfg.h,
                                    fmax=cfg.fmax, df=cfg.df, nthita=cfg.nthita, eps=cfg.eps)
    kw = dict(N2=cfg.N2, M=cfg.M, NT=cfg.NT, h=cfg.h, tao=cfg.tao, f0=cfg.f0,
              adaptive=cfg.coef == "adaptive", compen=True, rec=cfg.receivers(), dv=dv,
              coef_table=table)
    ptrue = build_problem(vtrue, **kw)
    pmig = build_problem(vmig, **kw)
    return ptrue, pmig, cfg.shots()


class Clocks:
    """nvidia-smi sampling during the timed region (samples kept in a
    temporary file)."""

    def __init__(self):
        fd, self.path = tempfile.mkstemp(prefix="rtm_bench_clocks_", suffix=".csv")
        os.close(fd)
        self.p = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *exc):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(5)
            except Exception:
                self.p.kill()
            self.f.close()

    def summary(self, dev_index=0):
        try:
            rows = [l.split(",") for l in open(self.path) if l.strip()]
            os.unlink(self.path)
        except Exception:
            return None
        rows = [[c.strip() for c in r] for r in rows if len(r) >= 9 and r[0].strip() == str(dev_index)]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


def measured_peak():
    try:
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def measured_traffic(cfg, shots_per_launch):
    """DRAM bytes of one backward-stencil launch from the committed ncu
    capture of this workload (profiles/ncu_traffic.json), or None."""
    key = "k_step backward, %s M=%d, %dx%d, %d shots per launch" % (
        cfg.coef, cfg.M, cfg.nz, cfg.nx, shots_per_launch)
    try:
        d = json.load(open(os.path.join(ROOT, "profiles", "ncu_traffic.json")))[key]
        return {"bytes": d["dram_bytes_read"] + d["dram_bytes_write"], "source": "profiles/" + d["summary"]}
    except Exception:
        return None


def cpu_sample(prob, seis_row, nt_sample, threads):
    """Reference kernel bodies (oracle/_ref) or, failing that, the oracle's
    C restatement, timed on the host cores: one migration of one shot over
    the first nt_sample time steps.  Returns (seconds, cell-updates, kind)."""
    import dataclasses
    from oracle import oracle as orc
    kind = "reference"
    try:
        orc.ref()
    except Exception:
        kind = "port"
    orc.set_threads(threads)
    p = dataclasses.replace(prob, NT=nt_sample, wav=prob.wav[: nt_sample + 1])
    s = np.ascontiguousarray(seis_row[:, :nt_sample], np.float32)
    t0 = time.perf_counter()
    orc.migrate(p, s, use_ref=(kind == "reference"))
    dt = time.perf_counter() - t0
    return dt, cell_updates_per_shot(p.nz, p.nx, p.N2, nt_sample), kind


def cpu_baseline(pmig, shot, seis_row, nt_sample, threads):
    """cpu_baseline object of the bench line (one timed one-shot sample)."""
    dt, cu, kind = cpu_sample(pmig.with_source(*shot), seis_row, nt_sample, threads)
    return {"value": cu / dt / 1e9, "unit": METRIC, "cores": threads, "kind": kind,
            "sample": "one shot of the workload grid, %d time steps (%.3g cell-updates), %.1f s"
                      % (nt_sample, cu, dt)}


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    n = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / n) if n > 0 else float("nan")


FP64_PIPELINE_NOTE = ("image: same observed gathers on both sides (the migration's error); "
                      "image_fp64_pipeline: the oracle also models the synthetic gathers in FP64, "
                      "so FP32 rounding of the gathers, amplified by the Laplacian filter and the "
                      "illumination division, is included (the reference's own FP32 pipeline "
                      "shows the same, 2.4e-3 at one shot of the multi-shot workload)")


def fp64_check(eng, ptrue, pmig, shot, seis_row, whitecoe, what):
    """Image error of one shot of the benched workload against the FP64
    oracle.  The product migrates the shot (its ring storage and kernels as
    benched) and finishes it (Laplacian filter, illumination stabilisation,
    normalisation by the illumination); the oracle does the same in FP64 on
    the same observed gathers ("image"), and on gathers that it models itself
    in FP64 from the true and smoothed models ("image_fp64_pipeline", which
    adds the FP32 modelling error of the synthetic data)."""
    from oracle import oracle as orc
    orc.set_threads(os.cpu_count() or 1)
    q = pmig.with_source(*shot)
    src = q.src_flat()
    seis = np.ascontiguousarray(seis_row, np.float32)
    img = np.zeros((q.nz, q.nx), np.float32)
    ill = np.zeros_like(img)
    eng.migrate_stack([src], seis[None], whitecoe, 1, True, image=img, illum=ill)
    t0 = time.perf_counter()
    d1, d2 = orc.migrate(q, seis, precision="f64")
    up, dn = orc.finish_shot(q, d1, d2, whitecoe)  # column-major [nx, nz]
    out = {"image": rel_l2(img, (up / dn).T), "illumination": rel_l2(ill, dn.T)}
    g64 = orc.model(ptrue.with_source(*shot), precision="f64") - orc.model(q, precision="f64")
    e1, e2 = orc.migrate(q, g64.astype(np.float32), precision="f64")
    up2, dn2 = orc.finish_shot(q, e1, e2, whitecoe)
    out["image_fp64_pipeline"] = rel_l2(img, (up2 / dn2).T)
    out["note"] = FP64_PIPELINE_NOTE
    out["shot"] = [int(shot[0]), int(shot[1])]
    out["what"] = what
    out["oracle_s"] = time.perf_counter() - t0
    return out


def fp64_check_window(eng, ptrue, pmig, i, src_full, wsrc, xa, wn, seis_row, whitecoe, what):
    """fp64_check for shot i of a batch of aperture windows: the product
    migrates the shot on its window (migrate_stack_windows, kernels and ring
    storage as benched); the oracle migrates the window problem in FP64 on
    the same gathers and on gathers it models itself in FP64 on the whole
    survey (true minus smoothed model, as the bench's gathers are made)."""
    from oracle import oracle as orc
    from oracle.port_problem import window_problem
    orc.set_threads(os.cpu_count() or 1)
    x0, w = int(xa[i]), int(wn[i])
    q = window_problem(pmig, x0, w)
    q = q.with_source(wsrc[i] // q.NX, wsrc[i] % q.NX)
    seis = np.ascontiguousarray(seis_row, np.float32)
    img = np.zeros((pmig.nz, pmig.nx), np.float32)
    ill = np.zeros_like(img)
    eng.migrate_stack_windows([wsrc[i]], [x0], [w], seis[None], whitecoe, 1, True, image=img,
                              illum=ill)
    img, ill = img[:, x0:x0 + w], ill[:, x0:x0 + w]
    t0 = time.perf_counter()
    d1, d2 = orc.migrate(q, seis, precision="f64")
    up, dn = orc.finish_shot(q, d1, d2, whitecoe)
    out = {"image": rel_l2(img, (up / dn).T), "illumination": rel_l2(ill, dn.T)}
    zf, xf = divmod(int(src_full), pmig.NX)
    g64 = (orc.model(ptrue.with_source(zf, xf), precision="f64") -
           orc.model(pmig.with_source(zf, xf), precision="f64"))
    e1, e2 = orc.migrate(q, g64.astype(np.float32), precision="f64")
    up2, dn2 = orc.finish_shot(q, e1, e2, whitecoe)
    out["image_fp64_pipeline"] = rel_l2(img, (up2 / dn2).T)
    out["note"] = FP64_PIPELINE_NOTE
    out["shot"] = int(i)
    out["window"] = [x0, w]
    out["what"] = what
    out["oracle_s"] = time.perf_counter() - t0
    return out


def run_reference_arm(a, cfg):
    """The reference's own CPU implementation of the path (kernel.cu kernel
    bodies on all host cores) on one shot of the workload, each step a
    sample over a prefix of the shot's time steps sized so that the whole
    run stays within REF_BUDGET_S.  The problem is prepared by the oracle's
    restatement of the reference's host code (velocity padding, bins, the
    FP64 least-squares table of funMandC), so no product code runs."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as orc
    from oracle.port_problem import build_problem_port
    from rtm_gpu_gb300 import synth
    threads = os.cpu_count() or 1
    orc.set_threads(threads)
    vmig = synth.smooth_model(cfg.true_model(), 10.0)
    prob = build_problem_port(vmig, N2=cfg.N2, M=cfg.M, NT=cfg.NT, h=cfg.h, tao=cfg.tao, f0=cfg.f0,
                              adaptive=cfg.coef == "adaptive", compen=True, rec=cfg.receivers(),
                              fmax=cfg.fmax, df=cfg.df, nthita=cfg.nthita, eps=cfg.eps,
                              nfdmin=cfg.nfdmin)
    shots = cfg.shots()
    p1 = prob.with_source(*shots[len(shots) // 2])
    rng = np.random.default_rng(7)
    seis = (rng.standard_normal((p1.nrec, cfg.NT)) * 1e-3).astype(np.float32)
    # rate from a short run, then samples of about min(10 s, budget / steps)
    dt, cu, kind = cpu_sample(p1, seis, min(100, cfg.NT), threads)
    rate = cu / dt
    per_step_s = min(10.0, REF_BUDGET_S / max(1, a.steps + a.warmup))
    nt = int(min(cfg.NT, max(20, per_step_s * rate / (cu / min(100, cfg.NT)))))
    for _ in range(a.warmup):
        cpu_sample(p1, seis, nt, threads)
    times = [cpu_sample(p1, seis, nt, threads)[0] for _ in range(a.steps)]
    cu_s = cell_updates_per_shot(cfg.nz, cfg.nx, cfg.N2, nt)
    v = cu_s * len(times) / sum(times) / 1e9
    ms = 1e3 * sum(times) / len(times)
    cu_all = cell_updates_per_shot(cfg.nz, cfg.nx, cfg.N2, cfg.NT) * cfg.nshot
    sample = ("one shot of the workload grid (seeded random gathers), the first %d of its %d time "
              "steps of the forward and backward runs (%.3g cell-updates per step)" % (nt, cfg.NT, cu_s))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": METRIC, "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": cfg.workload(),
            "workload_seconds_at_this_rate": cu_all / (v * 1e9),
            "cpu_baseline": {"value": v, "unit": METRIC, "cores": threads, "kind": kind,
                             "sample": sample},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "reference_gpu": reference_gpu(p1, seis)}
    print(json.dumps(line))


def reference_gpu(prob, seis):
    """The reference's own GPU kernels (kernel.cu:18-517, unchanged, nvcc for
    sm_103a) with its per-shot launch sequence (kernel.cu:788-933, stock
    16x16 blocks), timed on one full shot after one warm-up shot."""
    from oracle import oracle as orc
    try:
        orc.ref_gpu_migrate(prob, seis)
        _, _, sec = orc.ref_gpu_migrate(prob, seis)
    except Exception as exc:
        return {"unavailable": str(exc).splitlines()[0][:200]}
    cu = cell_updates_per_shot(prob.nz, prob.nx, prob.N2, prob.NT)
    return {"seconds_per_shot": sec, "shots_per_hour": 3600.0 / sec, "value": cu / sec / 1e9,
            "unit": METRIC,
            "what": "kernel.cu's 17 kernels compiled unchanged by nvcc for sm_103a, driven by its "
                    "per-shot launch sequence (16x16 blocks, default stream, per-step receiver "
                    "copy), one full shot, host wall clock"}


def rvsp_geometry(cfg, nshot=128, seed=1237, wmin=300, wmax=1201, well_x=600, z0=50, nrec=300):
    """Reverse-VSP survey on the multi-shot model: nshot surface sources, each
    with a seeded aperture window of width U[wmin, wmax] columns around it
    that contains the well (origin rounded down to a multiple of 4 columns,
    the width grown to match); nrec receivers down the well at interior column
    well_x, depths z0 .. z0+nrec-1.  Returns (sources (z, x) in the survey's
    padded grid, window starts, window widths, receiver line)."""
    rng = np.random.default_rng(seed)
    N2, nx = cfg.N2, cfg.nx
    xs = np.linspace(0, nx - 1, nshot).round().astype(int)
    w = rng.integers(wmin, min(wmax, nx) + 1, nshot)
    xa = np.clip(xs - w // 2, np.maximum(0, well_x - w + 1), np.minimum(well_x, nx - w))
    # window origins on multiples of 4 columns (the engine then reads the
    # window-interior model from the survey grid); the window grows by the
    # columns the origin moved, so it still ends where it did
    r = xa % 4
    xa, w = xa - r, np.minimum(w + r, nx - (xa - r))
    sx = np.clip(xs, xa, xa + w - 1)
    src = [(N2 + 1, N2 + int(x)) for x in sx]
    return src, xa.astype(np.int32), w.astype(np.int32), (N2 + z0, N2 + well_x, 1, 0, nrec)


def windowed_roofline(eng, step, NZ, nz, N2, wn, nbl):
    """Roofline of the backward stencil (the dominant kernel) for shots of
    uneven windows: the algorithmic bytes of all its launches in one
    migration (per launch and shot: 16 B per receiver-field cell of the
    padded window, 16 B per source-field cell and 32 B of compensated
    imaging per interior cell) over their summed CUDA-event durations."""
    eng.set_timing(True)
    step()
    tm = eng.timing()
    eng.set_timing(False)
    nbatch = -(-len(wn) // nbl)
    steps = tm["bwd_n"] / max(nbatch, 1)  # backward launches of one batch
    bwd_step = sum(16 * (NZ * (int(w) + 2 * N2) + nz * int(w)) + 32 * nz * int(w) for w in wn)
    fwd_step = sum(16 * NZ * (int(w) + 2 * N2) for w in wn)
    achieved = bwd_step * steps / (tm["bwd_ms"] / 1e3) / 1e9
    peak, peak_kind = measured_peak()
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": None,
            "kernel": "k_step<backward> (source reconstruction + receiver step + imaging)",
            "bytes_per_launch": bwd_step / max(nbatch, 1), "launch_ms": tm["bwd_ms"] / max(tm["bwd_n"], 1),
            "peak_kind": peak_kind,
            "forward_kernel": {"launch_ms": tm["fwd_ms"] / max(tm["fwd_n"], 1),
                               "achieved": fwd_step * steps / (tm["fwd_ms"] / 1e3) / 1e9},
            "pad_kernel_ms": tm["pad_ms"] / max(tm["pad_n"], 1)}


def run_rvsp(a, cfg):
    """Batched uneven shots (reverse VSP): all shots' windows advance
    together; kernel form and shots per launch from the autotuner; FP32."""
    import torch
    from rtm_gpu_gb300 import Engine, capi, synth
    from rtm_gpu_gb300.problem import build_problem
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    nshot = a.shots or 128
    src, xa, wn, rec = rvsp_geometry(cfg, nshot=nshot)
    vtrue = synth.model_c2(nz=cfg.nz, nx=cfg.nx)
    vmig = synth.smooth_model(vtrue, 10.0)
    table = None
    if cfg.coef == "adaptive":
        from rtm_gpu_gb300 import coeffs
        table = coeffs.table_source(nfdmax=cfg.M, nfdmin=cfg.nfdmin, tao=cfg.tao, h=cfg.h,
                                    fmax=cfg.fmax, df=cfg.df, nthita=cfg.nthita, eps=cfg.eps)
    kw = dict(N2=cfg.N2, M=cfg.M, NT=cfg.NT, h=cfg.h, tao=cfg.tao, f0=cfg.f0,
              adaptive=cfg.coef == "adaptive", compen=True, rec=rec, coef_table=table)
    ptrue, pmig = build_problem(vtrue, **kw), build_problem(vmig, **kw)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sh = stream.cuda_stream
    batch = a.batch or nshot
    # observed data on the whole survey (true minus smoothed model)
    full_src = [pmig.src_flat(z, x) for z, x in src]
    seis = torch.zeros((nshot, pmig.nrec, pmig.NT), dtype=torch.float32, device="cuda")
    tmp = torch.zeros_like(seis)
    with Engine(ptrue, batch=min(batch, 64), stream=sh) as e:
        e.model(full_src, out=seis)
    with Engine(pmig, batch=min(batch, 64), stream=sh) as e:
        e.model(full_src, out=tmp)
    seis -= tmp
    del tmp
    # sources in each shot's own padded grid
    wsrc = [z * (int(w) + 2 * cfg.N2) + (x - int(x0)) for (z, x), x0, w in zip(src, xa, wn)]
    ring = ring_flag(cfg)
    eng = Engine(pmig, batch=batch, stream=sh, ring_precision=ring)
    tuned = None
    if a.kernel == "auto":
        tuned = eng.autotune(wsrc, xa, wn, nsteps=20)
    else:
        eng.set_kernel(*kernel_forms(a))
    kern = eng.kernel()
    img = torch.zeros((pmig.nz, pmig.nx), dtype=torch.float32, device="cuda")
    ill = torch.zeros_like(img)

    def step():
        eng.migrate_stack_windows(wsrc, xa, wn, seis, cfg.whitecoe, nshot, True, image=img, illum=ill)

    for _ in range(max(3, a.warmup)):
        step()
    torch.cuda.synchronize()
    eng.launches(reset=True)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks() as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(a.steps):
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / a.steps
    launches = eng.launches()
    NZ = pmig.NZ
    cu = sum(cfg.NT * (2 * NZ * (int(w) + 2 * cfg.N2) + cfg.nz * int(w)) for w in wn)
    # end to end: gathers from pinned host memory, image back to the host
    seis_h = seis.cpu().pin_memory()
    img_h = torch.zeros((pmig.nz, pmig.nx), dtype=torch.float32).pin_memory()
    ill_h = torch.zeros_like(img_h).pin_memory()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(a.steps):
        eng.migrate_stack_windows(wsrc, xa, wn, seis_h, cfg.whitecoe, nshot, True, image=img_h,
                                  illum=ill_h)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_e2e = e0.elapsed_time(e1) / a.steps
    roofline = windowed_roofline(eng, step, NZ, cfg.nz, cfg.N2, wn, kern["shots_per_launch"])
    fp64 = None
    if not a.no_fp64_check:
        i = nshot // 2
        fp64 = fp64_check_window(eng, ptrue, pmig, i, full_src[i], wsrc, xa, wn,
                                 seis_h[i].numpy(), cfg.whitecoe,
                                 "shot %d of %d on its window, %s rings, kernels as benched"
                                 % (i, nshot, cfg.ring.upper()))
    line = {"metric": METRIC, "value": cu / (ms / 1e3) / 1e9, "unit": METRIC, "n_gpus": 1,
            "steps": a.steps, "warmup": max(3, a.warmup), "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "batched uneven shots, reverse VSP: %dx%d model, %d surface "
                                   "sources with aperture windows of 300-1201 columns, %d well "
                                   "receivers at x=600, z=50..%d, %d steps, M=%d %s, %s rings"
                                   % (cfg.nz, cfg.nx, nshot, rec[4], 50 + rec[4] - 1, cfg.NT,
                                      cfg.M, cfg.coef, cfg.ring.upper()),
                       "shots": nshot, "mean_window": float(np.mean(wn)), "batch": batch,
                       "autotuned": {"fwd_kernel": FORMS[kern["fwd"]],
                                     "bwd_kernel": FORMS[kern["bwd"]],
                                     "shots_per_launch": kern["shots_per_launch"],
                                     "tuning_gcells_per_s": tuned},
                       "l2": "inputs larger than L2 (%.1f GB of wavefields and rings)"
                             % (eng.device_bytes / 1e9)},
            "shots_per_hour": nshot / (ms / 1e3) * 3600,
            "e2e": {"value": cu / (ms_e2e / 1e3) / 1e9, "unit": METRIC,
                    "h2d_bytes_per_step": int(seis_h.numel() * 4),
                    "d2h_bytes_per_step": int((img_h.numel() + ill_h.numel()) * 4)},
            "roofline": roofline, "nrmse_vs_fp64": fp64,
            "clocks": clk.summary(0), "gpu_launches": launches,
            "gpu_launches_per_step": launches // a.steps}
    print(json.dumps(line))
    eng.close()


def run_c5(a, cfg):
    """Learned coefficients plus the full stack on the 1201x4001 model
    (dx=dz=10 m, 1500-6000 m/s gradients with salt-like 4500 m/s bodies):
    the coefficient table comes from the MLP (inputs r, kmax*h, M in 4..10)
    trained on the GPU on 200k FP64 optimiser samples of the survey's (r, kh)
    range, judged by the FP64 dispersion error in the reference's own
    measure, with the optimiser's set kept wherever the network's misses 1e-4
    and the optimiser's is better; shots with uneven aperture windows, int16
    rings (--ring), autotuned kernels.  --shots / --nt set the shot count and
    steps (defaults 8 x 8000; the configuration has 256 x 8000); shots run
    in launches of --batch (default up to 64)."""
    import torch
    from rtm_gpu_gb300 import Engine, coeffs, mlp, synth
    from rtm_gpu_gb300.problem import build_problem, f32
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    nz, nx, N2, h, tao, f0, M = 1201, 4001, 30, 10.0, 0.001, 25.0, 8
    nshot = a.shots or 8
    nt = a.nt or 8000
    batch = a.batch or min(nshot, 64)
    vtrue = synth.model_c5(nz=nz, nx=nx)
    vmig = synth.smooth_model(vtrue, 10.0)
    fmax = 2 * f0
    tol = 1e-4
    vlo, vhi = float(vmig.min()), float(vmig.max())
    t0 = time.perf_counter()
    net, train_loss = mlp.train_default(n=200_000, epochs=30, seed=5, batch=512, lr=3e-3,
                                        r_range=(vlo * tao / h * 0.98, vhi * tao / h * 1.02),
                                        kh_range=(2 * np.pi * fmax * h / vhi * 0.98,
                                                  2 * np.pi * fmax * h / vlo * 1.02),
                                        m_range=(4, 10))
    t_train = time.perf_counter() - t0
    info_box = {}

    def table(vmin, dv, nvel, need, hzx):
        assert dv == 1.0
        length, index, coef, info = net.table(M=M, tol=tol, tao=tao, h=h, fmax=fmax, vmin=vmin,
                                              nvel=nvel, need=need, metric=mlp.DISP_REFERENCE)
        info_box.update(info, coef=coef, index=index)
        return length, index, coef

    # surface receivers on interior columns 1500..2499, common to every
    # window; windows of seeded widths 1500..4001 placed to contain them
    rec = (N2 + 1, N2 + 1500, 0, 1, 1000)
    kw = dict(N2=N2, M=M, NT=nt, h=h, tao=tao, f0=f0, adaptive=True, compen=True, rec=rec)
    pmig = build_problem(vmig, coef_table=table, **kw)
    info = dict(info_box)
    # optimiser alone on the same bins, for the comparison
    sel = np.nonzero(info["err_used"] >= 0)[0]
    r = (pmig.vmin + sel) * float(f32(tao)) / float(f32(h))
    bb = 2.0 * 3.1415926535898 * float(f32(fmax)) * float(f32(tao)) / r
    t1 = time.perf_counter()
    copt = coeffs.ls_coefs(r, bb, M)
    t_opt = time.perf_counter() - t1
    Ms = np.full(len(sel), M)
    tab = np.stack([info["coef"][info["index"][i]:info["index"][i] + M + 1] for i in sel]).astype(np.float64)
    nk = int(fmax)
    dref = dict(nk=nk, metric=mlp.DISP_REFERENCE, tao=float(f32(tao)))
    errs = {"network": info["err_net"][sel], "optimiser": mlp.dispersion_error(copt, Ms, r, bb, **dref),
            "table": info["err_used"][sel]}
    rel = {"optimiser": mlp.dispersion_error(copt, Ms, r, bb, nk=nk),
           "table": mlp.dispersion_error(tab, Ms, r, bb, nk=nk)}
    ptrue = build_problem(vtrue, coef_table=table, **kw)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sh = stream.cuda_stream
    rng = np.random.default_rng(1240)
    wn = rng.integers(1500, nx + 1, nshot)
    xa = np.array([rng.integers(max(0, 2500 - w), min(1500, nx - w) + 1) for w in wn])
    xs = xa + wn // 2
    src_full = [pmig.src_flat(N2 + 1, N2 + int(x)) for x in xs]
    seis = step_gathers(Engine, ptrue, pmig, src_full, min(nshot, 8), sh, torch)
    wsrc = [(N2 + 1) * (int(w) + 2 * N2) + N2 + int(x) - int(x0) for x, x0, w in zip(xs, xa, wn)]
    eng = Engine(pmig, batch=batch, stream=sh, ring_precision=ring_flag(cfg))
    tuned = eng.autotune(wsrc[:batch], xa[:batch], wn[:batch], nsteps=10)
    kern = eng.kernel()
    img = torch.zeros((nz, nx), dtype=torch.float32, device="cuda")
    ill = torch.zeros_like(img)

    def step():
        eng.migrate_stack_windows(wsrc, xa, wn, seis, 1e-4, nshot, True, image=img, illum=ill)

    for _ in range(max(3, a.warmup)):
        step()
    torch.cuda.synchronize()
    eng.launches(reset=True)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks() as clk:
        ev0.record(stream)
        for _ in range(a.steps):
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / a.steps
    launches = eng.launches()
    NZ = nz + 2 * N2
    cu = sum(nt * (2 * NZ * (int(w) + 2 * N2) + nz * int(w)) for w in wn)
    roofline = windowed_roofline(eng, step, NZ, nz, N2, wn, kern["shots_per_launch"])
    fp64 = None
    if not a.no_fp64_check:
        seis_h = seis.cpu()
        i = 0
        fp64 = fp64_check_window(eng, ptrue, pmig, i, src_full[i], wsrc, xa, wn, seis_h[i].numpy(),
                                 1e-4, "shot %d of %d on its window, %s rings, kernels as benched"
                                 % (i, nshot, cfg.ring.upper()))
    line = {"metric": METRIC, "value": cu / (ms / 1e3) / 1e9, "unit": METRIC, "n_gpus": 1,
            "steps": a.steps, "warmup": max(3, a.warmup), "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "learned coefficients + full stack: 1201x4001 model, dx=dz=10 m, "
                                   "%d shots with aperture windows of 1500-4001 columns, 1000 surface "
                                   "receivers, %d steps, M=%d MLP table (optimiser kept where the "
                                   "network misses 1e-4 and the optimiser is better), %s rings"
                                   % (nshot, nt, M, cfg.ring.upper()),
                       "shots": nshot, "nt": nt, "mean_window": float(np.mean(wn)),
                       "l2": "inputs larger than L2 (%.1f GB)" % (eng.device_bytes / 1e9)},
            "engine": {"batch": batch, "fwd": FORMS[kern["fwd"]], "bwd": FORMS[kern["bwd"]],
                       "shots_per_launch": kern["shots_per_launch"], "chosen_by": "autotuner",
                       "tuning_gcells_per_s": tuned},
            "coefficients": {"bins": int(len(sel)), "from_network": int(len(sel) - info["fallback"]),
                             "tolerance": tol,
                             "measure": "(h/v)|v/v_FD-1| (the reference's operator-length test)",
                             "max_dispersion_error_network": float(errs["network"].max()),
                             "max_dispersion_error_optimiser": float(errs["optimiser"].max()),
                             "max_dispersion_error_table": float(errs["table"].max()),
                             "max_relative_phase_velocity_error_optimiser": float(rel["optimiser"].max()),
                             "max_relative_phase_velocity_error_table": float(rel["table"].max()),
                             "network_inputs": "r, kmax*h, M in 4..10; 200k optimiser samples",
                             "network_train_s": t_train, "network_train_loss": train_loss,
                             "table_s": info["seconds"], "optimiser_alone_s": t_opt},
            "roofline": roofline, "nrmse_vs_fp64": fp64,
            "clocks": clk.summary(0), "gpu_launches": launches}
    print(json.dumps(line))
    eng.close()


def step_gathers(Engine, ptrue, pmig, src, batch, stream_handle, torch):
    """Observed gathers [nshot, nrec, NT] on the device: modelled on the true
    model minus modelled on the smoothed model (direct wave removed)."""
    seis = torch.zeros((len(src), pmig.nrec, pmig.NT), dtype=torch.float32, device="cuda")
    tmp = torch.zeros_like(seis)
    with Engine(ptrue, batch=batch, stream=stream_handle) as e:
        e.model(src, out=seis)
    with Engine(pmig, batch=batch, stream=stream_handle) as e:
        e.model(src, out=tmp)
    seis -= tmp
    del tmp
    torch.cuda.synchronize()
    return seis


def storage_flag(name):
    from rtm_gpu_gb300 import capi
    return {"f32": capi.RTM_RING_F32, "bf16": capi.RTM_RING_BF16, "f16": capi.RTM_RING_F16,
            "i16": capi.RTM_RING_I16}[name]


def ring_flag(cfg):
    return storage_flag(cfg.ring)


def run_multishot(a, cfg):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from rtm_gpu_gb300 import Engine
    warm = max(3, a.warmup)

    ptrue, pmig, shots = build_problems(cfg)
    nshot = cfg.nshot
    if world > 1:
        # sharded survey: nshot shots per rank out of nshot * world along the
        # surface (weak scaling), stacks combined by one all-reduce per step
        from rtm_gpu_gb300 import synth
        from rtm_gpu_gb300.shard import shard_shots
        survey = synth.surface_shots(cfg.nx, nshot * world, cfg.N2)
        shots = [survey[i] for i in shard_shots(len(survey), rank, world)]
    batch = a.batch or nshot
    src = [pmig.src_flat(z, x) for z, x in shots]
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sh = stream.cuda_stream
    seis = step_gathers(Engine, ptrue, pmig, src, batch, sh, torch)

    eng = Engine(pmig, batch=batch, stream=sh, ring_precision=ring_flag(cfg))
    if cfg.snap:
        eng.set_snapshots(cfg.snap, storage_flag(cfg.snap_storage))
    tuned = None
    if a.kernel == "auto":
        tuned = eng.autotune(src, nsteps=20)
    else:
        eng.set_kernel(*kernel_forms(a))
    kern = eng.kernel()
    img = torch.zeros((pmig.nz, pmig.nx), dtype=torch.float32, device="cuda")
    ill = torch.zeros_like(img)

    s1 = torch.zeros((2, pmig.nz, pmig.nx), dtype=torch.float32, device="cuda")

    def step_dev():
        if not dist:
            eng.migrate_stack(src, seis, cfg.whitecoe, nshot, True, image=img, illum=ill)
            return
        # the rank's sums of the per-shot images (no normalisation), summed
        # over ranks in float64 (the combination rule of shard.combine_stacks),
        # then kernel.cu:1042-1059's normalisation
        eng.migrate_stack(src, seis, cfg.whitecoe, 1, False, image=s1[0], illum=s1[1])
        s64 = s1.double()
        dist.all_reduce(s64, op=dist.ReduceOp.SUM)
        ntot = float(nshot * world)
        ill.copy_(s64[1] / ntot)
        img.copy_((s64[0] / ntot) / (s64[1] / ntot))

    for _ in range(warm):
        step_dev()
    torch.cuda.synchronize()
    eng.launches(reset=True)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks() as clk:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(a.steps):
            step_dev()
        ev1.record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
    ms = ev0.elapsed_time(ev1) / a.steps
    launches = eng.launches()  # kernels launched inside the timed region (all K steps)
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    cu_step = cell_updates_per_shot(pmig.nz, pmig.nx, pmig.N2, pmig.NT) * nshot
    value = cu_step * world / (ms / 1e3) / 1e9

    # end to end through the public API with host buffers
    seis_h = seis.cpu().pin_memory()
    img_h = torch.zeros((pmig.nz, pmig.nx), dtype=torch.float32).pin_memory()
    ill_h = torch.zeros_like(img_h).pin_memory()
    eng.migrate_stack(src, seis_h, cfg.whitecoe, nshot, True, image=img_h, illum=ill_h)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(a.steps):
        eng.migrate_stack(src, seis_h, cfg.whitecoe, nshot, True, image=img_h, illum=ill_h)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_e2e = e0.elapsed_time(e1) / a.steps
    if dist:
        t = torch.tensor([ms_e2e], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_e2e = float(t.item())
    e2e = {"value": cu_step * world / (ms_e2e / 1e3) / 1e9, "unit": METRIC,
           "h2d_bytes_per_step": int(seis_h.numel() * 4),
           "d2h_bytes_per_step": int((img_h.numel() + ill_h.numel()) * 4)}

    # roofline of the dominant kernel (backward stencil) from a timed pass
    nb = min(kern["shots_per_launch"], nshot)  # shots of one launch
    eng.set_timing(True)
    r1d = torch.zeros((nb, pmig.NZ, pmig.NX), dtype=torch.float32, device="cuda")
    eng.migrate(src[:nb], seis[:nb], rel1=r1d, rel2=torch.zeros_like(r1d))
    del r1d
    tm = eng.timing()
    eng.set_timing(False)
    NZ, NX, nz, nx = pmig.NZ, pmig.NX, pmig.nz, pmig.nx
    bwd_bytes = nb * (16 * (NZ * NX + nz * nx) + 32 * nz * nx)
    fwd_bytes = nb * 16 * NZ * NX
    bwd_kernel = "k_step<backward> (source reconstruction + receiver step + imaging)"
    if cfg.snap:
        # the receiver step on every cell and its running sum on the interior
        # (the imaging at every snap-th step is a separate streaming kernel)
        bwd_bytes = nb * (16 * NZ * NX + 8 * nz * nx)
        fwd_bytes = nb * (16 * NZ * NX + 8 * nz * nx)  # plus the running sum's read and write
        bwd_kernel = "k_step<backward, snapshots> (receiver step and its running sum)"
    bwd_ms = tm["bwd_ms"] / max(tm["bwd_n"], 1)
    fwd_ms = tm["fwd_ms"] / max(tm["fwd_n"], 1)
    peak, peak_kind = measured_peak()
    traffic = None if cfg.snap else measured_traffic(cfg, nb)
    achieved = bwd_bytes / (bwd_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": (traffic or {}).get("bytes"),
                "traffic_source": (traffic or {}).get("source"),
                "kernel": bwd_kernel,
                "bytes_per_launch": bwd_bytes, "launch_ms": bwd_ms, "peak_kind": peak_kind,
                "forward_kernel": {"launch_ms": fwd_ms, "bytes_per_launch": fwd_bytes,
                                   "achieved": fwd_bytes / (fwd_ms / 1e3) / 1e9},
                "pad_kernel_ms": tm["pad_ms"] / max(tm["pad_n"], 1),
                "time_share": {"fwd": tm["fwd_ms"], "bwd": tm["bwd_ms"], "pad": tm["pad_ms"]}}

    # the plain single-shot GPU drop-in (the reference's per-shot launch
    # sequence on the rtm_k_* kernels) on one shot of the same workload
    plain = None
    if rank == 0 and not a.no_plain:
        plain = plain_dropin(pmig, src[0], seis_h[0].numpy(), torch)

    # CPU leg (rank 0, one GPU): the reference's loop on the host cores, and
    # one shot of this workload checked against the FP64 oracle
    cpu, fp64 = None, None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        nt_s = min(a.cpu_sample_nt or CPU_SAMPLE_NT, cfg.NT)
        cpu = cpu_baseline(pmig, shots[0], seis_h[0].numpy(), nt_s, os.cpu_count() or 1)
    if rank == 0 and world == 1 and not a.no_fp64_check:
        i = nshot // 2
        storage = ("source snapshots every %d steps in %s" % (cfg.snap, cfg.snap_storage.upper())
                   if cfg.snap else "%s rings" % cfg.ring.upper())
        fp64 = fp64_check(eng, ptrue, pmig, shots[i], seis_h[i].numpy(), cfg.whitecoe,
                          "shot %d of %d, %s, kernels as benched" % (i, nshot, storage))

    clocks = clk.summary(local)
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world,
                "steps": a.steps, "warmup": warm, "ms_per_step": ms, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": cfg.workload(),
                "engine": {"batch": batch, "fwd": FORMS[kern["fwd"]], "bwd": FORMS[kern["bwd"]],
                           "shots_per_launch": kern["shots_per_launch"],
                           "chosen_by": "autotuner" if tuned is not None else "flag",
                           "tuning_gcells_per_s": tuned, "device_bytes": eng.device_bytes},
                "shots_per_hour": nshot * world / (ms / 1e3) * 3600,
                "plain_dropin": plain,
                "speedup_vs_plain_shots_per_hour": (nshot * world / (ms / 1e3) * 3600 /
                                                    plain["shots_per_hour"]) if plain else None,
                "nrmse_vs_fp64": fp64,
                "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks,
                "gpu_launches": launches, "gpu_launches_per_step": launches // a.steps}
        print(json.dumps(line))
    eng.close()
    if dist:
        dist.destroy_process_group()


def plain_dropin(pmig, src_cell, seis_row, torch):
    """The plain single-shot GPU drop-in (rtm_plain_migrate_shot: the
    reference's per-shot launch sequence on the rtm_k_* kernels), one shot,
    host wall clock."""
    from rtm_gpu_gb300.engine import plain_migrate_shot
    plain_migrate_shot(pmig, src_cell, seis_row)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plain_migrate_shot(pmig, src_cell, seis_row)
    torch.cuda.synchronize()
    tp = time.perf_counter() - t0
    cu_shot = cell_updates_per_shot(pmig.nz, pmig.nx, pmig.N2, pmig.NT)
    return {"seconds_per_shot": tp, "shots_per_hour": 3600.0 / tp, "value": cu_shot / tp / 1e9,
            "unit": METRIC,
            "what": "rtm_plain_migrate_shot: kernel.cu's per-shot loop on the rtm_k_* drop-in "
                    "kernels, FP32 rings, host wall clock"}


def run_c1(a, cfg):
    """The single-shot configuration: one migration per step (forward run,
    reconstruction, receiver back-propagation, imaging, finishing) on the
    engine with a batch of one, L2 flushed before every timed step (the
    shot's working set fits in L2); each step timed with its own events."""
    import torch
    from rtm_gpu_gb300 import Engine
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    warm = max(3, a.warmup)
    ptrue, pmig, shots = build_problems(cfg)
    src = [pmig.src_flat(*shots[0])]
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sh = stream.cuda_stream
    seis = step_gathers(Engine, ptrue, pmig, src, 1, sh, torch)
    eng = Engine(pmig, batch=1, stream=sh, ring_precision=ring_flag(cfg))
    if a.kernel != "auto":
        eng.set_kernel(*kernel_forms(a))
    kern = eng.kernel()
    img = torch.zeros((pmig.nz, pmig.nx), dtype=torch.float32, device="cuda")
    ill = torch.zeros_like(img)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def step():
        eng.migrate_stack(src, seis, cfg.whitecoe, 1, True, image=img, illum=ill)

    for _ in range(warm):
        step()
    torch.cuda.synchronize()
    eng.launches(reset=True)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(a.steps)]
    with Clocks() as clk:
        for e0, e1 in evs:
            flush.fill_(1.0)
            e0.record(stream)
            step()
            e1.record(stream)
        torch.cuda.synchronize()
    ms = float(np.mean([e0.elapsed_time(e1) for e0, e1 in evs]))
    launches = eng.launches()
    cu = cell_updates_per_shot(pmig.nz, pmig.nx, pmig.N2, pmig.NT)
    seis_h = seis.cpu().pin_memory()
    img_h = torch.zeros((pmig.nz, pmig.nx), dtype=torch.float32).pin_memory()
    ill_h = torch.zeros_like(img_h).pin_memory()
    ee = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(a.steps)]
    for e0, e1 in ee:
        flush.fill_(1.0)
        e0.record(stream)
        eng.migrate_stack(src, seis_h, cfg.whitecoe, 1, True, image=img_h, illum=ill_h)
        e1.record(stream)
    torch.cuda.synchronize()
    ms_e2e = float(np.mean([e0.elapsed_time(e1) for e0, e1 in ee]))
    # backward-stencil roofline from a timed pass (working set in L2: stated,
    # not judged)
    eng.set_timing(True)
    r1d = torch.zeros((1, pmig.NZ, pmig.NX), dtype=torch.float32, device="cuda")
    eng.migrate(src, seis, rel1=r1d, rel2=torch.zeros_like(r1d))
    del r1d
    tm = eng.timing()
    eng.set_timing(False)
    NZ, NX, nz, nx = pmig.NZ, pmig.NX, pmig.nz, pmig.nx
    bwd_bytes = 16 * (NZ * NX + nz * nx) + 32 * nz * nx
    bwd_ms = tm["bwd_ms"] / max(tm["bwd_n"], 1)
    peak, peak_kind = measured_peak()
    achieved = bwd_bytes / (bwd_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": None,
                "kernel": "k_step<backward> (source reconstruction + receiver step + imaging)",
                "bytes_per_launch": bwd_bytes, "launch_ms": bwd_ms, "peak_kind": peak_kind,
                "note": "one shot's wavefields (about 8 MB) stay in L2 within a step; launch-bound",
                "pad_kernel_ms": tm["pad_ms"] / max(tm["pad_n"], 1)}
    plain = None if a.no_plain else plain_dropin(pmig, src[0], seis_h[0].numpy(), torch)
    cpu = fp64 = None
    if not a.no_cpu_baseline:
        cpu = cpu_baseline(pmig, shots[0], seis_h[0].numpy(), min(a.cpu_sample_nt or cfg.NT, cfg.NT),
                           os.cpu_count() or 1)
    if not a.no_fp64_check:
        fp64 = fp64_check(eng, ptrue, pmig, shots[0], seis_h[0].numpy(), cfg.whitecoe,
                          "the configuration's one shot, FP32 rings")
    line = {"metric": METRIC, "value": cu / (ms / 1e3) / 1e9, "unit": METRIC, "n_gpus": 1,
            "steps": a.steps, "warmup": warm, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": cfg.workload(),
            "engine": {"batch": 1, "fwd": FORMS[kern["fwd"]], "bwd": FORMS[kern["bwd"]]},
            "shots_per_hour": 3600.0 / (ms / 1e3), "plain_dropin": plain,
            "speedup_vs_plain_shots_per_hour": (3600.0 / (ms / 1e3) / plain["shots_per_hour"])
            if plain else None,
            "nrmse_vs_fp64": fp64,
            "e2e": {"value": cu / (ms_e2e / 1e3) / 1e9, "unit": METRIC,
                    "h2d_bytes_per_step": int(seis_h.numel() * 4),
                    "d2h_bytes_per_step": int((img_h.numel() + ill_h.numel()) * 4)},
            "roofline": roofline, "cpu_baseline": cpu, "clocks": clk.summary(0),
            "gpu_launches": launches, "gpu_launches_per_step": launches // a.steps}
    print(json.dumps(line))
    eng.close()


def main():
    a = parse()
    cfg = Config(a)
    if a.impl == "reference":
        if a.workload in ("rvsp", "c5") or a.snap:
            print(json.dumps({"impl": "reference", "unavailable":
                              "the reference arm is defined for the multishot and c1 workloads "
                              "with boundary rings (the reference stores no source snapshots)"}))
            return
        run_reference_arm(a, cfg)
        return
    if a.workload == "rvsp":
        run_rvsp(a, cfg)
        return
    if a.workload == "c5":
        run_c5(a, cfg)
        return
    if a.workload == "c1":
        run_c1(a, cfg)
        return
    run_multishot(a, cfg)


if __name__ == "__main__":
    main()
