"""Benchmark of the RTM propagate/migrate path on one GB300 (or N, one
process per GPU, shots sharded across ranks).

Workload (default): the plain multi-shot configuration -- a 401x1201 seeded
layered model (12 dipping layers 1500-5500 m/s, two normal faults, a
low-velocity lens), dx=dz=12.5 m, dt=1 ms, 4000 steps, M=8 adaptive
least-squares coefficients, 30-cell hybrid ABC, 64 surface shots with
full-spread receivers, images stacked with Kahan summation.  A step is the
full migration of the 64 shots: forward source run, boundary-ring
reconstruction, receiver back-propagation, imaging, per-shot finishing and
the stack.  The observed gathers are modelled first (true model minus
smoothed model, removing the direct wave) and stay resident in HBM for
`value`; `e2e` takes them from pinned host memory every step and returns the
image to the host.

Metric: grid-cell updates per second, one update = one grid point advanced
one time step; per shot NT*(2*NZ*NX + nz*nx) (forward on the padded grid,
receiver wavefield on the padded grid, source reconstruction on the interior).

--impl reference times the reference's own propagation + imaging loop
(kernel.cu kernel bodies, compiled for the host cores by oracle/build_ref.py)
on a bounded sample of the same workload, with all host threads.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
# time steps of the CPU baseline's one-shot sample (about 10 s of the
# reference's kernel bodies on 16 host cores for the multi-shot grid)
CPU_SAMPLE_NT = 2000
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
    ap.add_argument("--shots", type=int, default=64)
    ap.add_argument("--nt", type=int, default=4000)
    ap.add_argument("--batch", type=int, default=0, help="shots per batch (0: all)")
    ap.add_argument("--coef", default="adaptive", choices=["adaptive", "taylor"])
    ap.add_argument("--ring", default=None, choices=["f32", "bf16", "f16"],
                    help="boundary-ring storage (stencil and imaging stay FP32); default f16 "
                         "for the multi-shot workload, f32 for rvsp (FP32 throughout), bf16 for c5")
    ap.add_argument("--no-plain", action="store_true",
                    help="skip timing the plain single-shot drop-in for comparison")
    ap.add_argument("--cpu-sample-nt", type=int, default=0,
                    help="time steps of the one-shot CPU sample (0: %d, about 10 s on 16 cores)"
                         % CPU_SAMPLE_NT)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--small", action="store_true", help="reduced grid for quick checks")
    ap.add_argument("--kernel", default="auto", choices=["auto", "tiled", "persistent", "split", "x2", "x2-split"],
                    help="stencil kernel form (auto: the autotuner picks it and shots per launch)")
    ap.add_argument("--bwd-kernel", default="same", choices=["same", "tiled", "persistent", "split"],
                    help="backward stencil form with a fixed --kernel (same: --kernel's, tiled for x2 forms)")
    ap.add_argument("--workload", default="multishot", choices=["multishot", "rvsp", "c5"],
                    help="rvsp: batched uneven aperture windows, well receivers, autotuned; "
                         "c5: learned coefficients, 1201x4001 model, BF16 rings, uneven apertures")
    return ap.parse_args()


class Config:
    def __init__(self, a):
        self.small = a.small
        self.nz, self.nx = (101, 301) if a.small else (401, 1201)
        self.N2, self.M = 30, 8
        self.h, self.tao, self.f0 = 12.5, 0.001, 25.0
        self.NT = a.nt
        self.nshot = a.shots
        self.coef = a.coef
        self.ring = a.ring or {"multishot": "f16", "rvsp": "f32", "c5": "bf16"}[a.workload]
        self.whitecoe = 1e-4
        # optimiser settings (the reference's parameter file: nthita=1000,
        # eps=1e-5, df=1; fmax = 2*f0)
        self.fmax, self.df, self.nthita, self.eps, self.nfdmin = 2 * self.f0, 1.0, 1000, 1e-5, 2

    def workload(self):
        return {"workload": "multi-shot RTM %dx%d interior, 30-cell hybrid ABC, M=%d %s "
                            "coefficients, %d steps, %d surface shots, full-spread receivers, "
                            "FP32 stencil/imaging, %s boundary rings, Kahan stack"
                            % (self.nz, self.nx, self.M, self.coef, self.NT, self.nshot,
                               self.ring.upper()),
                "nz": self.nz, "nx": self.nx, "N2": self.N2, "M": self.M, "nt": self.NT,
                "shots": self.nshot, "dx_m": self.h, "dt_s": self.tao, "coefficients": self.coef,
                "ring_storage": self.ring}


def build_problems(cfg, dv=1.0):
    from rtm_gpu_gb300 import synth
    from rtm_gpu_gb300.problem import build_problem
    vtrue = synth.model_c2(nz=cfg.nz, nx=cfg.nx)
    vmig = synth.smooth_model(vtrue, 10.0)
    rec = synth.full_spread(cfg.nx, cfg.N2)
    table = None
    if cfg.coef == "adaptive":
        from rtm_gpu_gb300 import coeffs
        table = coeffs.table_source(nfdmax=cfg.M, nfdmin=cfg.nfdmin, tao=cfg.tao, h=cfg.h,
                                    fmax=cfg.fmax, df=cfg.df, nthita=cfg.nthita, eps=cfg.eps)
    kw = dict(N2=cfg.N2, M=cfg.M, NT=cfg.NT, h=cfg.h, tao=cfg.tao, f0=cfg.f0,
              adaptive=cfg.coef == "adaptive", compen=True, rec=rec, dv=dv, coef_table=table)
    ptrue = build_problem(vtrue, **kw)
    pmig = build_problem(vmig, **kw)
    shots = synth.surface_shots(cfg.nx, cfg.nshot, cfg.N2)
    return ptrue, pmig, shots


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, path):
        self.path = path
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


def cpu_baseline(cfg, pmig, shots, seis_host, nt_sample, threads):
    """Reference kernel bodies (oracle/_ref) or, failing that, the oracle's
    C restatement, timed on the host cores on one shot with nt_sample steps."""
    import dataclasses
    from oracle import oracle as orc
    kind = "reference"
    try:
        orc.ref()
    except Exception:
        kind = "port"
    orc.set_threads(threads)
    p = dataclasses.replace(pmig, NT=nt_sample, wav=pmig.wav[: nt_sample + 1])
    p = p.with_source(*shots[0])
    s = np.ascontiguousarray(seis_host[0][:, :nt_sample])
    t0 = time.perf_counter()
    orc.migrate(p, s, use_ref=(kind == "reference"))
    dt = time.perf_counter() - t0
    cu = cell_updates_per_shot(p.nz, p.nx, p.N2, nt_sample)
    return {"value": cu / dt / 1e9, "unit": METRIC, "cores": threads, "kind": kind,
            "sample": "one shot of the workload grid, %d time steps (%.3g cell-updates), %.1f s"
                      % (nt_sample, cu, dt)}


def run_reference_arm(a, cfg):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from rtm_gpu_gb300.problem import build_problem
    from rtm_gpu_gb300 import synth
    import dataclasses
    from oracle import oracle as orc
    # the reference arm needs no GPU: a Taylor problem of the same grid for
    # the loop (coefficient count M=8 per cell as the adaptive table at M=8)
    vmig = synth.smooth_model(synth.model_c2(nz=cfg.nz, nx=cfg.nx), 10.0)
    nt = min(a.cpu_sample_nt or CPU_SAMPLE_NT, cfg.NT)
    p = build_problem(vmig, N2=cfg.N2, M=cfg.M, NT=nt, h=cfg.h, tao=cfg.tao, f0=cfg.f0,
                      adaptive=False, compen=True, rec=synth.full_spread(cfg.nx, cfg.N2))
    shots = synth.surface_shots(cfg.nx, cfg.nshot, cfg.N2)
    rng = np.random.default_rng(7)
    seis = (rng.standard_normal((1, p.nrec, nt)) * 1e-3).astype(np.float32)
    threads = os.cpu_count() or 1
    for _ in range(a.warmup):
        cpu_baseline(cfg, p, shots, seis, nt, threads)
    vals = [cpu_baseline(cfg, p, shots, seis, nt, threads) for _ in range(a.steps)]
    v = float(np.median([x["value"] for x in vals]))
    cu = cell_updates_per_shot(cfg.nz, cfg.nx, cfg.N2, cfg.NT) * cfg.nshot
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": METRIC, "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": cu / (v * 1e9) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": cfg.workload(),
            "cpu_baseline": {"value": v, "unit": METRIC, "cores": threads, "kind": vals[0]["kind"],
                             "sample": vals[0]["sample"] + "; ms_per_step extrapolated to the full workload"},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def rvsp_geometry(cfg, nshot=128, seed=1237, wmin=300, wmax=1201, well_x=600, z0=50, nrec=300):
    """Reverse-VSP survey on the multi-shot model: nshot surface sources, each
    with a seeded aperture window of width U[wmin, wmax] columns around it
    that contains the well; nrec receivers down the well at interior column
    well_x, depths z0 .. z0+nrec-1.  Returns (sources (z, x) in the survey's
    padded grid, window starts, window widths, receiver line)."""
    rng = np.random.default_rng(seed)
    N2, nx = cfg.N2, cfg.nx
    xs = np.linspace(0, nx - 1, nshot).round().astype(int)
    w = rng.integers(wmin, min(wmax, nx) + 1, nshot)
    xa = np.clip(xs - w // 2, np.maximum(0, well_x - w + 1), np.minimum(well_x, nx - w))
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
    nshot = a.shots if a.shots != 64 else 128
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
    ring = {"f32": capi.RTM_RING_F32, "bf16": capi.RTM_RING_BF16, "f16": capi.RTM_RING_F16}[cfg.ring]
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
    with Clocks("/tmp/bench_clocks_rvsp.csv") as clk:
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
            "roofline": roofline,
            "clocks": clk.summary(0), "gpu_launches": launches,
            "gpu_launches_per_step": launches // a.steps}
    print(json.dumps(line))
    eng.close()


def run_c5(a, cfg):
    """Learned coefficients plus the full stack on the 1201x4001 model
    (dx=dz=10 m, 1500-6000 m/s gradients with salt-like 4500 m/s bodies):
    the coefficient table comes from the MLP trained on the GPU on FP64
    optimiser samples of the survey's (r, kh) range, with the optimiser as
    fallback wherever the network's dispersion error exceeds 1e-4; shots with
    uneven aperture windows, BF16 rings, autotuned kernels.  The shot count
    and steps are reduced from the 256 x 8000 of the full configuration
    (--shots / --nt) so the run fits a few minutes."""
    import torch
    from rtm_gpu_gb300 import Engine, capi, coeffs, mlp, synth
    from rtm_gpu_gb300.problem import build_problem, f32
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    nz, nx, N2, h, tao, f0, M = 1201, 4001, 30, 10.0, 0.001, 25.0, 8
    nshot = a.shots if a.shots != 64 else 8
    nt = a.nt if a.nt != 4000 else 8000
    vtrue = synth.model_c5(nz=nz, nx=nx)
    vmig = synth.smooth_model(vtrue, 10.0)
    fmax = 2 * f0
    vlo, vhi = float(vmig.min()), float(vmig.max())
    t0 = time.perf_counter()
    net, train_loss = mlp.train_default(n=50000, epochs=60, seed=5, batch=512, lr=3e-3,
                                        r_range=(vlo * tao / h * 0.98, vhi * tao / h * 1.02),
                                        kh_range=(2 * np.pi * fmax * h / vhi * 0.98,
                                                  2 * np.pi * fmax * h / vlo * 1.02),
                                        m_range=(M, M))
    t_train = time.perf_counter() - t0
    info_box = {}

    def table(vmin, dv, nvel, need, hzx):
        assert dv == 1.0
        length, index, coef, info = net.table(M=M, tol=1e-4, tao=tao, h=h, fmax=fmax, vmin=vmin,
                                              nvel=nvel, need=need)
        info_box.update(info)
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
    err_opt = mlp.dispersion_error(copt, np.full(len(sel), M), r, bb)
    err_net = info["err_net"][sel]
    ptrue = build_problem(vtrue, coef_table=table, **kw)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sh = stream.cuda_stream
    rng = np.random.default_rng(1240)
    wn = rng.integers(1500, nx + 1, nshot)
    xa = np.array([rng.integers(max(0, 2500 - w), min(1500, nx - w) + 1) for w in wn])
    xs = xa + wn // 2
    src_full = [pmig.src_flat(N2 + 1, N2 + int(x)) for x in xs]
    seis = torch.zeros((nshot, pmig.nrec, nt), dtype=torch.float32, device="cuda")
    tmp = torch.zeros_like(seis)
    with Engine(ptrue, batch=min(nshot, 8), stream=sh) as e:
        e.model(src_full, out=seis)
    with Engine(pmig, batch=min(nshot, 8), stream=sh) as e:
        e.model(src_full, out=tmp)
    seis -= tmp
    del tmp
    p2, seis2 = pmig, seis
    wsrc = [(N2 + 1) * (int(w) + 2 * N2) + N2 + int(x) - int(x0) for x, x0, w in zip(xs, xa, wn)]
    eng = Engine(p2, batch=nshot, stream=sh, ring_precision=capi.RTM_RING_BF16)
    tuned = eng.autotune(wsrc, xa, wn, nsteps=10)
    kern = eng.kernel()
    img = torch.zeros((nz, nx), dtype=torch.float32, device="cuda")
    ill = torch.zeros_like(img)

    def step():
        eng.migrate_stack_windows(wsrc, xa, wn, seis2, 1e-4, nshot, True, image=img, illum=ill)

    for _ in range(max(3, a.warmup)):
        step()
    torch.cuda.synchronize()
    eng.launches(reset=True)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks("/tmp/bench_clocks_c5.csv") as clk:
        ev0.record(stream)
        for _ in range(a.steps):
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / a.steps
    launches = eng.launches()
    NZ = nz + 2 * N2
    cu = sum(nt * (2 * NZ * (int(w) + 2 * N2) + nz * int(w)) for w in wn)
    used = info["err_used"][sel]
    roofline = windowed_roofline(eng, step, NZ, nz, N2, wn, kern["shots_per_launch"])
    line = {"metric": METRIC, "value": cu / (ms / 1e3) / 1e9, "unit": METRIC, "n_gpus": 1,
            "steps": a.steps, "warmup": max(3, a.warmup), "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "learned coefficients + full stack: 1201x4001 model, dx=dz=10 m, "
                                   "%d shots with aperture windows of 1500-4001 columns, 1000 surface "
                                   "receivers, %d steps, "
                                   "M=%d MLP table (optimiser fallback above 1e-4), BF16 rings"
                                   % (nshot, nt, M),
                       "shots": nshot, "nt": nt, "mean_window": float(np.mean(wn)),
                       "autotuned": {"fwd_kernel": FORMS[kern["fwd"]],
                                     "bwd_kernel": FORMS[kern["bwd"]],
                                     "shots_per_launch": kern["shots_per_launch"],
                                     "tuning_gcells_per_s": tuned},
                       "l2": "inputs larger than L2 (%.1f GB)" % (eng.device_bytes / 1e9)},
            "coefficients": {"bins": int(len(sel)), "from_network": int(len(sel) - info["fallback"]),
                             "tolerance": 1e-4, "max_dispersion_error_network": float(err_net.max()),
                             "max_dispersion_error_optimiser": float(err_opt.max()),
                             "max_dispersion_error_table": float(used.max()),
                             "network_train_s": t_train, "network_train_loss": train_loss,
                             "table_s": info["seconds"], "optimiser_alone_s": t_opt},
            "roofline": roofline,
            "clocks": clk.summary(0), "gpu_launches": launches}
    print(json.dumps(line))
    eng.close()


def main():
    a = parse()
    cfg = Config(a)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if a.impl == "reference":
        run_reference_arm(a, cfg)
        return
    if a.workload == "rvsp":
        run_rvsp(a, cfg)
        return
    if a.workload == "c5":
        run_c5(a, cfg)
        return
    import torch
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
    # observed data: true minus smoothed model (direct wave removed)
    seis = torch.zeros((nshot, pmig.nrec, pmig.NT), dtype=torch.float32, device="cuda")
    tmp = torch.zeros_like(seis)
    with Engine(ptrue, batch=batch, stream=sh) as e:
        e.model(src, out=seis)
    with Engine(pmig, batch=batch, stream=sh) as e:
        e.model(src, out=tmp)
    seis -= tmp
    del tmp
    torch.cuda.synchronize()

    from rtm_gpu_gb300 import capi
    ring = {"f32": capi.RTM_RING_F32, "bf16": capi.RTM_RING_BF16, "f16": capi.RTM_RING_F16}[cfg.ring]
    eng = Engine(pmig, batch=batch, stream=sh, ring_precision=ring)
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
        # over ranks, then kernel.cu:1042-1059's normalisation
        eng.migrate_stack(src, seis, cfg.whitecoe, 1, False, image=s1[0], illum=s1[1])
        dist.all_reduce(s1, op=dist.ReduceOp.SUM)
        ntot = float(nshot * world)
        torch.div(s1[1], ntot, out=ill)
        torch.div(torch.div(s1[0], ntot), ill, out=img)

    for _ in range(warm):
        step_dev()
    torch.cuda.synchronize()
    eng.launches(reset=True)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(os.path.join(ROOT, "gpurun_out", "bench_clocks.csv")
                if os.path.isdir(os.path.join(ROOT, "gpurun_out")) else "/tmp/bench_clocks.csv") as clk:
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
    bwd_ms = tm["bwd_ms"] / max(tm["bwd_n"], 1)
    fwd_ms = tm["fwd_ms"] / max(tm["fwd_n"], 1)
    peak, peak_kind = measured_peak()
    traffic = measured_traffic(cfg, nb)
    achieved = bwd_bytes / (bwd_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": (traffic or {}).get("bytes"),
                "traffic_source": (traffic or {}).get("source"),
                "kernel": "k_step<backward> (source reconstruction + receiver step + imaging)",
                "bytes_per_launch": bwd_bytes, "launch_ms": bwd_ms, "peak_kind": peak_kind,
                "forward_kernel": {"launch_ms": fwd_ms, "bytes_per_launch": fwd_bytes,
                                   "achieved": fwd_bytes / (fwd_ms / 1e3) / 1e9},
                "pad_kernel_ms": tm["pad_ms"] / max(tm["pad_n"], 1),
                "time_share": {"fwd": tm["fwd_ms"], "bwd": tm["bwd_ms"], "pad": tm["pad_ms"]}}

    # the plain single-shot GPU drop-in (the reference's per-shot launch
    # sequence on the rtm_k_* kernels) on one shot of the same workload
    plain = None
    if rank == 0 and not a.no_plain:
        from rtm_gpu_gb300.engine import plain_migrate_shot
        s0 = seis_h[0].numpy()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        plain_migrate_shot(pmig, src[0], s0)
        torch.cuda.synchronize()
        tp = time.perf_counter() - t0
        cu_shot = cell_updates_per_shot(pmig.nz, pmig.nx, pmig.N2, pmig.NT)
        plain = {"seconds_per_shot": tp, "shots_per_hour": 3600.0 / tp,
                 "value": cu_shot / tp / 1e9, "unit": METRIC,
                 "what": "rtm_plain_migrate_shot: kernel.cu's per-shot loop on the rtm_k_* "
                         "drop-in kernels, FP32 rings, host wall clock"}

    cpu = None
    if rank == 0 and not a.no_cpu_baseline:
        nt_s = min(a.cpu_sample_nt or CPU_SAMPLE_NT, cfg.NT)
        cpu = cpu_baseline(cfg, pmig, shots, seis_h.numpy(), nt_s, os.cpu_count() or 1)

    clocks = clk.summary(local)
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world,
                "steps": a.steps, "warmup": warm, "ms_per_step": ms, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": dict(cfg.workload(), batch=batch,
                               kernels={"fwd": FORMS[kern["fwd"]],
                                        "bwd": FORMS[kern["bwd"]],
                                        "shots_per_launch": kern["shots_per_launch"],
                                        "chosen_by": "autotuner" if tuned is not None else "flag",
                                        "tuning_gcells_per_s": tuned},
                               l2="inputs larger than L2 (%.1f GB of wavefields and rings)"
                                  % (eng.device_bytes / 1e9)),
                "shots_per_hour": nshot * world / (ms / 1e3) * 3600,
                "plain_dropin": plain,
                "speedup_vs_plain_shots_per_hour": (nshot * world / (ms / 1e3) * 3600 /
                                                    plain["shots_per_hour"]) if plain else None,
                "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks,
                "gpu_launches": launches, "gpu_launches_per_step": launches // a.steps}
        print(json.dumps(line))
    eng.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
