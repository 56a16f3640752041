"""Ring storage at the learned-coefficient configuration's length: one shot of
the 1201x4001 model (dx=dz=10 m, 8000 steps, M=8 table from the network,
1000 surface receivers) on a window of 1500 columns, migrated with FP32,
int16, FP16 and BF16 boundary rings and by the reference's own GPU build,
each against the FP64 oracle on the same observed gathers (finished image,
relative L2).  Over 8000 steps the 16-bit float codes' rounding of the
rings shows in the image: FP32 and the reference's GPU build land at 6.9e-4,
int16 at 8.4e-4 (held to the 1e-3 bar), FP16 at 1.0e-3 and BF16 at 6.1e-3
(reported)."""
import numpy as np
import pytest

from oracle import oracle as orc
from oracle.port_problem import window_problem
from rtm_gpu_gb300 import Engine, capi, mlp, synth
from rtm_gpu_gb300.problem import build_problem
from util import rel_l2

pytestmark = pytest.mark.gpu


def test_c5_ring_storage_vs_fp64(product_lib, cuda_ok):
    nz, nx, N2, h, tao, f0, M, nt = 1201, 4001, 30, 10.0, 0.001, 25.0, 8, 8000
    vtrue = synth.model_c5(nz=nz, nx=nx)
    vmig = synth.smooth_model(vtrue, 10.0)
    fmax, vlo, vhi = 2 * f0, float(vmig.min()), float(vmig.max())
    net, _ = mlp.train_default(n=200_000, epochs=30, seed=5, batch=512, lr=3e-3,
                               r_range=(vlo * tao / h * 0.98, vhi * tao / h * 1.02),
                               kh_range=(2 * np.pi * fmax * h / vhi * 0.98,
                                         2 * np.pi * fmax * h / vlo * 1.02),
                               m_range=(4, 10))

    def table(vmin, dv, nvel, need, hzx):
        length, index, coef, _ = net.table(M=M, tol=1e-4, tao=tao, h=h, fmax=fmax, vmin=vmin,
                                           nvel=nvel, need=need, metric=mlp.DISP_REFERENCE)
        return length, index, coef

    kw = dict(N2=N2, M=M, NT=nt, h=h, tao=tao, f0=f0, adaptive=True, compen=True,
              rec=(N2 + 1, N2 + 1500, 0, 1, 1000), coef_table=table)
    pmig, ptrue = build_problem(vmig, **kw), build_problem(vtrue, **kw)
    x0, w = 1500, 1500
    xs = x0 + w // 2
    src_full = pmig.src_flat(N2 + 1, N2 + xs)
    with Engine(ptrue, batch=1) as e:
        gt = e.model([src_full])[0]
    with Engine(pmig, batch=1) as e:
        gs = e.model([src_full])[0]
    seis = (gt - gs).astype(np.float32)
    wsrc = (N2 + 1) * (w + 2 * N2) + N2 + xs - x0
    q = window_problem(pmig, x0, w)
    q = q.with_source(wsrc // q.NX, wsrc % q.NX)
    up, dn = orc.finish_shot(q, *orc.migrate(q, seis, precision="f64"), 1e-4)
    ref = (up / dn).T
    err = {}
    for name, prec in (("f32", capi.RTM_RING_F32), ("i16", capi.RTM_RING_I16),
                       ("f16", capi.RTM_RING_F16), ("bf16", capi.RTM_RING_BF16)):
        with Engine(pmig, batch=1, ring_precision=prec) as e:
            img, _ = e.migrate_stack_windows([wsrc], [x0], [w], seis[None], 1e-4, 1, True)
        err[name] = rel_l2(img[:, x0:x0 + w], ref)
    up, dn = orc.finish_shot(q, *orc.ref_gpu_migrate(q, seis)[:2], 1e-4)
    err["reference_gpu_build"] = rel_l2((up / dn).T, ref)
    print("C5 shot, image rel-L2 against FP64 by ring storage:", err)
    assert err["f32"] <= err["reference_gpu_build"] + 1e-4
    assert err["i16"] <= 1e-3
    assert err["i16"] < err["f16"] < err["bf16"]
