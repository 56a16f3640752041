"""Generates the golden fixtures of tests/golden/ from the reference's own code.

Run in a checkout environment where caixh90/RTM_GPU's sources are available
(oracle/build_ref.py compiles its kernel bodies, LSMOrCon_rec_2D.cpp,
GPU_velocity_real.cpp, Resample.cpp, DisToTimeAndTimeToDis1D.cpp,
phase_correction_ricker_decon.cpp and the Ricker function for the CPU):

    python tests/golden/make_golden.py [/path/to/reference] [--only name ...]

Every array stored here was produced by the reference's code; the tests
compare the oracle (and, through it, the GPU engine) against them.
"""
from __future__ import annotations

import ctypes as C
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_ref  # noqa: E402
from oracle import oracle as orc  # noqa: E402

F32 = np.float32


def vp(a):
    return C.c_void_p(a.ctypes.data)


def ref_velocity(vin_colmajor, nz, nx, N2, tao, h, flip):
    L = orc.ref_host()
    NZ, NX = nz + 2 * N2, nx + 2 * N2
    with tempfile.NamedTemporaryFile(suffix=".dat", delete=False) as fh:
        fh.write(np.ascontiguousarray(vin_colmajor, F32).tobytes())
        path = fh.name
    out = [np.zeros(NZ * NX, F32) for _ in range(5)]
    L.ref_velocity(path.encode(), *out, NZ, NX, N2, tao, h, flip)
    os.unlink(path)
    v, v2, r, r1, r2 = out
    return v.reshape(NZ, NX), r1.reshape(NZ, NX)


def ref_table(nthita, nfdmax, nfdmin, tao, h, df, eps, fmax, vmin, vmax, dv, nvel, need, hzx):
    L = orc.ref_host()
    M = np.zeros(nvel, np.int32)
    idx = np.zeros(nvel + 1, np.int32)
    c = np.zeros(nvel * (nfdmax + 1), F32)
    nc = L.ref_funMandC(nthita, nfdmax, nfdmin, nvel, tao, h, df, eps, fmax, vmin, vmax, dv,
                        np.ascontiguousarray(need, np.int32), M, idx, c, c.size, hzx)
    return M, idx, c[:nc].copy()


def gen_lsm(out):
    L = orc.ref_host()
    orders = {}
    for N in range(2, 22, 2):
        c = np.zeros(N // 2 + 1, F32)
        L.ref_order(N, c)
        orders["order_%d" % N] = c
    cases = []
    coefs = []
    for M in (2, 4, 6, 8, 10):
        for r, bb in ((0.05, 1.5), (0.2, 2.0), (0.35, 2.5), (0.6, 2.9)):
            c = np.zeros(M + 1, np.float64)
            L.ref_cal2dfdcoe(c, r, bb, M, 1.0)
            cases.append((r, bb, M))
            coefs.append(np.pad(c, (0, 11 - c.size)))
    # anisotropic spacing hz != h
    c = np.zeros(7, np.float64)
    L.ref_cal2dfdcoe(c, 0.25, 2.2, 6, 1.6)
    lens = []
    for vel in (1500.0, 2500.0, 3500.0, 4500.0):
        lens.append(L.ref_callenfd(2, 10, vel, float(F32(0.001)), float(F32(10.0)), 1.0, 51, 40,
                                   1e-4, 1.0))
    need = np.ones(301, np.int32)
    need[5::11] = 0
    tab = ref_table(40, 8, 2, float(F32(0.001)), float(F32(10.0)), 1.0, 1e-4, 50.0, 1500.0,
                    1800.0, 1.0, 301, need, 1.0)
    np.savez_compressed(os.path.join(out, "lsm.npz"), cases=np.array(cases), coefs=np.array(coefs),
                        aniso=c, callen_vel=np.array([1500.0, 2500.0, 3500.0, 4500.0]),
                        callen=np.array(lens), table_need=need, table_len=tab[0],
                        table_index=tab[1], table_coef=tab[2], **orders)


def gen_velocity_ricker(out):
    rng = np.random.default_rng(42)
    nz, nx, N2 = 17, 23, 5
    vin = rng.uniform(1500, 3000, (nx, nz)).astype(F32)  # column-major file order
    res = {"vin": vin}
    for flip in (0, 1):
        v, r1 = ref_velocity(vin, nz, nx, N2, F32(0.001), F32(10.0), flip)
        res["v_flip%d" % flip] = v
        res["r1_flip%d" % flip] = r1
    R = orc.ref()
    t = (np.arange(300) * F32(0.001)).astype(F32)
    res["ricker_t"] = t
    res["ricker_f20"] = np.array([R.ref_ricker(float(x), 20.0) for x in t], F32)
    res["ricker_f25"] = np.array([R.ref_ricker(float(x), 25.0) for x in t], F32)
    np.savez_compressed(os.path.join(out, "velocity_ricker.npz"), **res)


def gen_kernels(out):
    """One call of every reference kernel on seeded random inputs."""
    R = orc.ref()
    rng = np.random.default_rng(7)
    NZ, NX, N2, M, NT = 37, 53, 5, 3, 6
    nz, nx = NZ - 2 * N2, NX - 2 * N2
    v = rng.uniform(1500, 1800, (NZ, NX)).astype(F32)
    r1 = (v * F32(0.001) / F32(10.0) / np.sqrt(F32(2))).astype(F32)
    w = np.array([F32(i / N2) for i in range(N2 + 1)], F32)
    vmin, vmax, nvel, need = orc.bin_velocity(v, 1.0)
    Ml, idx, coef = ref_table(30, M, 1, float(F32(0.001)), float(F32(10.0)), 1.0, 1e-6, 50.0,
                              vmin, vmax, 1.0, nvel, need, 1.0)
    ccon = np.array([-2.9, 1.6, -0.2, 0.03], F32)
    f = lambda: rng.standard_normal((NZ, NX)).astype(F32)
    u0, u1, u2, b = f(), f(), f(), f()
    ring = lambda n: rng.standard_normal(n).astype(F32)
    lf, rt = ring(M * nz * NT), ring(M * nz * NT)
    up, dw = ring(M * nx * NT), ring(M * nx * NT)
    seis = rng.standard_normal(nx).astype(F32)
    seis[::3] = 0
    sacc, racc, rel1, rel2 = f(), f(), f(), f()
    tao2, h2, hzx2_1, taoh, taoh2 = F32(1e-6), F32(0.01), F32(0.64), F32(1e-4), F32(5e-9)
    res = dict(NZ=NZ, NX=NX, N2=N2, M=M, NT=NT, v=v, r1=r1, w=w, vmin=vmin, dv=1.0, coef=coef,
               index=idx, ccon=ccon, u0=u0, u1=u1, u2=u2, b=b, lf=lf, rt=rt, up=up, dw=dw,
               seis=seis, sacc=sacc, racc=racc, rel1=rel1, rel2=rel2,
               scal=np.array([tao2, h2, hzx2_1, taoh, taoh2], F32))
    c = lambda a: np.ascontiguousarray(a).copy()
    # Add / Add_Con with a source at (12, 20)
    o = c(u2)
    R.ref_k_Add(vp(v), vp(o), vp(u0), vp(u1), vp(coef), vp(idx), C.c_float(tao2), C.c_float(h2),
                C.c_float(vmin), C.c_float(1.0), M, NZ, NX, NZ * NX, 12, 20, C.c_float(0.7),
                C.c_float(hzx2_1))
    res["out_Add"] = o
    o = c(u2)
    R.ref_k_Add_Con(vp(v), vp(o), vp(u0), vp(u1), vp(ccon), C.c_float(tao2), C.c_float(h2), M, NZ,
                    NX, NZ * NX, 12, 20, C.c_float(0.7), C.c_float(hzx2_1))
    res["out_Add_Con"] = o
    o = c(u2)
    R.ref_k_BKAdd_EFF(vp(v), vp(o), vp(u0), vp(u1), vp(coef), vp(idx), C.c_float(tao2),
                      C.c_float(h2), C.c_float(vmin), C.c_float(1.0), N2, NZ, NX, NZ * NX, 12, 20,
                      C.c_float(0.7), C.c_float(hzx2_1))
    res["out_BKAdd_EFF"] = o
    o = c(u2)
    R.ref_k_BKAdd_EFF_Con(vp(v), vp(o), vp(u0), vp(u1), vp(ccon), C.c_float(tao2), C.c_float(h2),
                          N2, NZ, NX, NZ * NX, 12, 20, M, C.c_float(0.7), C.c_float(hzx2_1))
    res["out_BKAdd_EFF_Con"] = o
    s_l, s_z, ds, n = N2, N2 + 1, 2, (nx + 1) // 2
    s_r = (n - 1) * ds + s_l
    o = c(u2)
    R.ref_k_BKAdd(vp(v), vp(o), vp(u1), vp(u0), vp(coef), vp(idx), vp(seis), C.c_float(tao2),
                  C.c_float(h2), C.c_float(vmin), C.c_float(1.0), M, NZ, NX, NZ * NX, s_l, s_r,
                  s_z, ds, C.c_float(hzx2_1))
    res["out_BKAdd"] = o
    o = c(u2)
    R.ref_k_BKAdd_Con(vp(v), vp(o), vp(u1), vp(u0), vp(ccon), vp(seis), C.c_float(tao2),
                      C.c_float(h2), M, NZ, NX, NZ * NX, s_l, s_r, s_z, ds, C.c_float(hzx2_1))
    res["out_BKAdd_Con"] = o
    res["line"] = np.array([s_l, s_r, s_z, ds], np.int32)
    # boundary
    ob = c(b)
    R.ref_k_Hybrid1(vp(u1), vp(u0), vp(u2), vp(ob), vp(lf), vp(rt), vp(up), vp(dw), vp(v), vp(r1),
                    vp(w), NZ, NX, N2, M, 3, C.c_float(taoh), C.c_float(taoh2))
    res["out_Hybrid1"] = ob
    o = c(u2)
    R.ref_k_Hybrid2(vp(u1), vp(u0), vp(o), vp(b), vp(lf), vp(rt), vp(up), vp(dw), vp(v), vp(r1),
                    vp(w), NZ, NX, N2, M, 3, C.c_float(taoh), C.c_float(taoh2))
    res["out_Hybrid2"] = o
    rings = [c(lf), c(rt), c(up), c(dw)]
    R.ref_k_Hybrid3(vp(u1), vp(u0), vp(u2), vp(b), *[vp(q) for q in rings], vp(v), vp(r1), vp(w),
                    NZ, NX, N2, M, 4, C.c_float(taoh), C.c_float(taoh2))
    res["out_Hybrid3"] = np.concatenate(rings)
    rings = [c(lf), c(rt), c(up), c(dw)]
    R.ref_k_Equal(*[vp(q) for q in rings], vp(u0), vp(u1), NZ, NX, N2, M)
    res["out_Equal"] = np.concatenate(rings)
    o = c(u1)
    R.ref_k_BKEqual(vp(lf), vp(rt), vp(up), vp(dw), vp(o), NZ, NX, N2, M, 2)
    res["out_BKEqual"] = o
    o1, o0 = c(u1), c(u0)
    R.ref_k_Deliver(vp(o1), vp(o0), vp(u2), NZ, NX)
    res["out_Deliver"] = np.stack([o1, o0])
    o1, o0 = c(u1), c(u0)
    R.ref_k_Deliver_EFF(vp(o1), vp(o0), vp(u2), N2, NZ, NX)
    res["out_Deliver_EFF"] = np.stack([o1, o0])
    # imaging: receiver wavefield R=u1, source S=u2
    q1, q2 = c(rel1), c(rel2)
    R.ref_k_Rel_NonCompen(vp(u1), vp(u2), vp(q1), vp(q2), NZ, NX)
    res["out_Rel_NonCompen"] = np.stack([q1, q2])
    q1, q2, sa, ra = c(rel1), c(rel2), c(sacc), c(racc)
    R.ref_k_Rel_Compen(vp(u1), vp(u2), vp(ra), vp(sa), vp(q1), vp(q2), NZ, NX)
    res["out_Rel_Compen"] = np.stack([q1, q2, sa, ra])
    np.savez_compressed(os.path.join(out, "kernels.npz"), **res)


def gen_shot(out):
    """A complete small migration and forward modelling through the
    reference's kernels (per-shot loop of kernel.cu:791-933)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from util import layered_model
    import dataclasses
    nz, nx, N2, M, NT = 40, 56, 8, 4, 160
    tao, h, f0 = F32(0.001), F32(10.0), 25.0
    vin = layered_model(nz, nx, 1500.0, 1800.0, 1)
    v, r1 = ref_velocity(vin.T.copy(), nz, nx, N2, tao, h, 0)
    vmin, vmax, nvel, need = orc.bin_velocity(v, 1.0)
    Ml, idx, coef = ref_table(24, M, 2, float(tao), float(h), 1.0, 1e-4, 50.0, vmin, vmax, 1.0,
                              nvel, need, 1.0)
    R = orc.ref()
    wav = np.array([R.ref_ricker(float(F32(i) * tao), f0) for i in range(NT + 1)], F32)
    w = np.array([F32(i / N2) for i in range(N2 + 1)], F32)
    res = dict(nz=nz, nx=nx, N2=N2, M=M, NT=NT, tao=tao, h=h, f0=f0, vin=vin, v=v, r1=r1, w=w,
               vmin=vmin, vmax=vmax, nvel=nvel, need=need, length=Ml, index=idx, coef=coef, wav=wav)

    class P:  # problem view for oracle.make_params
        pass

    from rtm_gpu_gb300.problem import Problem
    rng = np.random.default_rng(3)
    for compen in (1, 0):
        prob = Problem(nz=nz, nx=nx, N2=N2, M=M, NT=NT, h=float(h), hz=float(h), tao=float(tao),
                       f0=f0, adaptive=True, compen=bool(compen), v=v, r1=r1, w=w, vmin=vmin,
                       vmax=vmax, dv=1.0, nvel=nvel, length=Ml, index=idx, coef=coef, wav=wav,
                       rec=(N2 + 1, N2, 0, 2, (nx + 1) // 2), src_cell=(N2 + 2, N2 + nx // 2))
        seis = (rng.standard_normal((prob.nrec, NT)) * 1e-2).astype(F32)
        seis[:, ::5] = 0
        r1_, r2_ = orc.migrate(prob, seis, use_ref=True)
        res["seis_c%d" % compen] = seis
        res["rel1_c%d" % compen] = r1_
        res["rel2_c%d" % compen] = r2_
    res["rec"] = orc.model(prob, use_ref=True)
    np.savez_compressed(os.path.join(out, "shot.npz"), **res)


def gen_resample(out):
    """Resample.cpp:193-225 on seeded traces for several interval ratios
    (kernel.cu:839-845 resamples each trace from tao1 to tao)."""
    L = orc.ref_host()
    rng = np.random.default_rng(21)
    res = {}
    cases = [(101, 1.0, 0.33), (500, 0.002, 0.001), (400, 0.001, 0.0015), (300, 0.004, 0.001),
             (64, 0.0005, 0.00025), (257, 0.001, 0.001), (33, 0.003, 0.0007)]
    for i, (nxin, dxin, dxout) in enumerate(cases):
        y = rng.standard_normal(nxin).astype(F32)
        nxout = int((nxin - 1) * F32(dxin) / F32(dxout) + 1.5)  # kernel.cu:610 for NT
        r = np.zeros(nxout, F32)
        L.ref_resample(nxin, dxin, y, nxout, dxout, r)
        res["case%d_param" % i] = np.array([nxin, dxin, dxout, nxout], np.float64)
        res["case%d_in" % i] = y
        res["case%d_out" % i] = r
    np.savez_compressed(os.path.join(out, "resample.npz"), **res)


def poststack_inputs(seed=31, ntr=48, nz=700):
    """Seeded image traces and depth velocities of the post-stack pins (the
    pin test regenerates them)."""
    rng = np.random.default_rng(seed)
    v = np.sort((2000.0 + rng.uniform(0, 2500, (ntr, nz))).astype(F32), axis=1)
    img = rng.standard_normal((ntr, nz)).astype(F32)
    return v, img


def gen_poststack(out):
    """D2T, T2D and phase_correction of the reference on seeded traces.
    The outputs are stored as SHA-256 digests (plus short slices): the
    arrays are large and the pins are bit-for-bit.  The sizes keep the
    reference's work arrays above the allocator's mmap threshold, so the
    entry it reads uninitialised is zero."""
    import hashlib
    # fixed mmap threshold (no dynamic growth): the reference's work arrays
    # then come from fresh zero-filled pages whatever this process freed before
    C.CDLL("libc.so.6").mallopt(-3, 64 * 1024)  # M_MMAP_THRESHOLD
    L = orc.ref_post()
    v, img = poststack_inputs()
    ntr, nz = img.shape
    dz, dt = 5.0, 0.003
    scratch = os.path.join(tempfile.mkdtemp(), "post.bin").encode()
    buf = np.zeros(ntr * 20000, F32)
    nt = L.ref_d2t(scratch, v, img, ntr, nz, dz, dz, dt, buf, buf.size)
    t = buf[:ntr * nt].reshape(ntr, nt).copy()
    buf2 = np.zeros(ntr * 20000, F32)
    nz2 = L.ref_t2d(scratch, v, t, ntr, nt, nz, dz, dt, dz, buf2, buf2.size)
    d = buf2[:ntr * nz2].reshape(ntr, nz2).copy()
    res = {"params": np.array([31, ntr, nz, dz, dt, nt, nz2], np.float64)}
    res["d2t_sha"] = np.frombuffer(hashlib.sha256(t.tobytes()).digest(), np.uint8)
    res["t2d_sha"] = np.frombuffer(hashlib.sha256(d.tobytes()).digest(), np.uint8)
    res["d2t_slice"] = t[:2, :64].copy()
    res["t2d_slice"] = d[:2, :64].copy()
    for i, ang in enumerate((90.0, 37.5, -60.0)):
        ph = np.zeros_like(t)
        L.ref_phase_correction(t, ph, ntr, nt, ang)
        res["phase%d_angle" % i] = np.array([ang])
        res["phase%d_sha" % i] = np.frombuffer(hashlib.sha256(ph.tobytes()).digest(), np.uint8)
        res["phase%d_slice" % i] = ph[:2, :64].copy()
    np.savez_compressed(os.path.join(out, "poststack.npz"), **res)


GENERATORS = {"lsm": gen_lsm, "velocity_ricker": lambda o: gen_velocity_ricker(o),
              "kernels": lambda o: gen_kernels(o), "shot": lambda o: gen_shot(o),
              "resample": gen_resample, "poststack": gen_poststack}


def main():
    args = sys.argv[1:]
    only = None
    if "--only" in args:
        i = args.index("--only")
        only, args = args[i + 1:], args[:i]
    checkout = args[0] if args else build_ref.DEFAULT_CHECKOUT
    got = build_ref.build_ref(checkout, force=True)
    if "host" not in got or "kernels" not in got or "post" not in got:
        raise SystemExit("the reference's sources are needed to regenerate the fixtures")
    orc.set_threads(1)
    for name, gen in GENERATORS.items():
        if only is None or name in only:
            gen(HERE)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
