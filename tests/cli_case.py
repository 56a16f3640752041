"""A small run directory in the reference's file layout (kernel.cu:542-605,
686-691, 827-838; GPU_velocity_real.cpp:11-19) and the images the
reference's flow produces from it, computed with the oracle."""
from __future__ import annotations

import os

import numpy as np

from oracle import oracle as orc
from rtm_gpu_gb300.problem import Problem, f32

LABELS = ["nfdmax", "nfdmin", "N2", "f0", "fmax", "df", "nthita", "eps", "dv", "iLSTE", "ifv",
          "whitecoe", "hz", "tao", "iNorm", "iCompen", "Nsmooth", "wthite_phase", "angle", "NX_BG",
          "NX_ED", "NZ_BG", "NZ_ED", "OutNameseis", "OutNameVp", "OutNameDPR", "OutPara", "Result"]


def default_case(**kw):
    c = dict(nfdmax=4, nfdmin=2, N2=8, f0=25.0, fmax=50.0, df=1.0, nthita=360, eps=1e-5, dv=1.0,
             iLSTE=0, ifv=0, whitecoe=1e-4, hz=10.0, tao=0.001, iNorm=1, iCompen=1, Nsmooth=3,
             wthite_phase=0.1, angle=0.0, NX_BG=5, NX_ED=50, NZ_BG=2, NZ_ED=35,
             OutNameseis="gathers/", OutNameVp="vel.dat", OutNameDPR="depths.txt",
             OutPara="Parameter.txt", Result="out/",
             # parameter file
             h=10.0, tao1=0.001, mod_NZ=40, mod_NX=60, NT1=160, s_l=1, s_z=1, n=30, ds=2, r_x=20,
             depths=(30, 100, 200), dr=1, seed=3)
    c.update(kw)
    c["nrec"] = len(c["depths"])
    return c


def write_case(d, c):
    """Writes the run directory; returns (vin [nx][nz], gathers per shot)."""
    rng = np.random.default_rng(c["seed"])
    os.makedirs(os.path.join(d, c["OutNameseis"]), exist_ok=True)
    os.makedirs(os.path.join(d, c["Result"]), exist_ok=True)
    with open(os.path.join(d, "2D_Real_RVSP_RTM.txt"), "w") as fh:
        for k in LABELS:
            v = c[k]
            fh.write("The value of %s\n%s\n" % (k, v if not isinstance(v, float) else repr(v)))
    with open(os.path.join(d, c["OutPara"]), "w") as fh:
        vals = [c["h"], c["tao1"], c["mod_NZ"], c["mod_NX"], c["NT1"], c["s_l"], c["s_z"], c["n"],
                c["ds"], c["r_x"], c["nrec"], c["dr"]]
        fh.write(" \n".join(str(v) for v in vals) + "\n")
    with open(os.path.join(d, c["OutNameDPR"]), "w") as fh:
        fh.write(" ".join(str(v) for v in c["depths"]) + "\n")
    nz, nx = c["mod_NZ"], c["mod_NX"]
    z = np.arange(nz)[None, :]
    x = np.arange(nx)[:, None]
    vin = (1500.0 + 8.0 * z + 2.0 * np.sin(x / 7.0) + rng.uniform(0, 30, (nx, nz))).astype(np.float32)
    vin.tofile(os.path.join(d, c["OutNameVp"]))  # x-major interior
    gathers = []
    for N in c["depths"]:
        g = (rng.standard_normal((c["n"], c["NT1"])) * 1e-2).astype(np.float32)
        g.tofile(os.path.join(d, c["OutNameseis"] + "NEW_L10-1932-X_%d.dat" % N))
        gathers.append(g)
    return vin, gathers


def oracle_outputs(c, vin, gathers):
    """{file name: array} of what the reference's flow writes."""
    N2, nz, nx = c["N2"], c["mod_NZ"], c["mod_NX"]
    NZ, NX = nz + 2 * N2, nx + 2 * N2
    tao, tao1, h = f32(c["tao"]), f32(c["tao1"]), f32(c["h"])
    NT = int(float((c["NT1"] - 1) * np.float32(tao1) / np.float32(tao)) + 1.5)  # kernel.cu:610
    v, r1 = orc.pad_velocity(vin, NZ, NX, N2, np.float32(tao), np.float32(h), c["ifv"])
    vmin, vmax, nvel, need = orc.bin_velocity(v, f32(c["dv"]))
    hzx = float(np.float32(c["hz"]) / np.float32(h))
    if c["iLSTE"] == 0:
        length, index, coef = orc.fun_m_and_c(c["nthita"], c["nfdmax"], c["nfdmin"], nvel, tao, h,
                                              f32(c["df"]), f32(c["eps"]), f32(c["fmax"]), vmin,
                                              f32(c["dv"]), need, hzx)
    else:
        coef = orc.taylor(c["nfdmax"])
        length = np.full(nvel, c["nfdmax"], np.int32)
        index = np.zeros(nvel + 1, np.int32)
    w = np.array([f32((1.0 * i) / (1.0 * N2)) for i in range(N2 + 1)], np.float32)
    wav = orc.wavelet_table(NT + 1, tao, f32(c["f0"]))
    s_l, s_z, r_x = c["s_l"] + N2 - 1, c["s_z"] + N2 - 1, c["r_x"] + N2 - 1
    p = Problem(nz=nz, nx=nx, N2=N2, M=c["nfdmax"], NT=NT, h=float(h), hz=float(c["hz"]),
                tao=float(tao), f0=float(c["f0"]), adaptive=c["iLSTE"] == 0,
                compen=bool(c["iCompen"]), v=v, r1=r1, w=w, vmin=vmin, vmax=vmax,
                dv=float(c["dv"]), nvel=nvel, length=np.asarray(length, np.int32),
                index=np.asarray(index, np.int32), coef=np.asarray(coef, np.float32), wav=wav,
                rec=(s_z, s_l, 0, c["ds"], c["n"]))
    out, ups, downs = {}, [], []
    for m, N in enumerate(c["depths"]):
        r_u = int(abs(np.float32(N) / np.float32(c["hz"])) + N2 - 1)
        q = p.with_source(r_u, r_x)
        seis = gathers[m]
        if NT != c["NT1"]:
            seis = orc.resample(seis, tao1, NT, tao)
        o1, o2 = orc.migrate(q, seis)
        up, dn = orc.finish_shot(q, o1, o2, c["whitecoe"])  # x-major [nx][nz]
        out["RVSP_RTM_up_%d.dat" % (m + 1)] = up
        out["RVSP_RTM_down_%d.dat" % (m + 1)] = dn
        ups.append(up)
        downs.append(dn)
    img, _ = orc.stack(np.stack(ups), np.stack(downs), nrec=len(ups), inorm=c["iNorm"], kahan=1)
    BG, ED, ZB, ZE = c["NX_BG"], c["NX_ED"], c["NZ_BG"], c["NZ_ED"]
    if c["ifv"] == 1:
        cols = list(range(ED, BG, -1))
        out["RVSP_Migration_Real_new2.dat"] = np.stack([img[j, ZB:ZE] for j in cols])
        vcols = list(range(ED + N2, BG + N2, -1))
        out["vnew.dat"] = np.stack([v[ZB + N2:ZE + N2, j] for j in vcols])
    else:
        out["RVSP_Migration_Real_new2.dat"] = img[BG:ED, ZB:ZE]
        out["vnew.dat"] = np.stack([v[ZB:ZE + N2, j] for j in range(BG + N2, ED + N2)])
    if ZB == 0 and ZE == nz:
        # post-stack chain (kernel.cu:1108-1196): both files read back flat as
        # ED-BG traces of nz samples
        ntr = ED - BG

        def flat(a):
            f = np.zeros(ntr * nz, np.float32)
            a = a.ravel()[:ntr * nz]
            f[:a.size] = a
            return f.reshape(ntr, nz)

        mig, vdt = flat(out["RVSP_Migration_Real_new2.dat"]), flat(out["vnew.dat"])
        hz = np.float32(c["hz"])
        t = orc.depth_to_time(vdt, mig, hz, np.float32(tao))
        tp = orc.phase_rotate(t, float(c["angle"]))
        out["RVSP_Migration_Real_T.dat"] = t
        out["RVSP_Migration_Real_T_phase.dat"] = tp
        out["RVSP_Migration_Real_D.dat"] = orc.time_to_depth(vdt, tp, np.float32(tao), hz)
        out["RVSP_migration_Real.sgy"] = mig
    return out, NT
