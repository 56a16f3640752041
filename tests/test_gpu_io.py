"""The reference's file flow on the GPU engine: trace resampling against the
oracle's restatement of Resample.cpp (bit for bit) and the golden vectors
made by the reference's own code."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import oracle as orc
from rtm_gpu_gb300 import capi

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def gpu_resample(y, dxin, nxout, dxout):
    y = np.ascontiguousarray(y, np.float32)
    flat = y.reshape(-1, y.shape[-1])
    out = np.zeros((flat.shape[0], nxout), np.float32)
    capi.check(capi.lib().rtm_resample(capi.fptr(flat), flat.shape[0], flat.shape[1], dxin,
                                       capi.fptr(out), nxout, dxout, 0), "resample")
    return out.reshape(y.shape[:-1] + (nxout,))


def test_resample_golden(product_lib, cuda_ok):
    G = dict(np.load(os.path.join(GOLD, "resample.npz")))
    n = len([k for k in G if k.endswith("_param")])
    for i in range(n):
        nxin, dxin, dxout, nxout = G["case%d_param" % i]
        got = gpu_resample(G["case%d_in" % i], np.float32(dxin), int(nxout), np.float32(dxout))
        assert np.array_equal(got, G["case%d_out" % i]), i


def test_resample_many_traces_vs_oracle(product_lib, cuda_ok):
    rng = np.random.default_rng(4)
    for nxin, dxin, dxout in ((2001, 0.002, 0.001), (4000, 0.001, 0.0025), (700, 0.0005, 0.0003)):
        y = rng.standard_normal((37, nxin)).astype(np.float32)
        nxout = int((nxin - 1) * np.float32(dxin) / np.float32(dxout) + 1.5)
        got = gpu_resample(y, np.float32(dxin), nxout, np.float32(dxout))
        exp = orc.resample(y, np.float32(dxin), nxout, np.float32(dxout))
        assert np.array_equal(got, exp)


def test_resample_rejects_bad_arguments(product_lib, cuda_ok):
    y = np.zeros(10, np.float32)
    o = np.zeros(10, np.float32)
    L = capi.lib()
    assert L.rtm_resample(capi.fptr(y), 1, 10, 0.0, capi.fptr(o), 10, 0.001, 0) != 0
    assert L.rtm_resample(capi.fptr(y), 1, 0, 0.001, capi.fptr(o), 10, 0.001, 0) != 0


def _run_cli(d):
    import subprocess
    from rtm_gpu_gb300 import _build
    r = subprocess.run([_build.CLI], cwd=d, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("kw", [dict(), dict(iLSTE=1, ifv=1, iNorm=0, iCompen=0),
                                dict(tao1=0.002, NT1=81),   # gathers resampled 2 ms -> 1 ms
                                dict(NZ_BG=0, NZ_ED=40, angle=90.0)])  # + the post-stack chain
def test_reference_run_directory(product_lib, cuda_ok, tmp_path, kw):
    """The reference's run directory through rtm_gb300_run, file for file
    against the oracle run of the same flow."""
    import cli_case
    from util import rel_l2
    c = cli_case.default_case(**kw)
    vin, gathers = cli_case.write_case(str(tmp_path), c)
    exp, NT = cli_case.oracle_outputs(c, vin, gathers)
    _run_cli(str(tmp_path))
    for name, e in exp.items():
        path = os.path.join(tmp_path, c["Result"], name)
        if name.endswith(".sgy"):
            b = open(path, "rb").read()
            ntr, ns = e.shape
            assert len(b) == 3600 + ntr * (240 + 4 * ns)
            got = np.stack([np.frombuffer(b[3600 + i * (240 + 4 * ns) + 240:3600 + (i + 1) * (240 + 4 * ns)],
                                          ">f4") for i in range(ntr)])
            assert rel_l2(got, e) < 1e-3
            continue
        got = np.fromfile(path, np.float32)
        assert got.size == e.size, name
        got = got.reshape(e.shape)
        if name == "vnew.dat":
            assert np.array_equal(got, e)
        else:
            tol = 1e-3 if name.startswith("RVSP_Migration") else 1e-4
            assert rel_l2(got, e) < tol, (name, rel_l2(got, e))
    if c["NZ_BG"] != 0 or c["NZ_ED"] != c["mod_NZ"]:  # the chain runs only for a full-depth window
        assert not os.path.exists(os.path.join(tmp_path, c["Result"], "RVSP_Migration_Real_T.dat"))
