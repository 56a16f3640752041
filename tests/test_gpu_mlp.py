"""Learned-coefficient network: GPU gradients against the FP64 CPU oracle,
training reduces the loss, and what the network gains over the optimiser
alone when building a coefficient table."""
import time

import numpy as np
import pytest

from oracle import mlp_oracle
from rtm_gpu_gb300 import coeffs, mlp
from rtm_gpu_gb300.problem import f32, prep_taylor

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def data():
    return mlp.training_set(4000, seed=3)


def test_gradient_matches_fp64_oracle(product_lib, cuda_ok, data):
    x, c = data
    net = mlp.Mlp(seed=5)
    norm = mlp.fit_norm(x, c)
    net.norm = norm
    xb, cb = x[:256], c[:256]
    loss, g = net.grad(xb, cb)
    lo, go = mlp_oracle.loss_and_grad(net.params, norm, xb, cb)
    # FP32 on the GPU (sin/cos of the symbol included) against FP64
    assert abs(loss - lo) <= 1e-3 * abs(lo)
    assert np.linalg.norm(g - go) <= 1e-3 * np.linalg.norm(go)


def test_training_reduces_loss(product_lib, cuda_ok, data):
    x, c = data
    net = mlp.Mlp(seed=1)
    net.norm = mlp.fit_norm(x, c)
    l0, _ = net.grad(x, c)
    l1 = net.train(x, c, epochs=40, batch=256, lr=3e-3)
    l2, _ = net.grad(x, c)
    print("loss before %.4g after %.4g (last epoch %.4g)" % (l0, l2, l1))
    assert l2 < 0.01 * l0


def test_table_gain_over_optimiser(product_lib, cuda_ok):
    """The C5 band (v 1500-6000 m/s, h=10 m, tao=1 ms, fmax=50 Hz; 4501 bins of
    1 m/s) at operator length 8: a table built with a network trained on 200k
    optimiser samples of the band, judged in the reference's own dispersion
    measure (h/v)|v/v_FD - 1| at tolerance 1e-4, against the FP64 optimiser
    for every bin.

    What the network gains: at this length the least-squares normal
    equations are ill-conditioned where the band is narrow, and the
    optimiser's worst bins miss the band by a wide margin; the network's sets
    are smooth in (r, kh) and the table's worst relative phase-velocity error
    is several times lower than the optimiser table's.  No bin keeps a set
    worse than the better of the two."""
    tao, h, fmax, M = 0.001, 10.0, 50.0, 8
    vmin, nvel = 1500.0, 4501
    r_lo, r_hi = vmin * tao / h, (vmin + nvel - 1) * tao / h
    kh = lambda v: 2.0 * np.pi * fmax * h / v
    t0 = time.perf_counter()
    net, loss = mlp.train_default(n=200_000, epochs=30, seed=2, batch=512, lr=3e-3,
                                  r_range=(r_lo * 0.98, r_hi * 1.02),
                                  kh_range=(kh(vmin + nvel - 1) * 0.98, kh(vmin) * 1.02),
                                  m_range=(M, M))
    t_train = time.perf_counter() - t0
    need = np.ones(nvel, np.int32)
    tol = 1e-4
    length, index, coef, info = net.table(M=M, tol=tol, tao=tao, h=h, fmax=fmax, vmin=vmin,
                                          nvel=nvel, need=need, metric=mlp.DISP_REFERENCE)
    r = (vmin + np.arange(nvel)) * float(f32(tao)) / float(f32(h))
    bb = 2.0 * 3.1415926535898 * float(f32(fmax)) * float(f32(tao)) / r
    t0 = time.perf_counter()
    copt = coeffs.ls_coefs(r, bb, M)
    t_opt = time.perf_counter() - t0
    nk = int(fmax)
    ref_opt = mlp.dispersion_error(copt, np.full(nvel, M), r, bb, nk=nk, metric=mlp.DISP_REFERENCE,
                                   tao=float(f32(tao)))
    rel_opt = mlp.dispersion_error(copt, np.full(nvel, M), r, bb, nk=nk)
    tab = np.zeros((nvel, M + 1), np.float64)
    for i in range(nvel):
        tab[i] = coef[index[i]:index[i] + M + 1]
    rel_tab = mlp.dispersion_error(tab, np.full(nvel, M), r, bb, nk=nk)
    used, en = info["err_used"], info["err_net"]
    print("trained in %.1f s (loss %.3g); table %.3f s, %d/%d bins from the network; "
          "reference measure max: network %.2e optimiser %.2e table %.2e; relative max: "
          "optimiser %.2e table %.2e (optimiser alone %.3f s)"
          % (t_train, loss, info["seconds"], nvel - info["fallback"], nvel, en.max(), ref_opt.max(),
             used.max(), rel_opt.max(), rel_tab.max(), t_opt))
    # the table never keeps the worse of the two sets (FP64 judge; the table
    # holds float copies, hence the small slack)
    assert np.all(used <= np.minimum(en, np.maximum(ref_opt, tol)) * (1 + 1e-6) + 1e-12)
    assert nvel - info["fallback"] > nvel // 2      # the network carries most bins
    assert used.max() <= tol                          # every bin within the tolerance
    assert rel_tab.max() < 0.2 * rel_opt.max()        # the gain at this operator length
    assert np.all(length == M) and index[-1] == (M + 1) * nvel
