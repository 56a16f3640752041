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
    """A table for 600 velocity bins at M=8 built with a network trained for
    the survey's range of (r, kh), the optimiser as fallback, against the
    optimiser for every bin.  Every bin stays within max(tol, optimiser's own
    error); the network must carry some bins."""
    tao, h, fmax = 0.001, 10.0, 45.0
    vmin, nvel = 2000.0, 600
    r_lo, r_hi = vmin * tao / h, (vmin + nvel) * tao / h
    kh = lambda v: 2.0 * np.pi * fmax * h / v
    net, loss = mlp.train_default(n=20000, epochs=150, seed=2, batch=512, lr=3e-3,
                                  r_range=(r_lo * 0.98, r_hi * 1.02),
                                  kh_range=(kh(vmin + nvel) * 0.98, kh(vmin) * 1.02),
                                  m_range=(8, 8))
    need = np.ones(nvel, np.int32)
    tol = 3e-3
    length, index, coef, info = net.table(M=8, tol=tol, tao=tao, h=h, fmax=fmax, vmin=vmin,
                                          nvel=nvel, need=need)
    r = (vmin + np.arange(nvel)) * float(f32(tao)) / float(f32(h))
    bb = 2.0 * 3.1415926535898 * float(f32(fmax)) * float(f32(tao)) / r
    t0 = time.perf_counter()
    copt = coeffs.ls_coefs(r, bb, 8)
    t_opt = time.perf_counter() - t0
    err_opt = mlp.dispersion_error(copt, np.full(nvel, 8), r, bb)
    taylor = np.tile(np.asarray(prep_taylor(8), np.float64), (nvel, 1))
    err_tay = mlp.dispersion_error(taylor, np.full(nvel, 8), r, bb)
    used, en = info["err_used"], info["err_net"]
    print("training loss %.3g; network error quantiles (10/50/90/max) %s; Taylor max %.2e"
          % (loss, " ".join("%.2e" % q for q in np.quantile(en, [0.1, 0.5, 0.9, 1.0])),
             err_tay.max()))
    print("network table: %.3f s, %d/%d bins from the network, max error %.2e "
          "(optimiser alone: %.3f s, max error %.2e)"
          % (info["seconds"], nvel - info["fallback"], nvel, used.max(), t_opt, err_opt.max()))
    assert np.all(used <= np.maximum(tol, err_opt) + 1e-12)
    assert info["fallback"] < nvel  # the network is used for some bins
    assert np.all(length == 8) and index[-1] == 9 * nvel
