"""Shots with uneven aperture windows advancing in one batch (the batched
reverse-VSP configuration): each shot against the oracle run on its own
window of the survey model (same coefficient table), stacked in the survey
frame."""
import numpy as np
import pytest

from oracle import oracle as orc
from oracle.port_problem import window_problem
from rtm_gpu_gb300 import Engine
from util import rel_l2, small_problem

pytestmark = pytest.mark.gpu
TOL = 1e-4


@pytest.mark.parametrize("precision,tol_ill,tol_img", [("f32", TOL, TOL), ("f64", 1e-3, 5e-3)])
def test_uneven_windows_batch(product_lib, cuda_ok, precision, tol_ill, tol_img):
    """Against the FP32 oracle (same arithmetic) and, for the stated error of
    the batched uneven-window configuration, the FP64 oracle."""
    N2 = 8
    # vertical well at survey interior column 70
    p = small_problem(nz=50, nx=160, N2=N2, M=4, NT=150, rec=(N2 + 4, N2 + 70, 2, 0, 18))
    wins = [(0, 160), (30, 90), (55, 100), (10, 120)]
    rng = np.random.default_rng(12)
    srcs, seis = [], []
    for i, (xa, nx) in enumerate(wins):
        q = window_problem(p, xa, nx)
        sx = N2 + nx // 2 + (i - 2) * 3
        srcs.append((N2 + 1) * q.NX + sx)
        seis.append((rng.standard_normal((p.nrec, p.NT)) * 1e-2).astype(np.float32))
    seis = np.stack(seis)
    whitecoe = 1e-4
    # oracle: each shot on its own window, stacked into the survey frame
    sum_up = np.zeros((p.nz, p.nx), np.float64)
    sum_dn = np.zeros((p.nz, p.nx), np.float64)
    for i, (xa, nx) in enumerate(wins):
        q = window_problem(p, xa, nx)
        q = q.with_source(srcs[i] // q.NX, srcs[i] % q.NX)
        r1, r2 = orc.migrate(q, seis[i], precision=precision)
        u, d = orc.finish_shot(q, r1, r2, whitecoe)
        sum_up[:, xa:xa + nx] += u.T
        sum_dn[:, xa:xa + nx] += d.T
    ill_o = sum_dn / len(wins)
    img_o = (sum_up / len(wins)) / np.where(ill_o != 0, ill_o, 1)
    with Engine(p, batch=4) as e:
        img, ill = e.migrate_stack_windows(srcs, [w[0] for w in wins], [w[1] for w in wins], seis,
                                           whitecoe, len(wins), True)
    e_ill, e_img = rel_l2(ill, ill_o), rel_l2(img, img_o)
    print("uneven windows vs %s oracle: illumination rel-L2 %.3e, image %.3e" % (precision, e_ill, e_img))
    assert e_ill < tol_ill
    assert e_img < tol_img


def test_uniform_windows_equal_plain_stack(product_lib, cuda_ok):
    p = small_problem(nz=40, nx=100, N2=8, M=4, NT=120)
    srcs = [p.src_flat(p.N2 + 1, p.N2 + x) for x in (10, 50, 90)]
    rng = np.random.default_rng(3)
    seis = (rng.standard_normal((3, p.nrec, p.NT)) * 1e-2).astype(np.float32)
    with Engine(p, batch=3) as e:
        a, b = e.migrate_stack(srcs, seis, 1e-4, 3, True)
        c, d = e.migrate_stack_windows(srcs, [0, 0, 0], [p.nx] * 3, seis, 1e-4, 3, True)
    assert np.array_equal(a, c) and np.array_equal(b, d)


def test_aligned_windows_read_the_survey_model(product_lib, cuda_ok):
    """Windows whose origin is a multiple of 4 columns read the model tiles of
    their interior from the survey grid (wide enough windows here that whole
    128-column tiles lie inside); the result still matches the oracle run on
    each window's own padded model."""
    N2 = 8
    p = small_problem(nz=40, nx=420, N2=N2, M=4, NT=120, rec=(N2 + 4, N2 + 200, 2, 0, 12))
    wins = [(0, 420), (4, 300), (120, 280), (8, 400)]
    rng = np.random.default_rng(5)
    srcs, seis = [], []
    for i, (xa, nx) in enumerate(wins):
        q = window_problem(p, xa, nx)
        srcs.append((N2 + 1) * q.NX + N2 + nx // 2 + i)
        seis.append((rng.standard_normal((p.nrec, p.NT)) * 1e-2).astype(np.float32))
    seis = np.stack(seis)
    sum_up = np.zeros((p.nz, p.nx), np.float64)
    sum_dn = np.zeros((p.nz, p.nx), np.float64)
    for i, (xa, nx) in enumerate(wins):
        q = window_problem(p, xa, nx)
        q = q.with_source(srcs[i] // q.NX, srcs[i] % q.NX)
        u, d = orc.finish_shot(q, *orc.migrate(q, seis[i]), 1e-4)
        sum_up[:, xa:xa + nx] += u.T
        sum_dn[:, xa:xa + nx] += d.T
    ill_o = sum_dn / len(wins)
    img_o = (sum_up / len(wins)) / ill_o
    with Engine(p, batch=4) as e:
        img, ill = e.migrate_stack_windows(srcs, [w[0] for w in wins], [w[1] for w in wins], seis,
                                           1e-4, len(wins), True)
    assert rel_l2(ill, ill_o) < TOL
    assert rel_l2(img, img_o) < TOL
