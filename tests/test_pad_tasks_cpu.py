"""Work split of the column-streaming pad kernel (k_pad_cols in
rtm_engine_kernels.cuh), restated on the CPU: every pad cell of a grid is
owned by exactly one lane of one warp task, owned cells lie inside the grid,
and every cell a lane reads stays inside the grid after the kernel's
clamping.  Grids of the benchmark configurations, narrower window grids of a
wider launch, and small odd shapes."""
import numpy as np
import pytest

COLS, WARPS = 30, 4  # PAD_COLS, PAD_WARPS (PAD_RCH, the rows per task, is a build
                     # parameter: 8 by default, checked at 4, 8 and 16)


def tasks(NZ, NXmax, N2, RCH):
    ncg_tb, nch_tb = -(-NXmax // COLS), -(-N2 // RCH)
    ncg_lr, nch_lr = -(-N2 // COLS), -(-(NZ - 2 * N2) // RCH)
    ntask = 2 * ncg_tb * nch_tb + 2 * ncg_lr * nch_lr
    return ncg_tb, nch_tb, ncg_lr, nch_lr, -(-ntask // WARPS)


def owned_cells(NZ, NX, NXmax, N2, RCH):
    ncg_tb, nch_tb, ncg_lr, nch_lr, nblk = tasks(NZ, NXmax, N2, RCH)
    ntb, nlr = ncg_tb * nch_tb, ncg_lr * nch_lr
    count = np.zeros((NZ, NX), np.int32)
    for task in range(nblk * WARPS):
        if task < 2 * ntb:
            band, t = divmod(task, ntb)
            cg, ch = divmod(t, nch_tb)
            r0 = NZ - N2 if band else 0
            r1, c0, c1 = r0 + N2, 0, NX
        else:
            t = task - 2 * ntb
            if t >= 2 * nlr:
                continue
            band, t = divmod(t, nlr)
            cg, ch = divmod(t, nch_lr)
            r0, r1 = N2, NZ - N2
            c0 = NX - N2 if band else 0
            c1 = c0 + N2
        xg = c0 + cg * COLS
        if xg >= c1:
            continue
        zb = r0 + ch * RCH
        ze = min(zb + RCH, r1)
        for lane in range(32):
            x = xg + lane - 1
            xc = min(max(x, 0), NX - 1)
            assert 0 <= xc < NX
            for j in range(RCH + 2):  # the rows a task loads, clamped
                assert 0 <= min(max(zb - 1 + j, 0), NZ - 1) < NZ
            for z in range(zb, ze):
                if 1 <= lane <= COLS and x < c1:
                    assert 0 <= z < NZ and 0 <= x < NX
                    count[z, x] += 1
    return count


@pytest.mark.parametrize("NZ,NX,NXmax,N2", [
    (461, 1261, 1261, 30),    # multi-shot grid
    (261, 461, 461, 30),      # single-shot grid
    (461, 364, 1261, 30),     # narrow window grid of a wide launch
    (56, 72, 72, 8),          # test-sized grids
    (37, 53, 61, 5),
    (140, 140, 140, 64),      # pad wider than a column group
])
@pytest.mark.parametrize("RCH", [4, 8, 16])
def test_every_pad_cell_owned_once(NZ, NX, NXmax, N2, RCH):
    count = owned_cells(NZ, NX, NXmax, N2, RCH)
    pad = np.ones((NZ, NX), bool)
    pad[N2:NZ - N2, N2:NX - N2] = False
    assert np.all(count[pad] == 1)
    assert np.all(count[~pad] == 0)
