"""The absorbing-pad cell classification used by the engine (side / corner
update, blend weight index) against an enumeration of the thread conditions
of the reference's Hybrid1/Hybrid2 (kernel.cu:116-183), and the compact pad
enumeration of the pad kernel."""
import pytest


def reference_sets(NZ, NX, N2):
    """Index sets of kernel.cu:116-183 for the reference's full thread grid."""
    side, corner, blend = {}, set(), {}
    gx = (NZ + 15) // 16 * 16
    gy = (NX + 15) // 16 * 16
    for x in range(gx):
        for y in range(gy):
            if 0 < x <= N2 and N2 - x + 2 <= y < NX - N2 - 2 + x:
                side[(N2 - x, y)] = "row"
                side[(NZ - N2 + x - 1, y)] = "row"
            if 0 < y <= N2 and N2 - y + 2 <= x < NZ - N2 - 2 + y:
                side[(x, N2 - y)] = "col"
                side[(x, NX - N2 + y - 1)] = "col"
            if 0 < x <= N2 and y < NX:
                for c in [(N2 - x + 1, N2 - x), (N2 - x, N2 - x + 1), (N2 - x, N2 - x),
                          (NZ - N2 + x - 2, NX - N2 + x - 1), (NZ - N2 + x - 1, NX - N2 + x - 2),
                          (NZ - N2 + x - 1, NX - N2 + x - 1), (NZ - N2 + x - 1, N2 - x + 1),
                          (NZ - N2 + x - 2, N2 - x), (NZ - N2 + x - 1, N2 - x),
                          (N2 - x + 1, NX - N2 + x - 1), (N2 - x, NX - N2 + x - 2),
                          (N2 - x, NX - N2 + x - 1)]:
                    corner.add(c)
            if 0 < x <= N2 and N2 - x + 1 <= y < NX - N2 + x:
                assert (N2 - x, y) not in blend
                blend[(N2 - x, y)] = x
            if 0 < y <= N2 and N2 - y <= x < NZ - N2 + y - 1:
                assert (x, N2 - y) not in blend
                blend[(x, N2 - y)] = y
            if 0 < x <= N2 and N2 - x <= y < NX - N2 + x - 1:
                assert (NZ - N2 + x - 1, y) not in blend
                blend[(NZ - N2 + x - 1, y)] = x
            if 0 < y <= N2 and N2 - y + 1 <= x < NZ - N2 + y:
                assert (x, NX - N2 + y - 1) not in blend
                blend[(x, NX - N2 + y - 1)] = y
    return side, corner, blend


def closed_form(NZ, NX, N2):
    side, corner, blend = {}, set(), {}
    for z in range(NZ):
        for x in range(NX):
            if N2 <= z < NZ - N2 and N2 <= x < NX - N2:
                continue
            a, e = min(z, NZ - 1 - z), min(x, NX - 1 - x)
            if e >= a + 2:
                side[(z, x)] = "row"
            elif a >= e + 2:
                side[(z, x)] = "col"
            else:
                corner.add((z, x))
            blend[(z, x)] = max(N2 - z, N2 - x, z - (NZ - N2) + 1, x - (NX - N2) + 1)
    return side, corner, blend


def compact_cells(NZ, NX, N2):
    """Python restatement of abc_cell() (rtm_common.cuh)."""
    out = []
    top = N2 * NX
    n = NZ * NX - (NZ - 2 * N2) * (NX - 2 * N2)
    for t in range(n):
        if t < top:
            out.append((t // NX, t % NX))
        elif t < 2 * top:
            u = t - top
            out.append((NZ - N2 + u // NX, u % NX))
        else:
            u = t - 2 * top
            r, q = u // (2 * N2), u % (2 * N2)
            out.append((N2 + r, q if q < N2 else NX - 2 * N2 + q))
    return out


@pytest.mark.parametrize("NZ,NX,N2", [(37, 53, 5), (40, 41, 6), (61, 33, 7), (30, 30, 4),
                                      (96, 150, 30), (261, 461, 30)])
def test_classification_matches_reference(NZ, NX, N2):
    s1, c1, b1 = reference_sets(NZ, NX, N2)
    s2, c2, b2 = closed_form(NZ, NX, N2)
    assert s1 == s2
    assert c1 == c2
    assert b1 == b2
    assert set(s1) | c1 == set(b1)  # every pad cell gets a one-way value and one blend
    assert not (set(s1) & c1)


@pytest.mark.parametrize("NZ,NX,N2", [(37, 53, 5), (461, 1261, 30)])
def test_compact_enumeration_covers_pad_once(NZ, NX, N2):
    cells = compact_cells(NZ, NX, N2)
    assert len(cells) == len(set(cells))
    _, _, blend = closed_form(NZ, NX, N2) if NZ < 100 else (None, None, None)
    pad = {(z, x) for z in range(NZ) for x in range(NX)
           if not (N2 <= z < NZ - N2 and N2 <= x < NX - N2)}
    assert set(cells) == pad
