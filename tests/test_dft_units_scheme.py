"""The tensor-core DFT's unit list, made on the device (grid_mma.cu: k_unit_offsets,
k_make_units), restated on the CPU.

uoff[p] = sum over q < p of ceil(nk_q / tp) * nparts; unit u belongs to the last
projection p with uoff[p] <= u (projections without points are skipped by that
rule), and within it local = u - uoff[p] = (nc * nkr + kr) * tiles + t.  Checked
against the host-side loop it replaced (projection, block, tile order): the same
units in the same order, for 128- and 64-point tiles and projections without
points."""
import numpy as np
import pytest


def device_units(nk, tp, nnc, nkr):
    P = len(nk)
    off = np.concatenate([[0], np.cumsum(nk)])
    nparts = nnc * nkr
    uoff = np.concatenate([[0], np.cumsum([(n + tp - 1) // tp * nparts for n in nk])])
    units = []
    for u in range(int(uoff[-1])):
        lo, hi = 0, P - 1                                   # the binary search of k_make_units
        while lo < hi:
            mid = (lo + hi + 1) >> 1
            if uoff[mid] <= u:
                lo = mid
            else:
                hi = mid - 1
        p = lo
        n = off[p + 1] - off[p]
        tiles = (n + tp - 1) // tp
        local = u - uoff[p]
        t, rest = local % tiles, local // tiles
        kr, nc = rest % nkr, rest // nkr
        units.append((int(off[p] + t * tp), p, int((p * nnc + nc) * nkr + kr), int(min(tp, n - t * tp))))
    return units


def host_units(nk, tp, nnc, nkr):
    off = np.concatenate([[0], np.cumsum(nk)])
    units = []
    for p in range(len(nk)):
        for nc in range(nnc):
            for kr in range(nkr):
                for j in range(0, nk[p], tp):
                    units.append((int(off[p] + j), p, (p * nnc + nc) * nkr + kr, int(min(tp, nk[p] - j))))
    return units


@pytest.mark.parametrize("tp", [128, 64])
@pytest.mark.parametrize("nnc,nkr", [(1, 1), (2, 1), (1, 2), (3, 2)])
def test_device_unit_list_equals_the_host_loop(tp, nnc, nkr):
    rng = np.random.default_rng(tp + 10 * nnc + nkr)
    for _ in range(5):
        P = int(rng.integers(1, 12))
        nk = [int(x) for x in rng.integers(0, 700, size=P)]
        nk[int(rng.integers(0, P))] = 0                     # a projection without points
        assert device_units(nk, tp, nnc, nkr) == host_units(nk, tp, nnc, nkr)
