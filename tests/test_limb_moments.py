"""The learned regression's bin moments (csrc/lsm_mlp_nodes.cu, lsm_mlp_binned)
are summed as 32-bit limbs of at most 16 bits per path over epochs of at most
kEpochChunks x kLsmChunk paths and recombined into the 64-bit moments
n 2^40 + sum t, sum t^2, sum y, sum t y (the last two modulo 2^64).  This
restates the limb split and the recombination with exact integers and checks,
on random inputs and on the extreme inputs (t = 2^16, y = +/-2^24, a full
epoch of equal paths), that no limb sum leaves 32 bits and that the
recombined moments equal the direct 64-bit sums bit for bit."""
import numpy as np

EPOCH = 32 * 1024           # kEpochChunks x kLsmChunk
COUNT_SHIFT = 40            # kCountShift
M64 = (1 << 64) - 1


def limbs(tq, yq):
    ut = tq
    yb = yq + (1 << 24)
    tt = ut * ut
    pp = ut * yb
    return [1, ut, tt & 0xFFFF, tt >> 16, yb & 0xFFFF, yb >> 16, pp & 0xFFFF, (pp >> 16) & 0xFFFF, pp >> 32]


def fold(tqs, yqs):
    lim = [0] * 9
    for tq, yq in zip(tqs, yqs):
        for q, v in enumerate(limbs(int(tq), int(yq))):
            lim[q] += v
    assert all(0 <= v < (1 << 32) for v in lim), lim
    st = lim[1]
    m0 = ((lim[0] << COUNT_SHIFT) + st) & M64
    m1 = (lim[2] + (lim[3] << 16)) & M64
    m2 = (lim[4] + (lim[5] << 16) - (lim[0] << 24)) & M64
    m3 = (lim[6] + (lim[7] << 16) + (lim[8] << 32) - (st << 24)) & M64
    return m0, m1, m2, m3


def direct(tqs, yqs):
    m = [0, 0, 0, 0]
    for tq, yq in zip(tqs, yqs):
        tq, yq = int(tq), int(yq)
        m[0] = (m[0] + (1 << COUNT_SHIFT) + tq) & M64
        m[1] = (m[1] + tq * tq) & M64
        m[2] = (m[2] + (yq & M64)) & M64
        m[3] = (m[3] + ((tq * yq) & M64)) & M64
    return tuple(m)


def test_random_epochs_match_direct_sums():
    rng = np.random.default_rng(11)
    for n in (1, 7, 1000, 5000):
        tq = rng.integers(0, (1 << 16) + 1, n)
        yq = rng.integers(-(1 << 24), (1 << 24) + 1, n)
        assert fold(tq, yq) == direct(tq, yq)


def test_extreme_full_epoch_fits_32_bit_limbs():
    for t, y in ((1 << 16, 1 << 24), (1 << 16, -(1 << 24)), (0, -(1 << 24)), ((1 << 16) - 1, (1 << 24) - 1)):
        tq = np.full(EPOCH, t)
        yq = np.full(EPOCH, y)
        assert fold(tq, yq) == direct(tq, yq)
