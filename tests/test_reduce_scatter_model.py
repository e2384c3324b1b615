"""The transposed warp sum of the Q-environment and solute-row kernels
(reduce_scatter in q6_gb300/csrc/qnb_kernels.cu), modelled lane by lane in
float32 on the CPU: every value's sum equals, bit for bit, what warp_sum
(__shfl_down_sync over offsets 16, 8, 4, 2, 1, lane 0's result) gives for
that value, and lane v (N = 32) or lanes 2v and 2v + 1 (N = 16) hold value
v.  The GPU kernels are checked against the oracle in the -m gpu tests; this
pins the index mapping and the claim that the sums are unchanged."""
import numpy as np
import pytest


def warp_sum_lane0(vals):
    """vals: (32,) float32 per lane; shfl_down tree, lane 0's result."""
    v = vals.astype(np.float32).copy()
    for o in (16, 8, 4, 2, 1):
        src = np.arange(32) + o
        other = np.where(src < 32, v[np.minimum(src, 31)], np.float32(0))
        v = (v + other).astype(np.float32)
    return v[0]


def reduce_scatter(g):
    """g: (32 lanes, N) float32; returns the (32,) value each lane ends with."""
    g = g.astype(np.float32).copy()
    n = g.shape[1]
    lanes = np.arange(32)
    o, ln = 16, n
    while ln > 1:
        half = ln // 2
        up = (lanes & o) != 0
        keep = np.where(up[:, None], g[:, half:ln], g[:, :half])
        send = np.where(up[:, None], g[:, :half], g[:, half:ln])
        g[:, :half] = (keep + send[lanes ^ o]).astype(np.float32)
        o >>= 1
        ln = half
    v = g[:, 0].copy()
    while o > 0:
        v = (v + v[lanes ^ o]).astype(np.float32)
        o >>= 1
    return v


@pytest.mark.parametrize("n", [16, 32])
def test_transposed_sum_matches_warp_sum_bit_for_bit(n):
    rng = np.random.default_rng(n)
    for trial in range(50):
        scale = 10.0 ** rng.uniform(-3, 3, size=(1, n))
        g = (rng.normal(size=(32, n)) * scale).astype(np.float32)
        out = reduce_scatter(g)
        for v in range(n):
            ref = warp_sum_lane0(g[:, v])
            lanes = [v] if n == 32 else [2 * v, 2 * v + 1]
            for lane in lanes:
                assert out[lane].tobytes() == ref.tobytes(), (n, trial, v, lane, out[lane], ref)
