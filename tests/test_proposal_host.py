"""Host-side pieces of the learned proposal: training targets and the FLOP count."""
import numpy as np


def test_quarter_target_median_and_mask():
    from patchmatch_cuda_gb300 import proposal
    near, far = 1.0, 20.0
    depth = np.full((8, 12), 4.0, np.float32)
    depth[0, 0] = 19.0                          # an outlier inside block (0, 0)
    cost = np.zeros((8, 12, 2), np.float32)
    cost[4:8, 8:12, :] = 0.9                    # block (1, 2): PatchMatch not confident
    t = proposal.quarter_target(depth, near, far, 16, 16, cost)
    want = (0.25 - 1 / far) / (1 / near - 1 / far)
    assert abs(t[0, 0] - want) < 1e-6           # the median ignores the outlier
    assert t[1, 2] == -1.0                      # masked
    assert np.all(t[2:, :] == -1.0) and np.all(t[:, 3:] == -1.0)   # padding
    t2 = proposal.quarter_target(depth, near, far, 16, 16)          # no costs: all pixels
    assert abs(t2[1, 2] - want) < 1e-6


def test_quarter_target_mean():
    from patchmatch_cuda_gb300 import proposal
    depth = np.full((8, 8), 5.0, np.float32)
    depth[:4, :4] = 2.0
    t = proposal.quarter_target_mean(depth, 1.0, 20.0, 16, 16)
    r = 1 / 1.0 - 1 / 20.0
    assert abs(t[0, 0] - (0.5 - 0.05) / r) < 1e-6 and abs(t[1, 1] - (0.2 - 0.05) / r) < 1e-6
    assert t[2, 0] == -1.0
