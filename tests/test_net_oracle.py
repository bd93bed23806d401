"""The learned proposal's CPU oracle (float64): its hand-written gradients against central
finite differences of its own loss, and its layer table against the engine's."""
import numpy as np


def _loss(params, x, t, inv_far, inv_range):
    from oracle import pm_net_oracle as O
    # the oracle's loss with the same 1/P scaling as its gradient
    _, (l1, bce, cnt), _ = O.forward_backward(params, x, t, inv_far, inv_range, use_bf16=False)
    P = t.size
    return (l1 + 0.1 * bce) * cnt / P


def test_oracle_gradients_match_finite_differences():
    from oracle import pm_net_oracle as O
    rng = np.random.default_rng(5)
    offs, n = O.param_offsets()
    params = np.zeros(n)
    for (cin, cout, k, s, relu, lv), o in zip(O.layers(), offs):
        K = k * k * cin
        params[o:o + cout * K] = rng.normal(0, np.sqrt(2.0 / K), cout * K)
        params[o + cout * K:o + cout * K + cout] = rng.normal(0, 0.05, cout)
    x = rng.normal(0, 1, (1, 16, 16, O.IN_CH))
    t = rng.uniform(0, 1, (1, 16, 16))
    inv_far, inv_range = 0.05, 0.95
    g, _, _ = O.forward_backward(params, x, t, inv_far, inv_range, use_bf16=False)
    # spot-check coordinates of several layers (weights and biases)
    for li in (0, 5, 9, 12, 17, 18):
        cin, cout, k, s, relu, lv = O.layers()[li]
        o = offs[li]
        for j in (o + 3, o + cout * k * k * cin + 1):
            e = 1e-5
            p1, p2 = params.copy(), params.copy()
            p1[j] += e
            p2[j] -= e
            fd = (_loss(p1, x, t, inv_far, inv_range) - _loss(p2, x, t, inv_far, inv_range)) / (2 * e)
            assert abs(fd - g[j]) <= 1e-6 + 1e-3 * abs(fd), (li, j, fd, g[j])


def test_bf16_rounding_is_nearest_even():
    from oracle import pm_net_oracle as O
    v = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e-3, 65504.0])
    r = O.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125 and r[3] == -2.5
    assert abs(r[4] - 3.0e-3) <= 3.0e-3 * 2 ** -8


def test_parameter_count():
    from oracle import pm_net_oracle as O
    _, n = O.param_offsets()
    assert 1_500_000 < n < 1_800_000


def test_package_layer_table_matches_oracle():
    from oracle import pm_net_oracle as O
    from patchmatch_cuda_gb300 import proposal
    assert proposal.layer_table() == O.layers()
    assert proposal.forward_flops(192, 320) > 1e9
