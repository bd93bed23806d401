"""The learned depth proposal's kernels on the GPU: the tcgen05 BF16 GEMM against an FP32
matrix product (torch, no TF32) of the same BF16 inputs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _stream():
    import torch
    return torch.cuda.current_stream().cuda_stream


@pytest.mark.parametrize("m,n,k", [(128, 16, 64), (256, 48, 320), (384, 128, 2048), (128, 160, 128),
                                   (512, 256, 64)])
@pytest.mark.parametrize("mode", [0, 1])
def test_gemm_matches_fp32_product(engine_lib, m, n, k, mode):
    import torch
    torch.backends.cuda.matmul.allow_tf32 = False
    g = torch.Generator(device="cuda").manual_seed(m + n + k)
    a = torch.randn(m, k, device="cuda", generator=g).bfloat16()
    b = torch.randn(n, k, device="cuda", generator=g).bfloat16()
    bias = torch.randn(n, device="cuda", generator=g)
    ref = a.float() @ b.float().t() + bias
    if mode == 0:
        c = torch.zeros(m, n, device="cuda", dtype=torch.bfloat16)
        ref = ref.relu()
    else:
        c = torch.zeros(m, n, device="cuda")
    st = engine_lib.pm_gemm_bf16(a.data_ptr(), k, b.data_ptr(), k, m, n, k, c.data_ptr(), n, mode,
                                 bias.data_ptr(), 1 if mode == 0 else 0, 1, _stream())
    torch.cuda.synchronize()
    assert st == 0
    import ctypes as C
    err = C.c_uint(7)
    assert engine_lib.pm_gemm_error(C.byref(err), 1) == 0 and err.value == 0
    got = c.float()
    # FP32 accumulation order only; a BF16 result adds its own rounding (2^-8 relative)
    tol = (2.0 ** -7) * ref.abs() + 1e-2 if mode == 0 else 1e-4 * (k ** 0.5) * (1 + ref.abs())
    assert torch.all((got - ref).abs() <= tol), float((got - ref).abs().max())


@pytest.mark.parametrize("splits", [1, 3, 8])
def test_gemm_split_k_accumulates(engine_lib, splits):
    import torch
    torch.backends.cuda.matmul.allow_tf32 = False
    g = torch.Generator(device="cuda").manual_seed(11)
    m, n, k = 128, 96, 64 * 20
    a = torch.randn(m, k, device="cuda", generator=g).bfloat16()
    b = torch.randn(n, k, device="cuda", generator=g).bfloat16()
    c = torch.full((m, n), 0.5, device="cuda")
    st = engine_lib.pm_gemm_bf16(a.data_ptr(), k, b.data_ptr(), k, m, n, k, c.data_ptr(), n, 2, None, 0,
                                 splits, _stream())
    torch.cuda.synchronize()
    assert st == 0
    ref = a.float() @ b.float().t() + 0.5
    assert torch.allclose(c, ref, atol=1e-3, rtol=1e-4)


def test_gemm_rejects_bad_shapes(engine_lib):
    import torch
    a = torch.zeros(100, 64, device="cuda", dtype=torch.bfloat16)
    c = torch.zeros(100, 16, device="cuda")
    assert engine_lib.pm_gemm_bf16(a.data_ptr(), 64, a.data_ptr(), 64, 100, 16, 64, c.data_ptr(), 16, 1,
                                   None, 0, 1, _stream()) != 0


class Net:
    """ctypes wrapper of a pm_net for the tests."""

    def __init__(self, lib, b, h, w, seed=1):
        import ctypes as C
        self.lib = lib
        self.h = C.c_void_p()
        assert lib.pm_net_create(b, h, w, seed, C.byref(self.h)) == 0
        n = C.c_size_t()
        assert lib.pm_net_num_params(self.h, C.byref(n)) == 0
        self.n = n.value

    def params(self):
        p = np.zeros(self.n, np.float32)
        assert self.lib.pm_net_get_params(self.h, p.ctypes.data, self.n) == 0
        return p

    def layout(self):
        import ctypes as C
        nl = C.c_int()
        d = np.zeros(8 * 64, np.int32)
        assert self.lib.pm_net_layout(self.h, C.byref(nl), d.ctypes.data, 64) == 0
        return d[:8 * nl.value].reshape(nl.value, 8)

    def gradients(self, x, t, inv_far, inv_range):
        g = np.zeros(self.n, np.float32)
        loss = np.zeros(3, np.float32)
        st = self.lib.pm_net_gradients(self.h, x.data_ptr(), t.data_ptr(), inv_far, inv_range, g.ctypes.data,
                                       self.n, loss.ctypes.data)
        assert st == 0
        return g, loss

    def close(self):
        self.lib.pm_net_destroy(self.h)


def test_network_layout_matches_oracle(engine_lib):
    from oracle import pm_net_oracle as O
    net = Net(engine_lib, 1, 32, 48)
    lay = net.layout()
    offs, n = O.param_offsets()
    assert net.n == n
    for row, (cin, cout, k, s, relu, lv), o in zip(lay, O.layers(), offs):
        assert tuple(row[:6]) == (cin, cout, k, s, relu, o)
        assert (row[6], row[7]) == (32 >> lv, 48 >> lv)
    net.close()


def test_network_gradients_match_cpu_oracle(engine_lib, parity_log):
    """Every layer's weight and bias gradient from the GPU's forward and backward kernels
    against the float64 oracle rounding to bfloat16 where the GPU stores bfloat16. BF16
    rounding makes this network's gradients sensitive at the several-percent level: the
    oracle against itself with the parameters perturbed by 1e-6 (relative) differs by up to
    ~14 % per layer at initialisation. The bar per layer: cosine similarity >= 0.99 and a
    relative error within twice that noise floor (and never above 25 %). The loss terms match
    to 1e-3."""
    import torch
    from oracle import pm_net_oracle as O
    B, H, W = 2, 32, 32
    net = Net(engine_lib, B, H, W, seed=3)
    g = torch.Generator().manual_seed(4)
    x = torch.randn(B, H, W, O.IN_CH, generator=g)
    t = torch.rand(B, H, W, generator=g)
    t[0, :4, :] = -1.0                                  # masked pixels
    inv_far, inv_range = 0.05, 0.95
    gg, loss = net.gradients(x.cuda(), t.cuda(), inv_far, inv_range)
    params = net.params().astype(np.float64)
    xd, td = x.numpy().astype(np.float64), t.numpy()
    go, stats, _ = O.forward_backward(params, xd, td, inv_far, inv_range)
    rng = np.random.default_rng(0)
    gp, _, _ = O.forward_backward(params * (1 + 1e-6 * rng.normal(size=params.size)), xd, td, inv_far, inv_range)
    offs, n = O.param_offsets()
    per_layer, bad = [], []
    for li, ((cin, cout, k, s, relu, lv), o) in enumerate(zip(O.layers(), offs)):
        K = k * k * cin
        for name, sl in (("w", slice(o, o + cout * K)), ("b", slice(o + cout * K, o + cout * K + cout))):
            a = gg[sl].astype(np.float64)
            b = go[sl]
            nb = np.linalg.norm(b) + 1e-30
            cos = float(a @ b / (np.linalg.norm(a) * nb))
            rel = float(np.linalg.norm(a - b) / nb)
            floor = float(np.linalg.norm(gp[sl] - b) / nb)
            per_layer.append((li, name, round(cos, 5), round(rel, 4), round(floor, 4)))
            if not (cos >= 0.99 and rel <= min(0.25, max(0.02, 2 * floor))):
                bad.append(per_layer[-1])
    parity_log("net_gradients_vs_oracle", per_layer=per_layer, loss_gpu=[float(v) for v in loss],
               loss_oracle=list(stats))
    assert abs(loss[0] - stats[0]) <= 1e-3 and abs(loss[1] - stats[1]) <= 1e-3 and loss[2] == stats[2]
    assert not bad, bad
    net.close()


def test_training_steps_reduce_the_loss(engine_lib, parity_log):
    """Adam steps on one batch with a smooth target the input encodes: the loss falls."""
    import ctypes as C
    import torch
    B, H, W = 4, 32, 64
    net = Net(engine_lib, B, H, W, seed=9)
    g = torch.Generator().manual_seed(2)
    x = torch.rand(B, H, W, 17, generator=g) - 0.5
    t = (0.5 + 0.4 * torch.tanh(3 * x[..., 0] + 2 * x[..., 5])).contiguous()
    xc, tc = x.cuda(), t.cuda()
    loss = np.zeros(3, np.float32)
    curve = []
    for it in range(150):
        assert engine_lib.pm_net_train_step(net.h, xc.data_ptr(), tc.data_ptr(), 0.05, 0.95, 3e-3,
                                             loss.ctypes.data) == 0
        curve.append(float(loss[0]))
    parity_log("net_training_curve", l1=curve[::10] + [curve[-1]])
    assert curve[-1] < 0.6 * curve[0], curve[::10]
    err = C.c_uint(1)
    assert engine_lib.pm_gemm_error(C.byref(err), 0) == 0 and err.value == 0
    net.close()


@pytest.fixture(scope="module")
def small_views():
    from patchmatch_cuda_gb300 import scene
    w = scene.WORKLOADS["plane3_320x240"]
    return w, scene.make_views(w)


def test_proposal_input_channels(small_views):
    """Channel 0 is the reference's 4x4 block mean; the 16 warped channels lie in [0, 1]; the
    padding to a multiple of 16 is zero."""
    import torch
    from patchmatch_cuda_gb300 import Engine
    w, sv = small_views
    eng = Engine(sv.images, sv.ref_id, w.params())
    hp, wp = eng.proposal_shape()
    assert (hp, wp) == (64, 80)
    x = torch.full((hp, wp, 17), 7.0, device="cuda")
    eng.proposal_input(x.data_ptr())
    x = x.cpu().numpy()
    ref = sv.images[sv.ref_id].image.astype(np.float64)
    q = ref[:240, :320].reshape(60, 4, 80, 4).mean(axis=(1, 3)) / 255.0
    np.testing.assert_allclose(x[:60, :80, 0], q, atol=1e-6)
    assert np.all(x[60:] == 0.0)
    assert x[:60, :80, 1:].min() >= 0.0 and x[:60, :80, 1:].max() <= 1.0
    assert x[:60, :80, 1:].std() > 0.05
    eng.close()


def test_proposal_initialisation(small_views):
    """init_mode = proposal: the depth is the network's inverse depth, bilinearly upsampled,
    where the confidence reaches the threshold, and the uniform random initialisation
    elsewhere (threshold 1 reproduces init_mode = random exactly)."""
    import torch
    from patchmatch_cuda_gb300 import INIT_PROPOSAL, Engine, proposal
    w, sv = small_views
    rnd = Engine(sv.images, sv.ref_id, w.params())
    rnd.init_depth()
    d_rand = rnd.depth()
    e0 = Engine(sv.images, sv.ref_id, w.params(init_mode=INIT_PROPOSAL, proposal_threshold=0.0))
    e1 = Engine(sv.images, sv.ref_id, w.params(init_mode=INIT_PROPOSAL, proposal_threshold=1.0))
    hp, wp = e0.proposal_shape()
    net = proposal.ProposalNet(1, hp, wp, seed=7)
    e0.set_proposal(net)
    e1.set_proposal(net)
    e1.init_depth()
    np.testing.assert_array_equal(e1.depth(), d_rand)
    e0.init_depth()
    d = e0.depth()
    x = torch.empty(hp, wp, 17, device="cuda")
    out = torch.empty(hp, wp, 2, device="cuda")
    e0.proposal_input(x.data_ptr())
    net.forward(x.data_ptr(), out.data_ptr())
    torch.cuda.synchronize()
    o = out.cpu().numpy().astype(np.float64)
    inv_far, inv_range = 1.0 / w.depth_far, 1.0 / w.depth_near - 1.0 / w.depth_far
    rng = np.random.default_rng(0)
    for y, x_ in zip(rng.integers(0, 240, 200), rng.integers(0, 320, 200)):
        qx = min(max((x_ - 1.5) / 4, 0.0), 79.0)
        qy = min(max((y - 1.5) / 4, 0.0), 59.0)
        x0, y0 = int(qx), int(qy)
        x1, y1 = min(x0 + 1, 79), min(y0 + 1, 59)
        ax, ay = qx - x0, qy - y0
        s = ((1 - ay) * ((1 - ax) * o[y0, x0, 0] + ax * o[y0, x1, 0]) +
             ay * ((1 - ax) * o[y1, x0, 0] + ax * o[y1, x1, 0]))
        want = min(max(1.0 / (inv_far + s * inv_range), w.depth_near), w.depth_far)
        assert abs(d[y, x_] - want) <= 1e-4 * want, (y, x_, d[y, x_], want)
    # a full run from the proposal, two sweeps
    e2 = Engine(sv.images, sv.ref_id, w.params(init_mode=INIT_PROPOSAL, num_sweeps=2))
    e2.set_proposal(net)
    e2.run()
    d2 = e2.depth()
    assert np.all(np.isfinite(d2)) and d2.min() >= w.depth_near and d2.max() <= w.depth_far
    assert e2.stats().cost_evals > 0
    for e in (rnd, e0, e1, e2):
        e.close()
    net.close()


def test_run_requires_an_attached_network(small_views):
    from patchmatch_cuda_gb300 import INIT_PROPOSAL, Engine, PatchMatchError
    w, sv = small_views
    e = Engine(sv.images, sv.ref_id, w.params(init_mode=INIT_PROPOSAL))
    with pytest.raises(PatchMatchError):
        e.run()
    e.close()


def test_learned_schedule_against_random_controls(parity_log):
    """What the committed network (trained on the GPU on plain-PatchMatch depth maps of 2000
    seeded 640x480 scenes) gains, on three held-out scenes of the same kind, 4 sweeps each:

    * the learned schedule's gain comes from the schedule: numOfSamples views from the first
      sweep and the local search leave far fewer bad pixels (> 1 % relative depth error) after
      4 sweeps than the plain schedule stopped there (about 13 points);
    * the network adds nothing: at the specified confidence threshold 0.5 its depths cost about
      a point against the same schedule from random starting depths (threshold 1, the control),
      and at a threshold of 0.8, where it seeds only its most confident pixels, it is within half
      a point of the control. Its prediction (about 27 % median depth error) is too coarse to
      improve on random starts; the test fails if that changes, in either direction."""
    from patchmatch_cuda_gb300 import INIT_PROPOSAL, Engine, proposal, scene
    if not proposal.WEIGHTS.exists():
        pytest.skip("no trained weights in the package")
    rows = []
    for seed in (987654, 987655, 987656):  # seeds outside the training range
        wl = proposal.training_workload(seed)
        sv = scene.make_views(wl)

        def bad(**over):
            e = Engine(sv.images, sv.ref_id, wl.params(**over))
            net = proposal.for_engine(e) if over.get("init_mode") == INIT_PROPOSAL else None
            e.run()
            r = 100 * scene.bad_pixel_rate(e.depth(), sv.gt_depth)
            e.close()
            if net is not None:
                net.close()
            return r

        sched = dict(init_mode=INIT_PROPOSAL, num_sweeps=4, perturbation=0.05)
        rows.append({"seed": seed, "learned_0p5": bad(**sched), "learned_0p8": bad(proposal_threshold=0.8, **sched),
                     "control": bad(proposal_threshold=1.0, **sched), "plain_4": bad(num_sweeps=4),
                     "plain_20": bad()})
    mean = {k: float(np.mean([r[k] for r in rows])) for k in rows[0] if k != "seed"}
    parity_log("trained_proposal_640x480_heldout", scenes=rows, mean_bad_pixel_pct=mean)
    assert mean["plain_4"] - mean["control"] > 5.0, mean
    assert -0.5 <= mean["learned_0p5"] - mean["control"] <= 2.0, mean
    assert abs(mean["learned_0p8"] - mean["control"]) <= 0.5, mean
