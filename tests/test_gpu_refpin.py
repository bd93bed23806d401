"""The engine against the reference's own outputs (needs a GPU).

tests/golden/ref_box200_96x64.npz holds what yhsa678/patchMatch_cuda's own kernels compute,
run on the CPU by oracle/ref_host.cpp (tests/test_ref_pin.py pins the oracle to the same file),
on a 96x64 crop of the benchmarked scene at its window, view and sample counts (15x15, 10
sources, numOfSamples 5). The engine is compared here directly with the parts that draw no
random numbers (the engine keys its draws by pixel and sweep, the reference draws per-pixel
streams, so sweeps are compared through the oracle instead):

* Array2d_refImg's window sums (array2d_refImg.cu:11-67);
* computeNCC (patchMatch.cu:433-612) at 1024 queries, a quarter of them at the borders, with
  exact bilinear weights and with the texture unit's (the widened reference computed with the
  1/256 weights the engine's texture-unit sampler is checked to use);
* computeAllCostGivenDepth (patchMatch.cu:775-818) at the reference's own initial depth;
* GaussianBlurCUDA::Filter (GaussianBlurCUDA.cu:185-191), the engine's box prefilter, at 5, 11
  and 45 taps.

The bounds are those the engine meets against the FP64 oracle (tests/test_gpu_headline.py):
the reference's float build itself is farther from the widened one (NCC 1.4e-4).
"""
import sys
from pathlib import Path

import numpy as np
import pytest

from parity_util import NCC_TOL, ncc_err, special_value_flips

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))
import make_ref_golden as G  # noqa: E402


@pytest.fixture(scope="module")
def golden():
    z = np.load(GOLDEN / "ref_box200_96x64.npz")
    return {k: z[k] for k in z.files}


def make_engine(golden, **over):
    from patchmatch_cuda_gb300 import Engine
    p = G.params()
    for k, v in over.items():
        setattr(p, k, v)
    return Engine(G.stored_views(golden), int(golden["ref_id"]), p)


def queries(golden):
    return golden["q_x"], golden["q_y"], golden["q_view"], golden["q_depth"].astype(np.float32), golden["q_axis"]


def test_window_sums_match_reference(golden, parity_log):
    eng = make_engine(golden)
    ref, si, sii = eng.ref_maps()
    np.testing.assert_array_equal(ref, golden[f"image_{int(golden['ref_id'])}"].astype(np.float32) / np.float32(255))
    e_i = np.abs(si - golden["sum_i_f64"]) / golden["sum_i_f64"]
    e_ii = np.abs(sii - golden["sum_ii_f64"]) / golden["sum_ii_f64"]
    parity_log("refpin_gpu_window_sums", rel_max_i=float(e_i.max()), rel_max_ii=float(e_ii.max()))
    assert e_i.max() <= 6e-8 and e_ii.max() <= 6e-8      # the engine stores the sums as float
    eng.close()


@pytest.mark.parametrize("sampler", [0, 1])
def test_ncc_matches_reference(golden, sampler, parity_log):
    eng = make_engine(golden, sampler=sampler)
    got = eng.eval_costs(*queries(golden))
    want = golden["ncc_f64" if sampler == 0 else "ncc_f64_fixed"]
    err = ncc_err(got, want)
    flips = special_value_flips(got, want)
    e32 = ncc_err(golden["ncc_f32"], golden["ncc_f64"])
    parity_log(f"refpin_gpu_ncc_sampler{sampler}", n=int(err.size), err_max=float(err[~flips].max()),
               err_q99=float(np.quantile(err, 0.99)), special_value_flips=int(flips.sum()),
               reference_float_build_err_max=float(e32.max()))
    assert flips.sum() == 0
    assert err.max() <= (NCC_TOL if sampler == 0 else 5 * NCC_TOL)
    eng.close()


def test_initial_costs_match_reference(golden, parity_log):
    eng = make_engine(golden)
    eng.set_depth(golden["depth0_f64"].astype(np.float32))
    eng.compute_costs(1)
    c = eng.costs()
    want = golden["costs0_f64"].astype(np.float64)
    err = ncc_err(c, want)
    flips = special_value_flips(c, want)
    parity_log("refpin_gpu_initial_costs", n=int(err.size), err_q9999=float(np.quantile(err, 0.9999)),
               err_max_other=float(err[~flips].max()), special_value_flips=int(flips.sum()))
    assert np.quantile(err, 0.9999) <= NCC_TOL
    assert flips.sum() <= 1 and err[~flips].max() <= 5 * NCC_TOL
    eng.close()


def test_box_prefilter_matches_reference_blur(golden, parity_log):
    """The engine's box prefilter of the reference image is GaussianBlurCUDA as written: 1/width
    taps, edge pixels repeated. The engine fuses each tap's multiply-add (as nvcc does for the
    reference's `sum += tex2D(..) * g_Kernel[..]`), the host-compiled float build does not: the
    two differ by float rounding, at most half an ulp of 1 (values lie in [0, 1]) per add of
    each pass's taps."""
    errs = []
    for i, sigma in enumerate(golden["blur_sigma"]):
        eng = make_engine(golden, prefilter=1, gaussian_sigma=float(sigma))
        ref, _, _ = eng.ref_maps()
        e32 = np.abs(ref.astype(np.float64) - golden[f"blur{i}_f32"])
        e64 = np.abs(ref.astype(np.float64) - golden[f"blur{i}_f64"])
        errs.append((float(e32.max()), float(e64.max())))
        bound = 2 * int(golden["blur_taps"][i]) * 2.0 ** -24
        assert e32.max() <= bound and e64.max() <= bound, (sigma, e32.max(), e64.max(), bound)
        eng.close()
    parity_log("refpin_gpu_box_prefilter", taps=[int(t) for t in golden["blur_taps"]],
               err_max_vs_float_build=[e[0] for e in errs], err_max_vs_widened=[e[1] for e in errs])
