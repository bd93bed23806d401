"""pm_box_moments_noalloc: the reference-window moments for callers that cannot allocate device
memory (for example work recorded into a stream capture that must not gain allocation nodes, or
a host framework that owns every allocation). The caller passes device buffers; the entry point
keeps its intermediate row sums in a fixed scratch array inside the library.

Checked against the engine's own preparation (pm_create then pm_get_ref_maps) on calls in a row
with different images and windows, so a stale scratch from one call cannot hide an error in the
next. The window sums are formed in the engine's order (zero rows add exactly 0.0), so S_I and
S_II must equal the engine's bit for bit; c1 is checked against the oracle. One case is wide
enough (8192 columns) that the image runs through several row strips of the fixed scratch, the
last one short. This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

RTOL = 1e-5  # the moment-map tolerance of the other parity tests


def _views(seed, width, height):
    from patchmatch_cuda_gb300 import scene
    w = scene.Workload(f"noalloc{seed}", width, height, 2, 3, 1, 2.0, 8.0, 3, 0, seed=seed)
    return w, scene.make_views(w)


@pytest.mark.gpu
def test_noalloc_moments_match_engine_on_two_calls():
    torch = pytest.importorskip("torch")
    from oracle import pm_oracle
    from patchmatch_cuda_gb300 import Engine, _native
    lib = _native.load_engine()
    # (seed, width, height, half-window): one strip each for the first two; the third needs
    # 2^20 / (2 * 8192) = 64 strip rows of scratch per strip, so 46 image rows per strip and
    # 5 strips, the last of 16 rows
    cases = [(3, 320, 240, 5), (4, 200, 150, 9), (6, 8192, 200, 9), (3, 320, 240, 5)]
    for seed, width, height, hw in cases:
        w, sv = _views(seed, width, height)
        eng = Engine(sv.images, sv.ref_id, w.params(half_window=hw))
        ref, si, sii = eng.ref_maps()
        eng.close()
        d_ref = torch.from_numpy(ref).cuda()
        out = torch.full((3, height, width), float("nan"), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        st = lib.pm_box_moments_noalloc(d_ref.data_ptr(), width * 4, width, height, hw,
                                        out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(),
                                        width * 4, None)
        assert st == 0, _native.STATUS_NAMES.get(st, st)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        np.testing.assert_array_equal(got[0], si)
        np.testing.assert_array_equal(got[1], sii)
        osi, osii = pm_oracle.box_moments(ref, hw)
        xs = np.arange(width)
        ys = np.arange(height)
        nx = np.minimum(xs + hw, width - 1) - np.maximum(xs - hw, 0) + 1
        ny = np.minimum(ys + hw, height - 1) - np.maximum(ys - hw, 0) + 1
        c1 = osii - osi ** 2 / (ny[:, None] * nx[None, :])
        c1 = np.where(c1 < 1e-5, 0.0, c1)
        np.testing.assert_allclose(got[2], c1, rtol=RTOL, atol=RTOL)


def test_noalloc_rejects_images_wider_than_its_scratch(engine_lib):
    from patchmatch_cuda_gb300 import _native
    limit = _native.load_engine()
    width = 1 << 19  # two rows plus the window margin need more than the fixed scratch
    st = limit.pm_box_moments_noalloc(C.c_void_p(16), width * 4, width, 4, 3, C.c_void_p(16), None, None,
                                      width * 4, None)
    assert _native.STATUS_NAMES[st] == "PM_ERR_SCRATCH_LIMIT"


def test_noalloc_rejects_unaligned_pitches(engine_lib):
    """Pitches that are not whole floats are refused before anything is launched."""
    from patchmatch_cuda_gb300 import _native
    lib = _native.load_engine()
    for ref_pitch, out_pitch in [(64 * 4 + 2, 64 * 4), (64 * 4, 64 * 4 + 1), (63 * 4, 64 * 4)]:
        st = lib.pm_box_moments_noalloc(C.c_void_p(16), ref_pitch, 64, 8, 3, C.c_void_p(16), None, None,
                                        out_pitch, None)
        assert _native.STATUS_NAMES[st] == "PM_ERR_INVALID_ARGUMENT"
