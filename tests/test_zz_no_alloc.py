"""The no-allocation render entry point (clv_render_device_noalloc).

It exists for callers that cannot allocate GPU memory while rendering; its
path state lives in a static device array instead.  Two calls in a row must
each reproduce the film of the regular entry point (clv_render_device) for
the same seed -- same paths, so equal up to the order of the f64 film
additions (relative tolerance 1e-9) -- and oversized requests must be
refused.  This file is collected last so that a failure here comes after
every other test has run.
"""

import ctypes

import numpy as np
import pytest

import clovers_gb300 as cg
from clovers_gb300 import _lib, scenes

pytestmark = pytest.mark.gpu

RTOL = 1e-9


def test_noalloc_matches_regular_render(tmp_path):
    torch = pytest.importorskip("torch")
    path = scenes.write_scene(scenes.enclosed_box(), str(tmp_path / "box.json"))
    w = h = 48
    spp = 24
    d = cg.Scene.from_json(path, w, h).upload()
    L = _lib.lib()
    opts = cg.render_opts(cg.RenderOptions(width=w, height=h, samples=spp, max_depth=12, seed=21))
    stream = torch.cuda.current_stream().cuda_stream
    ref = torch.zeros(w * h * 3, dtype=torch.float64, device="cuda")
    _lib.check(L.clv_render_device(d.handle, ctypes.byref(opts), ref.data_ptr(), stream))
    torch.cuda.synchronize()
    ref_np = ref.cpu().numpy()
    assert ref_np.max() > 0
    for call in range(2):  # the static array keeps the previous call's contents
        film = torch.zeros(w * h * 3, dtype=torch.float64, device="cuda")
        _lib.check(L.clv_render_device_noalloc(d.handle, ctypes.byref(opts), film.data_ptr(), stream))
        torch.cuda.synchronize()
        out = film.cpu().numpy()
        np.testing.assert_allclose(out, ref_np, rtol=RTOL, atol=1e-12, err_msg="call %d" % call)
    assert d.status() == 0


def test_noalloc_rejects_oversized_request(tmp_path):
    torch = pytest.importorskip("torch")
    path = scenes.write_scene(scenes.enclosed_box(), str(tmp_path / "box.json"))
    d = cg.Scene.from_json(path, 16, 16).upload()
    L = _lib.lib()
    opts = cg.render_opts(cg.RenderOptions(width=16, height=16, samples=1, max_depth=4, seed=1))
    opts.path_slots = 65536 + 128
    film = torch.zeros(16 * 16 * 3, dtype=torch.float64, device="cuda")
    rc = L.clv_render_device_noalloc(d.handle, ctypes.byref(opts), film.data_ptr(),
                                     torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.CLV_E_INVALID
    assert b"exceeds the static scratch" in L.clv_last_error()
