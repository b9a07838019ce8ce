"""The path guide on the GPU (tcgen05 kernels), checked against the oracle:

* tensor-core products through the guide's shared-memory operand layouts are
  exact on integer-valued bf16 operands (every shape the network uses);
* the network's outputs and the gradient of -f log q(w) agree with the
  oracle's bf16-emulating restatement (tolerances below; the GPU accumulates
  in fp32 in another order, which can move a bf16 rounding by one step);
* a guided render with an untrained network stays an unbiased estimate
  (converges to the golden crop like the reference's estimator);
* training on the renderer's own records lowers the loss, and a trained
  guide lowers the error of the caustic crop at equal samples per pixel.
"""

import ctypes
import os
import sys
import tempfile

import numpy as np
import pytest

import clovers_gb300 as cg
import oracle
from clovers_gb300 import _lib

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402

pytestmark = pytest.mark.gpu

P = oracle.GUIDE_PARAMS
W2, W3, W4 = 64 * 176, 64 * 176 + 64 * 64, 64 * 176 + 2 * 64 * 64
LAYERS = [("W1", 0, W2), ("W2", W2, W3), ("W3", W3, W4), ("W4", W4, P)]


def random_params(seed, out_scale=0.3):
    rng = np.random.default_rng(seed)
    p = np.empty(P, np.float32)
    p[:W2] = rng.uniform(-1, 1, W2) * np.sqrt(6 / 176)
    p[W2:W4] = rng.uniform(-1, 1, W4 - W2) * np.sqrt(6 / 64)
    p[W4:] = rng.normal(0, out_scale, P - W4)
    return p


def random_records(n, seed):
    rng = np.random.default_rng(seed)
    r = np.zeros((n, 12), np.float32)
    r[:, :7] = rng.random((n, 7))
    w = rng.normal(size=(n, 3))
    r[:, 8:11] = w / np.linalg.norm(w, axis=1, keepdims=True)
    r[:, 11] = rng.exponential(1.0, n) * (rng.random(n) > 0.2)
    return r


def relmse(img, ref):
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))


@pytest.mark.parametrize("n,k", [(64, 176), (48, 64), (64, 48), (176, 128), (64, 128), (16, 16), (256, 256)])
def test_tensor_core_operand_layouts(n, k):
    d = np.zeros((128, n), np.float32)
    err = ctypes.c_float(-1.0)
    _lib.check(_lib.lib().clv_guide_selftest_mma(n, k, 11, d.ctypes.data, ctypes.byref(err)))
    assert err.value == 0.0, "tensor-core product differs from the CUDA-core sum by %g" % err.value
    assert np.abs(d).max() > 0


def test_forward_matches_oracle():
    g = cg.Guide(seed=3)
    p = random_params(8)
    g.set_params(p)
    assert np.array_equal(g.params(), p)
    q = np.zeros((5000, 8), np.float32)
    q[:, :7] = np.random.default_rng(9).random((5000, 7))
    out = g.forward(q)
    ref = oracle.guide_forward(p, q, bf16=True)
    rel = np.linalg.norm(out - ref) / np.linalg.norm(ref)
    worst = np.abs(out - ref).max() / np.abs(ref).max()
    print("forward: relative L2 %.2e, worst %.2e" % (rel, worst))
    assert rel < 1e-2 and worst < 0.05
    assert g.status() == 0


def test_gradient_matches_oracle():
    g = cg.Guide(seed=4)
    p = random_params(10)
    g.set_params(p)
    rec = random_records(20000, 11)  # > 152 tiles: CTAs accumulate several tiles in TMEM
    gg, loss = g.gradient(rec)
    rg, rloss = oracle.guide_gradient(p, rec, bf16=True)
    print("loss gpu %.6g oracle %.6g" % (loss, rloss))
    assert abs(loss - rloss) <= 2e-3 * abs(rloss)
    for name, a, b in LAYERS:
        rel = np.linalg.norm(gg[a:b] - rg[a:b]) / np.linalg.norm(rg[a:b])
        print("%s gradient: relative L2 %.2e" % (name, rel))
        assert rel < 3e-2, name
    # records with f = 0 contribute nothing
    z = rec.copy()
    z[:, 11] = 0.0
    g0, l0 = g.gradient(z)
    assert l0 == 0.0 and not np.any(g0)


def _scene(name):
    w, h, depth, win = make_golden.WORKLOADS[name][1:5]
    with tempfile.TemporaryDirectory() as tmp:
        d = cg.Scene.from_json(make_golden.scene_file(name, tmp), w, h).upload()
    return d, w, h, depth, win


def _render(d, w, h, spp, depth, seed, guide, alpha, offset=0):
    film = cg.DeviceBuffer(w * h * 3 * 8).zero()
    opts = cg.RenderOptions(width=w, height=h, samples=spp, max_depth=depth, seed=seed)
    cg.render_guided(d, opts, guide, alpha, film, sample_offset=offset)
    return film.to_numpy(np.float64, (w * h, 3))


def _crop(img, w, h, win):
    x0, r0, x1, r1 = win
    return img.reshape(h, w, 3)[r0:r1, x0:x1].reshape(-1, 3)


def test_guided_render_with_untrained_guide_is_unbiased():
    d, w, h, depth, win = _scene("box")
    ref = np.load(os.path.join(HERE, "golden", "box_ref.npz"))["mean"]
    guide = cg.Guide(seed=1)
    spp = 256
    crop = _crop(_render(d, w, h, spp, depth, 4242, guide, 0.5) / spp, w, h, win)
    err = relmse(crop, ref)
    print("box, untrained guide, alpha 0.5: relMSE %.3g at %d spp" % (err, spp))
    assert err < 4e-3
    assert np.all(np.abs(crop.mean(0) - ref.mean(0)) <= 0.02 * ref.mean(0))
    assert guide.status() == 0


def test_records_and_training():
    d, w, h, depth, win = _scene("prism")
    guide = cg.Guide(seed=2)
    _render(d, w, h, 4, depth, 5, guide, 0.0)
    rec = guide.records()
    assert rec.shape[0] > 100000
    assert np.all((rec[:, :7] >= 0) & (rec[:, :7] <= 1))
    assert np.allclose(np.linalg.norm(rec[:, 8:11], axis=1), 1.0, atol=1e-5)
    f = rec[:, 11]
    assert np.all(np.isfinite(f)) and np.all(f >= 0) and np.count_nonzero(f) > 1000
    _, l0 = guide.gradient(rec)
    losses = [guide.train(50, 16384) for _ in range(4)]
    _, l1 = guide.gradient(rec)
    print("loss over the records: %.4g -> %.4g (training means %s)" % (l0, l1, ["%.4g" % x for x in losses]))
    assert l1 < l0 - 0.05 * abs(l0)
    assert guide.status() == 0


def test_trained_guide_lowers_caustic_error():
    d, w, h, depth, win = _scene("prism")
    ref = np.load(os.path.join(HERE, "golden", "prism_ref.npz"))["mean"]
    spp = 256
    plain = cg.draw(cg.GlobalOptions(quiet=True),
                    cg.RenderOptions(width=w, height=h, samples=spp, max_depth=depth, seed=99), d)
    e_plain = relmse(_crop(plain.astype(np.float64), w, h, win), ref)
    guide = cg.Guide(seed=7)
    for k in range(32):  # training passes, not part of the measured image
        _render(d, w, h, 4, depth, 1000 + k, guide, 0.0 if k == 0 else 0.5)
        guide.train(64, 32768)
    img = _render(d, w, h, spp, depth, 99, guide, 0.5) / spp
    e_guided = relmse(_crop(img, w, h, win), ref)
    print("prism crop at %d spp: plain relMSE %.4g, guided %.4g" % (spp, e_plain, e_guided))
    assert e_guided < 0.8 * e_plain
    assert guide.status() == 0


def test_bounded_wait_runs_out_and_frees_tmem():
    """A wait on an mbarrier that nothing arrives on (no copy, no MMA in
    flight) gives up after its clock limit: the kernel raises the guide's
    timeout flag, frees its TMEM and returns; the context stays usable and a
    normal guide call afterwards works."""
    L = _lib.lib()
    flags, freed = ctypes.c_uint32(), ctypes.c_uint32()
    _lib.check(L.clv_guide_selftest_timeout(2000000, ctypes.byref(flags), ctypes.byref(freed)))
    assert flags.value == 8  # CLV_ERR_GUIDE
    assert freed.value == 1
    g = cg.Guide(seed=3)
    params = random_params(4)
    g.set_params(params)
    q = np.random.default_rng(5).random((300, 8)).astype(np.float32)
    q[:, 7] = 0.0
    out = g.forward(q)
    ref = oracle.guide_forward(params, q)
    assert np.linalg.norm(out - ref) <= 1e-2 * np.linalg.norm(ref)
    assert g.status() == 0
