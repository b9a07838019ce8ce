"""The guide's CPU oracle checked against mathematics alone (no GPU):

* the analytic gradient of -f log q(w) equals central finite differences of
  the loss (double precision, no bf16 rounding);
* every vMF mixture integrates to 1 over the sphere;
* the mixture sampler draws from the mixture density (first and second
  moments against quadrature).
The tensor-core kernels are then checked against this oracle in
tests/test_gpu_guide.py.
"""

import numpy as np

import oracle

P = oracle.GUIDE_PARAMS
W4 = 64 * 176 + 2 * 64 * 64


def random_params(seed, out_scale=0.3):
    rng = np.random.default_rng(seed)
    p = np.empty(P, np.float32)
    p[:64 * 176] = rng.uniform(-1, 1, 64 * 176) * np.sqrt(6 / 176)
    p[64 * 176:W4] = rng.uniform(-1, 1, W4 - 64 * 176) * np.sqrt(6 / 64)
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


def fibonacci_sphere(n):
    i = np.arange(n) + 0.5
    z = 1 - 2 * i / n
    r = np.sqrt(1 - z * z)
    ph = np.pi * (3 - np.sqrt(5)) * i
    return np.stack([r * np.cos(ph), r * np.sin(ph), z], 1)


def test_gradient_matches_finite_differences():
    p = random_params(1)
    rec = random_records(12, 2)
    g, loss = oracle.guide_gradient(p, rec, bf16=False)
    assert np.isfinite(loss) and loss != 0.0
    rng = np.random.default_rng(3)
    # parameters of every layer, including output-layer rows of each kind
    idx = np.concatenate([rng.integers(0, 64 * 176, 8), rng.integers(64 * 176, W4, 8), rng.integers(W4, P, 16)])
    checked = 0
    for i in idx:
        h = 1e-3 * max(1.0, abs(float(p[i])))
        pp, pm = p.copy(), p.copy()
        pp[i] = p[i] + h
        pm[i] = p[i] - h
        _, lp = oracle.guide_gradient(pp, rec, bf16=False)
        _, lm = oracle.guide_gradient(pm, rec, bf16=False)
        fd = (lp - lm) / (float(pp[i]) - float(pm[i]))
        assert abs(fd - g[i]) <= 2e-3 * max(abs(fd), abs(g[i])) + 1e-6, (i, fd, g[i])
        checked += abs(g[i]) > 1e-4
    assert checked >= 10


def test_bf16_rounding_stays_close_to_exact():
    p = random_params(4)
    q = np.zeros((64, 8), np.float32)
    q[:, :7] = np.random.default_rng(5).random((64, 7))
    a = oracle.guide_forward(p, q, bf16=True)
    b = oracle.guide_forward(p, q, bf16=False)
    assert np.linalg.norm(a - b) <= 0.05 * np.linalg.norm(b)


def test_mixture_integrates_to_one():
    rng = np.random.default_rng(6)
    dirs = fibonacci_sphere(200000).astype(np.float32)
    for _ in range(3):
        o = rng.normal(0, 1, 40).astype(np.float32)
        o[3::5] = rng.uniform(-2.5, 3.3, 8)  # concentrations up to ~27
        total = np.mean([oracle.guide_pdf(o, d) for d in dirs[::20]]) * 4 * np.pi
        assert abs(total - 1.0) < 5e-3, total


def test_sampler_draws_from_the_density():
    rng = np.random.default_rng(7)
    o = rng.normal(0, 1, 40).astype(np.float32)
    o[3::5] = rng.uniform(0.0, 2.5, 8)
    dirs = fibonacci_sphere(40000).astype(np.float32)
    q = np.array([oracle.guide_pdf(o, d) for d in dirs])
    wq = q / q.sum()
    mean_ref = (dirs * wq[:, None]).sum(0)
    second_ref = np.einsum("ni,nj,n->ij", dirs, dirs, wq)
    n = 40000
    u = rng.random((n, 3)).astype(np.float32)
    s = np.array([oracle.guide_sample(o, *uu) for uu in u])
    assert np.allclose(np.linalg.norm(s, axis=1), 1.0, atol=1e-5)
    tol = 4.0 / np.sqrt(n)
    assert np.all(np.abs(s.mean(0) - mean_ref) < tol), (s.mean(0), mean_ref)
    assert np.all(np.abs(np.einsum("ni,nj->ij", s, s) / n - second_ref) < tol)
