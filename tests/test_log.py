"""The render path's own natural logarithm (clovers_gb300/csrc/clv_log.h).

ConstantMedium::hit draws its free-flight distance from ln(U)
(clovers/src/objects/constant_medium.rs:102).  CUDA's logf and the host libm's
round the last bit differently, so the product and the oracle share one
routine evaluated in double with correctly rounded operations.  Checked here:

* CPU: against numpy's double-precision log, on every draw value the random
  stream can produce (k * 2^-24, sampled) and on random f32 bit patterns in
  (0, 1]: error within 1 ulp (CUDA's stated bound for logf; measured 0.5);
* GPU: the same bound over every f32 in (0, 1], and the GPU's bits equal the
  oracle's on every draw value k * 2^-24 and on random bit patterns.
"""

import ctypes

import numpy as np
import pytest

import oracle

ULP_BOUND = 1.0  # CUDA's documented maximum error of logf, in ulps


def _ulp_error(x, y):
    ref = np.log(x.astype(np.float64))
    nz = ref != 0.0
    _, e = np.frexp(np.abs(ref[nz]))
    err = np.abs(y.astype(np.float64)[nz] - ref[nz]) / np.ldexp(1.0, e - 24)
    return err, np.count_nonzero(y[nz] != ref[nz].astype(np.float32)), ref


def _draw_values(stride):
    k = np.arange(1, 1 << 24, stride, dtype=np.float64)
    return (k * 2.0 ** -24).astype(np.float32)


def _random_bits(n, seed):
    rng = np.random.default_rng(seed)
    return rng.integers(1, 0x3F800001, n, dtype=np.uint32).view(np.float32)


def test_oracle_log_error_bound():
    x = np.concatenate([_draw_values(7), _random_bits(1 << 21, 1),
                        np.array([1.0, 0.5, 2.0 ** -126, 2.0 ** -149, 0.70710677, 0.70710683], np.float32)])
    y = oracle.log_f32(x)
    err, not_nearest, _ = _ulp_error(x, y)
    assert err.max() <= ULP_BOUND
    assert not_nearest <= 1e-6 * x.size + 2
    assert oracle.log_f32([1.0])[0] == 0.0


def test_oracle_log_special_values():
    y = oracle.log_f32(np.array([0.0, -0.0, -1.0, np.inf, np.nan], np.float32))
    assert y[0] == -np.inf and y[1] == -np.inf
    assert np.isnan(y[2]) and y[3] == np.inf and np.isnan(y[4])


@pytest.mark.gpu
def test_gpu_log_all_inputs_and_bits_equal_oracle():
    from clovers_gb300 import _lib
    L = _lib.lib()
    x = np.concatenate([_draw_values(1), _random_bits(1 << 20, 2), np.array([0.0, 1.0], np.float32)])
    y = np.empty_like(x)
    max_ulp, not_nearest = ctypes.c_double(), ctypes.c_uint64()
    _lib.check(L.clv_selftest_log(x.ctypes.data, y.ctypes.data, x.size, ctypes.byref(max_ulp),
                                  ctypes.byref(not_nearest)))
    print("GPU log over every f32 in (0, 1]: max %.4f ulp, %d results not nearest" % (max_ulp.value,
                                                                                      not_nearest.value))
    assert max_ulp.value <= ULP_BOUND
    assert not_nearest.value <= 16
    assert np.array_equal(y.view(np.uint32), oracle.log_f32(x).view(np.uint32))
