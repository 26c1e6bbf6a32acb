"""PiecewiseConstantFunc against the reference's piecewise tests (CPU).

The cases and expected values of piecewise_test.py:60-285: values and
integrals without a batch, with a batch of rank 2, with repeated jump
locations, with matrix and 3-d event shapes, and the shape errors.
"""

import numpy as np
import pytest

from tqf.math.piecewise import PiecewiseConstantFunc

DTYPES = [np.float32, np.float64]


@pytest.mark.parametrize("dtype", DTYPES)
def test_value_and_integral_no_batch(dtype):
    # :60-88
    f = PiecewiseConstantFunc(np.array([0.1, 10], dtype=dtype), np.array([3, 4, 5], dtype=dtype), dtype=dtype)
    value = f(np.array([0.0, 0.1, 2.0, 11.0]))
    assert value.dtype == dtype
    np.testing.assert_array_equal(value, [3.0, 3.0, 4.0, 5.0])
    g = PiecewiseConstantFunc(np.array([1, 2, 3, 4, 5], dtype=dtype), np.array([0.1, 0.2, 0.3, 0.4, 0.5, 0.6]),
                              dtype=dtype)
    x = np.array([-4.1, 0.0, 1.0, 1.5, 2.0, 4.5, 5.5])
    integral = g.integrate(x, x + 4.1)
    assert integral.dtype == dtype
    np.testing.assert_allclose(integral, [0.41, 1.05, 1.46, 1.66, 1.86, 2.41, 2.46], atol=1e-5, rtol=1e-5)


X_BATCH = np.array([[[0.0, 0.1, 2.0, 11.0], [0.0, 2.0, 3.0, 9.0]], [[0.0, 1.0, 2.0, 3.0], [4.0, 5.0, 6.0, 7.0]]])
JUMPS_BATCH = np.array([[[0.1, 10.0], [1.5, 10.0]], [[1.0, 2.0], [5.0, 6.0]]])
VALUES_BATCH = np.array([[[3, 4, 5], [3, 4, 5]], [[3, 4, 5], [3, 4, 5]]])


@pytest.mark.parametrize("dtype", DTYPES)
def test_value_and_integral_with_batch(dtype):
    # :86-113, :138-161
    f = PiecewiseConstantFunc(JUMPS_BATCH, VALUES_BATCH, dtype=dtype)
    value = f(X_BATCH, left_continuous=False)
    assert value.dtype == dtype
    np.testing.assert_array_equal(value, [[[3.0, 4.0, 4.0, 5.0], [3.0, 4.0, 4.0, 4.0]],
                                          [[3.0, 4.0, 5.0, 5.0], [3.0, 4.0, 5.0, 5.0]]])
    integral = f.integrate(X_BATCH, X_BATCH + 1.1)
    assert integral.dtype == dtype
    np.testing.assert_allclose(integral, [[[4.3, 4.4, 4.4, 5.5], [3.3, 4.4, 4.4, 4.5]],
                                          [[3.4, 4.5, 5.5, 5.5], [3.4, 4.5, 5.5, 5.5]]], atol=1e-5, rtol=1e-5)


@pytest.mark.parametrize("dtype", DTYPES + [None])
def test_value_with_batch_and_repetitions(dtype):
    # :111-136 (AutoDtype: the dtype of the jump locations)
    x = np.array([[-4.1, 0.1, 1.0, 2.0, 10, 11.0], [1.0, 2.0, 3.0, 2.0, 5.0, 9.0]], dtype=dtype or np.float32)
    jumps = np.array([[0.1, 0.1, 1.0, 1.0, 10.0, 10.0], [-1.0, 1.2, 2.2, 2.2, 2.2, 8.0]], dtype=dtype or np.float32)
    values = np.array([[3, 3, 4, 5, 5.0, 2, 6.0], [-1, -5, 2, 5, 5.0, 5.0, 1.0]], dtype=dtype or np.float32)
    f = PiecewiseConstantFunc(jumps, values, dtype=dtype)
    value = f(x, left_continuous=True)
    assert value.dtype == (dtype or jumps.dtype)
    np.testing.assert_array_equal(value, [[3.0, 3.0, 4.0, 5.0, 5.0, 6.0], [-5.0, 2.0, 5.0, 2.0, 5.0, 1.0]])


@pytest.mark.parametrize("dtype", DTYPES + [None])
def test_invalid_shapes(dtype):
    # :162-184
    jumps = np.array([[0.1, 10], [2.0, 10]])
    with pytest.raises(ValueError):  # batch shapes differ
        PiecewiseConstantFunc(jumps, np.array([[[3, 4, 5], [3, 4, 5]]]), dtype=dtype)
    with pytest.raises(ValueError):  # values not one longer than the jumps
        PiecewiseConstantFunc(jumps, np.array([[3, 4, 5, 6], [3, 4, 5, 7]]), dtype=dtype)


@pytest.mark.parametrize("dtype", DTYPES + [None])
def test_matrix_event_shape_no_batch_shape(dtype):
    # :186-215
    x = np.array([0.0, 0.1, 2.0, 11.0])
    f = PiecewiseConstantFunc([0.1, 10], [[[1, 2], [3, 4]], [[5, 6], [7, 8]], [[9, 10], [11, 12]]], dtype=dtype)
    assert f.dtype() == (dtype or np.float32)
    np.testing.assert_allclose(f(x), [[[1, 2], [3, 4]], [[1, 2], [3, 4]], [[5, 6], [7, 8]], [[9, 10], [11, 12]]],
                               atol=1e-5, rtol=1e-5)
    np.testing.assert_allclose(f.integrate(x, x + 1),
                               [[[4.6, 5.6], [6.6, 7.6]], [[5, 6], [7, 8]], [[5, 6], [7, 8]], [[9, 10], [11, 12]]],
                               atol=1e-5, rtol=1e-5)


@pytest.mark.parametrize("dtype", DTYPES + [None])
def test_3d_event_shape_with_batch_shape(dtype):
    # :217-285 (also the tf.function variant)
    x = np.array([[0, 1, 2, 3], [0.5, 1.5, 2.5, 3.5]])
    f = PiecewiseConstantFunc([[0.5, 2], [0.5, 1.5]],
                              [[[0, 1, 1.5], [2, 3, 0], [1, 0, 1]], [[0, 0.5, 1], [1, 3, 2], [2, 3, 1]]], dtype=dtype)
    np.testing.assert_allclose(f(x), [[[0, 1, 1.5], [2, 3, 0], [2, 3, 0], [1, 0, 1]],
                                      [[0, 0.5, 1], [1, 3, 2], [2, 3, 1], [2, 3, 1]]], atol=1e-5, rtol=1e-5)
    np.testing.assert_allclose(f.integrate(x, x + 1), [[[1, 2, 0.75], [2, 3, 0], [1, 0, 1], [1, 0, 1]],
                                                       [[1, 3, 2], [2, 3, 1], [2, 3, 1], [2, 3, 1]]],
                               atol=1e-5, rtol=1e-5)
