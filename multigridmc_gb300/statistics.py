"""Integrated autocorrelation time of a scalar chain observable.

Restates Statistics::tau_int (src/auxilliary/statistics.cc:65-79) for a
scalar time series: with the lag-k autocovariance
C(k) = <Q_i Q_{i-k}> - <Q>^2 (the mean of Q_i Q_{i-k} over the N-k products,
statistics.cc:26-38 and 54-62),

    tau_int = 1 + 2 sum_{k=1}^{K-1} (1 - k/K) C(k) / C(0)

over a window of K lags.
"""
import numpy as np


def autocovariance(q, window):
    q = np.asarray(q, dtype=np.float64)
    n = len(q)
    if n < window + 1:
        raise ValueError(f"need more than {window} samples, got {n}")
    mean = q.mean()
    return np.array([np.mean(q[k:] * q[:n - k]) - mean * mean for k in range(window)])


def tau_int(q, window=50):
    C = autocovariance(q, window)
    k = np.arange(1, window)
    return float(1.0 + 2.0 * np.sum((1.0 - k / window) * C[1:] / C[0]))
