"""Statistics (src/auxilliary/test_statistics.hh:35-166): running mean,
covariance, autocovariance and tau_int on the AR(1) process
Q_n = A Q_{n-1} + xi + v with known moments."""
import numpy as np
import pytest

import oracle as O


@pytest.fixture(scope="module")
def ar1():
    theta = 1.3
    rot = np.array([[np.cos(theta), np.sin(theta)], [-np.sin(theta), np.cos(theta)]])
    A = rot @ np.diag([0.6, 0.4]) @ rot.T
    v = np.array([1.4, 0.6])
    rng = np.random.default_rng(1241517)
    # run the recurrence in the eigenbasis of the symmetric A, where it
    # decouples into two scalar AR(1) filters
    d, R = np.linalg.eigh(A)
    nwarm, n = 1000, 2000000
    e = rng.standard_normal((nwarm + n, 2)) + v
    P = lfilter_ar1(e @ R, d)
    return A, v, (P @ R.T)[nwarm:]


def lfilter_ar1(u, d):
    from scipy.signal import lfilter
    out = np.empty_like(u)
    for j in range(u.shape[1]):
        out[:, j] = lfilter([1.0], [1.0, -d[j]], u[:, j])
    return out


def test_average_covariance(ar1):
    A, v, Q = ar1
    st = O.Statistics(2, 10)
    st.record(Q)
    assert np.linalg.norm(st.average() - np.linalg.solve(np.eye(2) - A, v)) < 3e-3
    assert np.linalg.norm(st.covariance() - np.linalg.inv(np.eye(2) - A @ A)) < 3e-3


def test_autocovariance(ar1):
    A, v, Q = ar1
    window = 6
    st = O.Statistics(2, window)
    st.record(Q)
    ac = st.auto_covariance(window)
    C = np.linalg.inv(np.eye(2) - A @ A)
    diff = 0.0
    for k in range(window):
        diff += np.linalg.norm(ac[k] - C)
        C = C @ A
    assert diff < 2e-2


def test_tau_int(ar1):
    A, v, Q = ar1
    window = 20
    st = O.Statistics(2, window)
    st.record(Q)
    vv = np.array([0.8, 0.0])  # the reference test sets v(0) twice
    w = np.linalg.inv(np.eye(2) - A @ A) @ vv
    wk = w.copy()
    tau = 1.0
    for k in range(1, window):
        wk = A @ wk
        tau += 2.0 * (1.0 - k / window) * vv @ wk / (vv @ w)
    assert abs(st.tau_int(vv) - tau) < 2e-2
