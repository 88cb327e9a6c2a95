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


@pytest.mark.parametrize("rho,n,mu,window", [(0.3, 20000, 0.5, 50), (0.9, 100000, -2.0, 200), (0.0, 1000, 0.0, 10),
                                             (0.6, 5000, 3.0, 20)])
def test_library_tau_int_equals_oracle_statistics(rho, n, mu, window):
    """multigridmc_gb300.statistics.tau_int (the IACT estimator of the
    benchmark) equals the oracle's Statistics::tau_int (statistics.cc:65-79,
    pinned on AR(1) above) on the same scalar series, to 1e-12 relative."""
    from scipy.signal import lfilter
    import multigridmc_gb300 as M
    q = lfilter([1.0], [1.0, -rho], np.random.default_rng(5).standard_normal(n)) + mu
    st = O.Statistics(1, window)
    st.record(q)
    want = st.tau_int(np.array([1.0]))
    got = M.statistics.tau_int(q, window)
    assert abs(got - want) <= 1e-12 * abs(want)


def test_library_tau_int_on_an_mgmc_chain():
    """The same comparison on the observable b^T x of the oracle's MGMC chain
    (2D 32^2 prior, 4 levels, CLCG noise) with the benchmark's window 50."""
    import multigridmc_gb300 as M
    op = O.Operator.fd([32, 32], 10.0)
    s = O.mgmc_sampler(op, O.Source(), 4)
    bidx, bval = O.measurement_vector([32, 32], [0.5, 0.5], 0.1)
    x = np.zeros(op.n)
    z = s.observe(np.zeros(op.n), x, 3000, bidx, bval)
    st = O.Statistics(1, 50)
    st.record(z)
    want = st.tau_int(np.array([1.0]))
    assert abs(M.statistics.tau_int(z, 50) - want) <= 1e-12 * abs(want)
