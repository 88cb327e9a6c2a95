"""Gauss-Legendre quadrature of the oracle (src/auxilliary/test_quadrature.hh:53-76):
(a+1)(b+1)(c+1) int x^a y^b z^c over [0,1]^3 equals 1 up to the rule's degree."""
import numpy as np
import pytest

import oracle as O


@pytest.mark.parametrize("order,maxdeg", [(0, 1), (1, 3), (2, 5)])
def test_quadrature_exact(order, maxdeg):
    w, p = O.quadrature(3, order)
    for a in range(maxdeg + 1):
        for b in range(maxdeg + 1):
            for c in range(maxdeg + 1):
                if order == 0 and (a, b, c) != (1, 1, 1):
                    continue
                val = (a + 1) * (b + 1) * (c + 1) * np.sum(w * p[:, 0] ** a * p[:, 1] ** b * p[:, 2] ** c)
                assert abs(val - 1.0) < 1e-12
