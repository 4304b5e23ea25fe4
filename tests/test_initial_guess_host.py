"""Extrapolation weights of the EXTRAP initial-guess strategy (host computation of the
library, no GPU) against the CPU restatement of Extrap::extrapCoeffs, and their defining
property: exact one step ahead for polynomials up to the degree."""
import numpy as np
import pytest

import libparanumal_gb300 as lpg
from oracle import initial_guess as ig


@pytest.mark.parametrize("cpqr", [False, True])
@pytest.mark.parametrize("m,M", [(0, 1), (1, 2), (1, 3), (2, 4), (2, 6), (3, 8), (4, 12)])
def test_extrap_coeffs_match_restatement(m, M, cpqr):
    c = lpg.extrap_coeffs(m, M, cpqr)
    ref = ig.extrap_coeffs(m, M, cpqr)
    assert np.allclose(c, ref, rtol=1e-11, atol=1e-11), (c, ref)
    t = np.arange(M, dtype=float)
    for p in range(m + 1):
        assert abs((c * t ** p).sum() - float(M) ** p) <= 1e-9 * max(1.0, float(M) ** p)
    if cpqr:
        assert int((np.abs(c) > 1e-14).sum()) <= m + 1


def test_extrap_coeffs_reject_short_history():
    with pytest.raises(lpg.LPGError):
        lpg.extrap_coeffs(3, 2)
