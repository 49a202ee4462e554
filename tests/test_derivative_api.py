"""Host-side validation of the derivative API (eri_derivative_batches,
_eri_derivative_batch, eri_derivative_contraction): every error is raised
before any device work, with the reference's messages
(python/giao_integrals/eri.py:220-284, derivative_assembly.py:14-148)."""

from __future__ import annotations

import numpy as np
import pytest

import giaoint_gb300 as gi
from giaoint_gb300.eri import _eri_derivative_batch


def _basis():
    return gi.Basis([gi.Shell((0.1, -0.2, 0.3), 0, [0.8, 1.2], [0.7, -0.2]),
                     gi.Shell((-0.3, 0.4, 0.2), 1, [0.6], [1.0])])


@pytest.mark.parametrize("bad", [0, -1, True, 1.5])
def test_invalid_target_bytes(bad):
    with pytest.raises(ValueError, match="target_bytes"):
        list(gi.eri_derivative_batches(_basis(), target_bytes=bad))


@pytest.mark.parametrize("bad", [-1.0, float("nan"), float("inf")])
def test_invalid_screening(bad):
    with pytest.raises(ValueError, match="screening_threshold"):
        list(gi.eri_derivative_batches(_basis(), screening_threshold=bad))


def test_empty_and_invalid_quartets():
    assert list(gi.eri_derivative_batches(gi.Basis([]))) == []
    assert list(gi.eri_derivative_batches(_basis(), quartets=[])) == []
    with pytest.raises(IndexError):
        list(gi.eri_derivative_batches(_basis(), quartets=[(0, 0, 0, 9)]))
    for bad in [(0, 0, 0, True), (0, 0, 0, 0.5)]:
        with pytest.raises(ValueError):
            list(gi.eri_derivative_batches(_basis(), quartets=[bad]))
    with pytest.raises(ValueError, match="requires derivative bounds"):
        _eri_derivative_batch(_basis(), [(0, 0, 0, 0)], screening_threshold=1e-8)
    with pytest.raises(ValueError, match="finite and non-negative"):
        _eri_derivative_batch(_basis(), [(0, 0, 0, 0)], screening_threshold=-1.0)


def test_contraction_validation():
    b = _basis()
    n = b.ao_count
    P = np.zeros((n, n), dtype=np.complex128)
    with pytest.raises(ValueError, match="at least one density"):
        gi.eri_derivative_contraction(b, [0, 1], 2)
    with pytest.raises(ValueError, match="shell_atoms"):
        gi.eri_derivative_contraction(b, [0], 2, coulomb_pairs=[(P, P)])
    with pytest.raises(ValueError, match="shell_atoms"):
        gi.eri_derivative_contraction(b, [0, 2], 2, coulomb_pairs=[(P, P)])
    with pytest.raises(ValueError, match="integers"):
        gi.eri_derivative_contraction(b, [0, 1], True, coulomb_pairs=[(P, P)])
    with pytest.raises(ValueError, match="P and Q"):
        gi.eri_derivative_contraction(b, [0, 1], 2, coulomb_pairs=[(P,)])
    with pytest.raises(ValueError, match="shape"):
        gi.eri_derivative_contraction(b, [0, 1], 2, exchange_pairs=[(P[:2], P)])
    with pytest.raises(ValueError, match="gamma"):
        gi.eri_derivative_contraction(b, [0, 1], 2, gamma=np.zeros((n, n, n, n), dtype=np.float32))
    with pytest.raises(ValueError, match="out must be"):
        gi.eri_derivative_contraction(b, [0, 1], 2, coulomb_pairs=[(P, P)], out=np.zeros((2, 2), np.complex128))
    with pytest.raises(ValueError, match="target_bytes"):
        gi.eri_derivative_contraction(b, [0, 1], 2, coulomb_pairs=[(P, P)], target_bytes=0)
