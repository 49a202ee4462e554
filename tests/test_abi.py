"""C ABI and host-side logic (no GPU needed)."""

import re
from pathlib import Path

import numpy as np
import pytest

import giaoint_gb300 as gi
from giaoint_gb300 import _native as nat

HEADER = Path(__file__).resolve().parents[1] / "include" / "giao_gb300.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"\b(gx_[a-z0-9_]+)\s*\(", text)))


def test_library_loads_and_exports_every_declared_symbol():
    lib = nat.lib()
    names = declared_symbols()
    assert len(names) >= 18
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) == set(nat.SIGNATURES)


def test_shell_normalisation_matches_oracle(oracle):
    rng = np.random.default_rng(3)
    for l in range(5):
        exps = np.exp(rng.uniform(np.log(0.1), np.log(50), 4))
        coefs = rng.uniform(-1, 1, (2, 4))
        s = gi.Shell((0.1, 0.2, 0.3), l, exps, coefs)
        from oracle.oracle import ShellSpec

        expected = oracle.normalized_coefficients(ShellSpec((0.1, 0.2, 0.3), l, list(exps), coefs.tolist(), True))
        np.testing.assert_allclose(s.coefficients, expected, rtol=1e-14)
        assert s.ao_count == 2 * (l + 1) * (l + 2) // 2
    for l in range(4):
        for comp in gi.cartesian_components(l):
            assert gi.primitive_normalization(0.7, comp) == pytest.approx(oracle.primitive_normalization(0.7, comp),
                                                                          rel=1e-14)


def test_shell_and_field_validation_messages():
    with pytest.raises(ValueError, match="one- or two-dimensional"):
        gi.Shell((0, 0, 0), 0, [1.0], np.ones((1, 1, 1)))
    with pytest.raises(ValueError, match="final coefficient dimension"):
        gi.Shell((0, 0, 0), 0, [1.0, 2.0], [1.0])
    with pytest.raises(ValueError, match="finite and positive"):
        gi.Shell((0, 0, 0), 0, [-1.0], [1.0])
    with pytest.raises(ValueError, match="all-zero"):
        gi.Shell((0, 0, 0), 0, [1.0], [0.0])
    with pytest.raises(ValueError, match="length 3"):
        gi.MagneticField((0, 0))
    with pytest.raises(ValueError, match="finite"):
        gi.MagneticField((0, np.inf, 0))
    with pytest.raises(ValueError, match="normalize must be a bool"):
        gi.Shell((0, 0, 0), 0, [1.0], [1.0], normalize=1)
    assert gi.cartesian_components(2) == ((2, 0, 0), (1, 1, 0), (1, 0, 1), (0, 2, 0), (0, 1, 1), (0, 0, 2))


def test_api_validation_before_device_work():
    b = gi.Basis([gi.Shell((0, 0, 0), 0, [1.0], [1.0])])
    with pytest.raises(ValueError, match="storage must be"):
        gi.eri(b, storage="dense")
    with pytest.raises(ValueError, match="explicit max_bytes"):
        gi.eri(b, storage="full")
    with pytest.raises(MemoryError, match="requires 16 bytes"):
        gi.eri(b, storage="full", max_bytes=15)
    with pytest.raises(ValueError, match="target_bytes"):
        next(gi.eri_batches(b, target_bytes=0))
    with pytest.raises(IndexError, match="out of range"):
        next(gi.eri_batches(b, quartets=[(0, 0, 0, 1)]))
    with pytest.raises(ValueError, match="four indices"):
        next(gi.eri_batches(b, quartets=[(0, 0, 0)]))
    with pytest.raises(ValueError, match="positive integer"):
        gi.eri(b, threads=0)
    with pytest.raises(ValueError, match="pivot_batch_size"):
        gi.cholesky_eri(b, pivot_batch_size=0)
    with pytest.raises(ValueError, match="finite and non-negative"):
        gi.cholesky_eri(b, threshold=-1.0)
    with pytest.raises(ValueError, match="through 32"):
        gi.boys(1.0, 33)
    # the streaming entry point refuses a null consumer before it needs a device
    rc = nat.lib().gx_eri_for_each(None, None, None, None, None, 0, 0, 0.0, 0.0, nat.QUARTET_CONSUMER(), None, None)
    assert rc == -1 and "must not be null" in nat.last_error()
    consumer = nat.QUARTET_CONSUMER(lambda blk, user: 0)
    rc = nat.lib().gx_eri_for_each(None, None, None, None, None, 0, 0, 0.0, 0.0, consumer, None, None)
    assert rc == -1 and "null context or basis" in nat.last_error()
    # host-output copy modes: argument checks before any device work
    assert nat.lib().gx_context_set_copy_parts(None, 0, 0.0) == -1


def test_no_cpu_fallback_without_a_device():
    import ctypes

    handle = ctypes.c_void_p()
    rc = nat.lib().gx_context_create(0, ctypes.byref(handle))
    if rc == 0:
        nat.lib().gx_context_destroy(handle)
        pytest.skip("a CUDA device is present")
    with pytest.raises(RuntimeError, match="CUDA"):
        nat.check(rc)
