"""The C-ABI library loads, exports every entry point of include/mpdo_gb300.h
and fails loudly (no CPU fallback) where no GPU is present.  No device
compute; the engine's host-side truncation rule is checked against the
oracle's."""
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _declared():
    hdr = (ROOT / 'include' / 'mpdo_gb300.h').read_text()
    return sorted(set(re.findall(r'^\s*(?:mpdo_status|int|const char \*)\s*(mpdo_\w+)\s*\(', hdr, re.M)))


@pytest.fixture(scope='module')
def lib():
    from mpdo_gb300 import _build, _lib
    try:
        _build.build()
    except RuntimeError as e:  # pragma: no cover - toolchain missing
        pytest.skip(str(e))
    return _lib.load()


def test_header_declares_entry_points():
    names = _declared()
    for n in ('mpdo_engine_create', 'mpdo_apply_1q', 'mpdo_apply_2q', 'mpdo_truncate', 'mpdo_reduced_dm',
              'mpdo_expect_pauli_batch'):
        assert n in names


def test_exports_every_declared_symbol(lib):
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_signatures_cover_header(lib):
    from mpdo_gb300._lib import SIGNATURES
    assert set(_declared()) <= set(SIGNATURES), set(_declared()) - set(SIGNATURES)


def test_abi_version(lib):
    assert lib.mpdo_abi_version() == 1


def test_no_device_fails_loudly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip('GPU present')
    from mpdo_gb300 import Engine
    from mpdo_gb300._lib import MPDOError
    with pytest.raises(MPDOError, match='no CUDA device'):
        Engine(0)


def test_status_codes_map_to_reference_exceptions(lib):
    # the reference raises torch.linalg.LinAlgError when its SVD fails
    # (Circuit.py:127-136) and ValueError on bad arguments
    import torch
    from mpdo_gb300 import _lib
    cases = [(_lib.MPDO_ERR_INVALID, ValueError), (_lib.MPDO_ERR_BAD_SHAPE, ValueError),
             (_lib.MPDO_ERR_NOT_CONVERGED, torch.linalg.LinAlgError), (_lib.MPDO_ERR_NONFINITE, torch.linalg.LinAlgError),
             (_lib.MPDO_ERR_OOM, MemoryError), (_lib.MPDO_ERR_CUDA, _lib.MPDOError),
             (_lib.MPDO_ERR_NO_DEVICE, _lib.MPDOError)]
    for status, exc in cases:
        with pytest.raises(exc):
            _lib.check(status)
        assert lib.mpdo_status_string(status)
    _lib.check(_lib.MPDO_OK)


def test_batch_arguments_checked_before_any_device_work(lib):
    import ctypes as C
    from mpdo_gb300 import _lib
    h = C.c_void_p()
    assert lib.mpdo_batch_create(0, 0, C.byref(h)) == _lib.MPDO_ERR_INVALID
    assert b'workers' in lib.mpdo_last_error()
    assert lib.mpdo_batch_run(None, 1, None, None, None, None) == _lib.MPDO_ERR_INVALID
    assert lib.mpdo_batch_error(None, 0) == b''


def test_engine_truncation_rule_matches_the_oracle(lib):
    # decompositions.py:121-140 as the engine applies it on the host (split
    # cutoff and sweep error rule) against the oracle's keep_count, on random
    # graded spectra, with zero-extended spectra (nsv > len), exact ties at
    # the cut and caps; needs no device
    import ctypes as C

    import numpy as np
    import torch

    from oracle import mpdo_oracle as O
    rng = np.random.default_rng(0)
    out = C.c_int()
    cases = 0
    for trial in range(400):
        ln = int(rng.integers(1, 40))
        s = np.sort(np.exp(rng.uniform(-25, 0, ln)))[::-1].copy()
        if trial % 7 == 0:
            s[ln // 2:] = 0.0
        if trial % 11 == 0 and ln > 3:
            s[1:3] = s[1]
        nsv = ln + int(rng.integers(0, 5))
        for max_sv in (nsv, max(1, ln // 2), 1):
            for err, rel in ((-1.0, 0), (2.718281828459045e-8, 0), (1e-3, 1), (1e-7, 1), (0.5, 1)):
                assert lib.mpdo_keep_count(s.ctypes.data_as(C.POINTER(C.c_double)), ln, nsv, max_sv, err, rel,
                                           C.byref(out)) == 0
                full = torch.from_numpy(np.concatenate([s, np.zeros(nsv - ln)]))
                want = O.keep_count(full, max_sv, None if err < 0 else err, bool(rel))
                assert out.value == want, (trial, ln, nsv, max_sv, err, rel, out.value, want)
                cases += 1
    assert cases == 400 * 15
