"""The C-ABI library loads on a host without a GPU and exports the header's symbols."""
import numpy as np
import pytest

from aurora_gb300 import api


def test_library_exports_every_declared_symbol(built):
    L = api.lib()
    names = api.exported_symbols()
    assert len(names) >= 29
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert b"sm_103a" in L.aur_version()


def _subtree(k, n):
    s, f, w = 0, k, 1
    while f < n:
        s += min(w, n - f)
        f, w = 2 * f + 1, 2 * w
    return s


def test_nmh_layout_closed_forms(built):
    for n in list(range(1, 300)) + [1023, 1024, 1025, 5000]:
        ks = range(n) if n < 300 else range(0, n, 7)
        for k in ks:
            lv = (k + 1).bit_length() - 1
            L0 = (1 << lv) - 1
            start = 2 * sum(_subtree(q, n) for q in range(L0, k))
            numl = 2 * _subtree(2 * k + 1, n) if 2 * k + 1 < n else 0
            lbase = 2 * sum(_subtree(2 * q + 1, n) if 2 * q + 1 < n else 0 for q in range(L0, k))
            assert api.debug_nmh_layout(n, k) == (start, numl, lbase)


def test_errors_are_reported(built):
    with pytest.raises(api.AuroraError):
        api.debug_nmh_layout(4, 9)
    msg = api.lib().aur_last_error().decode()
    assert "k >= n" in msg
