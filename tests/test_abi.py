"""The C-ABI library builds for sm_103a and exports every entry point that
include/hitengpu.h declares (no GPU needed: nothing is called but hg_create,
which must fail cleanly without a device)."""
import ctypes
import os
import re

import pytest

from conftest import REPO


def _declared():
    src = open(os.path.join(REPO, "include", "hitengpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(hg_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    names = _declared()
    for n in ("hg_create", "hg_destroy", "hg_propagate_fixed", "hg_propagate_dop853", "hg_last_error_string"):
        assert n in names


def test_library_exports_all_declared_symbols():
    from hiten_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    for n in _declared():
        assert hasattr(lib, n), f"{n} declared in hitengpu.h but not exported"


def test_binding_covers_all_symbols():
    from hiten_gb300 import _lib
    assert sorted(_lib.EXPORTED) == _declared()


def test_create_without_device_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    from hiten_gb300 import _lib
    with pytest.raises(_lib.HitenGpuError):
        _lib.Handle(0)


def test_segmented_workspace_query():
    """Pure host arithmetic: 256-byte aligned sub-buffers, grows with N."""
    from hiten_gb300 import _lib
    L = _lib.load()
    assert L.hg_dop853_segmented_workspace_bytes(-1, 6, 0) == -1
    assert L.hg_dop853_segmented_workspace_bytes(10, 7, 0) == -1
    assert L.hg_dop853_segmented_workspace_bytes(10, 6, -1) == -1
    for dim in (6, 42):
        for hits in (0, 1, 8):
            prev = L.hg_dop853_segmented_workspace_bytes(0, dim, hits)
            assert prev > 0 and prev % 256 == 0
            for n in (1, 63, 64, 65, 16384, 1 << 20):
                b = L.hg_dop853_segmented_workspace_bytes(n, dim, hits)
                # lists and step-size state, plus one saved step (15 dim + 3
                # doubles, trajectory and hit index) per possible crossing
                assert b % 256 == 0 and b >= prev
                assert b >= n * (3 * 4 + 3 * 8) + n * hits * ((15 * dim + 3) * 8 + 8)
                prev = b


def test_integration_table_names_every_entry_point():
    """Every entry point of the header has a row (its reference counterpart or
    none) in the integration notes."""
    import re
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    hdr = open(os.path.join(root, "include", "hitengpu.h")).read()
    notes = open(os.path.join(root, "INTEGRATION.md")).read()
    names = sorted(set(re.findall(r"\b(hg_[a-z0-9_]+)\s*\(", hdr)))
    assert names
    assert [n for n in names if f"`{n}`" not in notes] == []
