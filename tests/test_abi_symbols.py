"""The C-ABI library loads without a GPU and exports every function the header declares."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "endobeams_gb300.h")


def declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(eb_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared()
    for must in ("eb_create", "eb_step", "eb_commit", "eb_rollback", "eb_destroy", "eb_element_eval",
                 "eb_contact_eval", "eb_contact_eval_noalloc"):
        assert must in names


def test_library_exports_every_declared_symbol(eb):
    from endobeams_gb300 import _lib
    lib = _lib.load()
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding covers every declared symbol
    assert set(declared()) <= set(_lib.SIGNATURES)


def test_library_has_no_cpu_compute_path(eb):
    """Without a usable GPU the compute entry points fail loudly instead of falling back."""
    import numpy as np
    import pytest
    from endobeams_gb300 import _lib
    n, _ = _lib.device_info()
    if n > 0:
        pytest.skip("a GPU is visible")
    with pytest.raises(_lib.EbError):
        eb.element_eval(np.zeros((1, 96)))
