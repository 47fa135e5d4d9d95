"""The C-ABI libraries load and export every symbol their headers declare.

No compute calls: this runs on a machine without a GPU.
"""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header, prefix):
    text = open(header).read()
    return sorted(set(re.findall(r"\b(%s\w+)\s*\(" % prefix, text)))


def test_product_library_exports_header():
    import whir_gb300 as W
    lib = ctypes.CDLL(W.lib_path())
    names = declared(os.path.join(ROOT, "include", "whir_gb300.h"), "whir_")
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_oracle_library_exports_header(oracle):
    lib = ctypes.CDLL(oracle.LIB_PATH)
    names = declared(os.path.join(ROOT, "oracle", "whir_oracle.h"), "wo_")
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_product_does_not_link_the_oracle():
    import subprocess
    import whir_gb300 as W
    out = subprocess.run(["nm", "-D", W.lib_path()], capture_output=True, text=True).stdout
    assert " wo_" not in out and "whir_oracle" not in out


def test_every_entry_point_has_a_ctypes_signature():
    # a function called without argtypes passes pointers as 32-bit ints
    import re
    import whir_gb300 as W
    header = open(os.path.join(ROOT, "include", "whir_gb300.h")).read()
    declared = set(re.findall(r"WHIR_API\s+[\w\s\*]+?\b(whir_\w+)\s*\(", header))
    # the allocation-free entry point is bound by its own test with its signature
    missing = declared - set(W._SIGS) - {"whir_compress_hi_noalloc"}
    assert not missing, sorted(missing)


def test_batch_limits_follow_the_dft_indexing():
    # a lock-step group's batched codewords must fit the DFT's 2^16-word rows
    # and 32-bit word indexing (no GPU needed: parameter arithmetic only)
    import whir_gb300 as W
    assert W.batch_max((16, 4, 2, 1, 1, 100)) == 1023   # extension rows of 64 words
    assert W.batch_max((22, 4, 2, 1, 1, 100)) == 127    # round 0: 2^19 rows x 64 words
    assert W.batch_max((10, 4, 1, 1, 1, 100)) == 1024   # no extension round
    assert W.batch_max((24, 4, 2, 1, 1, 100)) >= 1
    with pytest.raises(W.WhirError):
        W.batch_max((3, 4, 1, 1, 1, 100))               # k below the folding
