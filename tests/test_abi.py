"""The C-ABI libraries load and export every symbol their headers declare.

No compute calls: this runs on a machine without a GPU.
"""
import ctypes
import os
import re

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
