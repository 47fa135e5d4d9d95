"""Every `file.rs:N-M` citation in the sources falls inside the cited file.

Docstrings and comments cite the Rust reference by file and line so that a
reader can check each restatement against it.  This test reads the
reference's sources (the checkout at WHIR_REFERENCE, default
/root/reference) and checks that each cited line lies within the cited
file; a bare file name may match several files (lib.rs, mod.rs, test.rs),
and then the longest of them bounds it.  Skipped where the reference is not
checked out.
"""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("WHIR_REFERENCE", "/root/reference")
SCANNED = ["include", "oracle", "whir_gb300", "tests", "bench.py", "__graft_entry__.py",
           "DESIGN.md", "INTEGRATION.md", "README.md"]
CITE = re.compile(r"([A-Za-z0-9_/]+\.rs):(\d+(?:-\d+)?(?:,\s?\d+(?:-\d+)?)*)")


def _reference_lengths():
    lengths = {}
    for d, _, files in os.walk(REF):
        for f in files:
            if f.endswith(".rs"):
                p = os.path.join(d, f)
                with open(p, errors="replace") as fh:
                    lengths[os.path.relpath(p, REF)] = sum(1 for _ in fh)
    return lengths


def _sources():
    for entry in SCANNED:
        path = os.path.join(ROOT, entry)
        if os.path.isfile(path):
            yield path
            continue
        for d, dirs, files in os.walk(path):
            dirs[:] = [x for x in dirs if x not in ("_build", "_lib", "__pycache__")]
            for f in files:
                if f.endswith((".py", ".c", ".h", ".cu", ".cuh", ".cpp", ".md")):
                    yield os.path.join(d, f)


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "crates")),
                    reason="reference sources not checked out here")
def test_every_citation_is_inside_its_file():
    lengths = _reference_lengths()
    bad, seen = [], 0
    for path in _sources():
        with open(path, errors="replace") as fh:
            for ln, line in enumerate(fh, 1):
                for m in CITE.finditer(line):
                    name, spans = m.group(1), m.group(2)
                    cands = [n for f, n in lengths.items() if ("/" + f).endswith("/" + name)]
                    where = f"{os.path.relpath(path, ROOT)}:{ln} {m.group(0)}"
                    if not cands:
                        bad.append(where + " (no such file)")
                        continue
                    longest = max(cands)
                    for span in spans.replace(" ", "").split(","):
                        ends = [int(x) for x in span.split("-")]
                        seen += 1
                        if max(ends) > longest or ends[0] < 1 or ends[0] > ends[-1]:
                            bad.append(f"{where} (file has {longest} lines)")
    assert seen > 200
    assert not bad, "\n".join(bad)
