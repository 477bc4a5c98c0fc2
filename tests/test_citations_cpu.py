"""Every `File.jl:N` citation in the sources and notes points inside the cited reference file, and every
`function_name! (File.jl:a-b)` citation names a function that appears in those lines.

Reads the reference's Julia sources from HCC_REFERENCE_DIR (default /root/reference); skipped where they are absent.
"""
import os
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
REF = Path(os.environ.get("HCC_REFERENCE_DIR", "/root/reference"))
SCANNED = ["hypercloudcore.jl_gb300", "oracle", "include", "tests", "bench.py", "__graft_entry__.py", "DESIGN.md",
           "INTEGRATION.md", "README.md"]
SUFFIXES = {".cu", ".cuh", ".h", ".cpp", ".py", ".jl", ".md"}

# `NeighborLogic.jl:22-40` or `src/Grid/NeighborLogic.jl:22-40,:43-76`
CITE = re.compile(r"((?:[\w]+/)*)(\w+\.jl)((?::\d+(?:-\d+)?)(?:\s*,\s*:\d+(?:-\d+)?)*)")
# `_write_neighbours! (NeighborLogic.jl:309-329)`: an identifier with a bang or a leading underscore
NAMED = re.compile(r"(?<![\w])`?((?:_\w+|\w+!))`?\s*\(`?(?:[\w]+/)*(\w+\.jl):(\d+)(?:-(\d+))?")


def _reference_files():
    out = {}
    for p in REF.rglob("*.jl"):
        if "reviews" in p.parts:
            continue
        out.setdefault(p.name, []).append(p.read_text(errors="replace").splitlines())
    return out


def _scanned_lines():
    for entry in SCANNED:
        root = ROOT / entry
        paths = [root] if root.is_file() else sorted(root.rglob("*"))
        for f in paths:
            if f.is_file() and f.suffix in SUFFIXES and "_build" not in f.parts:
                for no, line in enumerate(f.read_text(errors="replace").splitlines(), 1):
                    yield f.relative_to(ROOT), no, line


@pytest.fixture(scope="module")
def ref_files():
    if not (REF / "src").is_dir():
        pytest.skip("reference sources not present")
    return _reference_files()


def test_citations_inside_cited_files(ref_files):
    bad = []
    for f, no, line in _scanned_lines():
        for m in CITE.finditer(line):
            texts = ref_files.get(m.group(2))
            if texts is None:
                continue            # a file of this repository or of a third party
            longest = max(len(t) for t in texts)
            for a, b in re.findall(r":(\d+)(?:-(\d+))?", m.group(3)):
                lo, hi = int(a), int(b or a)
                if lo < 1 or hi < lo or hi > longest:
                    bad.append(f"{f}:{no}: {m.group(0)} (the file has {longest} lines)")
    assert not bad, "citations outside the cited file:\n" + "\n".join(bad)


def test_named_citations_point_at_the_function(ref_files):
    bad = []
    for f, no, line in _scanned_lines():
        for m in NAMED.finditer(line):
            name, fname, a, b = m.groups()
            texts = ref_files.get(fname)
            if texts is None:
                continue
            lo, hi = int(a), int(b or a)
            if not any(name in "\n".join(t[lo - 1:hi]) for t in texts):
                bad.append(f"{f}:{no}: {m.group(0)}")
    assert not bad, "cited names not found in the cited lines:\n" + "\n".join(bad)
