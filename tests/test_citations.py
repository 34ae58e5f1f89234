"""Every reference citation `path:line` or `path:first-last` in the boundary header, INTEGRATION.md and
the product and oracle sources names a file of the reference and lines inside it.

The reference checkout is read from the SHOCOVOX_REFERENCE environment variable (its root, holding
src/); the test is skipped where it is not set.  A citation's path may be shortened to its last
components (`insert.rs`, `update/mod.rs`): it then has to fit at least one reference file ending so.
"""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("SHOCOVOX_REFERENCE", "")
CITE = re.compile(r"((?:[A-Za-z0-9_.]+/)*[A-Za-z0-9_]+\.(?:rs|wgsl|toml)):(\d+)(?:-(\d+))?")
SOURCES = ["include/svo.h", "INTEGRATION.md"]


def _cited_files():
    out = list(SOURCES)
    for top in ("shocovox_gb300", "oracle"):
        for d, dirs, names in os.walk(os.path.join(ROOT, top)):
            dirs[:] = sorted(x for x in dirs if not x.startswith(("_", ".")))  # build output, caches
            out += sorted(os.path.relpath(os.path.join(d, n), ROOT) for n in names
                          if n.endswith((".h", ".cuh", ".cu", ".cpp", ".py")))
    return out


@pytest.fixture(scope="module")
def reference_lines():
    if not REF or not os.path.isdir(os.path.join(REF, "src")):
        pytest.skip("SHOCOVOX_REFERENCE does not point at a reference checkout")
    lines = {}
    for d, _, names in os.walk(REF):
        for n in names:
            if n.endswith((".rs", ".wgsl", ".toml")):
                p = os.path.join(d, n)
                with open(p, errors="replace") as f:
                    lines[os.path.relpath(p, REF)] = sum(1 for _ in f)
    return lines


@pytest.mark.parametrize("source", _cited_files())
def test_citations_exist(reference_lines, source):
    with open(os.path.join(ROOT, source), errors="replace") as f:
        text = f.read()
    bad = []
    for m in CITE.finditer(text):
        path, first = m.group(1), int(m.group(2))
        last = int(m.group(3)) if m.group(3) else first
        cands = [n for p, n in reference_lines.items() if p == path or p.endswith("/" + path)]
        if not cands or first < 1 or last < first or not any(last <= n for n in cands):
            bad.append(m.group(0))
    assert not bad, "%s cites lines that the reference does not have: %s" % (source, bad)
