"""Reference citations stay inside the files they cite.

Every `name.jl:a-b` (or `name.md:a-b`) citation in the sources and design
notes must fall within the cited file of the reference checkout.  A citation
whose path does not name a test file refers to the package source (`src/`,
`docs/`), which resolves names shared by a source file and a test file.
The checkout is named by the NQCD_REFERENCE environment variable; the test
is skipped when the variable is unset or names no checkout.
"""
import collections
import os
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
REF = Path(os.environ["NQCD_REFERENCE"]) if os.environ.get("NQCD_REFERENCE") else None
CITE = re.compile(r"([\w./-]+\.(?:jl|md)):(\d+)(?:-(\d+))?((?:, ?\d+(?:-\d+)?)*)")


def _reference_files():
    files = collections.defaultdict(list)
    for d, _, names in os.walk(REF):
        for n in names:
            if n.endswith((".jl", ".md")):
                files[n].append(Path(d) / n)
    return files


def _sources():
    for sub in ("nqcdynamics.jl_gb300", "oracle", "tests", "include"):
        for p in (ROOT / sub).rglob("*"):
            if p.suffix in (".py", ".cu", ".cuh", ".h", ".cpp") and "_lib" not in p.parts and "__pycache__" not in p.parts:
                yield p
    for name in ("bench.py", "__graft_entry__.py", "DESIGN.md", "INTEGRATION.md", "README.md"):
        yield ROOT / name


@pytest.mark.skipif(REF is None or not (REF / "src").is_dir(), reason="NQCD_REFERENCE unset or not a checkout")
def test_reference_citations_are_in_range():
    files = _reference_files()
    nlines = {p: sum(1 for _ in open(p, errors="ignore")) for v in files.values() for p in v}
    bad = []
    for src in _sources():
        for ln, text in enumerate(open(src, errors="ignore"), 1):
            for m in CITE.finditer(text):
                name = os.path.basename(m.group(1))
                if name not in files:
                    continue
                cands = files[name]
                if len(cands) > 1:
                    sub = [c for c in cands if str(c).endswith(m.group(1).lstrip("./"))]
                    if len(sub) != 1:
                        want_test = "test/" in m.group(1)
                        sub = [c for c in (sub or cands) if ("/test/" in str(c)) == want_test] or cands
                    cands = sub
                nums = [int(m.group(2))] + ([int(m.group(3))] if m.group(3) else [])
                nums += [int(x) for x in re.findall(r"\d+", m.group(4) or "")]
                if max(nums) > max(nlines[c] for c in cands):
                    bad.append(f"{src.relative_to(ROOT)}:{ln}: {m.group(0)}")
    assert not bad, "\n".join(bad)
