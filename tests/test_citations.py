"""Every reference citation in this repository points at lines that exist.

The C interface, the oracle and the kernels name the reference code they replace or restate as
`file:line` or `file:a-b` (paths inside etano/simpimc). This test parses every such citation in the
tracked sources and documents and checks that each cited line lies inside the cited file, using the
line counts in tests/golden/reference_line_counts.json (written by make_reference_line_counts.py
beside it). Where the reference checkout is present, the manifest itself is checked against it.
"""
import json
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MANIFEST = os.path.join(ROOT, "tests", "golden", "reference_line_counts.json")
# Of the documents, only this repository's own are checked; other parties' files are not its citations.
OWN_DOCS = ("DESIGN.md", "INTEGRATION.md", "README.md", "profiles/")
SKIP_PREFIX = ("tests/golden/",)
CITE = re.compile(r"([A-Za-z_][A-Za-z0-9_./-]*\.(?:h|cc|cpp|py|xml|cmake))(?::|\s+lines?\s+)(\d+)(?:\s*-\s*(\d+))?"
                  r"((?:\s*,\s*\d+(?:\s*-\s*\d+)?)*)")


def _manifest():
    with open(MANIFEST) as fh:
        return json.load(fh)


def _by_basename(counts):
    out = {}
    for path, n in counts.items():
        out.setdefault(os.path.basename(path), []).append((path, n))
    return out


def _tracked():
    try:
        out = subprocess.check_output(["git", "ls-files"], cwd=ROOT, text=True)
        return [f for f in out.split()
                if not f.startswith(SKIP_PREFIX) and not f.endswith(".json") and (not f.endswith(".md") or f.startswith(OWN_DOCS))]
    except Exception:
        pytest.skip("not a git checkout")


def citations(text, by_name):
    """(line number, citation text, cited numbers, candidate files) for every citation of a
    reference file in `text`."""
    for ln, line in enumerate(text.splitlines(), 1):
        for m in CITE.finditer(line):
            name = os.path.basename(m.group(1))
            if name not in by_name:
                continue
            cands = by_name[name]
            if "/" in m.group(1):  # a path: keep the files whose path ends with it
                narrowed = [c for c in cands if c[0].endswith(m.group(1).lstrip("./"))]
                cands = narrowed or cands
            nums = [int(m.group(2))] + ([int(m.group(3))] if m.group(3) else [])
            nums += [int(x) for x in re.findall(r"\d+", m.group(4) or "")]
            yield ln, m.group(0), nums, cands


def test_manifest_matches_reference_checkout():
    ref = "/root/reference"
    if not os.path.isdir(os.path.join(ref, "src")):
        pytest.skip("reference checkout absent")
    import importlib.util
    spec = importlib.util.spec_from_file_location("mk", os.path.join(ROOT, "tests", "golden", "make_reference_line_counts.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    assert mk.counts(ref) == _manifest()


def test_every_citation_is_inside_its_file():
    by_name = _by_basename(_manifest())
    bad, seen = [], 0
    for rel in _tracked():
        try:
            with open(os.path.join(ROOT, rel), encoding="utf-8") as fh:
                text = fh.read()
        except (UnicodeDecodeError, FileNotFoundError, IsADirectoryError):
            continue
        for ln, cite, nums, cands in citations(text, by_name):
            seen += 1
            if all(max(nums) > n or min(nums) < 1 for _, n in cands):
                bad.append(f"{rel}:{ln}: {cite} (file lengths {[n for _, n in cands]})")
            if len(nums) == 2 and nums[1] < nums[0] and "," not in cite:
                bad.append(f"{rel}:{ln}: {cite} (reversed range)")
    assert seen > 200, seen  # the parser still finds the citations
    assert not bad, "\n".join(bad)
