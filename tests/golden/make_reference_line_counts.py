"""Writes reference_line_counts.json: the line count of every source file of etano/simpimc, keyed
by its path inside that project. tests/test_citations.py checks every file:line citation in this
repository against it, so the test runs where the reference checkout is absent.

Usage: python tests/golden/make_reference_line_counts.py [/root/reference]
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SUFFIXES = (".h", ".cc", ".cpp", ".py", ".xml", ".txt", ".cmake", ".rst", ".yml", ".sh", ".md")


def counts(root):
    out = {}
    for dp, dn, fn in os.walk(root):
        dn[:] = [d for d in dn if d != ".git"]
        for f in fn:
            if f.endswith(SUFFIXES) or f == "Makefile":
                p = os.path.join(dp, f)
                with open(p, errors="ignore") as fh:
                    out[os.path.relpath(p, root)] = sum(1 for _ in fh)
    return dict(sorted(out.items()))


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    with open(os.path.join(HERE, "reference_line_counts.json"), "w") as fh:
        json.dump(counts(root), fh, indent=0)
        fh.write("\n")
