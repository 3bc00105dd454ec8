"""Test infrastructure: every `path:line` or `path:first-last` citation of a
reference file in this repository's tracked files names a file of the
reference tree and lines inside it.

The reference tree is read where the oracle's Makefile reads it: $REF, or by
default a directory named `reference` beside this repository's root; without
it the check reports nothing to check.  Files that the build's review and
driver write (reviews, surveys, measurement records) quote this repository's
own paths and are not checked.
"""
from __future__ import annotations

import os
import re
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("REF") or os.path.join(os.path.dirname(ROOT), "reference")
# written outside the product by the review and measurement steps
NOT_CHECKED = {"SURVEY.md", "VERDICT.md", "ADVICE.md"}
_CITE = re.compile(r"((?:src|include|tools|test|training_pipeline)/[A-Za-z0-9_./-]+"
                   r"\.(?:c|h|cu|cpp|py|md)):(\d+)(?:-(\d+))?")


def reference_present() -> bool:
    return os.path.isdir(os.path.join(REF, "src"))


def bad_citations() -> list[tuple[str, str, str]]:
    """(file, citation, problem) for every citation that does not resolve."""
    files = subprocess.run(["git", "ls-files"], cwd=ROOT, capture_output=True, text=True,
                           check=True).stdout.split()
    lengths: dict[str, int] = {}
    bad = []
    for f in files:
        if f.endswith((".json", ".so")) or f in NOT_CHECKED:
            continue
        try:
            text = open(os.path.join(ROOT, f), encoding="utf-8").read()
        except (OSError, UnicodeDecodeError):
            continue
        for m in _CITE.finditer(text):
            path, a, b = m.group(1), int(m.group(2)), m.group(3)
            full = os.path.join(REF, path)
            if not os.path.isfile(full):
                bad.append((f, path, "no such reference file"))
                continue
            if path not in lengths:
                with open(full, errors="replace") as fh:
                    lengths[path] = sum(1 for _ in fh)
            last = int(b) if b else a
            if a < 1 or last < a or last > lengths[path]:
                bad.append((f, m.group(0), f"the file has {lengths[path]} lines"))
    return bad


if __name__ == "__main__":
    for row in bad_citations():
        print(*row)
