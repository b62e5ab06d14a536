"""Every file:line citation of the reference in this repository points inside
the cited file.

Citations have the form ``Name.ext:N``, ``Name.ext:N-M`` or lists of those
(``Name.ext:N-M,P``); the cited file is named by its base name.  The line
counts come from tests/golden/reference_lines.json (written by
``make_golden.py lines`` from the reference checkout), so the range check
runs anywhere.  Where the checkout is present (PHYBS_REFERENCE), citations
written as ``function (File:N...)`` are also checked to land on that
function: its name must appear within two lines of the first cited line.
"""
import json
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LINES = os.path.join(ROOT, "tests", "golden", "reference_lines.json")
# files of the build that quote the reference's line numbers but are not
# this repository's own text
SKIP_FILES = {"VERDICT.md", "ADVICE.md", "SURVEY.md", "BASELINE.md"}
SKIP_DIRS = {".git", "_work", "gpurun_out", "_build", "_ref", "__pycache__", ".pytest_cache", "baseline"}
TEXT_EXT = (".py", ".cu", ".cuh", ".h", ".hpp", ".cpp", ".c", ".md", ".txt")

CITE = re.compile(r"\b([A-Za-z_][A-Za-z_0-9]*\.(?:cpp|cu|cuh|h|hpp)):(\d+(?:-\d+)?(?:,\s?\d+(?:-\d+)?)*)")
NAMED = re.compile(r"\b(?:[A-Za-z_][A-Za-z_0-9]*::)?([A-Za-z_][A-Za-z_0-9]*)\s*\(\s*`?(?:FVM/)?"
                   r"([A-Za-z_][A-Za-z_0-9]*\.(?:cpp|cu|cuh|h|hpp)):(\d+(?:-\d+)?(?:,\s?\d+(?:-\d+)?)*)")


def _ranges(spec):
    for part in spec.split(","):
        a, _, b = part.strip().partition("-")
        yield int(a), int(b) if b else int(a)


def _files():
    for dp, dn, fn in os.walk(ROOT):
        dn[:] = [d for d in dn if d not in SKIP_DIRS]
        for f in fn:
            if f.endswith(TEXT_EXT) and not (dp == ROOT and f in SKIP_FILES):
                yield os.path.join(dp, f)


def _citations():
    counts = json.load(open(LINES))
    out = []
    for path in _files():
        try:
            text = open(path, encoding="utf-8").read()
        except UnicodeDecodeError:
            continue
        for ln, line in enumerate(text.splitlines(), 1):
            for m in CITE.finditer(line):
                if m.group(1) not in counts:
                    continue  # a file of this repository, or not a reference source
                for a, b in _ranges(m.group(2)):
                    out.append((os.path.relpath(path, ROOT), ln, m.group(1), a, b))
    return counts, out


def test_citations_lie_inside_the_reference_files():
    counts, cites = _citations()
    assert len(cites) > 100  # the scan found the repository's citations
    bad = [c for c in cites if not (1 <= c[3] <= c[4] <= counts[c[2]])]
    assert not bad, "citations outside the cited file:\n" + "\n".join(
        f"{p}:{ln}: {f}:{a}-{b} (file has {counts[f]} lines)" for p, ln, f, a, b in bad)


def test_named_citations_land_on_the_function():
    tree = os.environ.get("PHYBS_REFERENCE")
    if not tree or not os.path.isdir(os.path.join(tree, "FVM")):
        pytest.skip("the reference checkout (PHYBS_REFERENCE) is not present")
    src = {}
    for sub in ("FVM", os.path.join("3rd", "CUDA_helper")):
        for f in os.listdir(os.path.join(tree, sub)):
            src.setdefault(f, os.path.join(tree, sub, f))
    bad, n = [], 0
    for path in _files():
        try:
            text = open(path, encoding="utf-8").read()
        except UnicodeDecodeError:
            continue
        for ln, line in enumerate(text.splitlines(), 1):
            for m in NAMED.finditer(line):
                name, f = m.group(1), m.group(2)
                # function names only: camelCase or snake_case identifiers
                if f not in src or not re.search(r"[A-Z_]", name[1:]):
                    continue
                lines = open(src[f], errors="replace").read().splitlines()
                pat = re.compile(r"\b" + re.escape(name) + r"\b")
                # the name within one of the cited ranges (its definition may
                # sit up to two lines above a range that starts at the body)
                if not any(pat.search("\n".join(lines[max(0, a - 3):b])) for a, b in _ranges(m.group(3))):
                    # only names that the reference defines somewhere are claims about it
                    if re.search(r"\b" + re.escape(name) + r"\s*\(", "\n".join(lines)):
                        bad.append(f"{os.path.relpath(path, ROOT)}:{ln}: {name} ({f}:{m.group(3)})")
                n += 1
    assert n > 10
    assert not bad, "citations that miss the named function:\n" + "\n".join(bad)
