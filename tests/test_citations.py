"""Every reference citation `name.F:line` / `name.F:a-b` (also `.inc`) in the
tracked files must point at lines that exist in the MOLFDIR source tree.

A citation may carry a directory prefix (`rotran/trout.F:30`,
`source/reltwel/wrbuf.F:38`); without one, the base name must be unique in
the tree or, when several directories hold a file of that name, the
rotran one is meant (the path this library replaces).  Skipped where the
reference tree is absent."""

from __future__ import annotations

import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("MOLFDIR_REFERENCE", "/root/reference")
CITE = re.compile(r"(?<![\w/.-])((?:[\w.-]+/)*)([A-Za-z]\w*(?:\.par)?\.(?:F|inc|f|c)):(\d+)(?:-(\d+))?")


def _tree():
    files = {}
    for d, _, fs in os.walk(os.path.join(REF, "source")):
        for f in fs:
            if f.endswith((".F", ".inc", ".f", ".c")):
                files.setdefault(f, []).append(os.path.join(d, f))
    return files


def _nlines(path, cache={}):
    if path not in cache:
        with open(path, "rb") as fh:
            cache[path] = fh.read().count(b"\n")
    return cache[path]


def _resolve(prefix, name, files):
    cands = files.get(name, [])
    if prefix:
        pre = prefix.rstrip("/")
        if pre.startswith("source/"):
            pre = pre[len("source/"):]
        cands = [c for c in cands if os.path.dirname(c).endswith(os.sep + pre)]
    elif len(cands) > 1:
        rot = [c for c in cands if os.path.basename(os.path.dirname(c)) == "rotran"]
        cands = rot or cands
    return cands


def citations():
    out = subprocess.run(["git", "ls-files"], cwd=ROOT, capture_output=True, text=True).stdout.split()
    skip = ("VERDICT.md", "ADVICE.md", "SURVEY.md", "BASELINE.md")
    for rel in out:
        if rel.endswith(skip) or rel.endswith((".npz", ".json", ".jsonl")):
            continue
        path = os.path.join(ROOT, rel)
        try:
            text = open(path, encoding="utf-8").read()
        except (UnicodeDecodeError, OSError):
            continue
        for ln, line in enumerate(text.splitlines(), 1):
            for m in CITE.finditer(line):
                yield rel, ln, m.group(1), m.group(2), int(m.group(3)), int(m.group(4) or m.group(3))


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "source", "rotran")),
                    reason="MOLFDIR reference tree not present")
def test_reference_citations_resolve():
    files = _tree()
    bad = []
    n = 0
    for rel, ln, prefix, name, a, b in citations():
        cands = _resolve(prefix, name, files)
        if not cands:
            if name in ("rt_io.c", "rotran_oracle.c") or name.startswith(("rt_", "k_")):
                continue
            bad.append(f"{rel}:{ln}: {prefix}{name}:{a}-{b} (no such file)")
            continue
        n += 1
        if not any(1 <= a <= b <= _nlines(c) for c in cands):
            bad.append(f"{rel}:{ln}: {prefix}{name}:{a}-{b} (file has {_nlines(cands[0])} lines)")
    assert n > 50, "too few citations found: the pattern is broken"
    assert not bad, "citations past the end of the cited file:\n" + "\n".join(bad)
