"""Every `file:line` citation of the reference in the sources resolves.

Scans the headers, kernels, host code, oracle, tests, bench and the design
documents for citations such as `shader/src/NN_nv.glsl:178-196` or
`src/VkNRCState.cpp:25-31, 39-44`, and checks each cited file exists in the
reference tree and each cited line lies within it. A citation by bare file name
(`NRCRecord.glsl:47-49`) resolves when exactly one file of that name exists,
or to the one under shader/src/.
Skipped when the reference tree is not present (REF_DIR, default
/root/reference).
"""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("REF_DIR", "/root/reference")
EXTS = ("glsl", "comp", "frag", "vert", "cpp", "hpp", "h", "txt", "md")
CITE = re.compile(
    r"(?<![\w/.-])((?:[\w.-]+/)*[\w.-]+\.(?:%s)):(\d+(?:-\d+)?(?:,\s?\d+(?:-\d+)?)*)" % "|".join(EXTS)
)
SCAN_DIRS = ["include", "vknrc_gb300", "oracle", "tests"]
SCAN_FILES = ["bench.py", "__graft_entry__.py", "DESIGN.md", "INTEGRATION.md", "README.md"]
SCAN_EXT = (".h", ".cu", ".cuh", ".c", ".cpp", ".py", ".sh", ".md")


def _sources():
    for d in SCAN_DIRS:
        for base, dirs, files in os.walk(os.path.join(ROOT, d)):
            dirs[:] = [x for x in dirs if not x.startswith(("_", "."))]
            for f in files:
                if f.endswith(SCAN_EXT) and f != os.path.basename(__file__):
                    yield os.path.join(base, f)
    for f in SCAN_FILES:
        p = os.path.join(ROOT, f)
        if os.path.exists(p):
            yield p


def _ref_index():
    by_name = {}
    for base, dirs, files in os.walk(REF):
        dirs[:] = [x for x in dirs if x not in (".git", "eigen", "glm", "half")]
        for f in files:
            by_name.setdefault(f, []).append(os.path.join(base, f))
    return by_name


def _resolve(path, by_name):
    full = os.path.join(REF, path)
    if os.path.isfile(full):
        return full
    # a path given relative to a directory of the reference (e.g. rg/NNTrain.hpp)
    cands = [p for p in by_name.get(os.path.basename(path), []) if p.endswith("/" + path)]
    if len(cands) > 1:  # a bare shader name means the renderer's shader, not the test copy
        cands = [p for p in cands if "/shader/src/" in p]
    return cands[0] if len(cands) == 1 else None


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "shader")), reason="reference tree not present")
def test_reference_citations_resolve():
    by_name = _ref_index()
    lengths = {}
    bad = []
    n = 0
    for src in _sources():
        with open(src, encoding="utf-8", errors="replace") as fh:
            text = fh.read()
        for m in CITE.finditer(text):
            path, ranges = m.group(1), m.group(2)
            if path.startswith(("tests/", "oracle/", "include/", "vknrc_gb300/", "csrc/", "profiles/")):
                continue  # this repository's own files
            if os.path.basename(path) in ("nrc.h", "nrc_oracle.h", "nrc_kernels.h", "ptx.cuh"):
                continue
            target = _resolve(path, by_name)
            if target is None:
                if path in ("README.md",) or path.endswith(".md") and not os.path.isfile(os.path.join(REF, path)):
                    continue  # this repository's documents
                bad.append(f"{os.path.relpath(src, ROOT)}: {path} not found in the reference")
                continue
            if target not in lengths:
                with open(target, encoding="utf-8", errors="replace") as fh:
                    lengths[target] = sum(1 for _ in fh)
            for part in ranges.split(","):
                lo, _, hi = part.strip().partition("-")
                hi = hi or lo
                n += 1
                if not (1 <= int(lo) <= int(hi) <= lengths[target]):
                    bad.append(f"{os.path.relpath(src, ROOT)}: {path}:{part.strip()} (file has {lengths[target]} lines)")
    assert n > 100, f"only {n} citations found: the scanner is not matching"
    assert not bad, "unresolved citations:\n" + "\n".join(sorted(set(bad)))
