"""Every reference citation in the sources (a Swalbe.jl project path with a
line or line range, e.g. src/collide.jl:76-89) names a file of the
reference and lines inside it.

The reference checkout is read from $SWALBE_REFERENCE (default: the
read-only checkout this repository was built beside); where it is absent the
test is skipped.
"""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("SWALBE_REFERENCE", "/root/reference")
CITE = re.compile(r"\b((?:src|test|scripts|paper)/[\w./-]+\.(?:jl|md)):(\d+)(?:-(\d+))?"
                  r"((?:,\s*\d+(?:-\d+)?)*)")
# the source trees and top-level scripts (build outputs and caches skipped)
TREES = ("swalbe.jl_gb300", "oracle", "include", "tests", "bench.py", "__graft_entry__.py")
SKIP_DIRS = {"_build", "lib", "__pycache__", "_ref"}
EXTS = (".py", ".cu", ".cuh", ".h", ".c", ".jl", ".json")


def source_files():
    for top in TREES:
        p = os.path.join(ROOT, top)
        if os.path.isfile(p):
            yield p
            continue
        for root, dirs, files in os.walk(p):
            dirs[:] = [d for d in dirs if d not in SKIP_DIRS]
            for f in files:
                if f.endswith(EXTS):
                    yield os.path.join(root, f)


def cites():
    for p in source_files():
        with open(p, errors="replace") as fh:
            for ln, line in enumerate(fh, 1):
                for m in CITE.finditer(line):
                    nums = [int(m.group(2))] + ([int(m.group(3))] if m.group(3) else [])
                    for extra in re.findall(r"\d+(?:-\d+)?", m.group(4) or ""):
                        nums += [int(x) for x in extra.split("-")]
                    yield os.path.relpath(p, ROOT), ln, m.group(1), nums


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")), reason="reference not present")
def test_citations_point_inside_reference_files():
    lengths = {}
    bad = []
    n = 0
    for where, ln, path, nums in cites():
        n += 1
        full = os.path.join(REF, path)
        if not os.path.isfile(full):
            bad.append(f"{where}:{ln}: {path} does not exist")
            continue
        if full not in lengths:
            with open(full, errors="replace") as fh:
                lengths[full] = sum(1 for _ in fh)
        if min(nums) < 1 or max(nums) > lengths[full]:
            bad.append(f"{where}:{ln}: {path}:{nums} outside its {lengths[full]} lines")
        if len(nums) >= 2 and nums[1] < nums[0]:
            bad.append(f"{where}:{ln}: {path}:{nums} is a reversed range")
    assert n > 100
    assert not bad, "\n".join(bad)
