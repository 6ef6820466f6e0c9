"""The working tree that travels to a GPU host stays small.

Files matched by the copy's ignore list (build output, caches, raw profiles) stay
behind; everything else is copied to the GPU host before a run, and a copy above
512 MiB is refused there.  This test sums the sizes of the files that would
travel and fails above 400 MiB, so that study dumps written into the tree are
caught here first.
"""
import fnmatch
import os

from conftest import ROOT

LIMIT = 400 << 20


def ignore_patterns():
    pats = [".git/"]
    path = os.path.join(ROOT, ".gpurunignore")
    if os.path.exists(path):
        for line in open(path):
            line = line.strip()
            if line and not line.startswith("#"):
                pats.append(line)
    return pats


def ignored(rel, is_dir, pats):
    name = os.path.basename(rel)
    for p in pats:
        if p.endswith("/"):
            p = p[:-1]
            if is_dir and (fnmatch.fnmatch(name, p) or fnmatch.fnmatch(rel, p)):
                return True
        elif fnmatch.fnmatch(rel, p) or ("/" not in p and fnmatch.fnmatch(name, p)):
            return True
    return False


def travelling_bytes():
    pats = ignore_patterns()
    total, biggest = 0, []
    for d, dirs, files in os.walk(ROOT):
        reld = os.path.relpath(d, ROOT)
        reld = "" if reld == "." else reld + "/"
        dirs[:] = [x for x in dirs if not ignored(reld + x, True, pats)]
        for f in files:
            rel = reld + f
            if ignored(rel, False, pats):
                continue
            try:
                n = os.path.getsize(os.path.join(d, f))
            except OSError:
                continue
            total += n
            biggest.append((n, rel))
    return total, sorted(biggest, reverse=True)[:5]


def test_ignore_list_drops_build_output():
    pats = ignore_patterns()
    for rel, is_dir in [("climaatmos.jl_gb300/_build", True), ("_work/study.npz", False),
                        ("climaatmos.jl_gb300/gbdycore/libgbdycore.so", False), ("x/prof.ncu-rep", False)]:
        assert ignored(rel, is_dir, pats), rel


def test_tree_copied_to_the_gpu_host_is_below_400_mib():
    total, biggest = travelling_bytes()
    assert total < LIMIT, "tree to copy is %.1f MiB; largest: %s" % (total / 2**20, biggest)
