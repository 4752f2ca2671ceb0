"""The segmented render's segment plan (plan_segments in csrc/seg_plan.h, the
function k_seg_plan runs on the device), built for the host and checked on
random and extreme per-octave histograms: every work item of the sorted
list lands in exactly one segment, at most 64 segments, a segment's items
come from at most two consecutive octaves (bar the pathological widening),
and the plan ends even when the deposit scales span every octave."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(REPO, "dm-annihilation-cxx_gb300", "csrc")
K_CLASSES, K_SPAN, K_SLOTS = 256, 2, 64


@pytest.fixture(scope="module")
def plan(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("plan") / "libsegplan.so")
    subprocess.run(["g++", "-O1", "-std=c++17", "-shared", "-fPIC", "-I", CSRC,
                    os.path.join(REPO, "tests", "cpp", "seg_plan_shim.cpp"), "-o", so], check=True)
    lib = C.CDLL(so)
    lib.plan.restype = C.c_int
    lib.plan.argtypes = [C.c_void_p] * 3 + [C.c_longlong, C.c_void_p]

    def run(n, px, budget):
        n = np.ascontiguousarray(n, dtype=np.int32)
        end = np.cumsum(n).astype(np.int32)
        px = np.ascontiguousarray(px, dtype=np.int64)
        out = np.zeros(4 * K_SLOTS, dtype=np.int64)
        ns = lib.plan(n.ctypes.data, end.ctypes.data, px.ctypes.data, int(budget), out.ctypes.data)
        return ns, out.reshape(-1, 4)[:min(ns, K_SLOTS)], end
    return run


def covered(spans, total):
    hits = np.zeros(total, dtype=np.int64)
    for lo, hi, stride, off in spans:
        idx = np.arange(lo + off, hi, stride)
        hits[idx] += 1
    return hits


def check_plan(run, n, px, budget, span_limit=K_SPAN):
    ns, spans, end = run(n, px, budget)
    total = int(end[-1])
    assert 1 <= ns <= K_SLOTS or (ns == 0 and total == 0)
    hits = covered(spans, total)
    assert np.all(hits == 1), "every item in exactly one segment"
    cls_of = np.repeat(np.arange(K_CLASSES), n)
    for lo, hi, stride, off in spans:
        cs = np.unique(cls_of[np.arange(lo + off, hi, stride)])
        if cs.size and cs[0] == 0:
            assert cs.size == 1, "class 0 is a segment of its own"
        elif cs.size:
            assert cs[-1] - cs[0] < span_limit, (cs, "a segment spans more octaves than allowed")
    return ns, spans


@pytest.mark.parametrize("seed", range(20))
def test_random_histograms(plan, seed):
    rng = np.random.default_rng(seed)
    n = np.zeros(K_CLASSES, dtype=np.int64)
    live = rng.choice(np.arange(K_CLASSES), size=rng.integers(1, 40), replace=False)
    n[live] = rng.integers(1, 5000, size=live.size)
    px = n * rng.integers(1000, 40000, size=K_CLASSES)
    budget = int(rng.choice([1e5, 1e7, 1e9, 2.6e10]))
    check_plan(plan, n, px, budget)


def test_one_huge_octave_is_dealt_round_robin(plan):
    n = np.zeros(K_CLASSES, dtype=np.int64)
    n[130] = 10000
    px = n * 100000                      # 1e9 deposits in one octave
    ns, spans = check_plan(plan, n, px, budget=int(1e8))
    assert ns == 10 and all(s[2] == 10 for s in spans)


def test_every_octave_used_ends(plan):
    # deposit scales over every octave: more two-octave groups than slots, so
    # the plan widens the span (after the budget stops helping) and ends
    n = np.full(K_CLASSES, 3, dtype=np.int64)
    px = n * 10
    ns, _ = check_plan(plan, n, px, budget=1 << 40, span_limit=K_CLASSES)
    assert ns <= K_SLOTS


def test_empty_and_single_pixel_class(plan):
    n = np.zeros(K_CLASSES, dtype=np.int64)
    ns, _, _ = plan(n, np.zeros(K_CLASSES, dtype=np.int64), 100)
    assert ns == 0
    n[0] = 7
    ns, spans = check_plan(plan, n, np.zeros(K_CLASSES, dtype=np.int64), 100)
    assert ns == 1 and tuple(spans[0]) == (0, 7, 1, 0)
