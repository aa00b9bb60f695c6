"""The SpMV task schedule of the mixed engine (host code, no device): the rules
of make_schedule (csrc/mixed.cu) checked on segment lengths of the refinery
and random LPs.

* every light segment (length <= the instance's light_max) is in exactly one
  light task of its instance, every longer one exactly once in a list task;
* a light task holds at most max_segs segments and task_nnz light nonzeros
  (one longer segment alone excepted);
* no light task starts on a run of 32 or more long segments: after the
  renumbering by descending length the long segments are each instance's
  prefix, and the first light task starts after it;
* a shorter run of long segments stays in the first task (the small LPs keep
  their schedules)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import PKG_DIR, REPO

SKIP_RUN = 32  # kSkipRun in csrc/mixed.cu

HARNESS = r"""
#include <cstdio>
#include <vector>

#include "mixed.h"

int main() {
    int B, task_nnz, lanes, max_segs, nseg;
    if (std::scanf("%d %d %d %d %d", &B, &task_nnz, &lanes, &max_segs, &nseg) != 5) return 2;
    std::vector<int> off(B + 1), ptr(nseg + 1);
    for (int& v : off)
        if (std::scanf("%d", &v) != 1) return 2;
    for (int& v : ptr)
        if (std::scanf("%d", &v) != 1) return 2;
    sihg::SideSchedule s;
    sihg::make_schedule(ptr, off, task_nnz, s, lanes, max_segs);
    std::printf("L");
    for (int v : s.light_max) std::printf(" %d", v);
    std::printf("\n");
    for (const sihg::Task& t : s.tasks) std::printf("T %d %d %d %d\n", t.seg_begin, t.seg_end, t.inst, t.flags);
    std::printf("I");
    for (int v : s.list_idx) std::printf(" %d", v);
    std::printf("\n");
    return 0;
}
"""


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    from sih_pdhg import _lib

    if not os.path.exists(_lib.LIB_PATH):
        pytest.fail(f"{_lib.LIB_PATH} is missing: build the library first")
    d = tmp_path_factory.mktemp("schedule")
    src = d / "schedule_check.cu"
    src.write_text(HARNESS)
    exe = d / "schedule_check"
    lib_dir = os.path.dirname(_lib.LIB_PATH)
    subprocess.check_call(["nvcc", "-std=c++17", "-O1", "-I", os.path.join(PKG_DIR, "csrc"), "-I",
                           os.path.join(REPO, "include"), str(src), "-o", str(exe), "-L", lib_dir, "-lsih_pdhg",
                           "-Xlinker", "-rpath", "-Xlinker", lib_dir])
    return str(exe)


def schedule(exe, lengths_per_inst, task_nnz, max_segs=1024, lanes=0):
    """(light_max, tasks [(begin, end, inst, flags)], list_idx, ptr) for the
    instances' segment lengths laid out one after another."""
    lens = np.concatenate([np.asarray(l, dtype=np.int64) for l in lengths_per_inst])
    ptr = np.concatenate([[0], np.cumsum(lens)])
    off = np.concatenate([[0], np.cumsum([len(l) for l in lengths_per_inst])])
    text = " ".join(map(str, [len(lengths_per_inst), task_nnz, lanes, max_segs, len(lens)]))
    text += "\n" + " ".join(map(str, off)) + "\n" + " ".join(map(str, ptr)) + "\n"
    out = subprocess.run([exe], input=text, capture_output=True, text=True, timeout=120, check=True).stdout
    light_max, tasks, lst = None, [], []
    for line in out.splitlines():
        f = line.split()
        if f[0] == "L":
            light_max = [int(v) for v in f[1:]]
        elif f[0] == "T":
            tasks.append(tuple(int(v) for v in f[1:]))
        elif f[0] == "I":
            lst = [int(v) for v in f[1:]]
    return light_max, tasks, lst, ptr, off


def check_rules(light_max, tasks, lst, ptr, off, task_nnz, max_segs):
    lens = np.diff(ptr)
    nseg = len(lens)
    inst_of = np.repeat(np.arange(len(off) - 1), np.diff(off))
    is_long = lens > np.asarray(light_max)[inst_of]
    light_cover = np.zeros(nseg, dtype=np.int64)
    list_cover = np.zeros(nseg, dtype=np.int64)
    for b, e, inst, flags in tasks:
        if flags & 1:  # list task: entries [b, e) of list_idx
            segs = np.asarray(lst[b:e])
            assert np.all(inst_of[segs] == inst) and np.all(is_long[segs])
            list_cover[segs] += 1
            continue
        assert off[inst] <= b < e <= off[inst + 1]
        assert e - b <= max_segs
        light = ~is_long[b:e]
        light_cover[b:e] += light
        if light.sum() > 1:
            assert lens[b:e][light].sum() <= task_nnz
        # the task does not start on a run of SKIP_RUN long segments
        run = 0
        while b + run < e and is_long[b + run]:
            run += 1
        if run == e - b:  # the run may continue past the task
            k = e
            while k < off[inst + 1] and is_long[k]:
                k += 1
            run = k - b
        assert run < SKIP_RUN, (b, e, run)
    assert np.all(light_cover[~is_long] == 1)
    assert np.all(light_cover[is_long] == 0)
    assert np.all(list_cover[is_long] == 1)
    assert np.all(list_cover[~is_long] == 0)


def row_lengths(p):
    return np.bincount(p.A._ri, minlength=p.A._m)


@pytest.mark.parametrize("max_segs", [64, 1024])
def test_refinery_rows_skip_the_long_prefix(harness, max_segs):
    from sih_pdhg.generators import refinery_lp

    lens = np.sort(row_lengths(refinery_lp(168, 0)))[::-1]  # the engine's renumbering
    light_max, tasks, lst, ptr, off = schedule(harness, [lens], 128, max_segs)
    check_rules(light_max, tasks, lst, ptr, off, 128, max_segs)
    n_long = int((lens > light_max[0]).sum())
    assert n_long >= SKIP_RUN
    first_light = min(b for b, e, i, f in tasks if not f & 1)
    assert first_light == n_long


def test_one_nonzero_columns_are_cut_at_max_segs(harness):
    from sih_pdhg.generators import refinery_lp

    lens = np.sort(np.diff(refinery_lp(24, 0).A._cp))[::-1]
    for max_segs in (64, 1024):
        light_max, tasks, lst, ptr, off = schedule(harness, [lens], 128, max_segs)
        check_rules(light_max, tasks, lst, ptr, off, 128, max_segs)
        widest = max(e - b for b, e, i, f in tasks if not f & 1)
        assert widest == min(max_segs, 128)  # 128 one-nonzero columns fill a 128-nonzero task


def test_short_long_run_stays_in_the_first_task(harness):
    from sih_pdhg.generators import small_random_lp

    lens = np.sort(row_lengths(small_random_lp(2000, 5000, 8, 0)))[::-1]
    light_max, tasks, lst, ptr, off = schedule(harness, [lens], 128, 64)
    check_rules(light_max, tasks, lst, ptr, off, 128, 64)
    assert 0 < int((lens > light_max[0]).sum()) < SKIP_RUN
    assert min(b for b, e, i, f in tasks if not f & 1) == 0


def test_batch_of_unsorted_instances(harness):
    """Three instances, lengths in no order, one with a run of 40 long segments in
    the middle and one that starts with such a run."""
    rng = np.random.default_rng(5)
    a = rng.integers(1, 12, 300)
    a[100:140] = 200  # interior run
    b = rng.integers(0, 6, 500)  # empty segments too
    c = np.concatenate([np.full(50, 90), rng.integers(1, 9, 200)])  # leading run
    light_max, tasks, lst, ptr, off = schedule(harness, [a, b, c], 64, 64)
    check_rules(light_max, tasks, lst, ptr, off, 64, 64)
    starts_c = [t[0] for t in tasks if t[2] == 2 and not t[3] & 1]
    assert min(starts_c) == off[2] + 50
