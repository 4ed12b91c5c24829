"""The round trip's plan (vaikkari_gb300/csrc/gpe_round_trip_plan.h), compiled
on the CPU: instance groups are non-empty contiguous runs of the work-item order
(at most four) that hold every instance once; every group is active in exactly
K consecutive rounds; groups join and leave in order, one to K rounds apart, so
no round is idle; each piece of the schedule has one contiguous set of active
groups.  Without groups, one group of all instances in index order steps in
every round.  The 64-condensate batch's joins are pinned to the schedule its
GPU timeline was measured with."""
import json
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

DRIVER = r"""
#include <cstdio>
#include <vector>
#include "gpe_round_trip_plan.h"
int main()
{
    int n, split;
    long long steps;
    double R;
    if (std::scanf("%d %d %lld %lf", &n, &split, &steps, &R) != 4) return 1;
    std::vector<long long> values(n);
    std::vector<int> order(n);
    for (auto &v : values)
        if (std::scanf("%lld", &v) != 1) return 1;
    for (auto &o : order)
        if (std::scanf("%d", &o) != 1) return 1;
    const gpe::RoundTripPlan p = gpe::plan_round_trip(values, order, split != 0, steps, R);
    std::printf("{\"groups\": [");
    for (size_t g = 0; g < p.groups.size(); g++) {
        std::printf("%s[", g ? ", " : "");
        for (size_t k = 0; k < p.groups[g].size(); k++) std::printf("%s%d", k ? ", " : "", p.groups[g][k]);
        std::printf("]");
    }
    std::printf("], \"join\": [");
    for (size_t g = 0; g < p.join.size(); g++) std::printf("%s%lld", g ? ", " : "", p.join[g]);
    std::printf("], \"pieces\": [");
    for (size_t c = 0; c < p.pieces.size(); c++)
        std::printf("%s[%lld, %lld, %d, %d]", c ? ", " : "", p.pieces[c].r0, p.pieces[c].r1, p.pieces[c].lo,
                    p.pieces[c].hi);
    std::printf("]}\n");
    return 0;
}
"""


@pytest.fixture(scope="module")
def planner(tmp_path_factory):
    d = tmp_path_factory.mktemp("plan")
    src = d / "plan.cpp"
    src.write_text(DRIVER)
    exe = d / "plan"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I",
                    os.path.join(ROOT, "vaikkari_gb300", "csrc"), str(src), "-o", str(exe)], check=True)

    def run(values, order, split, steps, R):
        inp = f"{len(values)} {int(split)} {steps} {R!r}\n" + " ".join(map(str, values)) + "\n" + \
              " ".join(map(str, order)) + "\n"
        out = subprocess.run([str(exe)], input=inp, capture_output=True, text=True, check=True).stdout
        return json.loads(out)
    return run


def _order(values):
    """Work-item order: decreasing size, stable (as the library sorts)."""
    return sorted(range(len(values)), key=lambda i: -values[i])


def _check(plan, values, order, split, steps):
    n = len(values)
    groups, join, pieces = plan["groups"], plan["join"], plan["pieces"]
    G = len(groups)
    assert sorted(i for g in groups for i in g) == list(range(n))
    assert all(groups)
    if split and n > 1 and steps > 0:
        assert G <= min(n, 4)
        assert [i for g in groups for i in g] == order   # contiguous runs of the item order
    else:
        assert groups == [list(range(n))]
    assert len(join) == G and join[0] == 0
    for a, b in zip(join, join[1:]):
        assert 1 <= b - a <= steps
    if steps == 0:
        assert pieces == []
        return
    # pieces cover rounds 0 .. join[-1] + steps - 1 without gaps; active sets
    # contiguous, non-empty and constant inside each piece
    assert pieces[0][0] == 0 and pieces[-1][1] == join[-1] + steps
    rounds = [0] * G
    for (r0, r1, lo, hi), nxt in zip(pieces, pieces[1:] + [None]):
        assert r0 < r1
        if nxt is not None:
            assert nxt[0] == r1
        assert 0 <= lo <= hi < G
        for r in (r0, r1 - 1):
            assert [g for g in range(G) if join[g] <= r < join[g] + steps] == list(range(lo, hi + 1))
        for g in range(lo, hi + 1):
            rounds[g] += r1 - r0
    assert rounds == [steps] * G


@pytest.mark.parametrize("seed", range(40))
def test_plan_invariants_random_batches(planner, seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 70))
    values = [int(v) for v in rng.choice([1, 27, 1000, 27648, 65536, 884736 * 2], size=n)]
    if seed % 5 == 0:
        values = [int(rng.integers(1, 10 ** 7)) for _ in range(n)]
    order = _order(values)
    steps = int(rng.choice([0, 1, 2, 5, 20, 100, 1000]))
    R = float(rng.choice([0.5, 8.6, 10.0, 17.1, 1e3]))
    for split in (True, False):
        plan = planner(values, order, split, steps, R)
        _check(plan, values, order, split, steps)


def test_plan_of_the_64_condensate_batch(planner):
    """The batch's groups hold 18/28/28/26 % of the values, and with float host
    fields in GPE_FP32C (R = 16 B / 200 GB/s against 56 B / 6 TB/s) groups join
    at rounds 0, 13, 19 and 23 of a 20-step call, all four being active from
    round 23 to 79 of an 80-step one."""
    rng = np.random.default_rng(2)
    ns = rng.choice(np.asarray((24, 32, 48, 64, 96)), size=64)
    values = [2 * int(v) ** 3 for v in ns]
    order = _order(values)
    R = 4 * 4 / 200 * 6000 / 56
    plan = planner(values, order, True, 20, R)
    _check(plan, values, order, True, 20)
    shares = [sum(values[i] for i in g) / sum(values) for g in plan["groups"]]
    assert [round(s, 2) for s in shares] == [0.18, 0.28, 0.28, 0.26]
    assert plan["join"] == [0, 13, 19, 23]
    plan80 = planner(values, order, True, 80, R)
    assert [23, 80, 0, 3] in plan80["pieces"]


def test_plan_single_instance_and_no_split(planner):
    for split in (True, False):
        plan = planner([500], [0], split, 7, 8.6)
        assert plan == {"groups": [[0]], "join": [0], "pieces": [[0, 7, 0, 0]]}
    plan = planner([5, 9, 2], [1, 0, 2], False, 3, 8.6)
    assert plan == {"groups": [[0, 1, 2]], "join": [0], "pieces": [[0, 3, 0, 0]]}
