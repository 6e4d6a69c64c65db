"""The partial-sum schedule of one time step (SumPlan, sum_plan in
3d-ose_gb300/csrc/ose_internal.h), compiled from the library's own header as
a host program and checked against the reference's summation
(ose_3d_lib.cu:736-744, 839-860): there a_{n+1} is added to S at application
n and S is multiplied by the sponge after every addition, so in the new state
(S after application M) term a_j carries att^e with e = M for j <= 1 and
M - j + 2 for j >= 2.  For every series order M the schedule must add each
a_j (j = 0 .. M + 1) exactly once, with that total power of att (the power it
is added with plus the powers S is multiplied by at the applications that
touch it later), touch S at the last application, and use powers 0 .. 3 only."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
CSRC = os.path.join(ROOT, "3d-ose_gb300", "csrc")

PROGRAM = r'''
#include <cstdio>
#include "ose_internal.h"
int main()
{
    for (int M = 1; M <= 47; ++M)
        for (int n = 0; n <= M; ++n) {
            const ose::SumPlan p = ose::sum_plan(n, M);
            std::printf("%d %d %d %d %d %d %d %d %d\n", M, n, p.add_prev, p.add_new, p.s_read, p.touch, p.kS,
                        p.kP, p.kN);
        }
    return 0;
}
'''


@pytest.fixture(scope="module")
def plans(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    d = tmp_path_factory.mktemp("sumplan")
    src, exe = d / "sum_plan.cu", d / "sum_plan"
    src.write_text(PROGRAM)
    subprocess.run([nvcc, "-std=c++17", "-I" + CSRC, "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    rows = [tuple(int(v) for v in line.split()) for line in out.splitlines()]
    by_m = {}
    for M, n, ap, an, sr, t, ks, kp, kn in rows:
        by_m.setdefault(M, []).append(dict(n=n, add_prev=ap, add_new=an, s_read=sr, touch=t, kS=ks, kP=kp, kN=kn))
    return by_m


def test_every_term_added_once_with_the_reference_power(plans):
    for M, apps in plans.items():
        added = {}
        for p in apps:
            n = p["n"]
            if p["add_prev"]:
                assert p["touch"]
                added.setdefault(n - 1, []).append((n, p["kP"]))
            if p["add_new"]:
                assert p["touch"]
                added.setdefault(n + 1, []).append((n, p["kN"]))
        assert sorted(added) == list(range(M + 2)), M
        touches = [p["n"] for p in apps if p["touch"]]
        assert touches[-1] == M
        for j, ((n_add, k),) in ((j, v) for j, v in added.items()):
            # S is multiplied by att^(n - n') at each later touch: in total att^(M - n_add)
            later = sum(p["kS"] for p in apps if p["n"] > n_add and p["touch"])
            assert later == M - n_add, (M, j)
            expect = M if j <= 1 else M - j + 2
            assert k + later == expect, (M, j, k, later)


def test_stored_sum_is_read_back_with_the_gap_power(plans):
    for M, apps in plans.items():
        last = None
        for p in apps:
            if not p["touch"]:
                assert p["s_read"] == 0 and p["kS"] == 0
                continue
            if last is None:
                assert p["s_read"] == 0
            else:
                assert p["s_read"] == 1 and p["kS"] == p["n"] - last
            last = p["n"]


def test_powers_within_the_three_weights(plans):
    for M, apps in plans.items():
        for p in apps:
            assert 0 <= p["kS"] <= 3 and 0 <= p["kP"] <= 3 and 0 <= p["kN"] <= 1, (M, p)


def test_m10_touches_six_applications(plans):
    assert [p["n"] for p in plans[10] if p["touch"]] == [1, 2, 5, 6, 9, 10]
