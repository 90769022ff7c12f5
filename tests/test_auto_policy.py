"""CPU test of the automatic sweep configuration's policy
(pbf_gb300/csrc/auto_policy.h): trial schedule, the 3% switching margin,
separate solver and vorticity choices, period doubling and its cap, the
reset on a time drift, and the sit-outs of candidates that lose by 2x.  A
C++ harness compiled against the header drives it through scripted trials."""
import os
import shutil
import subprocess

import pytest

from tests.conftest import ROOT

HARNESS = r"""
#include <cstdio>
#include <vector>
#include "auto_policy.h"
using namespace pbf;
static int bad = 0;
#define CHECK(c) do { if (!(c)) { std::printf("FAILED line %d: %s\n", __LINE__, #c); ++bad; } } while (0)
static bool same(const std::vector<uint32_t>& a, std::vector<uint32_t> b) { return a == b; }
int main() {
    const uint32_t M = PBF_PASS_MASKED, D = PBF_PASS_DIRECT, C = PBF_PASS_COOP;
    AutoPolicy p;
    p.reset(0);
    CHECK(p.base == 32 && p.period == 32 && p.next == 32 && !p.trial_due());
    p.count = 31; CHECK(!p.trial_due());
    p.count = 32; CHECK(p.trial_due());
    uint32_t solver = M, vort = M;
    // trial 1: direct 10% faster for the solver, vorticity a tie; coop loses by > 2x
    std::vector<uint32_t> c = p.candidates(solver, vort, true);
    CHECK(same(c, {M, D, C}));
    {
        double s[] = {10.0, 9.0, 40.0}, v[] = {5.0, 5.0, 5.0};
        p.count = 34;
        p.finish(c, s, v, true, solver, vort);
    }
    CHECK(solver == D && vort == M);
    CHECK(p.period == 32 && p.next == 34 + 1 + 32 && p.trials == 1);
    CHECK(p.skip[C] == 3 && p.skip_len[C] == 3 && p.skip[M] == 0 && p.skip[D] == 0);
    {   // the mixed configuration joins the candidates where the caller asks for it
        AutoPolicy q;
        q.reset(0);
        const uint32_t X = PBF_PASS_MIXED;
        CHECK(same(q.candidates(X, X, false, true), {M, D, X}));
        CHECK(same(q.candidates(X, X, false, false), {M, D, X}));  // the current choice runs
        CHECK(same(q.candidates(M, M, true, true), {M, D, X, C}));
        double s[] = {10.0, 9.5, 6.0, 30.0}, v[] = {5.0, 5.0, 4.0, 20.0};
        uint32_t a = M, b = M;
        std::vector<uint32_t> cq = q.candidates(a, b, true, true);
        q.count = 32;
        q.finish(cq, s, v, true, a, b);
        CHECK(a == X && b == X && q.skip[C] == 3);
    }
    // trial 2: coop sits out; a candidate only 2% faster does not switch
    c = p.candidates(solver, vort, true);
    CHECK(same(c, {M, D}) && p.skip[C] == 2);
    {
        double s[] = {8.9, 9.0}, v[] = {5.0, 4.9};
        p.count = 70;
        p.finish(c, s, v, true, solver, vort);
    }
    CHECK(solver == D && vort == M);
    CHECK(p.period == 64 && p.next == 70 + 1 + 64);  // no change, no drift: doubled
    // trials 3-5: steady, the period doubles up to 256 and stays there
    for (uint32_t want : {128u, 256u, 256u}) {
        c = p.candidates(solver, vort, true);
        std::vector<double> s(c.size(), 9.0), v(c.size(), 5.0);
        for (size_t k = 0; k < c.size(); ++k) if (c[k] == M) s[k] = 9.5;
        p.finish(c, s.data(), v.data(), true, solver, vort);
        CHECK(p.period == want);
    }
    CHECK(p.skip[C] == 0);  // sat out trials 2-4, ran (not losing) in trial 5
    // trial 6: coop loses by 2x again (a new first loss: 3); the state drifted
    c = p.candidates(solver, vort, true);
    CHECK(same(c, {M, D, C}));
    {
        double s[] = {12.0, 11.7, 50.0}, v[] = {6.5, 6.5, 6.5};
        p.finish(c, s, v, true, solver, vort);
    }
    CHECK(solver == D && vort == M);
    CHECK(p.period == 32);  // drift resets the period
    CHECK(p.skip[C] == 3 && p.skip_len[C] == 3);
    // losing again each time it returns doubles the sit-out, up to 64
    for (uint32_t want : {6u, 12u, 24u, 48u, 64u, 64u}) {
        p.skip[C] = 0;
        c = p.candidates(solver, vort, true);
        std::vector<double> s(c.size(), 11.7), v(c.size(), 6.5);
        for (size_t k = 0; k < c.size(); ++k) if (c[k] == C) s[k] = 60.0;
        p.finish(c, s.data(), v.data(), true, solver, vort);
        CHECK(p.skip_len[C] == want);
    }
    // winning (or not losing by 2x) clears the sit-out length
    p.skip[C] = 0;
    c = p.candidates(solver, vort, true);
    {
        std::vector<double> s(c.size(), 11.7), v(c.size(), 6.5);
        p.finish(c, s.data(), v.data(), true, solver, vort);
    }
    CHECK(p.skip_len[C] == 0 && p.skip[C] == 0);
    // a current configuration always runs, even while it would sit out
    p.skip[D] = 5;
    c = p.candidates(solver, vort, true);
    CHECK(c.size() >= 2 && c[1] == D && p.skip[D] == 5);
    p.skip[D] = 0;
    // without vorticity only the solver choice moves
    c = p.candidates(solver, vort, false);
    CHECK(same(c, {M, D}));
    {
        double s[] = {5.0, 11.7}, v[] = {100.0, 1.0};
        p.finish(c, s, v, false, solver, vort);
    }
    CHECK(solver == M && vort == M);
    // reset restores the schedule and clears the sit-outs
    p.skip[C] = 9; p.skip_len[C] = 12;
    p.reset(5);
    CHECK(p.base == 5 && p.period == 5 && p.next == 5 && p.count == 0 && p.trials == 0);
    CHECK(p.skip[C] == 0 && p.skip_len[C] == 0 && p.last_ms == 0.0);
    // a base period above the cap is kept as the cap
    p.reset(1000);
    c = p.candidates(solver, vort, true);
    {
        std::vector<double> s(c.size(), 1.0), v(c.size(), 1.0);
        p.finish(c, s.data(), v.data(), true, solver, vort);
    }
    CHECK(p.period == 1000);
    std::printf("%d failures\n", bad);
    return bad != 0;
}
"""


def test_auto_policy(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "policy.cpp"
    src.write_text(HARNESS)
    exe = tmp_path / "policy"
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "pbf_gb300", "csrc"),
                    str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stdout + out.stderr
