// auto_policy.h — the bookkeeping of the automatic sweep configuration
// (PBF_SWEEP_AUTO, include/pbf.h): when to run a trial, which configurations
// it steps, and what it keeps.  Plain C++ (no CUDA): api.cu runs the trial
// substeps and feeds their stage times in; the CPU tests drive it directly.
//
// Rules:
//  - the first trial comes `base` substeps after a reset (state upload,
//    tuning change);
//  - a trial steps one substep under each candidate: masked and direct, and
//    mixed and cooperative where the scene size suits them (the caller
//    decides);
//  - a candidate replaces the current configuration of the solver pass or
//    the vorticity pass when its time for that pass is below kAutoMargin
//    times the current one's;
//  - the period returns to `base` when a choice changed or the chosen
//    configurations' time drifted by more than kAutoDrift either way since
//    the last trial, and doubles up to kAutoPeriodMax otherwise;
//  - a candidate whose total time exceeded kAutoPrune times the best one's
//    sits out the next kAutoPruneFirst trials, twice as many each time it
//    loses that way again (up to kAutoPruneMax); the current configurations
//    always run.
#pragma once

#include <algorithm>
#include <cstdint>
#include <vector>

#include "../../include/pbf.h"

namespace pbf {

constexpr uint32_t kAutoPeriod = 32;
constexpr uint32_t kAutoPeriodMax = 256;
constexpr double kAutoMargin = 0.97;
constexpr double kAutoDrift = 1.25;
constexpr double kAutoPrune = 2.0;
constexpr uint32_t kAutoPruneFirst = 3;
constexpr uint32_t kAutoPruneMax = 64;

struct AutoPolicy {
    uint32_t base = kAutoPeriod;   // first trial and period while things change
    uint32_t period = kAutoPeriod;
    uint64_t count = 0;            // substeps since the last reset
    uint64_t next = kAutoPeriod;   // substep at which the next trial starts
    double last_ms = 0.0;          // the chosen configurations' time at the last trial
    uint32_t skip[5] = {};         // trials a configuration still sits out
    uint32_t skip_len[5] = {};     // its last sit-out
    uint32_t trials = 0;

    void reset(uint32_t base_period) {
        base = period = base_period ? base_period : kAutoPeriod;
        count = 0;
        next = period;
        last_ms = 0.0;
        for (uint32_t& k : skip) k = 0;
        for (uint32_t& k : skip_len) k = 0;
        trials = 0;
    }

    bool trial_due() const { return count >= next; }

    // The next trial's candidates (PBF_PASS_*), given the current choices.
    std::vector<uint32_t> candidates(uint32_t solver, uint32_t vort, bool try_coop,
                                     bool try_mixed = false) {
        std::vector<uint32_t> all = {PBF_PASS_MASKED, PBF_PASS_DIRECT};
        if (try_mixed) all.push_back(PBF_PASS_MIXED);
        if (try_coop) all.push_back(PBF_PASS_COOP);
        std::vector<uint32_t> out;
        for (uint32_t p : all) {
            if (p == solver || p == vort || skip[p] == 0) out.push_back(p);
            else --skip[p];
        }
        // a current choice outside the list above (set before a reset) still runs
        for (uint32_t p : {solver, vort})
            if (std::find(out.begin(), out.end(), p) == out.end()) out.push_back(p);
        return out;
    }

    // After a trial: cands[c] took solver_ms[c] in the solver sweeps and
    // vort_ms[c] in the vorticity passes (ignored without vorticity).
    // Updates the choices, the sit-outs and the schedule; `count` is the
    // substep count at the trial's last substep (before it is counted).
    void finish(const std::vector<uint32_t>& cands, const double* solver_ms,
                const double* vort_ms, bool use_vort, uint32_t& solver, uint32_t& vort) {
        const size_t nc = cands.size();
        auto index_of = [&](uint32_t p) {
            size_t c = 0;
            while (c + 1 < nc && cands[c] != p) ++c;
            return c;
        };
        auto pick = [&](uint32_t cur, const double* ms) {
            size_t best = 0;
            for (size_t c = 1; c < nc; ++c)
                if (ms[c] < ms[best]) best = c;
            return ms[best] < kAutoMargin * ms[index_of(cur)] ? cands[best] : cur;
        };
        const uint32_t ns = pick(solver, solver_ms);
        const uint32_t nv = use_vort ? pick(vort, vort_ms) : vort;
        double now = solver_ms[index_of(ns)] + (use_vort ? vort_ms[index_of(nv)] : 0.0);
        const bool drifted =
            last_ms > 0.0 && (now > kAutoDrift * last_ms || now * kAutoDrift < last_ms);
        last_ms = now;
        double best = 0.0;
        for (size_t c = 0; c < nc; ++c) {
            const double t = solver_ms[c] + (use_vort ? vort_ms[c] : 0.0);
            best = c == 0 ? t : std::min(best, t);
        }
        for (size_t c = 0; c < nc; ++c) {
            const double t = solver_ms[c] + (use_vort ? vort_ms[c] : 0.0);
            uint32_t& len = skip_len[cands[c]];
            if (t > kAutoPrune * best) {
                len = len ? std::min(2 * len, kAutoPruneMax) : kAutoPruneFirst;
                skip[cands[c]] = len;
            } else {
                len = 0;
            }
        }
        const bool changed = ns != solver || nv != vort || drifted;
        solver = ns;
        vort = nv;
        period = changed ? base : std::min(2 * period, std::max(base, kAutoPeriodMax));
        next = count + 1 + period;
        ++trials;
    }
};

}  // namespace pbf
