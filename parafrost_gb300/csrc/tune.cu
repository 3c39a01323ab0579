// Autotuner of the launch shapes (pfg_tuning).
//
// Replaces the reference's launch-configuration macros (OPTIMIZEBLOCKS and
// its variants, src/gpu/grid.cuh:137-232), which size every grid from the
// device properties alone, by measurement on the caller's own instances:
// each trial uploads them, simplifies with per-kernel timing, and reads the
// time of every tuned pass's kernel group. Passes whose knobs belong to
// different kernel groups are swept together (trial j sets every knob to its
// j-th candidate: the passes run one after another on one stream and see the
// same inputs whatever the shapes, so each group's time answers for its own
// knob). Knobs that share a group (the BVE phase 3 grid and its ticket) are
// swept one after the other. Results never depend on the shapes.
#include <vector>

#include "engine.cuh"

namespace {

struct Knob {
    uint32_t pfg_tuning::*field;
    std::vector<uint32_t> cand;       // candidates; 0 is the built-in choice
    std::vector<int> groups;          // profiler groups whose time the knob moves
};

// one upload + simplify with the shapes `t`; ms[k] = time of the groups of knob k
int trial(pfg_ctx* o, uint32_t n, const pfg_instance* in, const pfg_tuning& t, const std::vector<Knob>& knobs,
          std::vector<double>& ms) {
    int rc = pfg_tuning_set(o, &t);
    if (rc != PFG_OK) return rc;
    rc = pfg_batch_upload(o, n, in);
    if (rc != PFG_OK) return rc;
    pfg_profile_reset(o);
    pfg_stats st;
    rc = pfg_simplify(o, &st);
    if (rc != PFG_OK) return rc;
    ms.assign(knobs.size(), 0.0);
    for (size_t k = 0; k < knobs.size(); k++)
        for (int g : knobs[k].groups) {
            uint64_t launches = 0, bytes = 0;
            double t_ms = 0;
            pfg_profile_get(o, g, &launches, &t_ms, &bytes);
            ms[k] += t_ms;
        }
    return PFG_OK;
}

// sweeps `knobs` together from `best`; every knob keeps its fastest candidate
int sweep(pfg_ctx* o, uint32_t n, const pfg_instance* in, uint32_t repeats, const std::vector<Knob>& knobs,
          pfg_tuning& best) {
    size_t ncand = 0;
    for (const Knob& k : knobs) ncand = std::max(ncand, k.cand.size());
    std::vector<double> best_ms(knobs.size(), 1e300);
    std::vector<uint32_t> best_v(knobs.size());
    for (size_t k = 0; k < knobs.size(); k++) best_v[k] = best.*(knobs[k].field);
    std::vector<double> ms;
    for (size_t j = 0; j < ncand; j++) {
        pfg_tuning t = best;
        for (const Knob& k : knobs) t.*(k.field) = k.cand[std::min(j, k.cand.size() - 1)];
        for (uint32_t r = 0; r < repeats; r++) {
            const int rc = trial(o, n, in, t, knobs, ms);
            if (rc != PFG_OK) return rc;
            for (size_t k = 0; k < knobs.size(); k++)
                if (ms[k] < best_ms[k]) { best_ms[k] = ms[k]; best_v[k] = t.*(knobs[k].field); }
        }
    }
    for (size_t k = 0; k < knobs.size(); k++) best.*(knobs[k].field) = best_v[k];
    return PFG_OK;
}

}  // namespace

extern "C" int pfg_autotune(pfg_ctx* o, uint32_t n, const pfg_instance* in, uint32_t repeats, pfg_tuning* out) {
    if (!o) return PFG_INVALID;
    if (!n || !in) { pfg::set_error(o, "autotune needs at least one instance"); return PFG_INVALID; }
    if (repeats == 0) repeats = 1;
    pfg_tuning start;
    pfg_tuning_get(o, &start);
    const bool was_on = pfg::profiling(o);
    pfg_profile_enable(o, 1);
    // blocks per SM: 0 = every block the SM holds (the kernels' occupancy)
    const std::vector<Knob> together = {
        {&pfg_tuning::sub_blocks_per_sm, {2, 4, 6, 0}, {pfg::K_SUB}},
        {&pfg_tuning::ve1_blocks_per_sm, {2, 4, 6, 0}, {pfg::K_VE1}},
        {&pfg_tuning::ve3_blocks_per_sm, {2, 4, 6, 0}, {pfg::K_VE3}},
        {&pfg_tuning::mis_threads, {64, 128, 256, 512}, {pfg::K_MIS_WIN, pfg::K_MIS_APPLY}},
        {&pfg_tuning::list_threads, {64, 128, 256, 512}, {pfg::K_FILL}},
        {&pfg_tuning::bcp_blocks_per_sm, {2, 4, 8, 16}, {pfg::K_BCP}},
    };
    const std::vector<Knob> then = {
        {&pfg_tuning::ve3_ticket, {1, 4, 16, 64}, {pfg::K_VE3}},
    };
    pfg_tuning best = start;
    int rc = sweep(o, n, in, repeats, together, best);
    if (rc == PFG_OK) rc = sweep(o, n, in, repeats, then, best);
    pfg_profile_enable(o, was_on ? 1 : 0);
    if (rc != PFG_OK) {
        pfg_tuning_set(o, &start);
        return rc;
    }
    pfg_tuning_set(o, &best);
    if (out) *out = best;
    return PFG_OK;
}
