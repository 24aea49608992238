// Launch-shape autotuner: the run-time launch shapes of the E+F sequence, timed on the staged
// batch through its captured CUDA graph.
//
// Knobs (each 0 = the built-in rule):
//   tune_tc[t]  warps per TMEM lane quadrant of the tensor-core network kernel for type t (1, 2, 4;
//               4 / G CTAs per SM, never more than tensor memory admits: the kernel's shared-memory
//               request caps the CTAs per SM at 512 / allocated columns whatever G is)
//   tune_bp     resident blocks per SM of the symmetry-function and force passes (the grid; both
//               passes take atoms from an atomic counter, so the grid only sets the residency)
//   tune_nbr    blocks per SM of the neighbour search (likewise counter-scheduled)
// The search is coordinate-wise. Each candidate is timed as the median of `reps` graph replays
// (CUDA events on the context's stream), after one replay that captures the graph and settles
// the capacities. A candidate is kept only when it beats the best so far by more than 1 %.
#include <algorithm>
#include <vector>
#include "context.hpp"

static bool valid_groups(int g) { return g == 0 || g == 1 || g == 2 || g == 4; }

static void check_tuning(const ann_tuning& t) {
    for (int k = 0; k < 4; ++k)
        if (!valid_groups(t.tc_groups[k])) throw ann_error(ANN_ERR_ARG, "tc_groups must be 0, 1, 2 or 4");
    if (t.bp_blocks_per_sm < 0 || t.bp_blocks_per_sm > 16) throw ann_error(ANN_ERR_ARG, "bp_blocks_per_sm must be in [0, 16]");
    if (t.nbr_blocks_per_sm < 0 || t.nbr_blocks_per_sm > 64) throw ann_error(ANN_ERR_ARG, "nbr_blocks_per_sm must be in [0, 64]");
}

static void apply(ann_ctx* c, const ann_tuning& t) {
    for (int k = 0; k < MAXT; ++k) c->tune_tc[k] = k < 4 ? t.tc_groups[k] : 0;
    c->tune_bp = t.bp_blocks_per_sm;
    c->tune_nbr = t.nbr_blocks_per_sm;
    drop_graphs(c);
}

// one evaluation of the staged batch with the context's current shapes (ms, median of reps). Every
// replay clears the status word, so each one's status is read after it: a negative result means
// that a replay's bounded device waits gave up (its early return would look fast)
static double time_batch(ann_ctx* c, int prec, int reps) {
    run_batch(c, prec, true, true);
    finish_batch(c);
    cudaEvent_t e0, e1;
    ck(cudaEventCreate(&e0), "event create");
    ck(cudaEventCreate(&e1), "event create");
    std::vector<float> t(reps);
    bool gave_up = false;
    try {
        for (int r = 0; r < reps; ++r) {
            ck(cudaEventRecord(e0, c->stream), "event record");
            run_batch(c, prec, true, true);
            ck(cudaEventRecord(e1, c->stream), "event record");
            ck(cudaEventSynchronize(e1), "event synchronize");
            ck(cudaEventElapsedTime(&t[r], e0, e1), "event time");
            int32_t s0 = 0;
            ck(cudaMemcpyAsync(&s0, c->status.p, sizeof(s0), cudaMemcpyDeviceToHost, c->stream), "D2H status");
            ck(cudaStreamSynchronize(c->stream), "synchronize");
            if (s0 & ST_TIMEOUT) gave_up = true;
        }
        finish_batch(c);
    } catch (...) {
        cudaEventDestroy(e0); cudaEventDestroy(e1);
        throw;
    }
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    if (gave_up) return -1.0;
    std::nth_element(t.begin(), t.begin() + reps / 2, t.end());
    return t[reps / 2];
}

extern "C" {

int ann_set_wait_limit(ann_ctx* c, int32_t polls) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    if (polls < -1 || polls > (1 << 24)) return fail(c, ANN_ERR_ARG, "polls must be -1 (built-in bounds) or in [0, 2^24]");
    c->wait_polls = polls < 0 ? 0 : polls + 1;
    drop_graphs(c);   // the limit is a kernel argument of the captured launches
    return ANN_OK;
}

int ann_set_tuning(ann_ctx* c, const ann_tuning* t) {
    if (!c || !t) return fail(c, ANN_ERR_ARG, "NULL argument");
    ANN_TRY(c, {
        check_tuning(*t);
        apply(c, *t);
    })
}

int ann_autotune(ann_ctx* c, int32_t prec, int32_t reps, ann_tuning* out) {
    if (!c) return fail(c, ANN_ERR_ARG, "NULL context");
    ANN_TRY(c, {
        set_device(c);
        if (prec != ANN_FP64 && prec != ANN_MIXED) throw ann_error(ANN_ERR_ARG, "invalid precision");
        if (c->md_ready) throw ann_error(ANN_ERR_STATE, "the autotuner times a staged batch, not an MD run (ann_compute first)");
        if (!c->have_batch || c->N <= 0) throw ann_error(ANN_ERR_STATE, "no batch staged (ann_compute first)");
        reps = std::max(1, std::min((int)reps, 1000));
        ann_tuning prior{};
        for (int k = 0; k < 4 && k < MAXT; ++k) prior.tc_groups[k] = c->tune_tc[k];
        prior.bp_blocks_per_sm = c->tune_bp;
        prior.nbr_blocks_per_sm = c->tune_nbr;
        try {
            ann_tuning best{};
            apply(c, best);
            const double t_default = time_batch(c, prec, reps);
            if (t_default < 0) throw ann_error(ANN_ERR_TIMEOUT, "a bounded device wait gave up with the built-in launch shapes");
            double t_best = t_default;
            // a candidate whose bounded waits gave up is dropped, not kept as fast, and the search goes on
            auto trial = [&](ann_tuning cand) {
                apply(c, cand);
                double t = -1.0;
                try { t = time_batch(c, prec, reps); }
                catch (ann_error& e) { if (e.code != ANN_ERR_TIMEOUT) throw; }
                if (t > 0 && t < 0.99 * t_best) { t_best = t; best = cand; }
            };
            if (prec == ANN_MIXED && use_tc(c)) {
                for (int ty = 0; ty < std::min(c->pot.ntypes(), 4); ++ty) {
                    const ann_tuning base = best;
                    for (int g : {1, 2, 4}) { ann_tuning cand = base; cand.tc_groups[ty] = g; trial(cand); }
                }
            }
            {
                const ann_tuning base = best;
                for (int b : {2, 3, 4}) { ann_tuning cand = base; cand.bp_blocks_per_sm = b; trial(cand); }
            }
            {
                const ann_tuning base = best;
                for (int b : {4, 8, 32}) { ann_tuning cand = base; cand.nbr_blocks_per_sm = b; trial(cand); }
            }
            apply(c, best);
            // leave the staged batch's results computed with the chosen shapes
            run_batch(c, prec, true, true);
            finish_batch(c);
            best.ms = t_best;
            best.ms_default = t_default;
            if (out) *out = best;
        } catch (...) {   // a failed search leaves the shapes the context had before it
            apply(c, prior);
            throw;
        }
    })
}

}  // extern "C"
