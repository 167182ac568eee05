// Autotuner of the narrow phase's launch shapes on a caller's workload.
//
// Seven shapes are searched, one after the other, each by timing the call
// it shapes (one warm-up, then the median of three runs) on the context's
// own scenes:
//  * k_ccd's resident blocks per SM (1 .. the occupancy limit): fewer blocks
//    leave the FP64 pipes less contended, more hide latency;
//  * the CCD frame cache's slots per body (256 .. 4096): fewer slots clear
//    faster, more keep frames of deep searches;
//  * the CCD searches per candidate (1 .. 32, from the nodes of its
//    subdivision tree at that depth): more fill the GPU when candidates are
//    few or deep, fewer skip the nodes above that depth;
//  * one CCD search per lane (k_ccd), per warp (k_ccd_group<32>, as
//    compiled or fitted to 4 or 5 blocks per SM) or per half-warp
//    (k_ccd_group<16>, as compiled or fitted to 4 blocks per SM), first;
//  * the CCD's first time window (none, 2^-4 .. 2^-8): small windows search
//    the boxes of all candidates closer to time order, so the running minimum
//    skips more of them, each window costs a launch;
//  * the CCD boxes a search piece evaluates before it hands its pending
//    boxes to a further launch (never, 16, the built-in 64, 256): short
//    pieces spread deep searches over the GPU, each hand-off costs a launch;
//  * k_barrier_local's constraints per warp (1 .. 32): one thread per
//    constraint fills the SMs for small sets, a full warp per 32 constraints
//    shares the PSD projections for large ones.
// The choice stays in the context (Ctx::tune) for every later call.
#include <algorithm>
#include <chrono>
#include <vector>

#include "common.cuh"

namespace rigc {

int detect_and_count(Ctx& c, const double* x0, const double* x1, bool continuous, double infl);
int construct_constraints(Ctx& c, const double* x, double dhat, double dmin);
int run_ccd(Ctx& c, const double* x0, const double* x1, double toi_tol, int flags, double* toi_host,
            double* per);
int barrier_term_impl(Ctx& c, const double* x, double dhat, double dmin, int flags,
                      rigc_barrier_out* out);
int ccd_max_blocks_per_sm(int* out, int mode);
int ccd_search_mode(const Ctx& c);

namespace {

// median wall time (ms) of fn over 3 runs after one warm-up; fn ends with a
// stream synchronisation (every call timed here reads a result back)
template <class F> int median_ms(F fn, double* ms)
{
    std::vector<double> t;
    RIGC_TRY(fn());
    for (int r = 0; r < 3; r++) {
        auto a = std::chrono::steady_clock::now();
        RIGC_TRY(fn());
        auto b = std::chrono::steady_clock::now();
        t.push_back(std::chrono::duration<double, std::milli>(b - a).count());
    }
    std::sort(t.begin(), t.end());
    *ms = t[1];
    return RIGC_OK;
}

} // namespace

int autotune(Ctx& c, const double* x0, const double* x1, double dhat, double dmin,
             rigc_tune_report* rep)
{
    rigc_tune_report r {};
    c.tune = Ctx::Tune {};
    // CCD over the continuous candidates of x0 -> x1
    RIGC_TRY(detect_and_count(c, x0, x1, true, dmin / 2.0));
    auto ccd = [&]() -> int {
        double toi;
        int s = run_ccd(c, x0, x1, 1e-4, 0, &toi, nullptr);
        return (s == RIGC_ERR_QUEUE_OVERFLOW || s == RIGC_ERR_ITER_LIMIT) ? RIGC_OK : s;
    };
    RIGC_TRY(median_ms(ccd, &r.ccd_ms_default));
    double best = r.ccd_ms_default;
    // one search per lane, per warp (as compiled, at 4 or 5 blocks per SM)
    // or per half-warp (as compiled, at 4 blocks per SM); the default: per warp
    int best_mode = ccd_search_mode(c);
    for (int mode : { 0, 1, 2, 3, 4, 5 }) {
        if (mode == best_mode) continue;
        c.tune.ccd_warp = mode;
        double ms;
        RIGC_TRY(median_ms(ccd, &ms));
        if (ms < best) {
            best = ms;
            best_mode = mode;
        }
    }
    c.tune.ccd_warp = best_mode;
    // the CCD's first time window (searches of one search per lane take none)
    int best_window = -1;
    if (best_mode != 0)
        for (int w : { 0, 4, 5, 7, 8 }) {
            c.tune.ccd_window_log2 = w;
            double ms;
            RIGC_TRY(median_ms(ccd, &ms));
            if (ms < best) {
                best = ms;
                best_window = w;
            }
        }
    c.tune.ccd_window_log2 = best_window;
    int occ;
    RIGC_TRY(ccd_max_blocks_per_sm(&occ, c.tune.ccd_warp));
    int best_bps = 0;
    for (int bps = 1; bps <= occ; bps++) {
        c.tune.ccd_blocks_per_sm = bps;
        double ms;
        RIGC_TRY(median_ms(ccd, &ms));
        if (ms < best) {
            best = ms;
            best_bps = bps;
        }
    }
    c.tune.ccd_blocks_per_sm = best_bps;
    int best_slots = 0;
    for (int slots : { 256, 512, 2048, 4096 }) {
        c.tune.cache_slots_per_body = slots;
        double ms;
        RIGC_TRY(median_ms(ccd, &ms));
        if (ms < best) {
            best = ms;
            best_slots = slots;
        }
    }
    c.tune.cache_slots_per_body = best_slots;
    int best_seeds = -1;
    for (int d = 0; d <= 5; d++) {
        c.tune.ccd_seeds_log2 = d;
        double ms;
        RIGC_TRY(median_ms(ccd, &ms));
        if (ms < best) {
            best = ms;
            best_seeds = d;
        }
    }
    c.tune.ccd_seeds_log2 = best_seeds;
    int best_ho = -1;
    for (int ho : { 0, 16, 256 }) {
        c.tune.ccd_hand_off = ho;
        double ms;
        RIGC_TRY(median_ms(ccd, &ms));
        if (ms < best) {
            best = ms;
            best_ho = ho;
        }
    }
    c.tune.ccd_hand_off = best_ho;
    r.ccd_ms = best;
    // barrier terms over the constraint set at x0
    RIGC_TRY(detect_and_count(c, x0, x0, false, (dhat + dmin) / 2.0));
    RIGC_TRY(construct_constraints(c, x0, dhat, dmin));
    auto barrier = [&]() -> int {
        rigc_barrier_out o;
        return barrier_term_impl(c, x0, dhat, dmin, RIGC_GRAD | RIGC_HESS | RIGC_PROJECT_PSD, &o);
    };
    RIGC_TRY(median_ms(barrier, &r.barrier_ms_default));
    best = r.barrier_ms_default;
    int best_pw = 0;
    for (int pw : { 1, 2, 4, 8, 16, 32 }) {
        c.tune.barrier_per_warp = pw;
        double ms;
        RIGC_TRY(median_ms(barrier, &ms));
        if (ms < best) {
            best = ms;
            best_pw = pw;
        }
    }
    c.tune.barrier_per_warp = best_pw;
    r.barrier_ms = best;
    r.ccd_blocks_per_sm = c.tune.ccd_blocks_per_sm;
    r.cache_slots_per_body = c.tune.cache_slots_per_body;
    r.barrier_per_warp = c.tune.barrier_per_warp;
    r.ccd_seeds_log2 = c.tune.ccd_seeds_log2;
    r.ccd_hand_off = c.tune.ccd_hand_off;
    r.ccd_warp = c.tune.ccd_warp;
    r.ccd_window_log2 = c.tune.ccd_window_log2;
    if (rep) *rep = r;
    return RIGC_OK;
}

} // namespace rigc
