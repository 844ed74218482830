// bp_autotune.cu -- picks the neighbour-walk variant that runs fastest for a
// solver's scene and step configuration.
//
// The walk variants (staging each CTA's neighbourhood in shared memory,
// testing candidates in chunks before the pair terms, the post passes'
// neighbour lists), the launch shapes of the unstaged scans (threads per
// CTA, persistent CTAs), iteration fusion (plane collision and commit in the
// reorder's and the position pass's epilogues) and the contact walks' cell
// culling give bit-identical results, so the choice only affects speed.
// Each candidate runs one update from the same state (the first call of a
// configuration captures its CUDA graph; it is run once untimed), timed with
// CUDA events on the solver's stream; the state is put back after every
// trial and the fastest variant is kept in the solver's parameters.
#include "bp_solver_state.h"

using namespace bp;

extern "C" bp_status bp_solver_autotune(bp_solver *s, int32_t num_substeps, float dt, int32_t iterations,
                                        int32_t *out_walk_options, float *out_ms)
{
    if (!s) return fail_with(BP_ERR_INVALID_ARGUMENT, "solver is NULL");
    if (num_substeps <= 0 || !(dt > 0.f) || iterations < 0)
        return fail_with(BP_ERR_INVALID_ARGUMENT, "num_substeps > 0, dt > 0 and iterations >= 0 required");
    if (s->tape) return fail_with(BP_ERR_INVALID_ARGUMENT, "not available while a tape records");
    static const int32_t kCandidates[] = {0,
                                          BP_WALK_NO_STAGING,
                                          BP_WALK_NO_SPLIT,
                                          BP_WALK_NO_LISTS,
                                          BP_WALK_NO_STAGING | BP_WALK_NO_SPLIT,
                                          BP_WALK_NO_STAGING | BP_WALK_NO_LISTS,
                                          BP_WALK_NO_SPLIT | BP_WALK_NO_LISTS,
                                          BP_WALK_NO_STAGING | BP_WALK_NO_SPLIT | BP_WALK_NO_LISTS};
    constexpr int kNum = (int)(sizeof(kCandidates) / sizeof(kCandidates[0]));
    // then the launch shape of the unstaged scans, on the fastest walk variant:
    // 128 and 64 threads per CTA, and persistent 256-thread CTAs
    static const int32_t kShapes[][2] = {{128, 0}, {64, 0}, {256, 1}};
    constexpr int kNumShapes = (int)(sizeof(kShapes) / sizeof(kShapes[0]));
    constexpr int kTrials = kNum + kNumShapes + 2;  // + iteration fusion, + contact culling
    if (out_ms)
        for (int c = 0; c < kTrials; ++c) out_ms[c] = 0.f;
    if (s->n <= 0) {
        if (out_walk_options) *out_walk_options = s->prm.walk_options;
        return BP_OK;
    }
    BP_CUDA_OR_FAIL(cudaStreamSynchronize(s->stream));
    StateSnapshot snap;
    bp_status st = snap.take(s);
    if (st != BP_OK) return st;
    cudaEvent_t e0, e1;
    BP_CUDA_OR_FAIL(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return fail_with(BP_ERR_CUDA, "cudaEventCreate");
    }
    // one update with parameters p from the saved state (after an untimed one
    // that captures its graph); its time in ms, or -1 after an error (in st)
    auto trial = [&](const bp_params &p) -> float {
        if ((st = bp_solver_set_params(s, &p)) != BP_OK) return -1.f;
        if ((st = bp_solver_update(s, num_substeps, dt, iterations, -1, nullptr, nullptr)) != BP_OK) return -1.f;
        snap.restore(s);
        cudaEventRecord(e0, s->stream);
        if ((st = bp_solver_update(s, num_substeps, dt, iterations, -1, nullptr, nullptr)) != BP_OK) return -1.f;
        cudaEventRecord(e1, s->stream);
        if (cudaEventSynchronize(e1) != cudaSuccess) {
            st = fail_with(BP_ERR_CUDA, "autotune: event");
            return -1.f;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        snap.restore(s);
        return ms;
    };
    const int32_t tuned = BP_WALK_NO_SPLIT | BP_WALK_NO_LISTS | BP_WALK_NO_STAGING | BP_WALK_NO_FUSION |
                          BP_WALK_NO_CONTACT_CULLING;
    const int32_t keep = s->prm.walk_options & ~tuned;
    // the walk variants run without contact culling (as the parameters' default)
    const int32_t base = keep | BP_WALK_NO_CONTACT_CULLING;
    float best = -1.f;
    bp_params bestp = s->prm;
    for (int c = 0; c < kNum && st == BP_OK; ++c) {
        bp_params p = s->prm;
        p.walk_options = base | kCandidates[c];
        p.scan_block = 0;
        p.scan_persistent = 0;
        const float ms = trial(p);
        if (ms < 0.f) break;
        if (out_ms) out_ms[c] = ms;
        if (best < 0.f || ms < best) {
            best = ms;
            bestp = p;
        }
    }
    for (int c = 0; c < kNumShapes && st == BP_OK; ++c) {
        if (!(bestp.walk_options & BP_WALK_NO_STAGING)) break;  // staged launches keep 256-thread CTAs
        bp_params p = bestp;
        p.scan_block = kShapes[c][0];
        p.scan_persistent = kShapes[c][1];
        const float ms = trial(p);
        if (ms < 0.f) break;
        if (out_ms) out_ms[kNum + c] = ms;
        if (ms < best) {
            best = ms;
            bestp = p;
        }
    }
    bp_params shaped = bestp;  // the shape trials compare against each other; the switches below
    // need a lead of more than 1 % (smaller leads are timing noise)
    // iteration fusion split into launches of their own
    if (st == BP_OK) {
        bp_params p = shaped;
        p.walk_options |= BP_WALK_NO_FUSION;
        const float ms = trial(p);
        if (ms >= 0.f) {
            if (out_ms) out_ms[kNum + kNumShapes] = ms;
            if (ms < 0.99f * best) {
                best = ms;
                bestp = p;
            }
        }
    }
    // contact culling, where the scene has contacts
    const bool contacts = (s->prm.stage_mask & BP_STAGE_PARTICLE_COLLISION) && s->has_solid && s->hash_pos;
    if (st == BP_OK && contacts) {
        bp_params p = bestp;
        p.walk_options &= ~BP_WALK_NO_CONTACT_CULLING;
        const float ms = trial(p);
        if (ms >= 0.f) {
            if (out_ms) out_ms[kNum + kNumShapes + 1] = ms;
            if (ms < 0.99f * best) {
                best = ms;
                bestp = p;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    snap.restore(s);
    const bp_status st2 = bp_solver_set_params(s, &bestp);
    cudaStreamSynchronize(s->stream);
    if (st != BP_OK) return st;
    if (st2 != BP_OK) return st2;
    if (out_walk_options) *out_walk_options = bestp.walk_options;
    return BP_OK;
}
