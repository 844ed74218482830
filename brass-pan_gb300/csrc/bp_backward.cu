// bp_backward.cu -- differentiable rollouts: recording, checkpoints and the
// adjoint driver behind bp_solver_backward.
//
// While a tape is open, every bp_solver_update is recorded (its substep
// constants and parameters) and the state is checkpointed at the start of an
// update once `checkpoint_every` substeps have passed since the last
// checkpoint.  bp_solver_backward walks the recorded substeps backwards: per
// segment between checkpoints it re-runs the forward substeps from the
// checkpoint, keeping each substep's start state, every stage's input
// (SubstepTape) and the grid the substep ran with; then, last substep first,
// it applies the adjoint kernels of the stages in reverse order
// (bp_adjoint.cu).  Each position in a segment has its own buffers, so its
// recording re-run and its adjoint are each captured once as a CUDA graph and
// replayed for every segment.  The neighbour sets of the adjoint walks are those
// of the re-run forward pass.  Finally the solver's state is put back as it
// was before the call.
#include <algorithm>
#include <vector>

#include "bp_solver_state.h"

namespace bp {

// launchers in bp_adjoint.cu
void adj_reorder(cudaStream_t st, const SimConsts &C, const int *order, const float4 *Xprev, const float4 *Vprev,
                 int stabilize, int inv_scaled, const float4 *gP, const float4 *gXs, const float4 *gVs,
                 const float *gW, float4 *gXprev, float4 *gVprev);
void adj_planes(cudaStream_t st, const SimConsts &C, const float4 *Xs, const float4 *Pin, float4 *gP, float4 *gXs);
void adj_commit(cudaStream_t st, int n, float inv_dt, const float4 *gX, const float4 *gV, float4 *gP, float4 *gXs,
                float4 *gVs, float *gW);
void adj_immovable(cudaStream_t st, int k, const int *ids, const int *to_new, float4 *gP, float4 *gXs);
void adj_distance(cudaStream_t st, const DistanceArgs &a, const float4 *Pin, const float *w, const int *to_new,
                  float4 *gP, float *gW, float4 *G1, float4 *G2, float *g_stiff, float *g_rest);
void adj_wind(cudaStream_t st, const SimConsts &C, const WindArgs &a, const float4 *Pin, const float4 *Vs,
              const float *mass, const int *to_new, float4 *gP, float4 *gVs, float4 *FG, float4 *FV, float4 *FW,
              float4 *g_wind);
void adj_fluid(cudaStream_t st, const SimConsts &C, const float4 *Pin, const float *mass, const float *lam,
               const float *rho, const int *off, const float4 *gOut, const float *gRho, float *gLam, float4 *gPart,
               float4 *GD, float *rhob, float4 *gIn);
void adj_xsph(cudaStream_t st, const SimConsts &C, const float4 *P, const float4 *V, const int *off,
              const float *mass, const float *rho, const float4 *gVout, float4 *gVin, float4 *gX, float *gRho);
void adj_shape_matching(cudaStream_t st, const RigidArgs &a, const float4 *rot, const float4 *Pin, const int *to_new,
                        float4 *gP);
void adj_contacts(cudaStream_t st, const SimConsts &C, const float4 *Pin, const float4 *Xs, const float *w,
                  const int *off, int *count, const float4 *gOut, float4 *gIn, float4 *gXs, float *gW);
void adj_unpick(cudaStream_t st, int id, const int *to_new, float4 *g1, float4 *g2);
void adj_unpick_orig(cudaStream_t st, int n, int id, const int *orig, float4 *g1, float4 *g2);
void adj_bending(cudaStream_t st, const BendingArgs &a, float kb, const float4 *Pin, const float *w, const int *to_new,
                 float4 *gP, float *gW);
void adj_post(cudaStream_t st, const SimConsts &C, const float4 *P, const float4 *V, const float4 *Om,
              const float4 *Nm, const float *rho, const int *off, const float4 *gVb, float4 *gV, float4 *gX,
              float *gRho, float4 *etab, float4 *omb, float4 *ombo, float4 *nmb);

namespace {

// Device buffers owned by a tape (freed with it).
struct DevPool {
    std::vector<void *> ptrs;
    ~DevPool()
    {
        for (void *p : ptrs) cudaFree(p);
    }
    template <class T>
    T *get(size_t count)
    {
        void *p = nullptr;
        if (cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess) return nullptr;
        ptrs.push_back(p);
        return (T *)p;
    }
};

// The state a substep starts from.
struct StateBuf {
    float4 *X = nullptr, *V = nullptr, *rot = nullptr, *cm = nullptr;
    int *orig = nullptr;
    int *to_new = nullptr;  // the inverse of orig (picking finds the picked particle through it)
};

// What a substep leaves in the solver's buffers that its adjoint reads: the
// reordered positions, the order and maps, masses, the cell keys and offsets.
struct SubCtx {
    float4 *Xs = nullptr;
    int *order = nullptr, *to_new = nullptr, *keys = nullptr, *off = nullptr;
    float *mass = nullptr, *w = nullptr;
};

}  // namespace

struct Tape {
    int every = 1;
    struct Sub {
        SimConsts C;
        bp_params prm;
        int iterations;
        int ckpt;  // checkpoint taken at the start of this substep, or -1
        // picking (original id, or -1): the target position, and after the
        // last substep of its update (last) the velocity the particle gets
        int picked;
        float3 ppos, pvel;
        bool last;
    };
    std::vector<Sub> subs;
    std::vector<StateBuf> ckpts;
    int since = 0;
    DevPool pool;
    // per position in a segment: the substep's start state, its stage records,
    // the grid and order it ran with, and the CUDA graphs of its recording
    // re-run and of its adjoint (captured for the configuration in the keys)
    std::vector<StateBuf> seg;
    std::vector<SubstepTape *> tapes;
    std::vector<SubCtx> ctxs;
    std::vector<cudaGraphExec_t> g_fwd, g_bwd;
    std::vector<std::vector<char>> key_fwd, key_bwd, key_warm;
    // adjoint buffers
    bool grads_ready = false;
    float4 *gX = nullptr, *gV = nullptr, *gXn = nullptr, *gVn = nullptr, *gP = nullptr, *gP2 = nullptr;
    float4 *gXs = nullptr, *gVs = nullptr, *gPart = nullptr;
    float *gW = nullptr, *gLam = nullptr;
    float4 *G1 = nullptr, *G2 = nullptr, *FG = nullptr, *FV = nullptr, *FW = nullptr, *g_wind = nullptr;
    float *g_stiff = nullptr, *g_rest = nullptr;
    int *contacts = nullptr;  // per particle: its friction contacts (the collision adjoint's pass A)
    // the post passes' adjoint: density gradient (read by the last fluid stage's adjoint), eta-bar,
    // omega-bar of the confinement term, full omega-bar, normal-bar
    float *gRho = nullptr;
    float4 *etab = nullptr, *omb = nullptr, *ombo = nullptr, *nmb = nullptr;
    // the textbook fluid adjoint: (G, D-bar) and rho-bar per particle
    float4 *GD = nullptr;
    float *rhob = nullptr;
};

void destroy_tape(Tape *t)
{
    if (!t) return;
    for (cudaGraphExec_t g : t->g_fwd)
        if (g) cudaGraphExecDestroy(g);
    for (cudaGraphExec_t g : t->g_bwd)
        if (g) cudaGraphExecDestroy(g);
    for (SubstepTape *st : t->tapes) {
        for (float4 *p : st->pool4) cudaFree(p);
        for (float *p : st->pool1) cudaFree(p);
        delete st;
    }
    delete t;
}

int SubstepTape::snap4(const float4 *src, size_t count)
{
    if (count == 0) count = (size_t)s->n;
    if (used4 == (int)pool4.size()) {
        void *p = nullptr;
        if (cudaMalloc(&p, (size_t)std::max(s->n, 1) * sizeof(float4)) != cudaSuccess) {
            ok = false;
            return -1;
        }
        pool4.push_back((float4 *)p);
    }
    cudaMemcpyAsync(pool4[used4], src, count * sizeof(float4), cudaMemcpyDeviceToDevice, s->stream);
    return used4++;
}

int SubstepTape::snap1(const float *src)
{
    if (used1 == (int)pool1.size()) {
        void *p = nullptr;
        if (cudaMalloc(&p, (size_t)std::max(s->n, 1) * sizeof(float)) != cudaSuccess) {
            ok = false;
            return -1;
        }
        pool1.push_back((float *)p);
    }
    cudaMemcpyAsync(pool1[used1], src, (size_t)s->n * sizeof(float), cudaMemcpyDeviceToDevice, s->stream);
    return used1++;
}

namespace {

bool alloc_state(Tape &t, const bp_solver *s, StateBuf &b)
{
    const int nb = s->rigid.num_bodies;
    b.X = t.pool.get<float4>(s->n);
    b.V = t.pool.get<float4>(s->n);
    b.orig = t.pool.get<int>(s->n);
    b.to_new = t.pool.get<int>(s->n);
    b.rot = t.pool.get<float4>(nb);
    b.cm = t.pool.get<float4>(nb);
    return b.X && b.V && b.orig && b.to_new && b.rot && b.cm;
}

void save_state(const bp_solver *s, const StateBuf &b)
{
    const size_t n = (size_t)s->n;
    cudaMemcpyAsync(b.X, s->Xc, n * sizeof(float4), cudaMemcpyDeviceToDevice, s->stream);
    cudaMemcpyAsync(b.V, s->Vc, n * sizeof(float4), cudaMemcpyDeviceToDevice, s->stream);
    cudaMemcpyAsync(b.orig, s->orig_c, n * sizeof(int), cudaMemcpyDeviceToDevice, s->stream);
    cudaMemcpyAsync(b.to_new, s->to_new, n * sizeof(int), cudaMemcpyDeviceToDevice, s->stream);
    if (s->rigid.num_bodies > 0) {
        const size_t nb = (size_t)s->rigid.num_bodies;
        cudaMemcpyAsync(b.rot, s->rigid.rot, nb * sizeof(float4), cudaMemcpyDeviceToDevice, s->stream);
        cudaMemcpyAsync(b.cm, s->rigid.cm, nb * sizeof(float4), cudaMemcpyDeviceToDevice, s->stream);
    }
}

void load_state(bp_solver *s, const StateBuf &b)
{
    const size_t n = (size_t)s->n;
    cudaMemcpyAsync(s->Xc, b.X, n * sizeof(float4), cudaMemcpyDeviceToDevice, s->stream);
    cudaMemcpyAsync(s->Vc, b.V, n * sizeof(float4), cudaMemcpyDeviceToDevice, s->stream);
    cudaMemcpyAsync(s->orig_c, b.orig, n * sizeof(int), cudaMemcpyDeviceToDevice, s->stream);
    cudaMemcpyAsync(s->to_new, b.to_new, n * sizeof(int), cudaMemcpyDeviceToDevice, s->stream);
    if (s->rigid.num_bodies > 0) {
        const size_t nb = (size_t)s->rigid.num_bodies;
        cudaMemcpyAsync(s->rigid.rot, b.rot, nb * sizeof(float4), cudaMemcpyDeviceToDevice, s->stream);
        cudaMemcpyAsync(s->rigid.cm, b.cm, nb * sizeof(float4), cudaMemcpyDeviceToDevice, s->stream);
    }
}

bool alloc_ctx(Tape &t, const bp_solver *s, SubCtx &c)
{
    const size_t n = (size_t)s->n;
    c.Xs = t.pool.get<float4>(n);
    c.order = t.pool.get<int>(n);
    c.to_new = t.pool.get<int>(n);
    c.keys = t.pool.get<int>(n);
    c.off = t.pool.get<int>(s->ncells + 1);
    c.mass = t.pool.get<float>(n);
    c.w = t.pool.get<float>(n);
    return c.Xs && c.order && c.to_new && c.keys && c.off && c.mass && c.w;
}

// direction: true saves the solver's buffers into c, false loads them back
void copy_ctx(bp_solver *s, const SubCtx &c, bool save)
{
    const size_t n = (size_t)s->n;
    auto cp = [&](void *solver_buf, void *ctx_buf, size_t bytes) {
        cudaMemcpyAsync(save ? ctx_buf : solver_buf, save ? solver_buf : ctx_buf, bytes, cudaMemcpyDeviceToDevice,
                        s->stream);
    };
    cp(s->Xs, c.Xs, n * sizeof(float4));
    cp(s->order, c.order, n * sizeof(int));
    cp(s->to_new, c.to_new, n * sizeof(int));
    cp(s->sorted_keys, c.keys, n * sizeof(int));
    cp(s->off, c.off, (s->ncells + 1) * sizeof(int));
    cp(s->mass, c.mass, n * sizeof(float));
    cp(s->w, c.w, n * sizeof(float));
}

bool stage_on(const bp_params &p, int bit) { return (p.stage_mask & bit) != 0; }

bp_status ensure_grads(Tape &t, const bp_solver *s)
{
    if (t.grads_ready) return BP_OK;
    const size_t n = (size_t)s->n;
    const size_t m = (size_t)s->dist.num_edges, f = (size_t)s->wind.num_faces;
    t.gX = t.pool.get<float4>(n);
    t.gV = t.pool.get<float4>(n);
    t.gXn = t.pool.get<float4>(n);
    t.gVn = t.pool.get<float4>(n);
    t.gP = t.pool.get<float4>(n);
    t.gP2 = t.pool.get<float4>(n);
    t.gXs = t.pool.get<float4>(n);
    t.gVs = t.pool.get<float4>(n);
    t.gPart = t.pool.get<float4>(n);
    t.gW = t.pool.get<float>(n);
    t.gLam = t.pool.get<float>(n);
    t.G1 = t.pool.get<float4>(m);
    t.G2 = t.pool.get<float4>(m);
    t.FG = t.pool.get<float4>(3 * f);
    t.FV = t.pool.get<float4>(f);
    t.FW = t.pool.get<float4>(f);
    t.g_wind = t.pool.get<float4>(1);
    t.g_stiff = t.pool.get<float>(m);
    t.g_rest = t.pool.get<float>(m);
    t.contacts = t.pool.get<int>(n);
    t.gRho = t.pool.get<float>(n);
    t.etab = t.pool.get<float4>(n);
    t.omb = t.pool.get<float4>(n);
    t.ombo = t.pool.get<float4>(n);
    t.nmb = t.pool.get<float4>(n);
    t.GD = t.pool.get<float4>(n);
    t.rhob = t.pool.get<float>(n);
    if (!(t.gX && t.gV && t.gXn && t.gVn && t.gP && t.gP2 && t.gXs && t.gVs && t.gPart && t.gW && t.gLam && t.G1 &&
          t.G2 && t.FG && t.FV && t.FW && t.g_wind && t.g_stiff && t.g_rest && t.contacts && t.gRho && t.etab &&
          t.omb && t.ombo && t.nmb && t.GD && t.rhob))
        return fail_with(BP_ERR_OUT_OF_MEMORY, "backward: gradient buffers");
    t.grads_ready = true;
    return BP_OK;
}

// The adjoint of one substep whose taped re-run just finished; (gX, gV) are
// the gradients w.r.t. its committed state on entry and w.r.t. its start
// state (start.X, start.V, in the previous order) on exit.  Every buffer
// keeps its role (results are copied back rather than swapped), so the
// sequence can be captured once and replayed for every substep.
void adjoint_substep(bp_solver *s, Tape &t, const Tape::Sub &u, const StateBuf &start, const SubstepTape &T)
{
    const cudaStream_t st = s->stream;
    SimConsts C = u.C;  // the adjoint walks take the 27 cells, recording their pairs in the list buffer
    C.vl = nullptr;
    C.nl_pos = nullptr;
    C.nl_stats = nullptr;
    // nor the alias classes: their class-order positions are gathered only
    // for the forward walks (the same candidates in the same order remain)
    C.cls_perm = nullptr;
    C.cls_post = 0;
    if (!(u.prm.walk_options & BP_WALK_NO_LISTS)) {
        C.nbr = s->nbr;
        C.nbr_count = s->nbr_count;  // the fluid adjoint's pass A leaves its lists for pass B
        C.nbr_cap = kPostListCap;
    }
    const bp_params &p = u.prm;
    const bool planes = stage_on(p, BP_STAGE_PLANES) && s->nplanes > 0;
    const bool distance = stage_on(p, BP_STAGE_DISTANCE) && s->dist.num_edges > 0;
    const bool pcoll = stage_on(p, BP_STAGE_PARTICLE_COLLISION) && s->has_solid;
    const bool bending = stage_on(p, BP_STAGE_BENDING) && s->bend.num_quads > 0;
    // the post passes' and XSPH's density gradient, for the last fluid stage (the density they read)
    cudaMemsetAsync(t.gRho, 0, (size_t)s->n * sizeof(float), st);
    bool last_fluid = true;
    // the velocity the update gave the picked particle after its last substep
    if (u.last && u.picked >= 0) adj_unpick(st, u.picked, s->to_new, t.gV, nullptr);
    for (int r = (int)T.recs.size() - 1; r >= 0; --r) {
        const TapeRec &rec = T.recs[r];
        switch (rec.stage) {
        case TS_POST_AB: {  // positions: the commit's input; velocities before pass A in the slot
            int c = r - 1;
            while (c >= 0 && T.recs[c].stage != TS_COMMIT) --c;
            const float4 *Pc = T.pool4[T.recs[c].slot];
            const size_t bytes = (size_t)s->n * sizeof(float4);
            const float *rho = T.pool1[rec.aux1];
            if (C.use_xsph) {  // pass C first: gV -> the gradient of pass B's velocities
                adj_xsph(st, C, Pc, T.pool4[rec.aux + 2], s->off, s->mass, rho, t.gV, t.gVn, t.gX, t.gRho);
                cudaMemcpyAsync(t.gV, t.gVn, bytes, cudaMemcpyDeviceToDevice, st);
            }
            adj_post(st, C, Pc, T.pool4[rec.slot], T.pool4[rec.aux], T.pool4[rec.aux + 1], rho, s->off, t.gV, t.gVn,
                     t.gX, t.gRho, t.etab, t.omb, t.ombo, t.nmb);
            cudaMemcpyAsync(t.gV, t.gVn, bytes, cudaMemcpyDeviceToDevice, st);
            break;
        }
        case TS_PICK:  // the iteration's target position
            adj_unpick(st, u.picked, s->to_new, t.gP, nullptr);
            break;
        case TS_BENDING:
            adj_bending(st, s->bend, p.bending_stiffness, T.pool4[rec.slot], s->w, s->to_new, t.gP, t.gW);
            break;
        case TS_XSPH: {  // velocities before XSPH in the slot; positions: the commit's input
            int c = r - 1;
            while (c >= 0 && T.recs[c].stage != TS_COMMIT) --c;
            adj_xsph(st, C, T.pool4[T.recs[c].slot], T.pool4[rec.slot], s->off, s->mass, T.pool1[rec.aux1], t.gV,
                     t.gVn, t.gX, t.gRho);
            cudaMemcpyAsync(t.gV, t.gVn, (size_t)s->n * sizeof(float4), cudaMemcpyDeviceToDevice, st);
            break;
        }
        case TS_COMMIT:
            adj_commit(st, s->n, C.inv_dt, t.gX, t.gV, t.gP, t.gXs, t.gVs, t.gW);
            break;
        case TS_IMMOVABLE:
            adj_immovable(st, s->nimm, s->imm, s->to_new, t.gP, t.gXs);
            break;
        case TS_DISTANCE:
            adj_distance(st, s->dist, T.pool4[rec.slot], s->w, s->to_new, t.gP, t.gW, t.G1, t.G2, t.g_stiff,
                         t.g_rest);
            break;
        case TS_FLUID:
            adj_fluid(st, C, T.pool4[rec.slot], s->mass, T.pool1[rec.aux], T.pool1[rec.aux + 1], s->off, t.gP,
                      last_fluid ? t.gRho : nullptr, t.gLam, t.gPart, t.GD, t.rhob, t.gP2);
            last_fluid = false;
            cudaMemcpyAsync(t.gP, t.gP2, (size_t)s->n * sizeof(float4), cudaMemcpyDeviceToDevice, st);
            break;
        case TS_PLANES:
            adj_planes(st, C, s->Xs, T.pool4[rec.slot], t.gP, t.gXs);
            break;
        case TS_PCOLL:
            adj_contacts(st, C, T.pool4[rec.slot], s->Xs, s->w, s->off, t.contacts, t.gP, t.gP2, t.gXs, t.gW);
            cudaMemcpyAsync(t.gP, t.gP2, (size_t)s->n * sizeof(float4), cudaMemcpyDeviceToDevice, st);
            break;
        case TS_SHAPE:
            adj_shape_matching(st, s->rigid, T.pool4[rec.aux], T.pool4[rec.slot], s->to_new, t.gP);
            break;
        case TS_WIND:
            adj_wind(st, C, s->wind, T.pool4[rec.slot], T.pool4[T.vs_slot], s->mass, s->to_new, t.gP, t.gVs, t.FG,
                     t.FV, t.FW, t.g_wind);
            break;
        default:  // excluded by check_supported
            break;
        }
    }
    const int inv_scaled = (distance || bending || pcoll) ? 1 : 0;  // the stages that read w
    adj_reorder(st, C, s->order, start.X, start.V, planes ? 1 : 0, inv_scaled, t.gP, t.gXs, t.gVs, t.gW, t.gXn,
                t.gVn);
    cudaMemcpyAsync(t.gX, t.gXn, (size_t)s->n * sizeof(float4), cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(t.gV, t.gVn, (size_t)s->n * sizeof(float4), cudaMemcpyDeviceToDevice, st);
    // the substep began by setting the picked particle's position and velocity
    if (u.picked >= 0) adj_unpick_orig(st, s->n, u.picked, start.orig, t.gX, t.gV);
}

// The bytes a captured substep depends on: its constants, iteration count and
// parameters (buffer pointers inside them are the solver's own, fixed).
std::vector<char> sub_key(const Tape::Sub &u)
{
    const float pick[8] = {(float)u.picked, u.ppos.x, u.ppos.y, u.ppos.z, u.pvel.x, u.pvel.y, u.pvel.z,
                           u.last ? 1.f : 0.f};
    std::vector<char> k(sizeof(SimConsts) + sizeof(int) + sizeof(bp_params) + sizeof(pick));
    char *p = k.data();
    memcpy(p, &u.C, sizeof(SimConsts));
    memcpy(p += sizeof(SimConsts), &u.iterations, sizeof(int));
    memcpy(p += sizeof(int), &u.prm, sizeof(bp_params));
    memcpy(p += sizeof(bp_params), pick, sizeof(pick));
    return k;
}

// Launches the graph of `enqueue` (captured again when the substep differs
// from the captured one).
template <class F>
bp_status replay(bp_solver *s, cudaGraphExec_t &exec, std::vector<char> &key, const Tape::Sub &u, F &&enqueue)
{
    std::vector<char> k = sub_key(u);
    if (!exec || k != key) {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return BP_ERR_CUDA;
        enqueue();
        if (cudaStreamEndCapture(s->stream, &g) != cudaSuccess) return BP_ERR_CUDA;
        const cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return BP_ERR_CUDA;
        key = k;
    }
    return cudaGraphLaunch(exec, s->stream) == cudaSuccess ? BP_OK : BP_ERR_CUDA;
}

}  // namespace

// Called by bp_solver_update before it enqueues an update while a tape is open.
bp_status tape_record_update(bp_solver *s, int nsub, float dt, int iterations, int picked, float3 ppos, float3 pvel)
{
    Tape &t = *s->tape;
    int ck = -1;
    if (t.subs.empty() || t.since >= t.every) {
        StateBuf b;
        if (!alloc_state(t, s, b)) return fail_with(BP_ERR_OUT_OF_MEMORY, "tape: checkpoint");
        save_state(s, b);
        t.ckpts.push_back(b);
        ck = (int)t.ckpts.size() - 1;
        t.since = 0;
    }
    const SimConsts C = make_consts(s, dt / (float)nsub);
    for (int k = 0; k < nsub; ++k)
        t.subs.push_back(Tape::Sub{C, s->prm, iterations, k == 0 ? ck : -1, picked, ppos, pvel, k == nsub - 1});
    t.since += nsub;
    return BP_OK;
}

}  // namespace bp

using namespace bp;

bool bp_solver::tape_empty() const { return !tape || tape->subs.empty(); }

extern "C" bp_status bp_solver_tape_begin(bp_solver *s, int32_t checkpoint_every)
{
    if (!s) return fail_with(BP_ERR_INVALID_ARGUMENT, "solver is NULL");
    if (checkpoint_every <= 0) return fail_with(BP_ERR_INVALID_ARGUMENT, "checkpoint_every must be positive");
    if (s->tape) destroy_tape(s->tape);
    s->tape = new (std::nothrow) Tape();
    if (!s->tape) return fail_with(BP_ERR_OUT_OF_MEMORY, "tape");
    s->tape->every = checkpoint_every;
    return BP_OK;
}

extern "C" bp_status bp_solver_tape_end(bp_solver *s)
{
    if (!s) return fail_with(BP_ERR_INVALID_ARGUMENT, "solver is NULL");
    if (s->stream) cudaStreamSynchronize(s->stream);
    destroy_tape(s->tape);
    s->tape = nullptr;
    return BP_OK;
}

extern "C" bp_status bp_solver_backward(bp_solver *s, const float *grad_positions, const float *grad_velocities,
                                        bp_gradients *out)
{
    if (!s || !out) return fail_with(BP_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!s->tape || s->tape->subs.empty()) return fail_with(BP_ERR_INVALID_ARGUMENT, "backward: nothing recorded");
    Tape &t = *s->tape;
    bp_status stt;
    if ((stt = ensure_grads(t, s)) != BP_OK) return stt;
    const cudaStream_t st = s->stream;
    const int n = s->n;
    const size_t N = (size_t)n;
    BP_CUDA_OR_FAIL(cudaStreamSynchronize(st));
    StateSnapshot snap;
    if ((stt = snap.take(s)) != BP_OK) return stt;

    // incoming gradients, original order -> the final state's sorted order
    cudaMemsetAsync(t.gX, 0, N * sizeof(float4), st);
    cudaMemsetAsync(t.gV, 0, N * sizeof(float4), st);
    if (grad_positions) {
        cudaMemcpyAsync(s->staging, grad_positions, N * 12, cudaMemcpyHostToDevice, st);
        launch_scatter_xyz(st, n, s->staging, s->to_new, t.gX);
    }
    if (grad_velocities) {
        cudaMemcpyAsync(s->staging + 3 * N, grad_velocities, N * 12, cudaMemcpyHostToDevice, st);
        launch_scatter_xyz(st, n, s->staging + 3 * N, s->to_new, t.gV);
    }
    cudaMemsetAsync(t.g_stiff, 0, std::max(s->dist.num_edges, 1) * sizeof(float), st);
    cudaMemsetAsync(t.g_rest, 0, std::max(s->dist.num_edges, 1) * sizeof(float), st);
    cudaMemsetAsync(t.g_wind, 0, sizeof(float4), st);

    const bp_params saved_prm = s->prm;
    LaunchLog L;
    L.stream = st;
    auto bail = [&](bp_status e, const char *msg) {
        s->prm = saved_prm;
        snap.restore(s);
        return fail_with(e, msg);
    };
    int seg_end = (int)t.subs.size();
    while (seg_end > 0) {
        int seg_begin = seg_end - 1;
        while (t.subs[seg_begin].ckpt < 0) --seg_begin;  // substep 0 always holds checkpoint 0
        const int len = seg_end - seg_begin;
        while ((int)t.seg.size() < len) {
            StateBuf b;
            SubCtx c;
            SubstepTape *tp = new (std::nothrow) SubstepTape();
            if (!tp || !alloc_state(t, s, b) || !alloc_ctx(t, s, c)) {
                delete tp;
                return bail(BP_ERR_OUT_OF_MEMORY, "backward: segment buffers");
            }
            tp->s = s;
            t.seg.push_back(b);
            t.ctxs.push_back(c);
            t.tapes.push_back(tp);
            t.g_fwd.push_back(nullptr);
            t.g_bwd.push_back(nullptr);
            t.key_fwd.emplace_back();
            t.key_bwd.emplace_back();
            t.key_warm.emplace_back();
        }
        // forward from the checkpoint, recording every substep: its start
        // state, each stage's input and the grid it ran with
        load_state(s, t.ckpts[t.subs[seg_begin].ckpt]);
        for (int k = seg_begin; k < seg_end; ++k) {
            const int q = k - seg_begin;
            const Tape::Sub &u = t.subs[k];
            s->prm = u.prm;
            auto body = [&] {
                save_state(s, t.seg[q]);
                t.tapes[q]->reset();
                enqueue_substep(s, u.C, u.iterations, u.picked, u.ppos, &L, t.tapes[q]);
                if (u.last && u.picked >= 0)  // the end of its update: the picked particle's velocity
                    launch_pick(s->stream, u.picked, s->to_new, s->Xc, u.ppos, 0, s->Vc, u.pvel, &L);
                copy_ctx(s, t.ctxs[q], true);
            };
            if (sub_key(u) != t.key_warm[q]) {  // a new configuration runs once directly, growing
                body();                          // the record pool outside any capture
                if (!t.tapes[q]->ok) return bail(BP_ERR_OUT_OF_MEMORY, "backward: stage records");
                t.key_warm[q] = sub_key(u);
            } else {
                const bp_status e = replay(s, t.g_fwd[q], t.key_fwd[q], u, body);
                if (e != BP_OK) return bail(e, "backward: recording graph");
            }
        }
        // last substep first: the adjoint of each, on the grid it ran with
        for (int k = seg_end - 1; k >= seg_begin; --k) {
            const int q = k - seg_begin;
            const Tape::Sub &u = t.subs[k];
            s->prm = u.prm;
            const bp_status e = replay(s, t.g_bwd[q], t.key_bwd[q], u, [&] {
                copy_ctx(s, t.ctxs[q], false);
                adjoint_substep(s, t, u, t.seg[q], *t.tapes[q]);
            });
            if (e != BP_OK) return bail(e, "backward: adjoint graph");
        }
        seg_end = seg_begin;
    }
    s->prm = saved_prm;

    // gradients w.r.t. the state at tape_begin, in its order -> original order
    const int *orig0 = t.ckpts[0].orig;
    bp_status result = BP_OK;
    if (out->positions) {
        launch_gather_xyz(st, n, t.gX, orig0, s->staging);
        cudaMemcpyAsync(out->positions, s->staging, N * 12, cudaMemcpyDeviceToHost, st);
    }
    if (out->velocities) {
        launch_gather_xyz(st, n, t.gV, orig0, s->staging + 3 * N);
        cudaMemcpyAsync(out->velocities, s->staging + 3 * N, N * 12, cudaMemcpyDeviceToHost, st);
    }
    const size_t m = (size_t)s->dist.num_edges;
    if (out->distance_stiffness && m)
        cudaMemcpyAsync(out->distance_stiffness, t.g_stiff, m * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (out->distance_rest_length && m)
        cudaMemcpyAsync(out->distance_rest_length, t.g_rest, m * sizeof(float), cudaMemcpyDeviceToHost, st);
    float4 gw = make_float4(0.f, 0.f, 0.f, 0.f);
    cudaMemcpyAsync(&gw, t.g_wind, sizeof(float4), cudaMemcpyDeviceToHost, st);
    snap.restore(s);
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) result = fail_with(BP_ERR_CUDA, std::string("backward: ") + cudaGetErrorString(e));
    if (out->wind_velocity) {
        out->wind_velocity[0] = gw.x;
        out->wind_velocity[1] = gw.y;
        out->wind_velocity[2] = gw.z;
    }
    if (result == BP_OK) {
        const cudaError_t le = cudaGetLastError();
        if (le != cudaSuccess) result = fail_with(BP_ERR_CUDA, std::string("backward: ") + cudaGetErrorString(le));
    }
    return result;
}
