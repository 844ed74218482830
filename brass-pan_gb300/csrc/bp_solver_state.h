// bp_solver_state.h -- the solver handle's state, shared by the step
// orchestration (bp_solver.cu) and the adjoint driver (bp_backward.cu).
#pragma once

#include <cstring>
#include <string>
#include <vector>

#include "bp_internal.h"

namespace bp {
struct SubstepTape;
struct Tape;

// Sets the message bp_last_error_string returns and passes the status on.
inline bp_status fail_with(bp_status st, const std::string &msg)
{
    set_last_error(msg.c_str());
    return st;
}
}  // namespace bp

#define BP_CUDA_OR_FAIL(call)                                                                        \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess)                                                                       \
            return bp::fail_with(e_ == cudaErrorMemoryAllocation ? BP_ERR_OUT_OF_MEMORY : BP_ERR_CUDA, \
                                 std::string(#call) + ": " + cudaGetErrorString(e_));                \
    } while (0)

using namespace bp;

namespace bp {
void destroy_tape(Tape *t);  // frees a recording (bp_backward.cu)

// Stages of a substep as recorded for the adjoint.
enum TapeStage : int {
    TS_WIND,
    TS_PLANES,
    TS_PCOLL,
    TS_FLUID,
    TS_DISTANCE,
    TS_SHAPE,
    TS_IMMOVABLE,
    TS_COMMIT,
    TS_XSPH,
    TS_POST_AB,
    TS_BENDING,
    TS_PICK  // the picked particle set to the target (no snapshot)
};
struct TapeRec {
    int stage;
    int slot;  // snapshot of the stage's input: positions, or velocities for TS_XSPH and TS_POST_AB
    // TS_FLUID: snapshots of lambda (aux) and density (aux + 1) in pool1; TS_SHAPE: the rotations after
    // it; TS_POST_AB: omega (aux) and normals (aux + 1) after pass A, and with XSPH the velocities
    // after pass B (aux + 2)
    int aux;
    int aux1 = -1;  // TS_POST_AB, TS_XSPH: the density the passes read (pool1)
};

// The intermediates of one substep re-run for its adjoint: each stage's
// input, copied into a pool of device buffers that persists across substeps.
struct SubstepTape {
    bp_solver *s = nullptr;
    std::vector<float4 *> pool4;
    std::vector<float *> pool1;
    int used4 = 0, used1 = 0;
    std::vector<TapeRec> recs;
    int vs_slot = -1;  // velocities after the reorder
    bool ok = true;    // false after a failed allocation
    void reset()
    {
        used4 = used1 = 0;
        recs.clear();
        vs_slot = -1;
    }
    int snap4(const float4 *src, size_t count = 0);  // count 0: one per particle (count <= particles)
    int snap1(const float *src);
    void push(int stage, const float4 *src, int aux = -1) { recs.push_back(TapeRec{stage, snap4(src), aux, -1}); }
    void mark(int stage) { recs.push_back(TapeRec{stage, -1, -1, -1}); }
};
}  // namespace bp

// Recorded neighbours per particle for the post passes: about 33 at rest
// density with h = 2 spacings, well over 128 in fluid compressed 2.5-fold
// (particles beyond the cap walk their cells; 64 / 128 / 192 measured
// 73.6 / 77.7 / 84.0 M particle-substeps/s over the mixed 200 frames).
#ifndef BP_POST_LIST_CAP
#define BP_POST_LIST_CAP 192
#endif
constexpr int kPostListCap = BP_POST_LIST_CAP;
static_assert(kPostListCap % 4 == 0, "lists are stored as records of four entries");

// Entries of a Verlet list (candidates within h + skin): about 1.3x the
// neighbours within h at a skin of 0.1 h (particles beyond it walk their cells).
constexpr int kVerletCap = 256;
static_assert(kVerletCap % 4 == 0, "lists are stored as records of four entries");

// Alias classes are kept for key spaces of at most this many cells (their
// offsets take 8 entries per cell: 64 MB at 2^21 cells, a 128^3 table).
constexpr size_t kClassMaxCells = size_t(1) << 21;

struct bp_solver {
    int n = 0;
    bp_params prm{};
    int nplanes = 0;
    float planes[kMaxPlanes][6];
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int device = 0;

    std::vector<void *> allocs;

    float4 *Xc = nullptr, *Vc = nullptr, *Xs = nullptr, *Vs = nullptr, *Pa = nullptr, *Pb = nullptr;
    float4 *Om = nullptr, *Nm = nullptr;
    float4 *Pcur = nullptr;  // predicted positions after the last substep
    int *orig_c = nullptr, *orig_s = nullptr, *to_new = nullptr, *group = nullptr;
    int *keys = nullptr, *sorted_keys = nullptr, *order = nullptr, *off = nullptr;
    float *mass = nullptr, *lam = nullptr, *rho = nullptr, *w = nullptr;
    float *staging = nullptr;  // 2 x N x 3 floats for host copies
    int *vl = nullptr, *vl_count = nullptr;  // Verlet lists [kVerletCap][N] (records of four), counts
    int *nl_cell = nullptr;
    float4 *nl_pos = nullptr;
    unsigned long long *nl_outlier = nullptr;  // outlier cell bits [D*D][ceil(D/64)]
    unsigned *nl_stats = nullptr;
    unsigned *err = nullptr;
    int *tile_solid = nullptr;  // per 256 sorted particles: the tile holds a solid
    int *solid_prefix = nullptr, *solid_list = nullptr, *solid_totals = nullptr;  // compacted solids
    unsigned long long *solid_cells = nullptr, *solid_near = nullptr;  // SolidCells masks (one scene with fluid)
    float4 *solid_pos = nullptr;  // positions of the compacted solids (launch_particle_collision)
    // contact walks: hash-time positions, the reach bounds and the solids'
    // walk order (allocated with solids at creation)
    float4 *hash_pos = nullptr;
    unsigned *contact_reach = nullptr;
    int *solid_walk = nullptr;
    int *nbr = nullptr, *nbr_count = nullptr;  // post-pass neighbour lists [kPostListCap][N], counts
    float2 *lm = nullptr;  // (lambda, mass) per sorted particle (SimConsts::lm)
    float *walk_xyz = nullptr;  // walk planes (SimConsts::walk_xyz): 4 planes of walk_stride floats
    int walk_stride = 0;
    SortScratch sort{};
    // alias classes (SimConsts::cls_perm); cls.perm == nullptr: not allocated
    // (key spaces above kClassMaxCells cells)
    ClassArrays cls{};
    int cls_dmin = 0;  // smallest grid dimension of the scenes

    bool has_solid = false;
    int num_solids = 0;
    size_t ncells = 0;   // cells of the key space (D^3 for one scene)
    int sort_dim = 0;    // a grid dimension whose key width covers every key (sort passes)
    // batched ensembles (num_scenes == 0: one scene)
    int num_scenes = 0;
    std::vector<int> scene_first;  // num_scenes + 1 particle offsets
    SceneConsts *scn = nullptr;
    int *scene_of = nullptr;
    DistanceArgs dist{};
    BendingArgs bend{};
    WindArgs wind{};
    RigidArgs rigid{};
    int nimm = 0;
    int *imm = nullptr;

    // graph cache
    cudaGraphExec_t exec = nullptr;
    int g_sub = -1, g_iter = -1;
    float g_dt = 0.f;
    uint64_t g_params_version = ~0ull;
    uint64_t params_version = 0;
    int64_t graph_launches = 0;
    int64_t last_launches = 0;

    bp::Tape *tape = nullptr;  // recording for bp_solver_backward (nullptr: not recording)
    bool tape_empty() const;   // no update recorded yet

    ~bp_solver()
    {
        if (tape) bp::destroy_tape(tape);
        if (exec) cudaGraphExecDestroy(exec);
        for (void *p : allocs) cudaFree(p);
        if (own_stream && stream) cudaStreamDestroy(stream);
    }

    template <class T>
    bp_status alloc(T **ptr, size_t count)
    {
        void *p = nullptr;
        const size_t bytes = count * sizeof(T) > 0 ? count * sizeof(T) : 16;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e != cudaSuccess)
            return bp::fail_with(BP_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        allocs.push_back(p);
        *ptr = (T *)p;
        return BP_OK;
    }
    template <class T>
    bp_status upload(T **ptr, const void *host, size_t count)
    {
        bp_status st = alloc(ptr, count);
        if (st != BP_OK) return st;
        if (count) BP_CUDA_OR_FAIL(cudaMemcpy(*ptr, host, count * sizeof(T), cudaMemcpyHostToDevice));
        return BP_OK;
    }
};


namespace bp {
// Substep constants of solver s for substep length sdt.
SimConsts make_consts(const bp_solver *s, float sdt);
// Records an update about to be enqueued while s->tape is open.
bp_status tape_record_update(bp_solver *s, int nsub, float dt, int iterations, int picked, float3 ppos, float3 pvel);
// Enqueues one substep on s->stream.  With a tape, the fused epilogues are
// replaced by their separate kernels and every stage's input is recorded.
void enqueue_substep(bp_solver *s, const SimConsts &C, int iterations, int picked, float3 ppos, LaunchLog *L,
                     SubstepTape *tape = nullptr);
}  // namespace bp

// Every buffer a caller can observe after an update (device pointer, bytes):
// what a later update reads (committed state, its cell-sorted order, rigid
// rotations) and what the queries return.
inline std::vector<std::pair<void *, size_t>> state_buffers(bp_solver *s)
{
    const size_t n = (size_t)s->n, nb = (size_t)s->rigid.num_bodies;
    std::vector<std::pair<void *, size_t>> bufs = {
        {s->Xc, n * 16},          {s->Vc, n * 16},       {s->Xs, n * 16},   {s->Vs, n * 16},
        {s->Pa, n * 16},          {s->Pb, n * 16},       {s->orig_c, n * 4}, {s->orig_s, n * 4},
        {s->to_new, n * 4},       {s->sorted_keys, n * 4}, {s->order, n * 4}, {s->off, (s->ncells + 1) * 4},
        {s->mass, n * 4},         {s->lam, n * 4},       {s->rho, n * 4},   {s->w, n * 4},
        {s->err, 4}};
    if (nb) {
        bufs.push_back({s->rigid.rot, nb * 16});
        bufs.push_back({s->rigid.cm, nb * 16});
    }
    return bufs;
}

// The state buffers copied aside on the device and put back (around
// backward() and the autotuner's trial updates).
struct StateSnapshot {
    std::vector<std::pair<void *, size_t>> bufs;  // solver buffer, bytes
    std::vector<void *> copies;
    float4 *pcur = nullptr;
    ~StateSnapshot()
    {
        for (void *p : copies) cudaFree(p);
    }
    bp_status take(bp_solver *s)
    {
        bufs = state_buffers(s);
        for (auto &b : bufs) {
            void *p = nullptr;
            if (cudaMalloc(&p, b.second) != cudaSuccess) return bp::fail_with(BP_ERR_OUT_OF_MEMORY, "state snapshot");
            copies.push_back(p);
            cudaMemcpyAsync(p, b.first, b.second, cudaMemcpyDeviceToDevice, s->stream);
        }
        pcur = s->Pcur;
        return BP_OK;
    }
    void restore(bp_solver *s)
    {
        for (size_t k = 0; k < bufs.size(); ++k)
            cudaMemcpyAsync(bufs[k].first, copies[k], bufs[k].second, cudaMemcpyDeviceToDevice, s->stream);
        s->Pcur = pcur;
    }
};
