// bp_internal.h -- host-side declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "bp_common.cuh"

namespace bp {

// Counts kernel launches and, when `events` is set (bp_solver_profile),
// records a CUDA event after each one so per-stage device time can be read
// back without a profiler.
struct LaunchLog {
    int64_t count = 0;
    cudaStream_t stream = nullptr;
    int max_events = 0;
    int num_events = 0;
    cudaEvent_t *events = nullptr;
    const char **names = nullptr;
    void done(const char *name)
    {
        ++count;
        if (events && num_events < max_events) {
            cudaEventRecord(events[num_events], stream);
            names[num_events++] = name;
        }
    }
};

// ---- stable LSD radix sort of (cell key, particle index) pairs -------------
// 9-bit digits; a tile of 4096 keys per CTA (512 threads x 8 keys).
constexpr int kRadixBits = 9;
constexpr int kRadixBins = 1 << kRadixBits;
constexpr int kSortThreads = 512;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;

inline int sort_tiles(int n) { return (n + kSortTile - 1) / kSortTile; }
inline int key_bits(int D)
{
    int b = 0;
    while ((1 << b) < D) ++b;
    return 3 * b;
}
inline int sort_passes(int D) { return (key_bits(D) + kRadixBits - 1) / kRadixBits; }

// Scratch the sort needs beyond its input and output arrays.
struct SortScratch {
    int *keys_alt[2];   // n each (only [0] is needed for <= 2 passes)
    int *vals_alt[2];
    int *hist;          // kRadixBins * tiles
    int *digit_total;   // kRadixBins
};
size_t sort_scratch_bytes(int n, int D);
void sort_scratch_carve(void *base, int n, int D, SortScratch *s);

// A device-side switch for kernels captured in a graph: they do nothing
// unless *word >= min (word == nullptr: always open).
struct Gate {
    const int *word = nullptr;
    int min = 0;
};
__device__ __forceinline__ bool gate_closed(const Gate &g) { return g.word && *g.word < g.min; }

// keys_in: cell keys (pass 0 histogram already in s.hist when hist_ready);
// vals_in == nullptr means the identity permutation.
void radix_sort_pairs(cudaStream_t st, int n, int D, const int *keys_in, const int *vals_in, int *keys_out,
                      int *vals_out, const SortScratch &s, bool hist_ready, LaunchLog *L, Gate gate = Gate{});

// ---- grid kernels launched by the solver and the stand-alone API ----
void launch_hash_f3(cudaStream_t st, int n, const float *pos3, float cell, int D, int *keys, int *hist,
                    LaunchLog *L);
void launch_hash_state(cudaStream_t st, const SimConsts &C, const float4 *X, const float4 *V, int *keys,
                       int *hist, LaunchLog *L);
void launch_find_start_end(cudaStream_t st, int n, const int *sorted, int *start, int *end, LaunchLog *L);
void launch_reset_start_end(cudaStream_t st, int n, const int *sorted, int *start, int *end,
                            LaunchLog *L);
void launch_cell_offsets(cudaStream_t st, int n, int ncells, const int *sorted, int *off, LaunchLog *L,
                         Gate gate = Gate{});

struct ReorderArgs {
    const int *order;      // sorted position -> old index
    const float4 *Xc, *Vc; // state in the old order
    const int *orig_c;
    float4 *Xs, *Vs, *P;   // new order
    float *mass;
    int *orig_s, *to_new;
    float *inv_scaled;     // nullptr: not needed
    int stabilize;         // run planeStabilize twice
    int collide;           // also run iteration 0's plane collision
    int *tile_solid;       // nullptr, or flags set for 256-particle tiles holding a solid (cleared before)
    int *cls;              // nullptr, or the alias class of each sorted particle at hash time
    float4 *pos0;          // with cls: the hash-time (predicted) position of each sorted particle
    float4 *hash_pos;      // nullptr, or the same for the contact walks' reach (k_contact_reach)
};
void launch_reorder(cudaStream_t st, const SimConsts &C, const ReorderArgs &a, LaunchLog *L);

// ---- alias classes (SimConsts::cls_perm) ----
struct ClassArrays {
    int *cls;        // [n] class of each sorted particle (k_reorder)
    float4 *pos0;    // [n] hash-time positions (k_reorder)
    int *keys;       // [n] class-order keys: class * T + cell key
    int *perm;       // [n] class order -> sorted index
    int *inv;        // [n] sorted index -> class order
    int *off;        // [8 T + 1]
    float4 *pos;     // [n] P in class order
    int *mixed;      // one word: particles whose class differs from their cell's first particle's
    int *moved;      // one word
    float *mass;     // [n] masses in class order (k_class_keys)
    float2 *lm;      // [n] (lambda, mass) in class order (k_lambda, slot lists)
    float *rho;      // [n] densities in class order (k_lambda, slot lists)
    float4 *vel, *om, *nm, *vb;  // [n] each: the post passes' class-order copies (SimConsts::cls_vel ...)
    int T;           // cell keys of all scenes
    float reach2;    // squared reach (see SimConsts::cls_perm)
};
// After k_reorder: class order (one radix pass), keys, inverse, offsets and
// the count of particles in cells holding two classes (off: the cell offsets).
void launch_class_order(cudaStream_t st, int n, const int *sorted_keys, const int *off, const float *mass,
                        const ClassArrays &a, const SortScratch &s, LaunchLog *L);
// Gathers P into class order and flags particles beyond the reach.
// V != nullptr: also gathers V into a.vel (before the post passes).
// planes != nullptr: also writes the walk planes (SimConsts::walk_xyz), in
// class order where the classes are open and in sorted order where not.
void launch_class_refresh(cudaStream_t st, int n, const float4 *P, const ClassArrays &a, LaunchLog *L,
                          const float4 *V = nullptr, float *planes = nullptr, int stride = 0);
// The walk planes in sorted order (scenes without alias classes).
void launch_walk_planes(cudaStream_t st, int n, const float4 *P, float *planes, int stride, LaunchLog *L);

// ---- fluid kernels ----
void launch_lambda(cudaStream_t st, const SimConsts &C, const float4 *P, const float *mass, const int *off,
                   float *lam, float *rho, LaunchLog *L);
struct DeltaArgs {
    const float4 *P;
    const float *mass, *lam;
    const int *off;
    float4 *Pout;
    int epilogue;          // 0 none, 1 plane collision (next iteration), 2 commit (+ plane none)
    const float4 *Xs;      // x for planes / commit
    float4 *Xc, *Vc;       // commit targets
    const float4 *Vs;      // for phase bits on commit
    const int *orig_s;
    int *orig_c;
};
void launch_deltap(cudaStream_t st, const SimConsts &C, const DeltaArgs &a, LaunchLog *L);
void launch_post_a(cudaStream_t st, const SimConsts &C, const float4 *P, const float4 *V, const float *rho,
                   const int *off, float4 *Om, float4 *Nm, LaunchLog *L);
void launch_post_b(cudaStream_t st, const SimConsts &C, const float4 *P, const float4 *V, const float4 *Om,
                   const float4 *Nm, const int *off, float4 *Vout, LaunchLog *L);
void launch_post_c(cudaStream_t st, const SimConsts &C, const float4 *P, const float4 *V, const int *off,
                   const float *mass, const float *rho, float4 *Vout, LaunchLog *L);
void launch_neighbor_counts_f3(cudaStream_t st, int n, const float *pos3, float cell, int D, float h,
                               const int *start, const int *end, int *counts);

// ---- per-particle and constraint kernels ----
void launch_planes(cudaStream_t st, const SimConsts &C, const float4 *Xs, float4 *P, LaunchLog *L);
void launch_commit(cudaStream_t st, const SimConsts &C, const float4 *P, const float4 *Xs, const float4 *Vs,
                   const int *orig_s, float4 *Xc, float4 *Vc, int *orig_c, LaunchLog *L);
// tile_solid: nullptr, or one flag per 256 sorted particles (the tile holds a solid);
// solid_prefix / solid_list: nullptr, or the compacted solids (launch_solid_list)
// solids_apart: the nsolid solids of the list walk in a second launch over the list.
// solid_near: nullptr, or SolidCells::near of the same sorted order.
// solid_pos: C.n + 1 float4 of scratch (the listed solids' positions, gathered
// first); the kernels take the solid count from solid_prefix[C.n] (this
// substep's compaction), nsolid (the count at creation) only sizes launches.
// solid_walk: nullptr, or the listed solids in the order their launch takes
// them (launch_solid_list).  With C.contact_reach the contact walks visit only
// the cells a partner can be stored in (launch_contact_reach, just before).
void launch_particle_collision(cudaStream_t st, const SimConsts &C, const float4 *P, const float4 *Xs,
                               const float *w, const int *off, const int *tile_solid, const int *solid_prefix,
                               const int *solid_list, const int *solid_walk, int nsolid, bool solids_apart,
                               const unsigned long long *solid_near, float4 *solid_pos, float4 *Pout, LaunchLog *L);
// reach[0] = the bits of the largest per-axis |P - hashed| over the n
// particles, reach[1] over the solids (NaN or infinite: +inf).  With a solid
// list and fewer than n / 2 solids (nsolid: the count at creation) only the
// solids are bounded, over the list, and reach[0] = +inf: the solid walkers
// then take all 27 cells.
void launch_contact_reach(cudaStream_t st, int n, const float4 *P, const float4 *hashed, unsigned *reach,
                          LaunchLog *L, int nsolid = 0, const int *solid_prefix = nullptr,
                          const int *solid_list = nullptr);
// Bit masks over the D^3 table cells of one scene (cells == nullptr: not built):
// cells marks the stored cells (keys) of the solids, near the cells whose 27
// cells hold one.
struct SolidCells {
    int D = 0;
    const int *keys = nullptr;  // stored cell of every sorted particle
    unsigned long long *cells = nullptr, *near = nullptr;  // D^3 / 64 words each
};
// solid_prefix[i] (i <= n): solids among sorted [0, i); solid_list: their sorted indices in order.
// totals: (n + 1023) / 1024 ints of scratch.
// With walk: the listed solids again, each tile of 256 entries grouped by the
// half of its cell each one's position lies in on every axis, for the solids'
// contact launch (the warps of a group walk the same cells).
void launch_solid_list(cudaStream_t st, int n, const float4 *P, int *totals, int *solid_prefix, int *solid_list,
                       const SolidCells &sc, LaunchLog *L, int nsolid = 0, float cell = 0.f, int *walk = nullptr);
struct DistanceArgs {
    int num_edges;
    const int2 *pairs;       // original ids
    const float2 *params;    // rest length, stiffness
    int num_nodes;           // particles with incident edges
    const int *node_ids;     // original ids of those particles
    const int *node_ptr;     // CSR row pointers (num_nodes + 1)
    const int *node_inc;     // edge*2 + side
    float4 *edge_k;          // per-edge correction vector
};
void launch_distance(cudaStream_t st, const SimConsts &C, const DistanceArgs &a, float4 *P, const float *w,
                     const int *to_new, unsigned *err, LaunchLog *L);
struct BendingArgs {
    int num_quads;
    const int4 *quads;       // original ids: hinge edge (x, y), wings z and w
    float stiffness;
    int num_nodes;           // particles with incident quads
    const int *node_ids;     // original ids of those particles
    const int *node_ptr;     // CSR row pointers (num_nodes + 1)
    const int *node_inc;     // quad*4 + corner
    float4 *terms;           // per quad and corner: the correction
};
void launch_bending(cudaStream_t st, const SimConsts &C, const BendingArgs &a, float4 *P, const float *w,
                    const int *to_new, LaunchLog *L);
struct WindArgs {
    int num_faces;
    const int *faces;        // [F][3] original ids
    int num_nodes;
    const int *node_ids;
    const int *node_ptr;
    const int *node_inc;     // face index
    float4 *face_move;
};
void launch_wind(cudaStream_t st, const SimConsts &C, const WindArgs &a, float4 *P, const float4 *Vs,
                 const float *mass, const int *to_new, LaunchLog *L);
struct RigidArgs {
    int num_bodies;
    const int2 *ranges;      // original ids
    const float4 *rest;      // by original id
    float4 *rot, *cm;
};
void launch_shape_matching(cudaStream_t st, const SimConsts &C, const RigidArgs &a, float4 *P,
                           const int *to_new, LaunchLog *L);
void launch_immovable(cudaStream_t st, const SimConsts &C, int k, const int *ids, const int *to_new, const float4 *Xs,
                      float4 *P, LaunchLog *L);
void launch_pick(cudaStream_t st, int id_orig, const int *to_new, float4 *pos, float3 p, int set_pos, float4 *vel,
                 float3 v, LaunchLog *L);
void launch_pack_infos(cudaStream_t st, int n, const float4 *X, const float4 *V, void *out);
// out[3*o..] = src[i].xyz with o = map ? map[i] : i (sorted -> original when map = orig ids)
void launch_gather_xyz(cudaStream_t st, int n, const float4 *src, const int *map, float *out);
// dst[i].xyz = in[3*k..] with i = map ? map[k] : k, w kept (original -> sorted when map = to_new)
void launch_scatter_xyz(cudaStream_t st, int n, const float *in, const int *map, float4 *dst);
void launch_check_finite(cudaStream_t st, int n, const float4 *X, unsigned *err, LaunchLog *L);

// Sets the message bp_last_error_string returns on this thread.
void set_last_error(const char *msg);

}  // namespace bp
