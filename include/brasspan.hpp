// brasspan.hpp -- C++ mirror of the reference's Scene / ParticleSolver API over
// the C ABI in brasspan.h (header only).
//
// Host code written against brass-pan (brasstower/scene.h, particlesolver.cuh)
// ports with the same names:
//
//   brasspan::Scene scene;                       // scene.h:455 (Scene)
//   scene.addFluidBlock(...); scene.addCloth(...); scene.addRigidBox(...);
//   brasspan::ParticleSolver solver(scene);      // particlesolver.cuh:148
//   solver.update(2, 1.f / 60.f);                // particlesolver.cuh:772
//   solver.queryNewParticleId(id);               // particlesolver.cuh:360
//
// Status codes of the C ABI become std::runtime_error here, as the reference
// throws std::exception on capacity errors (particlesolver.cuh:398-402).
#pragma once

#include <cmath>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "brasspan.h"

namespace brasspan {

struct float3_ {
    float x, y, z;
};

inline void check(bp_status st)
{
    if (st != BP_OK) throw std::runtime_error(std::string("brasspan: ") + bp_last_error_string());
}

// Flat scene vectors in original particle order plus the add* builders.
// Phases and ids follow ParticleSolver's add* methods (particlesolver.cuh:395-710):
// one negative phase per fluid block, one solid phase per self-colliding
// particle (granulars, ropes, cloths) or per rigid body, ids offset by the
// particle count before the object.
class Scene {
public:
    float particleRadius = 0.05f;                   // scene.h:500
    float fluidKernelRadius = 2.3f * 0.05f;         // scene.h:501
    float cellSize = 0.05f * 2.3f;
    int gridDim = 512;
    float fluidRestDensity = 1200.0f;

    std::vector<float> positions;  // [N][3]
    std::vector<float> velocities; // [N][3] (empty: zero)
    std::vector<float> masses;
    std::vector<int> phases;
    std::vector<int> groupIds;
    std::vector<float> planes;     // [P][6]
    std::vector<int> faces;        // [F][3]
    std::vector<float> rigidbodyInitialPositions;  // [N][3] by particle id
    std::vector<int> rigidbodyParticleIdRanges;    // [B][2]
    std::vector<int> distancePairs;                // [M][2]
    std::vector<float> distanceParams;             // [M][2]
    std::vector<int> immovableConstraints;
    std::vector<int> bendingConstraints;  // [Q][4]: "bending constraints - record all 4 ids" (scene.h:527-528)

    int groupIdCounter = 0;
    int solidPhaseCounter = 1;   // scene.h:534
    int fluidPhaseCounter = -1;  // scene.h:535

    int numParticles() const { return (int)masses.size(); }

    void addPlane(float3_ origin, float3_ normal)
    {
        const float row[6] = {origin.x, origin.y, origin.z, normal.x, normal.y, normal.z};
        planes.insert(planes.end(), row, row + 6);
    }

    // CreateFluidBlock + addFluids (scene.h:122-139, particlesolver.cuh:480-507)
    std::pair<int, int> addFluidBlock(const int dim[3], float3_ start, float3_ step, float mass)
    {
        const int n0 = numParticles();
        lattice(dim, start, step, mass, [&](int) { return fluidPhaseCounter; }, nullptr);
        fluidPhaseCounter -= 1;
        return {n0, numParticles()};
    }

    // Scene::addGranularsBlock (scene.cpp:130-146)
    std::pair<int, int> addGranularsBlock(const int dim[3], float3_ start, float3_ step, float mass)
    {
        const int n0 = numParticles();
        lattice(dim, start, step, mass, [&](int) { return solidPhaseCounter++; }, nullptr);
        return {n0, numParticles()};
    }

    // RigidBody::CreateRigidBox + addRigidBody (scene.h:51-85, particlesolver.cuh:424-478)
    std::pair<int, int> addRigidBox(const int dim[3], float3_ start, float3_ step, float mass)
    {
        const int n0 = numParticles();
        const int phase = solidPhaseCounter++;
        lattice(dim, start, step, mass, [&](int) { return phase; }, nullptr);
        const int n1 = numParticles();
        double c[3] = {0, 0, 0};
        for (int i = n0; i < n1; ++i)
            for (int a = 0; a < 3; ++a) c[a] += positions[3 * i + a];
        for (int a = 0; a < 3; ++a) c[a] /= (n1 - n0);
        for (int i = n0; i < n1; ++i)
            for (int a = 0; a < 3; ++a) rigidbodyInitialPositions[3 * i + a] = positions[3 * i + a] - (float)c[a];
        rigidbodyParticleIdRanges.push_back(n0);
        rigidbodyParticleIdRanges.push_back(n1);
        return {n0, n1};
    }

    // Rope::CreateRope + addNoodles (scene.h:141-179, particlesolver.cuh:510-573)
    std::pair<int, int> addRope(float3_ start, float3_ end, int numJoint, float mass)
    {
        const int n0 = numParticles();
        const float d[3] = {end.x - start.x, end.y - start.y, end.z - start.z};
        const float len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) / float(numJoint - 1);
        for (int i = 0; i < numJoint; ++i) {
            const float t = float(i) / float(numJoint - 1);
            push(start.x + t * d[0], start.y + t * d[1], start.z + t * d[2], mass, solidPhaseCounter++);
        }
        groupIdCounter++;
        for (int i = 0; i < numJoint - 1; ++i) pair(n0 + i, n0 + i + 1, len, 1.0f);
        for (int i = 1; i < numJoint - 1; ++i) pair(n0 + i - 1, n0 + i + 1, len * 2.0f, 0.1f);
        return {n0, numParticles()};
    }

    // Cloth::CreateCloth + addCloth (scene.h:226-330, particlesolver.cuh:576-710)
    std::pair<int, int> addCloth(float3_ start, float3_ offsetX, float3_ offsetY, int nx, int ny, float mass,
                                 bool c0 = false, bool c1 = false, bool c2 = false, bool c3 = false,
                                 float stretch = 0.2f, float shear = 0.2f, float bend = 0.1f,
                                 bool dihedral = false)
    {
        const int n0 = numParticles();
        const float lx = norm(offsetX), ly = norm(offsetY);
        const float3_ xy = {offsetX.x + offsetY.x, offsetX.y + offsetY.y, offsetX.z + offsetY.z};
        const float ld = norm(xy);
        if (c0) immovableConstraints.push_back(n0 + 0);
        if (c1) immovableConstraints.push_back(n0 + nx - 1);
        if (c2) immovableConstraints.push_back(n0 + nx * (ny - 1));
        if (c3) immovableConstraints.push_back(n0 + nx * ny - 1);
        for (int x = 0; x < nx; ++x)
            for (int y = 0; y < ny; ++y) {
                push(start.x + float(y) * offsetX.x + float(x) * offsetY.x,
                     start.y + float(y) * offsetX.y + float(x) * offsetY.y,
                     start.z + float(y) * offsetX.z + float(x) * offsetY.z, mass, solidPhaseCounter++);
                const int p1 = y * nx + x, p2 = y * nx + x + 1, p3 = (y + 1) * nx + x, p4 = (y + 1) * nx + x + 1;
                if (x < nx - 1 && y < ny - 1) {
                    const int f[6] = {p1, p2, p3, p2, p3, p4};
                    for (int k = 0; k < 6; ++k) faces.push_back(n0 + f[k]);
                    if (dihedral) {  // the commented-out quads of scene.h:308-320
                        const int odd[4] = {p3, p2, p1, p4}, even[4] = {p1, p4, p3, p2};
                        for (int k = 0; k < 4; ++k) bendingConstraints.push_back(n0 + ((x + y) % 2 ? odd[k] : even[k]));
                    }
                }
                if (x < nx - 1) pair(n0 + p1, n0 + p2, lx, stretch);
                if (y < ny - 1) pair(n0 + p1, n0 + p3, ly, stretch);
                if (x < nx - 1 && y < ny - 1) {
                    pair(n0 + p1, n0 + p4, ld, shear);
                    pair(n0 + p2, n0 + p3, ld, shear);
                }
                if (x > 0 && y > 0 && x < nx - 1 && y < ny - 1) {
                    int q[3][3];
                    for (int i = -1; i <= 1; ++i)
                        for (int j = -1; j <= 1; ++j) q[i + 1][j + 1] = (y + i) * nx + x + j;
                    for (int i = 0; i < 3; ++i) pair(n0 + q[i][0], n0 + q[i][2], lx * 2, bend);
                    for (int i = 0; i < 3; ++i) pair(n0 + q[0][i], n0 + q[2][i], ly * 2, bend);
                }
            }
        groupIdCounter++;
        return {n0, numParticles()};
    }

    void makeImmovable(int id) { immovableConstraints.push_back(id); }

    // View for bp_solver_create (valid while the scene is alive and unchanged).
    bp_scene_desc desc() const
    {
        bp_scene_desc d{};
        d.num_particles = numParticles();
        d.positions = positions.data();
        d.velocities = velocities.empty() ? nullptr : velocities.data();
        d.masses = masses.data();
        d.phases = phases.data();
        d.group_ids = groupIds.data();
        d.num_planes = (int)planes.size() / 6;
        d.planes = planes.empty() ? nullptr : planes.data();
        d.num_distance_constraints = (int)distancePairs.size() / 2;
        d.distance_pairs = distancePairs.empty() ? nullptr : distancePairs.data();
        d.distance_params = distanceParams.empty() ? nullptr : distanceParams.data();
        d.num_wind_faces = (int)faces.size() / 3;
        d.wind_faces = faces.empty() ? nullptr : faces.data();
        d.num_rigid_bodies = (int)rigidbodyParticleIdRanges.size() / 2;
        d.rigid_ranges = rigidbodyParticleIdRanges.empty() ? nullptr : rigidbodyParticleIdRanges.data();
        d.rigid_rest_positions = rigidbodyInitialPositions.data();
        d.num_immovables = (int)immovableConstraints.size();
        d.immovables = immovableConstraints.empty() ? nullptr : immovableConstraints.data();
        d.num_bendings = (int)bendingConstraints.size() / 4;
        d.bendings = bendingConstraints.empty() ? nullptr : bendingConstraints.data();
        return d;
    }

    bp_params params() const
    {
        bp_params p;
        bp_params_init(&p, particleRadius);
        p.kernel_radius = fluidKernelRadius;
        p.cell_size = cellSize;
        p.grid_dim = gridDim;
        p.rest_density = fluidRestDensity;
        return p;
    }

private:
    static float norm(float3_ v) { return std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }
    void push(float x, float y, float z, float m, int phase)
    {
        positions.insert(positions.end(), {x, y, z});
        rigidbodyInitialPositions.insert(rigidbodyInitialPositions.end(), {0.f, 0.f, 0.f});
        masses.push_back(m);
        phases.push_back(phase);
        groupIds.push_back(groupIdCounter);
    }
    void pair(int a, int b, float d, float k)
    {
        distancePairs.insert(distancePairs.end(), {a, b});
        distanceParams.insert(distanceParams.end(), {d, k});
    }
    template <class PhaseFn>
    void lattice(const int dim[3], float3_ s, float3_ st, float mass, PhaseFn phase, void *)
    {
        int k = 0;
        for (int i = 0; i < dim[0]; ++i)
            for (int j = 0; j < dim[1]; ++j)
                for (int l = 0; l < dim[2]; ++l)
                    push(s.x + st.x * float(i), s.y + st.y * float(j), s.z + st.z * float(l), mass, phase(k++));
        groupIdCounter++;
    }
};

class ParticleSolver {
public:
    explicit ParticleSolver(const Scene &scene, const bp_params *params = nullptr, void *stream = nullptr)
    {
        const bp_scene_desc d = scene.desc();
        const bp_params p = params ? *params : scene.params();
        check(bp_solver_create(&d, &p, stream, &s_));
        n_ = scene.numParticles();
    }
    ~ParticleSolver() { bp_solver_destroy(s_); }
    ParticleSolver(const ParticleSolver &) = delete;
    ParticleSolver &operator=(const ParticleSolver &) = delete;

    // particlesolver.cuh:772 -- iterations was the hard-coded 2 there
    void update(int numSubTimeStep, float deltaTime, int iterations = 2, int pickedOriginalParticleId = -1,
                const float *pickedParticlePosition = nullptr, const float *pickedParticleVelocity = nullptr)
    {
        check(bp_solver_update(s_, numSubTimeStep, deltaTime, iterations, pickedOriginalParticleId,
                               pickedParticlePosition, pickedParticleVelocity));
    }
    int queryOriginalParticleId(int newParticleId)
    {
        int32_t o;
        check(bp_solver_query_original_particle_id(s_, newParticleId, &o));
        return o;
    }
    int queryNewParticleId(int oldParticleId)
    {
        int32_t o;
        check(bp_solver_query_new_particle_id(s_, oldParticleId, &o));
        return o;
    }
    float3_ getParticlePosition(int particleIndex)
    {
        float v[3];
        check(bp_solver_get_particle_position(s_, particleIndex, v));
        return {v[0], v[1], v[2]};
    }
    std::vector<float> positions(bp_order order = BP_ORDER_ORIGINAL)
    {
        std::vector<float> out(3 * (size_t)n_);
        check(bp_solver_copy_positions(s_, out.data(), order));
        return out;
    }
    // devPositions & co. (particlesolver.cuh:1078-1146): device pointers, sorted order
    void *devicePointer(bp_field field)
    {
        void *p;
        size_t b;
        check(bp_solver_field(s_, field, &p, &b));
        return p;
    }
    bp_solver *handle() { return s_; }

    // Differentiable rollouts (no counterpart in the reference): record the
    // following updates, then gradients of a loss of the final state.
    struct Gradients {
        std::vector<float> positions, velocities, windVelocity, distanceStiffness, distanceRestLength;
    };
    void tapeBegin(int checkpointEvery) { check(bp_solver_tape_begin(s_, checkpointEvery)); }
    void tapeEnd() { check(bp_solver_tape_end(s_)); }
    // dLdx, dLdv: [N][3] in original order (either may be empty for zero);
    // numDistanceConstraints sizes the per-constraint gradients
    Gradients backward(const std::vector<float> &dLdx, const std::vector<float> &dLdv, int numDistanceConstraints)
    {
        Gradients g;
        g.positions.assign(3 * (size_t)n_, 0.f);
        g.velocities.assign(3 * (size_t)n_, 0.f);
        g.windVelocity.assign(3, 0.f);
        g.distanceStiffness.assign((size_t)numDistanceConstraints, 0.f);
        g.distanceRestLength.assign((size_t)numDistanceConstraints, 0.f);
        bp_gradients out;
        out.positions = g.positions.data();
        out.velocities = g.velocities.data();
        out.wind_velocity = g.windVelocity.data();
        out.distance_stiffness = numDistanceConstraints ? g.distanceStiffness.data() : nullptr;
        out.distance_rest_length = numDistanceConstraints ? g.distanceRestLength.data() : nullptr;
        check(bp_solver_backward(s_, dLdx.empty() ? nullptr : dLdx.data(), dLdv.empty() ? nullptr : dLdv.data(),
                                 &out));
        return g;
    }

private:
    bp_solver *s_ = nullptr;
    int n_ = 0;
};

// Many independent scenes stepped together (no counterpart in the reference).
class BatchSolver {
public:
    BatchSolver(const std::vector<const Scene *> &scenes, void *stream = nullptr)
    {
        std::vector<bp_scene_desc> d;
        std::vector<bp_params> p;
        for (const Scene *sc : scenes) {
            d.push_back(sc->desc());
            p.push_back(sc->params());
        }
        check(bp_batch_create((int32_t)d.size(), d.data(), p.data(), stream, &s_));
    }
    ~BatchSolver() { bp_solver_destroy(s_); }
    BatchSolver(const BatchSolver &) = delete;
    BatchSolver &operator=(const BatchSolver &) = delete;
    void step(float dt, int numSubTimeStep, int iterations) { check(bp_batch_step(s_, dt, numSubTimeStep, iterations)); }
    // first original id and particle count of one scene
    std::pair<int, int> sceneRange(int scene) const
    {
        int32_t first, count;
        check(bp_batch_scene_range(s_, scene, &first, &count));
        return {first, count};
    }
    bp_solver *handle() { return s_; }

private:
    bp_solver *s_ = nullptr;
};

}  // namespace brasspan
