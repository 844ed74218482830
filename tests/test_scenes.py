"""Scene builders: constraint counts of the reference's cloth factory, phase
and id conventions, and agreement of the C++ (include/brasspan.hpp) and
Python builders array for array."""
from __future__ import annotations

import subprocess

import numpy as np

from conftest import REPO


def test_cloth_counts_follow_reference_factory(bp):
    s = bp.scenes.Scene()
    n = 9
    s.add_cloth((0, 1, 0), (0.1, 0, 0), (0, 0, 0.1), n, n, 1.0, corners=(True, True, False, False))
    stretch = 2 * n * (n - 1)
    shear = 2 * (n - 1) ** 2
    bend = 6 * (n - 2) ** 2  # skip-one pairs of every interior 3x3 stencil, repeats included
    assert len(s.distance_pairs) == stretch + shear + bend
    assert len(s.faces) == 2 * (n - 1) ** 2
    assert list(s.immovables) == [0, n - 1]
    assert (s.phases == np.arange(1, n * n + 1)).all()  # self-colliding: one phase per particle
    # rest lengths: 0.1 stretch, 0.1*sqrt(2) shear, 0.2 bend
    d = np.unique(np.round(s.distance_params[:, 0].astype(np.float64), 5))
    np.testing.assert_allclose(d, [0.1, np.sqrt(0.02), 0.2], rtol=1e-5)


def test_dihedral_quads_follow_reference_pattern(bp):
    """The reference's commented-out cloth bending quads (scene.h:308-320):
    one per lattice quad, hinge along the diagonal p3-p2 when x + y is odd,
    p1-p4 when even."""
    s = bp.scenes.Scene()
    n = 5
    s.add_cloth((0, 1, 0), (0.1, 0, 0), (0, 0, 0.1), n, n, 1.0, dihedral=True)
    assert s.bendings.shape == ((n - 1) ** 2, 4)
    q = s.bendings.tolist()
    k = 0
    for x in range(n - 1):
        for y in range(n - 1):
            p1, p2, p3, p4 = y * n + x, y * n + x + 1, (y + 1) * n + x, (y + 1) * n + x + 1
            assert q[k] == ([p3, p2, p1, p4] if (x + y) % 2 else [p1, p4, p3, p2])
            k += 1


def test_phase_and_group_conventions(bp):
    s = bp.scenes.Scene()
    s.add_fluid_block((2, 2, 2), (0, 0, 0), (0.1, 0.1, 0.1), 1.0)
    s.add_fluid_block((2, 2, 2), (1, 0, 0), (0.1, 0.1, 0.1), 1.0)
    s.add_rigid_box((2, 2, 2), (2, 0, 0), (0.1, 0.1, 0.1), 1.0)
    s.add_granulars_block((1, 1, 2), (3, 0, 0), (0.1, 0.1, 0.1), 1.0)
    assert (s.phases[:8] == -1).all() and (s.phases[8:16] == -2).all()
    assert (s.phases[16:24] == 1).all() and list(s.phases[24:]) == [2, 3]
    assert list(np.unique(s.group_ids)) == [0, 1, 2, 3]
    assert s.rigid_ranges.tolist() == [[16, 24]]
    np.testing.assert_allclose(s.rigid_rest[16:24].mean(axis=0), 0, atol=1e-6)
    assert (s.rigid_rest[:16] == 0).all()


CPP = r"""
#include <cstdio>
#include "brasspan.hpp"
using namespace brasspan;
template <class T> void dump(FILE *f, const std::vector<T> &v) { long n = (long)v.size(); fwrite(&n, 8, 1, f); fwrite(v.data(), sizeof(T), v.size(), f); }
int main(int argc, char **argv) {
    Scene s;
    const int fd[3] = {3, 4, 5};
    s.addFluidBlock(fd, {0.1f, 0.1f, 0.1f}, {0.1f, 0.1f, 0.1f}, 1.0f);
    s.addCloth({0.2f, 1.25f, 0.2f}, {0.1f, 0.f, 0.f}, {0.f, 0.f, 0.1f}, 6, 6, 1.0f, true, false, false, true,
               0.2f, 0.2f, 0.1f, true);
    const int rd[3] = {3, 2, 3};
    s.addRigidBox(rd, {0.4f, 1.45f, 0.5f}, {0.1f, 0.1f, 0.1f}, 1.0f);
    s.addRope({2.5f, 3.0f, 0.5f}, {2.5f, 2.0f, 0.5f}, 7, 1.0f);
    FILE *f = fopen(argv[1], "wb");
    dump(f, s.positions); dump(f, s.masses); dump(f, s.phases); dump(f, s.groupIds); dump(f, s.distancePairs);
    dump(f, s.distanceParams); dump(f, s.faces); dump(f, s.rigidbodyParticleIdRanges);
    dump(f, s.rigidbodyInitialPositions); dump(f, s.immovableConstraints); dump(f, s.bendingConstraints);
    const bp_scene_desc d = s.desc();
    if (d.num_bendings * 4 != (int)s.bendingConstraints.size() || d.bendings != s.bendingConstraints.data()) return 2;
    fclose(f);
    bp_params p = s.params();
    return p.grid_dim == 512 ? 0 : 1;
}
"""


def test_cpp_scene_builder_matches_python(bp, tmp_path):
    src = tmp_path / "scene.cpp"
    src.write_text(CPP)
    exe = tmp_path / "scene"
    lib_dir = bp.abi.LIB_PATH.parent
    subprocess.run(["g++", "-std=c++17", "-O1", f"-I{REPO / 'include'}", str(src), "-o", str(exe),
                    f"-L{lib_dir}", "-lbrasspan", f"-Wl,-rpath,{lib_dir}"], check=True)
    out = tmp_path / "scene.bin"
    subprocess.run([str(exe), str(out)], check=True)
    raw = out.read_bytes()
    arrays, off = [], 0
    kinds = [np.float32, np.float32, np.int32, np.int32, np.int32, np.float32, np.int32, np.int32, np.float32,
             np.int32, np.int32]
    for k in kinds:
        n = int(np.frombuffer(raw, np.int64, 1, off)[0])
        off += 8
        arrays.append(np.frombuffer(raw, k, n, off))
        off += n * 4
    s = bp.scenes.Scene()
    s.add_fluid_block((3, 4, 5), (0.1, 0.1, 0.1), (0.1, 0.1, 0.1), 1.0)
    s.add_cloth((0.2, 1.25, 0.2), (0.1, 0, 0), (0, 0, 0.1), 6, 6, 1.0, corners=(True, False, False, True),
                dihedral=True)
    s.add_rigid_box((3, 2, 3), (0.4, 1.45, 0.5), (0.1, 0.1, 0.1), 1.0)
    s.add_rope((2.5, 3.0, 0.5), (2.5, 2.0, 0.5), 7, 1.0)
    np.testing.assert_array_equal(arrays[0].reshape(-1, 3), s.positions)
    np.testing.assert_array_equal(arrays[1], s.masses)
    np.testing.assert_array_equal(arrays[2], s.phases)
    np.testing.assert_array_equal(arrays[3], s.group_ids)
    np.testing.assert_array_equal(arrays[4].reshape(-1, 2), s.distance_pairs)
    np.testing.assert_allclose(arrays[5].reshape(-1, 2), s.distance_params, rtol=1e-6)
    np.testing.assert_array_equal(arrays[6].reshape(-1, 3), s.faces)
    np.testing.assert_array_equal(arrays[7].reshape(-1, 2), s.rigid_ranges)
    np.testing.assert_allclose(arrays[8].reshape(-1, 3), s.rigid_rest, atol=1e-6)
    np.testing.assert_array_equal(arrays[9], s.immovables)
    np.testing.assert_array_equal(arrays[10].reshape(-1, 4), s.bendings)
