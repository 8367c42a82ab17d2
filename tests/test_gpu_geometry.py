"""Mesh -> particle sampling on the GPU (GeometryLoading.cpp:10-143 via
load_point_cloud_from_obj, bind.cpp:531-538): the GPU winding numbers
against the oracle's FP64 restatement, and the kept lattice points against
the reference's own sampler recorded on a convex and a non-convex mesh
(tests/golden/reference_mesh_sampling.npz)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def meshes():
    from pathlib import Path
    return dict(np.load(Path(__file__).parent / "golden" / "reference_mesh_sampling.npz"))


def test_winding_numbers_match_oracle(dm, meshes):
    from diffmpm_bindings.geometry import winding_numbers
    from geometry_oracle import winding_numbers as oracle_wn
    rng = np.random.default_rng(0)
    for name in ("ellipsoid", "torus"):
        V, F = meshes[f"{name}_V"], meshes[f"{name}_F"]
        pts = (0.1 + 0.8 * rng.random((4000, 3))).astype(np.float32)
        pts = np.concatenate([pts, V[:50]])  # on the surface: exactly 0.5
        got, want = winding_numbers(pts, V, F), oracle_wn(pts, V, F)
        assert np.abs(got - want).max() < 1e-5, name
        assert (got[-50:] == 0.5).all()


@pytest.mark.parametrize("name", ["ellipsoid", "torus"])
def test_lattice_matches_reference_sampler(dm, meshes, name):
    from diffmpm_bindings.geometry import lattice_inside_mesh
    V, F, dx, ref = meshes[f"{name}_V"], meshes[f"{name}_F"], float(meshes[f"{name}_dx"]), meshes[f"{name}_points"]
    got = lattice_inside_mesh(V, F, dx)
    assert got.shape == ref.shape
    assert np.array_equal(got.astype(np.float32), ref.astype(np.float32))  # same points, same (lattice) order


def test_load_point_cloud_from_obj(dm, meshes, tmp_path):
    V, F, dx = meshes["torus_V"], meshes["torus_F"], float(meshes["torus_dx"])
    p = tmp_path / "torus.obj"
    p.write_text("".join(f"v {a} {b} {c}\n" for a, b, c in V) + "".join(f"f {a+1} {b+1} {c+1}\n" for a, b, c in F))
    opt = dm.OptInput()
    opt.p_density, opt.lam, opt.mu = 100.0, 5000.0, 3000.0
    opt.points_per_cell_cuberoot, opt.grid_dx = 1, dx
    pc = dm.load_point_cloud_from_obj(str(p), opt)
    assert len(pc) == len(meshes["torus_points"])
    assert np.allclose(pc.get_positions(), meshes["torus_points"].astype(np.float32))
