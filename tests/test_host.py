"""Host-side logic that needs no GPU: OptInput, Lame parameters, mesh
sampling, synthetic workloads."""
import math

import numpy as np
import pytest


def test_optinput_fields(dm):
    o = dm.OptInput()
    o.grid_dx = 1
    o.grid_min_point = [-16.0, -16.0, -16.0]
    o.num_timesteps = 10
    o.f_ext = (0, -9.8, 0)
    o.mpm_input_mesh_path = "a.obj"
    assert o.grid_dx == 1.0 and o.num_timesteps == 10
    assert np.allclose(o.grid_min_point, -16) and np.allclose(o.f_ext, [0, -9.8, 0])
    with pytest.raises(AttributeError):
        o.not_a_field = 1
    fields = ["mpm_input_mesh_path", "mpm_target_mesh_path", "grid_dx", "grid_min_point", "grid_max_point",
              "points_per_cell_cuberoot", "lam", "mu", "p_density", "dt", "drag", "f_ext", "num_animations",
              "num_timesteps", "control_stride", "max_gd_iters", "max_ls_iters", "initial_alpha", "gd_tol",
              "smoothing_factor", "current_episodes"]
    assert len(fields) == 21
    for f in fields:
        assert hasattr(o, f), f


def test_lame_parameters(dm, orc):
    lam, mu = dm.calculate_lame_parameters(1e4, 0.3)
    l2, m2 = orc.lame(1e4, 0.3)
    assert abs(lam - l2) / l2 < 1e-6 and abs(mu - m2) / m2 < 1e-6


def _cube_mesh(lo=-1.0, hi=1.0):
    V = np.array([[x, y, z] for x in (lo, hi) for y in (lo, hi) for z in (lo, hi)], np.float32)
    F = np.array([[0, 1, 3], [0, 3, 2], [4, 6, 7], [4, 7, 5], [0, 4, 5], [0, 5, 1], [2, 3, 7], [2, 7, 6],
                  [0, 2, 6], [0, 6, 4], [1, 5, 7], [1, 7, 3]])
    return V, F


def test_winding_number_oracle():
    from geometry_oracle import winding_numbers
    V, F = _cube_mesh()
    w = winding_numbers(np.array([[0, 0, 0], [0.9, 0.9, -0.9], [2, 0, 0], [0, -3, 0], [1, 0, 0], [1, 1, 1]], float),
                        V, F)
    assert np.allclose(np.abs(w[:4]), [1, 1, 0, 0], atol=1e-9)
    assert w[4] == 0.5 and w[5] == 0.5  # on a face, on a vertex


def test_lattice_sampling_matches_reference_rule(tmp_path):
    from diffmpm_bindings.geometry import lattice
    from geometry_oracle import winding_numbers
    V, F = _cube_mesh(-1.0, 1.0)
    pts = lattice(V, 0.5)
    assert len(pts) == 5 ** 3 and np.allclose(pts[0], -1) and np.allclose(pts[1], [-1, -1, -0.5])
    inside = pts[np.abs(winding_numbers(pts, V, F)) >= 0.5]
    assert len(inside) == 125  # the interior 27 and the 98 on the surface (signed distance 0)
    p = tmp_path / "cube.obj"
    p.write_text("".join(f"v {a} {b} {c}\n" for a, b, c in V) + "".join(f"f {a+1} {b+1} {c+1}\n" for a, b, c in F))
    from diffmpm_bindings.geometry import read_obj
    V2, F2 = read_obj(str(p))
    assert np.allclose(V2, V) and (F2 == F).all()


def test_workload_sizes():
    from diffmpm_bindings import workloads as W
    w = W.sphere32()
    assert w.n == round(8 * 4 / 3 * math.pi * 0.25 ** 3 * 32 ** 3) == 17157
    assert w.dims == (33, 33, 33)
    x = w.x
    assert ((x - 0.5) ** 2).sum(1).max() < 0.25 ** 2
    e = W.ellipsoid64(sort=False)
    assert abs(e.n - 153_729) < 10
    assert W.stable_density(5e4, 0.35, 5e-4, 1 / 64) > 300


def test_bindings_reject_bad_render_grad_shapes(dm):
    with pytest.raises(RuntimeError, match=r"dLdF must be \(N,3,3\)"):
        dm.CompGraph._render_arrays(np.zeros((4, 3)), np.zeros((4, 3)), "")
    with pytest.raises(RuntimeError, match=r"dLdx must be \(N,3\)"):
        dm.CompGraph._render_arrays(np.zeros((4, 3, 3)), np.zeros((4, 2)), "")


def test_diff_gauss_module_surface():
    """The rasterizer module keeps the reference diff_gauss API (no GPU needed)."""
    pytest.importorskip("torch")
    import diff_gauss as dg
    assert dg.GaussianRasterizationSettings._fields == (
        "image_height", "image_width", "tanfovx", "tanfovy", "bg", "scale_modifier", "viewmatrix", "projmatrix",
        "sh_degree", "campos", "prefiltered", "debug")
    import inspect
    params = list(inspect.signature(dg.GaussianRasterizer.forward).parameters)
    assert params == ["self", "means3D", "means2D", "opacities", "shs", "colors_precomp", "scales", "rotations",
                      "cov3Ds_precomp", "norm3Ds_precomp", "extra_attrs"]
