"""diff_gauss: the differentiable Gaussian rasterizer the reference's renderer
imports (renderer/core/renderer.py:30-83), on the sm_103a kernels of
libmpm.so (include/gsplat.h).

Same module surface as the reference's diff_gauss
(gaussian-splatting/submodules/diff-gaussian-rasterization/diff_gauss/__init__.py):
``GaussianRasterizationSettings``, ``GaussianRasterizer`` (forward returns
color (3,H,W), depth (1,H,W), normal (3,H,W, unit length), alpha (1,H,W),
radii (P,) and extra (E,H,W)), ``rasterize_gaussians`` and ``markVisible``;
gradients flow to means3D, means2D (NDC-space, for densification
statistics), SH or precomputed colors, opacities, scales, rotations,
precomputed covariances and normals, and extra attributes.  All tensors live
on the GPU; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
from typing import NamedTuple

import torch
import torch.nn as nn

from diffmpm_bindings import _lib

_vp = C.c_void_p
GS_TILE = 16
GS_MAX_EXTRA = 34


# gradients: the reference's (default) or the exact derivative of the forward
# pass; they differ only in the rotation gradient through normals taken from
# scales and rotations (include/gsplat.h, GsScene.exact_adjoint)
_ADJOINT = {"exact": 0}


def set_adjoint(mode: str = "reference") -> None:
    """'reference': the reference rasterizer's gradients, including the sign
    its backward gives the rotation gradient through the normal (additive;
    the default); 'exact': the derivative of the forward pass."""
    if mode not in ("reference", "exact"):
        raise ValueError("adjoint must be 'reference' or 'exact'")
    _ADJOINT["exact"] = int(mode == "exact")


class _Scene(C.Structure):
    _fields_ = [("P", C.c_int), ("H", C.c_int), ("W", C.c_int), ("tanfovx", C.c_float), ("tanfovy", C.c_float),
                ("scale_modifier", C.c_float), ("sh_degree", C.c_int), ("sh_coeffs", C.c_int),
                ("extra_dims", C.c_int), ("bg", _vp), ("viewmatrix", _vp), ("projmatrix", _vp), ("campos", _vp),
                ("means3D", _vp), ("opacities", _vp), ("shs", _vp), ("colors", _vp), ("scales", _vp),
                ("rotations", _vp), ("cov3D", _vp), ("norm3D", _vp), ("extra", _vp), ("exact_adjoint", C.c_int)]


class _Geom(C.Structure):
    _fields_ = [(n, _vp) for n in ("radii", "xy", "depth", "conic_opacity", "rgb", "normal", "cov3D", "clamped",
                                   "tiles_touched", "offsets")]


class _Binning(C.Structure):
    _fields_ = [(n, _vp) for n in ("keys", "keys_sorted", "ids", "ids_sorted", "ranges")]


class _Image(C.Structure):
    _fields_ = [(n, _vp) for n in ("color", "depth", "normal", "alpha", "extra", "n_contrib")]


class _Grads(C.Structure):
    _fields_ = [(n, _vp) for n in ("means3D", "means2D", "opacities", "colors", "shs", "scales", "rotations",
                                   "cov3D", "norm3D", "extra", "conic", "depth")]


def _ptr(t):
    return None if t is None or t.numel() == 0 else _vp(t.data_ptr())


def _f32(t):
    return t.detach().to(torch.float32).contiguous()


class GaussianRasterizationSettings(NamedTuple):
    image_height: int
    image_width: int
    tanfovx: float
    tanfovy: float
    bg: torch.Tensor
    scale_modifier: float
    viewmatrix: torch.Tensor
    projmatrix: torch.Tensor
    sh_degree: int
    campos: torch.Tensor
    prefiltered: bool
    debug: bool


def _scene(s: GaussianRasterizationSettings, means3D, opacities, sh, colors, scales, rotations, cov3D, norm3D,
           extra, keep):
    P = means3D.shape[0]
    t = {k: (_f32(v) if v is not None and v.numel() else None) for k, v in dict(
        bg=s.bg, view=s.viewmatrix, proj=s.projmatrix, campos=s.campos, means3D=means3D, opacities=opacities,
        sh=sh, colors=colors, scales=scales, rotations=rotations, cov3D=cov3D, norm3D=norm3D, extra=extra).items()}
    keep.append(t)
    sc = _Scene()
    sc.P, sc.H, sc.W = P, int(s.image_height), int(s.image_width)
    sc.tanfovx, sc.tanfovy, sc.scale_modifier = float(s.tanfovx), float(s.tanfovy), float(s.scale_modifier)
    sc.sh_degree = int(s.sh_degree)
    sc.sh_coeffs = int(t["sh"].shape[1]) if t["sh"] is not None else 0
    sc.extra_dims = int(t["extra"].shape[1]) if t["extra"] is not None else 0
    sc.bg, sc.viewmatrix, sc.projmatrix, sc.campos = _ptr(t["bg"]), _ptr(t["view"]), _ptr(t["proj"]), _ptr(t["campos"])
    sc.means3D, sc.opacities, sc.shs, sc.colors = _ptr(t["means3D"]), _ptr(t["opacities"]), _ptr(t["sh"]), _ptr(t["colors"])
    sc.scales, sc.rotations, sc.cov3D = _ptr(t["scales"]), _ptr(t["rotations"]), _ptr(t["cov3D"])
    sc.norm3D, sc.extra = _ptr(t["norm3D"]), _ptr(t["extra"])
    sc.exact_adjoint = _ADJOINT["exact"]
    return sc


def _stream():
    return _vp(torch.cuda.current_stream().cuda_stream)


class _RasterizeGaussians(torch.autograd.Function):
    @staticmethod
    def forward(ctx, means3D, means2D, sh, colors_precomp, opacities, scales, rotations, cov3Ds_precomp,
                norm3Ds_precomp, extra_attrs, raster_settings):
        if extra_attrs.numel() and extra_attrs.shape[1] > GS_MAX_EXTRA:
            raise ValueError(f"extra_attrs may have at most {GS_MAX_EXTRA} channels")
        s = raster_settings
        dev = means3D.device
        P, H, W = means3D.shape[0], int(s.image_height), int(s.image_width)
        keep = []
        sc = _scene(s, means3D, opacities, sh, colors_precomp, scales, rotations, cov3Ds_precomp, norm3Ds_precomp,
                    extra_attrs, keep)
        ED = sc.extra_dims
        f32 = dict(dtype=torch.float32, device=dev)
        i32 = dict(dtype=torch.int32, device=dev)
        geom = dict(radii=torch.zeros(P, **i32), xy=torch.zeros((P, 2), **f32), depth=torch.zeros(P, **f32),
                    conic_opacity=torch.zeros((P, 4), **f32), rgb=torch.zeros((P, 3), **f32),
                    normal=torch.zeros((P, 3), **f32), cov3D=torch.zeros((P, 6), **f32),
                    clamped=torch.zeros((P, 3), dtype=torch.uint8, device=dev), tiles_touched=torch.zeros(P, **i32),
                    offsets=torch.zeros(P, **i32))
        g = _Geom(**{k: _ptr(v) if v.numel() else None for k, v in geom.items()})
        tiles = ((W + GS_TILE - 1) // GS_TILE) * ((H + GS_TILE - 1) // GS_TILE)
        scan_b, sort_b = C.c_size_t(), C.c_size_t()
        _lib.check(_lib.lib.gs_scratch_bytes(P, 0, tiles, C.byref(scan_b), C.byref(sort_b)), "rasterize_gaussians")
        scan_tmp = torch.empty(max(1, scan_b.value), dtype=torch.uint8, device=dev)
        L = C.c_int()
        _lib.check(_lib.lib.gs_preprocess(C.byref(sc), C.byref(g), _vp(scan_tmp.data_ptr()), scan_b.value,
                                          C.byref(L), _stream()), "rasterize_gaussians")
        L = L.value
        _lib.check(_lib.lib.gs_scratch_bytes(P, L, tiles, C.byref(scan_b), C.byref(sort_b)), "rasterize_gaussians")
        binning = dict(keys=torch.empty(max(1, L), dtype=torch.int64, device=dev),
                       keys_sorted=torch.empty(max(1, L), dtype=torch.int64, device=dev),
                       ids=torch.empty(max(1, L), **i32), ids_sorted=torch.empty(max(1, L), **i32),
                       ranges=torch.zeros(2 * tiles, **i32))
        b = _Binning(**{k: _ptr(v) for k, v in binning.items()})
        sort_tmp = torch.empty(max(1, sort_b.value), dtype=torch.uint8, device=dev)
        img = dict(color=torch.empty((3, H, W), **f32), depth=torch.empty((1, H, W), **f32),
                   normal=torch.empty((3, H, W), **f32), alpha=torch.empty((1, H, W), **f32),
                   extra=torch.empty((ED, H, W), **f32), n_contrib=torch.empty((H, W), **i32))
        im = _Image(**{k: _ptr(v) for k, v in img.items()})
        _lib.check(_lib.lib.gs_render(C.byref(sc), C.byref(g), L, C.byref(b), _vp(sort_tmp.data_ptr()),
                                      sort_b.value, C.byref(im), _stream()), "rasterize_gaussians")
        ctx.set_materialize_grads(False)  # unused outputs arrive as None: their adjoint terms are skipped
        ctx.raster_settings = s
        ctx.num_rendered = L
        ctx.has = dict(sh=sh.numel() > 0, colors=colors_precomp.numel() > 0, scales=scales.numel() > 0,
                       rotations=rotations.numel() > 0, cov3D=cov3Ds_precomp.numel() > 0,
                       norm3D=norm3Ds_precomp.numel() > 0, extra=extra_attrs.numel() > 0)
        ctx.shapes = dict(opacities=opacities.shape, means2D=means2D.shape)
        ctx.save_for_backward(means3D, sh, colors_precomp, opacities, scales, rotations, cov3Ds_precomp,
                              norm3Ds_precomp, extra_attrs, *geom.values(), binning["ids_sorted"],
                              binning["ranges"], img["alpha"], img["n_contrib"])
        ctx.geom_keys = list(geom)
        ctx.mark_non_differentiable(geom["radii"])
        return img["color"], img["depth"], img["normal"], img["alpha"], geom["radii"], img["extra"]

    @staticmethod
    def backward(ctx, g_color, g_depth, g_norm, g_alpha, _g_radii, g_extra):
        s = ctx.raster_settings
        saved = ctx.saved_tensors
        (means3D, sh, colors, opacities, scales, rotations, cov3D, norm3D, extra) = saved[:9]
        geom = dict(zip(ctx.geom_keys, saved[9:9 + len(ctx.geom_keys)]))
        ids_sorted, ranges, alpha, n_contrib = saved[9 + len(ctx.geom_keys):]
        keep = []
        sc = _scene(s, means3D, opacities, sh, colors, scales, rotations, cov3D, norm3D, extra, keep)
        dev = means3D.device
        P = means3D.shape[0]
        g = _Geom(**{k: _ptr(v) if v.numel() else None for k, v in geom.items()})
        b = _Binning(keys=None, keys_sorted=None, ids=None, ids_sorted=_ptr(ids_sorted), ranges=_ptr(ranges))
        im = _Image(color=None, depth=None, normal=None, alpha=_ptr(alpha), extra=None, n_contrib=_ptr(n_contrib))
        f32 = dict(dtype=torch.float32, device=dev)
        grads = dict(means3D=torch.empty((P, 3), **f32), means2D=torch.empty((P, 3), **f32),
                     opacities=torch.empty(P, **f32), colors=torch.empty((P, 3), **f32),
                     shs=torch.empty((P, sc.sh_coeffs, 3), **f32) if ctx.has["sh"] else None,
                     scales=torch.empty((P, 3), **f32) if ctx.has["scales"] else None,
                     rotations=torch.empty((P, 4), **f32) if ctx.has["rotations"] else None,
                     cov3D=torch.empty((P, 6), **f32), norm3D=torch.empty((P, 3), **f32),
                     extra=torch.empty((P, sc.extra_dims), **f32) if ctx.has["extra"] else None,
                     conic=torch.empty((P, 3), **f32), depth=torch.empty(P, **f32))
        gr = _Grads(**{k: _ptr(v) for k, v in grads.items()})
        outs = [None if t is None else _f32(t) for t in (g_color, g_depth, g_norm, g_alpha, g_extra)]
        _lib.check(_lib.lib.gs_backward(C.byref(sc), C.byref(g), ctx.num_rendered, C.byref(b), C.byref(im),
                                        *[_ptr(t) for t in outs], C.byref(gr), _stream()), "rasterize_gaussians")
        h = ctx.has
        m2 = grads["means2D"]  # (P,3); the third entry is zero
        if tuple(ctx.shapes["means2D"]) == (P, 2):
            m2 = m2[:, :2].contiguous()
        return (grads["means3D"], m2,
                grads["shs"] if h["sh"] else None, grads["colors"] if h["colors"] else None,
                grads["opacities"].reshape(ctx.shapes["opacities"]),
                grads["scales"] if h["scales"] else None, grads["rotations"] if h["rotations"] else None,
                grads["cov3D"] if h["cov3D"] else None, grads["norm3D"] if h["norm3D"] else None,
                grads["extra"] if h["extra"] else None, None)


def rasterize_gaussians(means3D, means2D, sh, colors_precomp, opacities, scales, rotations, cov3Ds_precomp,
                        norm3Ds_precomp, extra_attrs, raster_settings):
    color, depth, norm, alpha, radii, extra = _RasterizeGaussians.apply(
        means3D, means2D, sh, colors_precomp, opacities, scales, rotations, cov3Ds_precomp, norm3Ds_precomp,
        extra_attrs, raster_settings)
    norm = torch.nn.functional.normalize(norm, p=2, dim=0)
    return color, depth, norm, alpha, radii, extra


class GaussianRasterizer(nn.Module):
    def __init__(self, raster_settings):
        super().__init__()
        self.raster_settings = raster_settings

    def markVisible(self, positions):
        """Near-plane test of each point (view-space z > 0.2)."""
        with torch.no_grad():
            v = self.raster_settings.viewmatrix.to(positions.dtype).reshape(4, 4)
            z = positions @ v[:3, 2] + v[3, 2]
            return z > 0.2

    def forward(self, means3D, means2D, opacities, shs=None, colors_precomp=None, scales=None, rotations=None,
                cov3Ds_precomp=None, norm3Ds_precomp=None, extra_attrs=None):
        s = self.raster_settings
        if (shs is None and colors_precomp is None) or (shs is not None and colors_precomp is not None):
            raise Exception('Please provide excatly one of either SHs or precomputed colors!')
        if ((scales is None or rotations is None) and cov3Ds_precomp is None) or \
                ((scales is not None or rotations is not None) and cov3Ds_precomp is not None):
            raise Exception('Please provide exactly one of either scale/rotation pair or precomputed 3D covariance!')
        dev = means3D.device
        empty = torch.empty(0, device=dev)
        if scales is None:
            raise ValueError('To support norm and depth prediction, scales == None is not allowed')
        if rotations is None:
            raise ValueError('To support norm and depth prediction, rotations == None is not allowed')
        return rasterize_gaussians(
            means3D, means2D, empty if shs is None else shs, empty if colors_precomp is None else colors_precomp,
            opacities, scales, rotations, empty if cov3Ds_precomp is None else cov3Ds_precomp,
            empty if norm3Ds_precomp is None else norm3Ds_precomp, empty if extra_attrs is None else extra_attrs,
            s)
