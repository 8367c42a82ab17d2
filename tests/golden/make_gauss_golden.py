"""Golden outputs of the reference's differentiable Gaussian rasterizer
(gaussian-splatting/submodules/diff-gaussian-rasterization), for the parity
test of diff_gauss in tests/test_gpu_gsplat.py.  TEST INFRASTRUCTURE: it
runs on a GPU host and writes an .npz; nothing in the package uses it.

The reference's kernels are its own sources compiled as sm_103a device
code into oracle/_ref/gs_{forward,backward,impl}.cubin
(oracle/build_oracle.py: build_ref_gauss).  This script loads them with the
CUDA driver API and drives them as the reference's host code does
(cuda_rasterizer/rasterizer_impl.cu:200-463, rasterize_points.cu:36-236):

* forward: preprocessCUDA -> inclusive prefix sum of tiles_touched ->
  duplicateWithKeys -> sort of the (tile | depth) keys -> identifyTileRanges
  -> renderCUDA;
* backward: renderCUDA (backward.cu) -> computeCov2DCUDA -> preprocessCUDA
  (backward.cu).

The prefix sum and the key sort, CUB's InclusiveSum and stable radix
SortPairs in the reference, are torch.cumsum and a stable torch.sort here:
the keys' upper bits are zero and the sort is stable in both, so the order
is the same.  Before every launch the kernel's parameter list (count, and
offset and size of each parameter, from cuFuncGetParamInfo) is checked
against the arguments built here; a mismatch stops the script before
anything runs.

Usage: python tests/golden/make_gauss_golden.py OUT.npz
"""
from __future__ import annotations

import ctypes as C
import struct
import sys
from pathlib import Path

import numpy as np
import torch

ROOT = Path(__file__).resolve().parents[2]
REF = ROOT / "oracle" / "_ref"
sys.path.insert(0, str(ROOT / "tests"))
sys.path.insert(0, str(ROOT / "shape-morphing-binder_gb300"))

BLOCK = 16


# ------------------------------------------------------------ driver API

class Dim3(C.Structure):
    _fields_ = [("x", C.c_uint), ("y", C.c_uint), ("z", C.c_uint)]


_cu = C.CDLL("libcuda.so.1")
_cu.cuModuleLoadData.argtypes = [C.POINTER(C.c_void_p), C.c_void_p]
_cu.cuModuleGetFunction.argtypes = [C.POINTER(C.c_void_p), C.c_void_p, C.c_char_p]
_cu.cuFuncGetParamInfo.argtypes = [C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
_cu.cuLaunchKernel.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                               C.c_void_p, C.POINTER(C.c_void_p), C.c_void_p]
_cu.cuCtxSynchronize.argtypes = []


def _ck(r, what):
    if r != 0:
        raise RuntimeError(f"{what}: CUresult {r}")


def elf_functions(blob: bytes) -> list[str]:
    """Names of the function symbols in an ELF64 image (a cubin built here)."""
    shoff, = struct.unpack_from("<Q", blob, 0x28)
    shentsize, shnum = struct.unpack_from("<HH", blob, 0x3A)
    secs = [struct.unpack_from("<IIQQQQIIQQ", blob, shoff + i * shentsize) for i in range(shnum)]
    out = []
    for sec in secs:
        if sec[1] != 2:  # SHT_SYMTAB
            continue
        strtab = secs[sec[6]]
        for k in range(sec[5] // 24):
            name, info, _, _, _, _ = struct.unpack_from("<IBBHQQ", blob, sec[4] + k * 24)
            if info & 0xF == 2:  # STT_FUNC
                end = blob.index(b"\0", strtab[4] + name)
                out.append(blob[strtab[4] + name:end].decode())
    return out


class Module:
    def __init__(self, path: Path):
        self.blob = path.read_bytes()
        self._buf = C.create_string_buffer(self.blob, len(self.blob))
        self.h = C.c_void_p()
        _ck(_cu.cuModuleLoadData(C.byref(self.h), C.cast(self._buf, C.c_void_p)), f"cuModuleLoadData {path.name}")
        self.names = elf_functions(self.blob)

    def function(self, stem: str):
        hits = [n for n in self.names if stem in n]
        if len(hits) != 1:
            raise RuntimeError(f"{stem}: {len(hits)} matching functions")
        f = C.c_void_p()
        _ck(_cu.cuModuleGetFunction(C.byref(f), self.h, hits[0].encode()), stem)
        return Kernel(stem, f)


def ptr(t):
    return C.c_void_p(0 if t is None else t.data_ptr())


class Kernel:
    def __init__(self, name, f):
        self.name, self.f = name, f

    def check(self, args):
        off, size = C.c_size_t(), C.c_size_t()
        for i, a in enumerate(args):
            _ck(_cu.cuFuncGetParamInfo(self.f, i, C.byref(off), C.byref(size)), f"{self.name} param {i}")
            if size.value != C.sizeof(a):
                raise RuntimeError(f"{self.name} param {i}: kernel size {size.value}, given {C.sizeof(a)}")
        if _cu.cuFuncGetParamInfo(self.f, len(args), C.byref(off), C.byref(size)) == 0:
            raise RuntimeError(f"{self.name}: the kernel has more than {len(args)} parameters")

    def __call__(self, grid, block, args):
        self.check(args)
        params = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        _ck(_cu.cuLaunchKernel(self.f, *grid, *block, 0, stream, params, None), f"launch {self.name}")
        _ck(_cu.cuCtxSynchronize(), f"run {self.name}")


# ------------------------------------------------------------ host flow

def forward(mods, s):
    """rasterizer_impl.cu:200-329 with rasterize_points.cu:36-130."""
    dev = s["means3D"].device
    P, H, W = s["means3D"].shape[0], s["H"], s["W"]
    shs, colors, extra = s.get("shs"), s.get("colors"), s.get("extra")
    cov3D_pre, norm3D_pre = s.get("cov3D"), s.get("norm3D")
    D = s.get("sh_degree", 0)
    M = 0 if shs is None else shs.shape[1]
    ED = 0 if extra is None else extra.shape[1]
    f32 = np.float32
    tanx, tany = f32(s["tanx"]), f32(s["tany"])
    focal_y, focal_x = f32(H) / (f32(2.0) * tany), f32(W) / (f32(2.0) * tanx)
    tg = ((W + BLOCK - 1) // BLOCK, (H + BLOCK - 1) // BLOCK, 1)
    z = lambda *shape, dt=torch.float32: torch.zeros(shape, dtype=dt, device=dev)  # noqa: E731
    g = dict(depths=z(P), clamped=z(P * 3, dt=torch.bool), means2D=z(P, 2), cov3D=z(P, 6), conic=z(P, 4),
             rgb=z(P, 3), norm3D=z(P, 3), tiles=z(P, dt=torch.int32), radii=z(P, dt=torch.int32))
    out = dict(color=z(3, H, W), depth=z(1, H, W), norm=z(3, H, W), alpha=z(1, H, W),
               extra=z(ED, H, W) if ED else None)
    nb = (P + 255) // 256
    mods["fwd"].function("preprocessCUDA")((nb, 1, 1), (256, 1, 1), [
        C.c_int(P), C.c_int(D), C.c_int(M), ptr(s["means3D"]), ptr(s.get("scales")), C.c_float(1.0),
        ptr(s.get("rotations")), ptr(s["opacities"]), ptr(shs), ptr(g["clamped"]), ptr(cov3D_pre), ptr(norm3D_pre),
        ptr(colors), ptr(s["view"]), ptr(s["proj"]), ptr(s["campos"]), C.c_int(W), C.c_int(H), C.c_float(tanx),
        C.c_float(tany), C.c_float(focal_x), C.c_float(focal_y), ptr(g["radii"]), ptr(g["means2D"]),
        ptr(g["depths"]), ptr(g["cov3D"]), ptr(g["norm3D"]), ptr(g["rgb"]), ptr(g["conic"]), Dim3(*tg),
        ptr(g["tiles"]), C.c_bool(False)])
    offsets = torch.cumsum(g["tiles"].to(torch.int64), 0).to(torch.int32)
    R = int(offsets[-1]) if P else 0
    g["offsets"] = offsets
    keys = z(max(R, 1), dt=torch.int64)
    vals = z(max(R, 1), dt=torch.int32)
    mods["impl"].function("duplicateWithKeys")((nb, 1, 1), (256, 1, 1), [
        C.c_int(P), ptr(g["means2D"]), ptr(g["depths"]), ptr(offsets), ptr(keys), ptr(vals), ptr(g["radii"]),
        Dim3(*tg)])
    keys, order = torch.sort(keys[:R], stable=True)
    vals = vals[:R][order].contiguous()
    keys = keys.contiguous()
    ranges = z(tg[0] * tg[1], 2, dt=torch.int32)
    if R > 0:
        mods["impl"].function("identifyTileRanges")(((R + 255) // 256, 1, 1), (256, 1, 1), [
            C.c_int(R), ptr(keys), ptr(ranges)])
    n_contrib = z(H * W, dt=torch.int32)
    feat = colors if colors is not None else g["rgb"]
    nrm = norm3D_pre if norm3D_pre is not None else g["norm3D"]
    mods["fwd"].function("renderCUDA")(tg, (BLOCK, BLOCK, 1), [
        ptr(ranges), ptr(vals), C.c_int(W), C.c_int(H), C.c_int(ED), ptr(g["means2D"]), ptr(feat), ptr(nrm),
        ptr(g["depths"]), ptr(extra), ptr(g["conic"]), ptr(out["alpha"]), ptr(n_contrib), ptr(s["bg"]),
        ptr(out["color"]), ptr(out["depth"]), ptr(out["norm"]), ptr(out["extra"])])
    state = dict(g=g, ranges=ranges, vals=vals, n_contrib=n_contrib, R=R, tg=tg, focal=(focal_x, focal_y), D=D,
                 M=M, ED=ED)
    return out, state


def backward(mods, s, out, st, up):
    """rasterizer_impl.cu:333-463 with rasterize_points.cu:132-236 and
    backward.cu:703-839."""
    dev = s["means3D"].device
    P, H, W = s["means3D"].shape[0], s["H"], s["W"]
    D, M, ED, g = st["D"], st["M"], st["ED"], st["g"]
    shs, colors, extra = s.get("shs"), s.get("colors"), s.get("extra")
    cov3D_pre, norm3D_pre = s.get("cov3D"), s.get("norm3D")
    z = lambda *shape: torch.zeros(shape, dtype=torch.float32, device=dev)  # noqa: E731
    d = dict(means3D=z(P, 3), means2D=z(P, 3), colors=z(P, 3), depths=z(P, 1), conic=z(P, 4), opacities=z(P, 1),
             cov3D=z(P, 6), norm3D=z(P, 3), shs=z(P, max(M, 1), 3), scales=z(P, 3), rotations=z(P, 4),
             extra=z(P, ED) if ED else None)
    color_ptr = colors if colors is not None else g["rgb"]
    norm_ptr = norm3D_pre if norm3D_pre is not None else g["norm3D"]
    tg = st["tg"]
    mods["bwd"].function("renderCUDA")(tg, (BLOCK, BLOCK, 1), [
        ptr(st["ranges"]), ptr(st["vals"]), C.c_int(W), C.c_int(H), C.c_int(ED), ptr(s["bg"]), ptr(g["means2D"]),
        ptr(g["conic"]), ptr(color_ptr), ptr(g["depths"]), ptr(norm_ptr), ptr(extra), ptr(out["alpha"]),
        ptr(st["n_contrib"]), ptr(up["color"]), ptr(up["depth"]), ptr(up["norm"]), ptr(up["alpha"]),
        ptr(up.get("extra")), ptr(d["means2D"]), ptr(d["conic"]), ptr(d["opacities"]), ptr(d["colors"]),
        ptr(d["depths"]), ptr(d["norm3D"]), ptr(d["extra"])])
    cov_ptr = cov3D_pre if cov3D_pre is not None else g["cov3D"]
    nb = (P + 255) // 256
    fx, fy = st["focal"]
    mods["bwd"].function("computeCov2DCUDA")((nb, 1, 1), (256, 1, 1), [
        C.c_int(P), ptr(s["means3D"]), ptr(g["radii"]), ptr(cov_ptr), C.c_float(fx), C.c_float(fy),
        C.c_float(np.float32(s["tanx"])), C.c_float(np.float32(s["tany"])), ptr(s["view"]), ptr(d["conic"]),
        ptr(d["means3D"]), ptr(d["cov3D"])])
    mods["bwd"].function("preprocessCUDA")((nb, 1, 1), (256, 1, 1), [
        C.c_int(P), C.c_int(D), C.c_int(M), ptr(s["means3D"]), ptr(g["radii"]), ptr(shs), ptr(norm_ptr),
        C.c_bool(norm3D_pre is not None), ptr(g["clamped"]), ptr(s.get("scales")), ptr(s.get("rotations")),
        C.c_float(1.0), ptr(s["view"]), ptr(s["proj"]), ptr(s["campos"]), ptr(d["means2D"]), ptr(d["means3D"]),
        ptr(d["colors"]), ptr(d["depths"]), ptr(d["cov3D"]), ptr(d["norm3D"]), ptr(d["shs"]), ptr(d["scales"]),
        ptr(d["rotations"])])
    if M == 0:
        d["shs"] = None
    return d


# ------------------------------------------------------------ scenes

def scenes():
    """Seeded small scenes: precomputed colors; SH degree 3 with extra
    channels; precomputed covariance, normals and colors."""
    import gs_reference as GR
    out = {}
    for name, seed, kind in (("rgb", 21, "rgb"), ("sh3", 22, "sh"), ("cov", 23, "cov")):
        g = torch.Generator().manual_seed(seed)
        d = torch.float64
        P, H, W = 400, 48, 72
        tanx, tany, view, proj, eye = GR.camera(H, W, fovx_deg=55.0)
        m = (torch.rand(P, 3, generator=g, dtype=d) - 0.5) * torch.tensor([2.0, 1.6, 1.5], dtype=d)
        sc = 0.02 + 0.12 * torch.rand(P, 3, generator=g, dtype=d)
        q = torch.randn(P, 4, generator=g, dtype=d)
        q = q / q.norm(dim=1, keepdim=True)
        s = dict(means3D=m, opacities=0.1 + 0.85 * torch.rand(P, 1, generator=g, dtype=d), H=H, W=W, tanx=tanx,
                 tany=tany, view=view, proj=proj, campos=eye, bg=torch.tensor([0.2, 0.4, 0.7], dtype=d))
        if kind == "cov":
            Rm = GR.quat_rot(q)
            Mx = sc[:, :, None] * Rm
            S = Mx.transpose(1, 2) @ Mx
            s["cov3D"] = torch.stack([S[:, 0, 0], S[:, 0, 1], S[:, 0, 2], S[:, 1, 1], S[:, 1, 2], S[:, 2, 2]], 1)
            s["norm3D"] = torch.nn.functional.normalize(torch.randn(P, 3, generator=g, dtype=d), dim=1)
            s["colors"] = torch.rand(P, 3, generator=g, dtype=d)
        else:
            s["scales"], s["rotations"] = sc, q
            if kind == "sh":
                s["shs"] = 0.4 * torch.randn(P, 16, 3, generator=g, dtype=d)
                s["sh_degree"] = 3
                s["extra"] = torch.randn(P, 4, generator=g, dtype=d)
            else:
                s["colors"] = torch.rand(P, 3, generator=g, dtype=d)
        ED = s["extra"].shape[1] if "extra" in s else 0
        up = dict(color=torch.randn(3, H, W, generator=g, dtype=d), depth=torch.randn(1, H, W, generator=g, dtype=d),
                  norm=torch.randn(3, H, W, generator=g, dtype=d), alpha=torch.randn(1, H, W, generator=g, dtype=d))
        if ED:
            up["extra"] = torch.randn(ED, H, W, generator=g, dtype=d)
        out[name] = (s, up)
    return out


def main() -> int:
    out_path = Path(sys.argv[1])
    dev = torch.device("cuda")
    torch.zeros(1, device=dev)  # the runtime's primary context, current on this thread
    mods = {k: Module(REF / f"gs_{v}.cubin") for k, v in (("fwd", "forward"), ("bwd", "backward"), ("impl", "impl"))}
    save = {}
    for name, (s, up) in scenes().items():
        t = {k: (v.to(dev, torch.float32).contiguous() if torch.is_tensor(v) else v) for k, v in s.items()}
        u = {k: v.to(dev, torch.float32).contiguous() for k, v in up.items()}
        out, st = forward(mods, t)
        grads = backward(mods, t, out, st, u)
        for k, v in s.items():
            save[f"{name}/in/{k}"] = v.numpy() if torch.is_tensor(v) else np.asarray(v)
        for k, v in up.items():
            save[f"{name}/up/{k}"] = v.to(torch.float32).numpy()
        for k, v in out.items():
            if v is not None:
                save[f"{name}/out/{k}"] = v.cpu().numpy()
        save[f"{name}/out/radii"] = st["g"]["radii"].cpu().numpy()
        save[f"{name}/num_rendered"] = np.asarray(st["R"])
        for k, v in grads.items():
            if v is not None:
                save[f"{name}/grad/{k}"] = v.cpu().numpy()
        print(name, "rendered", st["R"], "visible", int((st["g"]["radii"] > 0).sum()))
    out_path.parent.mkdir(parents=True, exist_ok=True)
    np.savez_compressed(out_path, **save)
    print("wrote", out_path)
    return 0


if __name__ == "__main__":
    sys.exit(main())
