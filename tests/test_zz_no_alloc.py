"""The allocation-free mass loss against the regular one.

mpm_mass_loss_noalloc serves callers that cannot allocate device memory
(a fixed device-memory budget that may not grow, a host runtime that owns
every allocation): it takes the caller's device buffers and keeps its own
scratch in a static device array.  Here it is called through the C ABI
twice in a row, on different inputs, and each result is compared with
mpm_compgraph_mass_loss (CompGraph.end_layer_mass_loss) on the same
particles: loss within 1e-6 relative, dL/dx within 1e-5 in norm (both FP32;
only the order of the atomic sums differs).  A call after the first one
leaves the device's free memory unchanged, and a stream under capture is
refused (the call is synchronous).
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _inputs(seed, shift):
    from diffmpm_bindings import workloads as W
    w = W.sphere32(seed=seed, G=20)
    g = O.Grid(w.dims, w.dx)
    tgt = np.zeros(g.n_nodes)
    O.Oracle().p2g_accumulate(g, w.x + shift, w.v, np.zeros((w.n, 3, 3)), w.m, tgt, np.zeros((g.n_nodes, 3)))
    return w, g, tgt


def _regular(dm, w, g, tgt, adjoint):
    pc = dm.PointCloud.from_arrays(w.x.astype(np.float32), m=w.m.astype(np.float32))
    grid = dm.Grid(*g.dims, g.dx, g.min)
    target = dm.Grid(*g.dims, g.dx, g.min)
    target.set_node_masses(tgt)
    cg = dm.CompGraph(pc, grid, target, adjoint=adjoint)
    loss = cg.end_layer_mass_loss()
    return loss, cg.get_grad(0, "x", np.float64)


def _noalloc(dm, torch, w, g, tgt, exact):
    dev = torch.device("cuda")
    x = torch.tensor(w.x, dtype=torch.float32, device=dev).contiguous()
    m = torch.tensor(w.m, dtype=torch.float32, device=dev).contiguous()
    t = torch.tensor(tgt, dtype=torch.float32, device=dev).contiguous()
    gx = torch.full((w.n, 3), float("nan"), dtype=torch.float32, device=dev)
    dims = (C.c_int * 3)(*g.dims)
    mn = (C.c_double * 3)(*g.min)
    loss = C.c_double()
    torch.cuda.synchronize()
    rc = dm._lib.lib.mpm_mass_loss_noalloc(w.n, C.c_void_p(x.data_ptr()), C.c_void_p(m.data_ptr()),
                                          C.c_void_p(t.data_ptr()), dims, C.c_double(g.dx), mn, int(exact),
                                          C.c_void_p(gx.data_ptr()), C.byref(loss), None)
    assert rc == 0, dm._lib.lib.mpm_last_error()
    return loss.value, gx.double().cpu().numpy()


@pytest.mark.parametrize("adjoint", ["reference", "exact"])
def test_noalloc_mass_loss_matches_regular_entry_point(dm, adjoint):
    torch = pytest.importorskip("torch")
    for call, (seed, shift) in enumerate(((0, 0.0), (5, 0.017))):
        w, g, tgt = _inputs(seed, shift)
        want_loss, want_gx = _regular(dm, w, g, tgt, adjoint)
        loss, gx = _noalloc(dm, torch, w, g, tgt, adjoint == "exact")
        assert abs(loss - want_loss) <= 1e-6 * abs(want_loss), (call, loss, want_loss)
        err = np.linalg.norm(gx - want_gx) / np.linalg.norm(want_gx)
        assert err <= 1e-5, (call, err)


def test_noalloc_call_leaves_free_device_memory_unchanged(dm):
    """After one call on the device (which loads the library's module and so
    its static scratch), a further call on other inputs changes the device's
    free memory by nothing: no allocation happens on the call path."""
    torch = pytest.importorskip("torch")
    a, b = _inputs(1, 0.0), _inputs(2, 0.011)
    _noalloc(dm, torch, *a, False)  # module load happens here, if not before
    dev = torch.device("cuda")
    w, g, tgt = b
    x = torch.tensor(w.x, dtype=torch.float32, device=dev).contiguous()
    m = torch.tensor(w.m, dtype=torch.float32, device=dev).contiguous()
    t = torch.tensor(tgt, dtype=torch.float32, device=dev).contiguous()
    gx = torch.empty((w.n, 3), dtype=torch.float32, device=dev)
    dims = (C.c_int * 3)(*g.dims)
    mn = (C.c_double * 3)(*g.min)
    loss = C.c_double()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    rc = dm._lib.lib.mpm_mass_loss_noalloc(w.n, C.c_void_p(x.data_ptr()), C.c_void_p(m.data_ptr()),
                                          C.c_void_p(t.data_ptr()), dims, C.c_double(g.dx), mn, 1,
                                          C.c_void_p(gx.data_ptr()), C.byref(loss), None)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert rc == 0, dm._lib.lib.mpm_last_error()
    assert free1 == free0, (free0, free1)
    assert np.isfinite(loss.value) and torch.isfinite(gx).all()


def test_noalloc_refuses_a_stream_under_capture(dm):
    """The call is synchronous, so a stream being captured is refused before
    any work is queued on it; the capture itself stays valid."""
    torch = pytest.importorskip("torch")
    w, g, tgt = _inputs(3, 0.0)
    dev = torch.device("cuda")
    x = torch.tensor(w.x, dtype=torch.float32, device=dev).contiguous()
    m = torch.tensor(w.m, dtype=torch.float32, device=dev).contiguous()
    t = torch.tensor(tgt, dtype=torch.float32, device=dev).contiguous()
    gx = torch.zeros((w.n, 3), dtype=torch.float32, device=dev)
    dims = (C.c_int * 3)(*g.dims)
    mn = (C.c_double * 3)(*g.min)
    loss = C.c_double()
    y = torch.zeros(4, device=dev)
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    torch.cuda.synchronize()
    with torch.cuda.graph(graph, stream=side):
        rc = dm._lib.lib.mpm_mass_loss_noalloc(w.n, C.c_void_p(x.data_ptr()), C.c_void_p(m.data_ptr()),
                                              C.c_void_p(t.data_ptr()), dims, C.c_double(g.dx), mn, 0,
                                              C.c_void_p(gx.data_ptr()), C.byref(loss),
                                              C.c_void_p(side.cuda_stream))
        y.add_(1.0)
    graph.replay()
    torch.cuda.synchronize()
    assert rc == dm._lib.MPM_ERR_STATE
    assert b"captured" in dm._lib.lib.mpm_last_error()
    assert float(y.sum()) == 4.0


def test_noalloc_rejects_oversized_grid(dm):
    lib = dm._lib.lib
    dims = (C.c_int * 3)(128, 128, 128)  # 2,097,152 nodes > MPM_NOALLOC_MAX_NODES
    loss = C.c_double()
    rc = lib.mpm_mass_loss_noalloc(0, None, None, C.c_void_p(1), dims, C.c_double(1.0), None, 0, None,
                                   C.byref(loss), None)
    assert rc == dm._lib.MPM_ERR_SHAPE
    assert b"MPM_NOALLOC_MAX_NODES" in lib.mpm_last_error()
