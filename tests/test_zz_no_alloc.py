"""gh1_shape_eval_noalloc: shape evaluation into caller-owned device memory with
the library's fixed scratch array, for callers that cannot let the library
allocate.  Checked against gh1_shape_eval (the allocating entry point) on
consecutive calls that share the scratch, and against the FP64 CPU oracle's
shape functions directly; collected last so that it also runs after every
other GPU test has used the library."""
import ctypes
import os
import re

import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.conftest import ROOT

pytestmark = pytest.mark.gpu


def _max_entries():
    src = open(os.path.join(ROOT, "include", "gh1.h")).read()
    return int(re.search(r"#define\s+GH1_SHAPE_NOALLOC_MAX_ENTRIES\s+(\d+)", src).group(1))


def _nloc(et, p):
    return (p + 1) * (p + 2) * (p + 3) // 6 if et == 4 else (p + 1) ** 3


def _call(ctx, et, p, vn, d_pts, val, grd, npts=None):
    vnc = (ctypes.c_int32 * len(vn))(*vn)
    n = d_pts.shape[0] if npts is None else npts
    return ctx.lib.gh1_shape_eval_noalloc(ctx.h, et, p, vnc, n, ctypes.c_void_p(d_pts.data_ptr()),
                                          ctypes.c_void_p(val.data_ptr()), ctypes.c_void_p(grd.data_ptr()))


def _outputs(et, p, npts):
    n = _nloc(et, p)
    val = torch.full((npts, n), float("nan"), dtype=torch.float64, device="cuda")
    grd = torch.full((npts, n, 3), float("nan"), dtype=torch.float64, device="cuda")
    return val, grd


def _cases():
    rng = np.random.default_rng(2024)
    return [(8, 4, [5, 3, 0, 7, 1, 6, 2, 4], rng.uniform(0, 1, (1500, 3))),
            (4, 3, [7, 2, 9, 4], rng.dirichlet(np.ones(4), size=600)[:, :3]),
            (8, 2, [0, 1, 2, 3, 4, 5, 6, 7], rng.uniform(0, 1, (40, 3)))]


def test_noalloc_matches_allocating_entry(gpu):
    """Two (here three) calls in a row agree with gh1_shape_eval within the
    shape-parity tolerance (1e-13 values, 1e-12 gradients); the scratch left by
    one call does not leak into the next."""
    ctx = gpu.context(0)
    outs = []
    for et, p, vn, pts in _cases():
        d_pts = torch.from_numpy(np.ascontiguousarray(pts)).cuda()
        val, grd = _outputs(et, p, len(pts))
        ctx.check(_call(ctx, et, p, vn, d_pts, val, grd))
        torch.cuda.synchronize()
        rv, rg = gpu.ShapeEval(et, p, vn, pts)
        v, g = val.cpu().numpy(), grd.cpu().numpy()
        assert np.isfinite(v).all() and np.isfinite(g).all()
        assert np.abs(v - rv).max() < 1e-13 and np.abs(g - rg).max() < 1e-12
        ov, og = O.shapes(et, p, vn, pts)
        assert np.abs(v - ov).max() < 1e-13 and np.abs(g - og).max() < 1e-12
        outs.append((v, g))
    # repeating the first case after the others reproduces it exactly
    et, p, vn, pts = _cases()[0]
    d_pts = torch.from_numpy(np.ascontiguousarray(pts)).cuda()
    val, grd = _outputs(et, p, len(pts))
    ctx.check(_call(ctx, et, p, vn, d_pts, val, grd))
    torch.cuda.synchronize()
    assert np.array_equal(val.cpu().numpy(), outs[0][0]) and np.array_equal(grd.cpu().numpy(), outs[0][1])


def test_noalloc_allocates_nothing(gpu):
    """After a first call, further calls leave the device's free memory unchanged."""
    ctx = gpu.context(0)
    et, p, vn, pts = _cases()[0]
    d_pts = torch.from_numpy(np.ascontiguousarray(pts)).cuda()
    val, grd = _outputs(et, p, len(pts))
    ctx.check(_call(ctx, et, p, vn, d_pts, val, grd))
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(2):
        ctx.check(_call(ctx, et, p, vn, d_pts, val, grd))
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_oversize_and_host_memory(gpu):
    """Requests beyond the fixed scratch, and host buffers, fail with ERR_ARG
    before any device work."""
    from ngsolve_gb300._lib import GH1Error
    ctx = gpu.context(0)
    cap = _max_entries()
    et, p, vn = 8, 4, list(range(8))
    too_many = cap // _nloc(et, p) + 1
    d_pts = torch.zeros((4, 3), dtype=torch.float64, device="cuda")
    val, grd = _outputs(et, p, 4)
    rc = _call(ctx, et, p, vn, d_pts, val, grd, npts=too_many)
    assert rc == 1
    with pytest.raises(GH1Error, match="exceeds the fixed scratch"):
        ctx.check(rc)
    h_pts = torch.zeros((4, 3), dtype=torch.float64)
    with pytest.raises(GH1Error, match="device memory"):
        ctx.check(_call(ctx, et, p, vn, h_pts, val, grd))
    # the largest accepted size still runs and matches the allocating entry
    npts = cap // _nloc(et, p)
    pts = np.random.default_rng(3).uniform(0, 1, (npts, 3))
    d_pts = torch.from_numpy(pts).cuda()
    val, grd = _outputs(et, p, npts)
    ctx.check(_call(ctx, et, p, vn, d_pts, val, grd))
    torch.cuda.synchronize()
    rv, rg = gpu.ShapeEval(et, p, vn, pts)
    assert np.abs(val.cpu().numpy() - rv).max() < 1e-13 and np.abs(grd.cpu().numpy() - rg).max() < 1e-12
