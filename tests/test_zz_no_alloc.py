"""pp_surfdist_noalloc (ion2surf with every buffer in a static device array)
against the allocating path -- pp_hull_upload + pp_run + pp_surfdist_fetch --
on two clouds, called twice in a row so the second call starts from the
scratch contents the first one left.  Results are bit-identical: both paths
take the minimum of the same per-triangle float distances.

Kept in a file of its own that pytest collects last; it passes alone in a
fresh process as well as after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from paraprobe_gb300 import native as N
from paraprobe_gb300 import synth

pytestmark = pytest.mark.gpu


def _noalloc(lib, torch, xyz, tri, rp):
    dx = torch.from_numpy(np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1)).to("cuda")
    dt = torch.from_numpy(np.ascontiguousarray(tri, dtype=np.float32).reshape(-1)).to("cuda")
    out = torch.full((xyz.shape[0],), -1.0, dtype=torch.float32, device="cuda")
    err = C.create_string_buffer(256)
    rc = lib.pp_surfdist_noalloc(C.c_void_p(dx.data_ptr()), xyz.shape[0], C.c_void_p(dt.data_ptr()), tri.shape[0],
                                 rp, C.c_void_p(out.data_ptr()), None, err, 256)
    assert rc == N.PP_OK, err.value.decode()
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _allocating(ctx, spec, carve, rmax):
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, carve)
    ctx.tasks([[1]], [[1]])
    ctx.hist(0.0, 0.01, rmax)
    ctx.run(cid, N.PP_RDF, [])
    ctx.fetch()
    d2 = ctx.surfdist_fetch(cid, spec.xyz.shape[0])
    ctx.free(cid)
    return d2


def test_noalloc_matches_allocating_path_twice(ctx):
    torch = pytest.importorskip("torch")
    lib = N.load()
    cone = synth.cone_specimen(n=60000, r_apex=8.0, half_angle_deg=10.0, length=20.0, n_clusters=20,
                               members=40, nspecies=3, seed=41, nseg=96, stack=3.0)
    cyl = synth.cylinder_specimen(n=25000, radius=6.0, height=12.0, nseg=48, stack=2.0, seed=43)
    cases = [(cone, 2.0, 1.2), (cyl, 1.0, 1.5)]
    for spec, carve, rmax in cases:
        ref = _allocating(ctx, spec, carve, rmax)
        got = _noalloc(lib, torch, spec.xyz, spec.hull, max(rmax, carve))
        assert got.dtype == np.float32 and got.shape == ref.shape
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
        assert (got < np.float32(max(rmax, carve)) ** 2).any()


def test_noalloc_rejects_oversized_hull(ctx):
    torch = pytest.importorskip("torch")
    lib = N.load()
    buf = torch.zeros(9, dtype=torch.float32, device="cuda")
    out = torch.zeros(1, dtype=torch.float32, device="cuda")
    err = C.create_string_buffer(256)
    rc = lib.pp_surfdist_noalloc(C.c_void_p(buf.data_ptr()), 1, C.c_void_p(buf.data_ptr()), 2_000_001, 2.0,
                                 C.c_void_p(out.data_ptr()), None, err, 256)
    assert rc == N.PP_ERR_UNSUPPORTED
    assert b"2000001 triangles" in err.value
