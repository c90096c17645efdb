"""The CUDA path against the reference-generated golden fixtures."""
import numpy as np
import pytest

import golden_cases as G

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", G.names())
def test_gpu_matches_reference(ctx, name):
    c = G.load(name)
    cid = ctx.upload(c["xyz"], c["labels"])
    if c["hull"].shape[0]:
        ctx.hull(cid, c["hull"], 2.0)
    ctx.tasks(c["trg"], c["env"])
    ctx.hist(c["rmin"], c["rincr"], c["rmax"])
    ctx.set_option("npcorr_order", c["npcorr_order"])
    ctx.run(cid, c["flags"], c["k"])
    out = ctx.fetch()
    st = ctx.stats()
    surf = ctx.surfdist_fetch(cid, c["xyz"].shape[0])
    assert np.array_equal(surf.view(np.uint32), c["surf"].view(np.uint32))
    assert st["centres"] == c["stats"]["centres"]
    assert st["pairs"] == c["stats"]["pairs"]
    assert np.array_equal(out, c["bins"])
    L = c["stats"]["cntnb_len"]
    if L:
        cn = ctx.fetch_cntnb()
        assert np.array_equal(cn, c["cntnb"].reshape(len(c["trg"]), L))
    if c["npcorr"].size:
        npc = ctx.fetch_npcorr()
        assert npc.size == c["npcorr"].size and np.array_equal(npc.reshape(-1), c["npcorr"])
    ctx.free(cid)


@pytest.mark.parametrize("name", G.names())
def test_gpu_voxelizer_matches_reference(ctx, name):
    c = G.load(name)
    cid = ctx.upload(c["xyz"], c["labels"])
    v = ctx.inside(cid, *c["bin_width"])
    ref = c["voxel"]
    assert v["nions_inside"] == ref["nions_inside"] and float(v["volume_inside"]) == ref["volume_inside"]
    assert (v["vacuum"], v["surface"], v["inside"]) == (ref["vacuum_bins"], ref["surface_bins"], ref["inside_bins"])
    assert (v["nx"], v["ny"], v["nz"]) == (ref["nx"], ref["ny"], ref["nz"])
    ctx.free(cid)
