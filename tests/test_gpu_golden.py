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


def _groups(flags, ntasks, nk, H):
    """(flag, offset, length) of each histogram group in the pp_fetch layout."""
    out, o = [], 0
    for f, n in ((1, ntasks), (2, ntasks), (4, ntasks), (8, ntasks * nk)):
        if flags & f:
            out.append((f, o, n * H))
            o += n * H
    return out


@pytest.mark.parametrize("lists", [0, 2])
@pytest.mark.parametrize("name", G.names())
def test_gpu_lanes_match_reference(ctx, name, lists):
    """The centre-per-lane scans on the reference fixtures, forced by a cell
    block shape: the fixture's RDF/RIPK analyses as one pass and its 1NN/kNN
    analyses as another, each against the matching groups of the reference's
    bins (passes the centre-per-lane kernels cannot take run the per-centre
    scan and must match all the same).  lists = 2 keeps the kNN lists as bin
    categories instead of distances."""
    c = G.load(name)
    flags = c["flags"] & (1 | 2 | 4 | 8)
    cid = ctx.upload(c["xyz"], c["labels"])
    if c["hull"].shape[0]:
        ctx.hull(cid, c["hull"], 2.0)
    ctx.tuning(cid, 4.0, ((4 | 2 << 8 | 2 << 12) << 16) | 0x100)
    ctx.tasks(c["trg"], c["env"])
    ctx.hist(c["rmin"], c["rincr"], c["rmax"])
    ctx.set_option("knn_lists", lists)
    try:
        _lanes_parts(ctx, c, cid, name, flags)
    finally:
        ctx.set_option("knn_lists", 0)
        ctx.free(cid)


def _lanes_parts(ctx, c, cid, name, flags):
    ntasks, nk = len(c["trg"]), len(c["k"]) if c["flags"] & 8 else 0
    H = c["stats"]["nbins"] + 2
    ref = {f: c["bins"][o:o + n] for f, o, n in _groups(c["flags"], ntasks, nk, H)}
    kernels = []
    for part in (flags & (1 | 4), flags & (2 | 8)):
        if not part:
            continue
        ks = c["k"] if part & 8 else []
        ctx.run(cid, part, ks)
        out, st = ctx.fetch(), ctx.stats()
        kernels.append(ctx.last_kernel())
        assert st["pairs"] == c["stats"]["pairs"] and st["centres"] == c["stats"]["centres"]
        want = np.concatenate([ref[f] for f, _, _ in _groups(part, ntasks, len(ks), H)])
        assert np.array_equal(out, want), (name, part, kernels[-1])
    if flags & (1 | 4) and flags & (2 | 8):
        # both in one pass: the RDF/RIPK and the kNN centre-per-lane passes
        # (or the per-centre scan for kNN with overlapping sets) one after the other
        ks = c["k"] if flags & 8 else []
        ctx.run(cid, flags, ks)
        out, st = ctx.fetch(), ctx.stats()
        kernels.append(ctx.last_kernel())
        assert kernels[-1].startswith("k_lanes+")
        assert st["pairs"] == c["stats"]["pairs"] and st["centres"] == c["stats"]["centres"]
        want = np.concatenate([ref[f] for f, _, _ in _groups(flags, ntasks, len(ks), H)])
        assert np.array_equal(out, want), (name, flags, kernels[-1])
    assert kernels
    print(f"{name}: {kernels}")
