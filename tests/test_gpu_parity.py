"""GPU path (through the C ABI) against the CPU oracle on seeded clouds.

Counts must be bit-identical: the oracle restates the reference's float
arithmetic, and the device evaluates the same expressions without
contraction, binning through an exact threshold table.
"""
import numpy as np
import pytest

from paraprobe_gb300 import native as N
from paraprobe_gb300 import synth

pytestmark = pytest.mark.gpu

ALL = N.PP_RDF | N.PP_1NN | N.PP_RIPK | N.PP_MKNN


def BRICK(cells, batch):
    """Tile code of the brick scan: cells per brick, centres per warp batch."""
    return (cells << 16) | batch


def _run_both(ctx, oracle, spec, rmin, rincr, rmax, flags, trg, env, ks, surf=None, perm_labels=None, carve=2.0):
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, carve)
    ctx.tasks(trg, env)
    ctx.hist(rmin, rincr, rmax)
    perm = None
    labels = spec.labels
    if perm_labels is not None:
        perm, labels = perm_labels
    ctx.run(cid, flags, ks, label_perm=perm)
    gpu = ctx.fetch()
    st = ctx.stats()
    gs = ctx.surfdist_fetch(cid, spec.xyz.shape[0])
    rp = max(np.float32(rmax), np.float32(carve))
    cs = oracle.surface_distance(spec.xyz, spec.hull, rp)
    assert np.array_equal(gs.view(np.uint32), cs.view(np.uint32)), "ion2surf differs"
    ref = oracle.spatstat(spec.xyz, labels, cs, rmin, rincr, rmax, flags, trg, env, ks)
    cnt = None
    if flags & N.PP_CNTNB:
        cnt = ctx.fetch_cntnb()
    ctx.free(cid)
    return gpu, st, ref, cnt


def test_cylinder_all_analyses(ctx, oracle):
    spec = synth.cylinder_specimen(n=40000, radius=6.0, height=24.0, seed=11, nseg=96, stack=4.0)
    trg = [[2], [1], [2, 3]]
    env = [[1, 2, 3], [2], [3]]
    gpu, st, ref, _ = _run_both(ctx, oracle, spec, 0.0, 0.01, 1.0, ALL, trg, env, [10, 5, 1])
    assert st["centres"] == ref["centres"]
    assert st["pairs"] == ref["pairs"]
    assert gpu.shape == ref["bins"].shape
    bad = np.nonzero(gpu != ref["bins"])[0]
    assert bad.size == 0, f"{bad.size} bins differ, first {bad[:10]}"


def test_cone_all_pairs_knn(ctx, oracle):
    spec = synth.cone_specimen(n=60000, r_apex=8.0, half_angle_deg=10.0, length=20.0, n_clusters=30,
                               members=40, nspecies=4, seed=5, nseg=96, stack=4.0)
    types = [1, 2, 3, 4]
    trg = [[a] for a in types for b in types]
    env = [[b] for a in types for b in types]
    gpu, st, ref, _ = _run_both(ctx, oracle, spec, 0.0, 0.005, 1.5, ALL, trg, env, [8, 3, 1])
    assert st["pairs"] == ref["pairs"]
    assert np.array_equal(gpu, ref["bins"])


def test_cntnb(ctx, oracle):
    spec = synth.cylinder_specimen(n=20000, radius=5.0, height=16.0, seed=3, nseg=64, stack=4.0)
    trg, env = [[2], [1, 2]], [[1, 2, 3], [3]]
    gpu, st, ref, cnt = _run_both(ctx, oracle, spec, 0.0, 0.02, 1.2, N.PP_RDF | N.PP_CNTNB, trg, env, [])
    L = cnt.shape[1]
    assert np.array_equal(cnt, ref["cntnb"][:, :L])
    assert ref["cntnb"][:, L:].sum() == 0


def test_nonzero_rmin_and_coarse_bins(ctx, oracle):
    spec = synth.cylinder_specimen(n=20000, radius=5.0, height=16.0, seed=4, nseg=64, stack=4.0)
    trg, env = [[1], [2]], [[1, 2, 3], [1]]
    # 0.1 nm bins over [0.3, 1.3]: (1.0/0.1f) truncates to 9 bins, d == R goes to the upper dump
    gpu, st, ref, _ = _run_both(ctx, oracle, spec, 0.3, 0.1, 1.3, ALL, trg, env, [40, 2])
    assert ref["nbins"] == 9
    assert np.array_equal(gpu, ref["bins"])


def test_large_k_register_rows(ctx, oracle):
    spec = synth.cylinder_specimen(n=30000, radius=5.0, height=20.0, seed=8, nseg=64, stack=4.0)
    trg, env = [[1], [2]], [[1, 2, 3], [1, 2]]
    gpu, st, ref, _ = _run_both(ctx, oracle, spec, 0.0, 0.01, 1.3, N.PP_MKNN | N.PP_1NN, trg, env, [100, 64, 33, 7])
    assert np.array_equal(gpu, ref["bins"])


def test_label_permutation(ctx, oracle):
    spec = synth.cylinder_specimen(n=20000, radius=5.0, height=16.0, seed=9, nseg=64, stack=4.0)
    rng = np.random.default_rng(1)
    perm = rng.permutation(spec.xyz.shape[0]).astype(np.uint32)
    shuffled = spec.labels[perm]
    trg, env = [[2]], [[1, 2, 3]]
    gpu, st, ref, _ = _run_both(ctx, oracle, spec, 0.0, 0.01, 1.0, ALL, trg, env, [5, 1],
                                perm_labels=(perm, shuffled))
    assert np.array_equal(gpu, ref["bins"])


def test_neighbor_sets(ctx, oracle):
    spec = synth.cylinder_specimen(n=20000, radius=5.0, height=16.0, seed=2, nseg=64, stack=4.0)
    cid = ctx.upload(spec.xyz, spec.labels)
    for ion in (0, 17, 12345):
        ids, d2 = ctx.neighbors(cid, ion, 1.0)
        rid, rd2 = oracle.neighbors(spec.xyz, ion, 1.0)
        assert np.array_equal(ids, rid)
        assert np.array_equal(d2.view(np.uint32), rd2.view(np.uint32))
    ctx.free(cid)


def test_batched_matches_plain(ctx, oracle):
    spec = synth.cone_specimen(n=40000, r_apex=8.0, half_angle_deg=10.0, length=16.0, n_clusters=20,
                               members=40, nspecies=3, seed=13, nseg=64, stack=4.0)
    types = [1, 2, 3]
    trg = [[a] for a in types for b in types]
    env = [[b] for a in types for b in types]
    rmin, rincr, rmax = 0.0, 0.01, 1.2
    ks = [8, 2, 1]
    flags = N.PP_RDF | N.PP_1NN | N.PP_MKNN
    sets = np.stack([N.shuffle_labels(spec.labels, 100 + s) for s in range(3)])
    rois = np.array([[0.0, 0.0, 8.0, 6.0], [2.0, -1.0, 5.0, 3.5]], dtype=np.float32)
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    ctx.tasks(trg, env)
    ctx.hist(rmin, rincr, rmax)
    ctx.run_batched(cid, flags, ks, include_original=True, label_sets=sets, rois=rois)
    assert ctx.batched_count() == 1 + 3 + 2
    surf = oracle.surface_distance(spec.xyz, spec.hull, 2.0)
    outs = [ctx.fetch_batched(r) for r in range(6)]
    ref0 = oracle.spatstat(spec.xyz, spec.labels, surf, rmin, rincr, rmax, flags, trg, env, ks)
    assert np.array_equal(outs[0], ref0["bins"])
    for q in range(3):
        refq = oracle.spatstat(spec.xyz, sets[q], surf, rmin, rincr, rmax, flags, trg, env, ks)
        assert np.array_equal(outs[1 + q], refq["bins"]), f"label set {q}"
    for q in range(2):
        c = rois[q]
        d = np.sqrt(((spec.xyz - c[:3]) ** 2).sum(axis=1, dtype=np.float32)).astype(np.float32)
        # the device evaluates |p-c| from the float d^2 expression; recompute it the same way
        dx = (spec.xyz[:, 0] - c[0]).astype(np.float32)
        dy = (spec.xyz[:, 1] - c[1]).astype(np.float32)
        dz = (spec.xyz[:, 2] - c[2]).astype(np.float32)
        d = np.sqrt((dx * dx + dy * dy) + dz * dz).astype(np.float32)
        mask = ((np.float32(c[3]) - d) >= np.float32(rmax)).astype(np.uint8)
        refq = oracle.spatstat(spec.xyz, spec.labels, surf, rmin, rincr, rmax, flags, trg, env, ks, centre_mask=mask)
        assert np.array_equal(outs[4 + q], refq["bins"]), f"roi {q}"
    ctx.free(cid)


@pytest.mark.parametrize("rincr,nsets", [(0.001, 5), (0.02, 1), (0.0005, 2)])
def test_batched_overlapping_sets(ctx, oracle, rincr, nsets):
    """Overlapping environment sets, cumulative RIPK and an unsorted k list;
    the bin widths select 2-, 4- and 1-realisation groups in the batched kernel."""
    spec = synth.cone_specimen(n=30000, r_apex=8.0, half_angle_deg=10.0, length=14.0, n_clusters=15,
                               members=40, nspecies=3, seed=31, nseg=64, stack=4.0)
    trg = [[1], [2], [3, 1], [1, 2, 3]]
    env = [[1, 2], [2, 3], [1, 2, 3], [3]]
    rmin, rmax = 0.0, 1.2
    ks = [3, 12, 1, 5]
    flags = ALL
    sets = np.stack([N.shuffle_labels(spec.labels, 700 + s) for s in range(nsets)])
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    ctx.tasks(trg, env)
    ctx.hist(rmin, rincr, rmax)
    ctx.run_batched(cid, flags, ks, include_original=True, label_sets=sets)
    assert ctx.batched_count() == 1 + nsets
    surf = oracle.surface_distance(spec.xyz, spec.hull, 2.0)
    ref0 = oracle.spatstat(spec.xyz, spec.labels, surf, rmin, rincr, rmax, flags, trg, env, ks)
    assert np.array_equal(ctx.fetch_batched(0), ref0["bins"])
    for q in range(nsets):
        refq = oracle.spatstat(spec.xyz, sets[q], surf, rmin, rincr, rmax, flags, trg, env, ks)
        assert np.array_equal(ctx.fetch_batched(1 + q), refq["bins"]), f"label set {q}"
    ctx.free(cid)


def test_batched_graph_replay(ctx, oracle):
    """A second batched run with the same plan replays the captured graph and
    gives the same bins; new label sets in the same buffers replay it too."""
    spec = synth.cone_specimen(n=30000, r_apex=8.0, half_angle_deg=10.0, length=14.0, n_clusters=15,
                               members=40, nspecies=3, seed=37, nseg=64, stack=4.0)
    types = [1, 2, 3]
    trg = [[a] for a in types for b in types]
    env = [[b] for a in types for b in types]
    ks = [4, 2, 1]
    flags = N.PP_RDF | N.PP_MKNN
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    ctx.tasks(trg, env)
    ctx.hist(0.0, 0.02, 1.2)
    sets = np.stack([N.shuffle_labels(spec.labels, 900 + s) for s in range(5)])
    ctx.run_batched(cid, flags, ks, include_original=True, label_sets=sets)
    first = [ctx.fetch_batched(r) for r in range(6)]
    g1 = ctx.batched_graph()
    assert g1["nodes"] >= 1
    ctx.run_batched(cid, flags, ks, include_original=True, label_sets=sets)
    g2 = ctx.batched_graph()
    assert g2["captures"] == g1["captures"] and g2["launches"] == g1["launches"] + 1
    for r in range(6):
        assert np.array_equal(ctx.fetch_batched(r), first[r])
    sets2 = np.stack([N.shuffle_labels(spec.labels, 950 + s) for s in range(5)])
    ctx.run_batched(cid, flags, ks, include_original=True, label_sets=sets2)
    assert ctx.batched_graph()["captures"] == g1["captures"]
    surf = oracle.surface_distance(spec.xyz, spec.hull, 2.0)
    ref = oracle.spatstat(spec.xyz, sets2[3], surf, 0.0, 0.02, 1.2, flags, trg, env, ks)
    assert np.array_equal(ctx.fetch_batched(4), ref["bins"])
    ctx.free(cid)


def test_results_independent_of_tuning(ctx, oracle):
    spec = synth.cone_specimen(n=50000, r_apex=8.0, half_angle_deg=10.0, length=20.0, n_clusters=25,
                               members=40, nspecies=3, seed=21, nseg=64, stack=4.0)
    types = [1, 2, 3]
    trg = [[a] for a in types for b in types]
    env = [[b] for a in types for b in types]
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    ctx.tasks(trg, env)
    ctx.hist(0.0, 0.01, 1.4)
    outs = []
    for ratio, tile in ((2.0, 1), (3.5, 64), (5.0, 7), (1.0, 1000), (4.0, BRICK(8, 16)), (2.0, BRICK(1, 1)),
                        (5.0, BRICK(16, 32)), (3.0, BRICK(3, 5))):
        ctx.tuning(cid, ratio, tile)
        ctx.run(cid, ALL, [6, 2, 1])
        outs.append(ctx.fetch())
    r, t = ctx.autotune(cid, ALL, [6, 2, 1], sample=2000)
    lanes = t >= 65536 and (t & 0xffff) == N.PP_TILE_LANES
    assert 2.0 <= r <= 5.0 and (t in (32, 128, 512) or (t >> 16) in (4, 8, 16) or lanes)
    ctx.run(cid, ALL, [6, 2, 1])
    outs.append(ctx.fetch())
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])
    surf = oracle.surface_distance(spec.xyz, spec.hull, 2.0)
    ref = oracle.spatstat(spec.xyz, spec.labels, surf, 0.0, 0.01, 1.4, ALL, trg, env, [6, 2, 1])
    assert np.array_equal(outs[0], ref["bins"])
    ctx.free(cid)


def test_symmetric_rdf_pass(ctx, oracle):
    """RDF/RIPK-only passes take each pair of two centres once; counts must equal
    the per-centre scan's, including non-centre neighbours, a label
    permutation and a non-zero lower radius."""
    spec = synth.cone_specimen(n=60000, r_apex=8.0, half_angle_deg=10.0, length=20.0, n_clusters=30,
                               members=40, nspecies=4, seed=31, nseg=96, stack=4.0)
    trg = [[1], [2, 3], [4]]
    env = [[1, 2], [1, 2, 3], [1]]
    rng = np.random.default_rng(5)
    perm = rng.permutation(spec.xyz.shape[0]).astype(np.uint32)
    for p in (None, perm):
        labels = spec.labels if p is None else spec.labels[p]
        gpu, st, ref, _ = _run_both(ctx, oracle, spec, 0.1, 0.02, 1.6, N.PP_RDF | N.PP_RIPK, trg, env, [],
                                    perm_labels=None if p is None else (p, labels))
        assert st["pairs"] == ref["pairs"]
        assert np.array_equal(gpu, ref["bins"])


@pytest.mark.parametrize("tile", [BRICK(8, 16), BRICK(1, 1), BRICK(16, 32), BRICK(5, 7)])
@pytest.mark.parametrize("ratio", [2.0, 3.0, 5.0])
def test_brick_scan(ctx, oracle, tile, ratio):
    """The brick scan against the oracle: a symmetric RDF/RIPK pass under a
    label permutation with a non-zero lower radius, and a kNN pass over all
    species pairs (disjoint environment sets)."""
    spec = synth.cone_specimen(n=40000, r_apex=8.0, half_angle_deg=10.0, length=16.0, n_clusters=20,
                               members=40, nspecies=3, seed=53, nseg=64, stack=4.0)
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    ctx.tuning(cid, ratio, tile)
    surf = oracle.surface_distance(spec.xyz, spec.hull, 2.0)
    rng = np.random.default_rng(int(ratio * 10) + (tile >> 16))
    perm = rng.permutation(spec.xyz.shape[0]).astype(np.uint32)
    lab = spec.labels[perm]
    trg, env = [[1], [2, 3], [3]], [[1, 2], [1, 2, 3], [1]]
    ctx.tasks(trg, env)
    ctx.hist(0.1, 0.02, 1.3)
    ctx.set_option("lanes", 0)  # both passes through the brick scan, not the centre-per-lane scan
    try:
        ctx.run(cid, N.PP_RDF | N.PP_RIPK, [], label_perm=perm)
        gpu, st = ctx.fetch(), ctx.stats()
        ref = oracle.spatstat(spec.xyz, lab, surf, 0.1, 0.02, 1.3, N.PP_RDF | N.PP_RIPK, trg, env, [])
        assert st["pairs"] == ref["pairs"] and np.array_equal(gpu, ref["bins"])
        types = [1, 2, 3]
        trg = [[a] for a in types for b in types]
        env = [[b] for a in types for b in types]
        ctx.tasks(trg, env)
        ctx.hist(0.0, 0.005, 1.2)
        ks = [12, 3, 1]
        ctx.run(cid, N.PP_1NN | N.PP_MKNN, ks)
        gpu, st = ctx.fetch(), ctx.stats()
    finally:
        ctx.set_option("lanes", 1)
    ref = oracle.spatstat(spec.xyz, spec.labels, surf, 0.0, 0.005, 1.2, N.PP_1NN | N.PP_MKNN, trg, env, ks)
    assert st["pairs"] == ref["pairs"] and np.array_equal(gpu, ref["bins"])
    ctx.free(cid)


@pytest.mark.parametrize("rincr", [0.02, 0.001])
def test_batched_chunked_geometry(ctx, oracle, rincr):
    """Pair lists held a chunk of centres at a time (batched_pair_cap) give the
    same bins as lists held whole, for the fused and the 32-realisation kNN
    kernels."""
    spec = synth.cone_specimen(n=30000, r_apex=8.0, half_angle_deg=10.0, length=14.0, n_clusters=15,
                               members=40, nspecies=3, seed=61, nseg=64, stack=4.0)
    types = [1, 2, 3]
    trg = [[a] for a in types for b in types]
    env = [[b] for a in types for b in types]
    ks = [5, 2, 1]
    flags = N.PP_RDF | N.PP_MKNN
    sets = np.stack([N.shuffle_labels(spec.labels, 300 + s) for s in range(4)])
    rois = np.array([[0.0, 0.0, 7.0, 5.0]], dtype=np.float32)
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    ctx.tasks(trg, env)
    ctx.hist(0.0, rincr, 1.2)
    ctx.run_batched(cid, flags, ks, include_original=True, label_sets=sets, rois=rois)
    whole = [ctx.fetch_batched(r) for r in range(6)]
    pairs = sum(ctx.batched_stats(r)["pairs"] for r in range(6))
    try:
        ctx.set_option("batched_pair_cap", 20000)
        ctx.run_batched(cid, flags, ks, include_original=True, label_sets=sets, rois=rois)
        for r in range(6):
            assert np.array_equal(ctx.fetch_batched(r), whole[r]), r
        assert sum(ctx.batched_stats(r)["pairs"] for r in range(6)) == pairs
    finally:
        ctx.set_option("batched_pair_cap", 0)
    surf = oracle.surface_distance(spec.xyz, spec.hull, 2.0)
    ref = oracle.spatstat(spec.xyz, sets[2], surf, 0.0, rincr, 1.2, flags, trg, env, ks)
    assert np.array_equal(whole[3], ref["bins"])
    ctx.free(cid)


@pytest.mark.parametrize("nsets", [33, 40])
def test_batched_32_lane_groups_and_rest(ctx, oracle, nsets):
    """More than 32 realisations: full 32-lane kNN groups, plus either a short
    rest taken by the rank walk (1 + 33 = 34: rest 2) or a partly filled group
    (1 + 40 = 41: rest 9); realisations on both sides of the split checked."""
    spec = synth.cone_specimen(n=20000, r_apex=8.0, half_angle_deg=10.0, length=10.0, n_clusters=10,
                               members=40, nspecies=3, seed=71, nseg=48, stack=4.0)
    types = [1, 2, 3]
    trg = [[a] for a in types for b in types]
    env = [[b] for a in types for b in types]
    ks = [4, 1]
    flags = N.PP_RDF | N.PP_MKNN
    sets = np.stack([N.shuffle_labels(spec.labels, 1200 + s) for s in range(nsets)])
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    ctx.tasks(trg, env)
    ctx.hist(0.0, 0.02, 1.1)
    ctx.run_batched(cid, flags, ks, include_original=True, label_sets=sets)
    assert ctx.batched_count() == 1 + nsets
    surf = oracle.surface_distance(spec.xyz, spec.hull, 2.0)
    for r in (0, 5, 31, 32, 33, nsets):
        lab = spec.labels if r == 0 else sets[r - 1]
        ref = oracle.spatstat(spec.xyz, lab, surf, 0.0, 0.02, 1.1, flags, trg, env, ks)
        assert np.array_equal(ctx.fetch_batched(r), ref["bins"]), r
    ctx.free(cid)


@pytest.mark.parametrize("nspecies,ks", [(10, [12, 3, 1]), (6, [20, 9, 2, 1]), (8, [5, 4, 3, 2, 1])])
def test_batched_walk_set_counts(ctx, oracle, nspecies, ks):
    """The 32-realisation kNN walk with one environment set per species for
    every centre type (six, eight or ten sets), k up to 20, realisations of the
    first 32-lane group and of the second."""
    spec = synth.cone_specimen(n=20000, r_apex=8.0, half_angle_deg=10.0, length=10.0, n_clusters=10,
                               members=40, nspecies=nspecies, seed=83 + nspecies, nseg=48, stack=4.0,
                               iid=(0.04, 0.03, 0.02))
    types = list(range(1, nspecies + 1))
    trg = [[a] for a in types[:3] for b in types]
    env = [[b] for a in types[:3] for b in types]
    flags = N.PP_1NN | N.PP_MKNN
    sets = np.stack([N.shuffle_labels(spec.labels, 1300 + s) for s in range(33)])
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    ctx.tasks(trg, env)
    ctx.hist(0.0, 0.01, 1.2)
    ctx.run_batched(cid, flags, ks, include_original=True, label_sets=sets)
    assert ctx.batched_count() == 34
    surf = oracle.surface_distance(spec.xyz, spec.hull, 2.0)
    for r in (0, 1, 31, 32, 33):
        lab = spec.labels if r == 0 else sets[r - 1]
        ref = oracle.spatstat(spec.xyz, lab, surf, 0.0, 0.01, 1.2, flags, trg, env, ks)
        assert np.array_equal(ctx.fetch_batched(r), ref["bins"]), r
    ctx.free(cid)


@pytest.mark.parametrize("order", [0, 4])
def test_npcorr_matches_oracle(ctx, oracle, order):
    """n-point correlations (analysis mode 5) with overlapping environment sets,
    beside RDF in the same pass."""
    spec = synth.cone_specimen(n=25000, r_apex=8.0, half_angle_deg=10.0, length=12.0, n_clusters=12,
                               members=40, nspecies=3, seed=81, nseg=64, stack=4.0)
    trg, env = [[1], [2, 3], [3]], [[1, 2], [1, 2, 3], [1]]
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    ctx.tasks(trg, env)
    ctx.hist(0.0, 0.04, 1.1)
    ctx.set_option("npcorr_order", order)
    ctx.run(cid, N.PP_RDF | N.PP_NPCORR, [])
    npc = ctx.fetch_npcorr()
    rdf = ctx.fetch()
    ctx.set_option("npcorr_order", 0)
    surf = oracle.surface_distance(spec.xyz, spec.hull, 2.0)
    ref = oracle.npcorr(spec.xyz, spec.labels, surf, 0.04, 1.1, trg, env, order)
    assert ref.sum() > 0 and np.array_equal(npc, ref)
    ref_rdf = oracle.spatstat(spec.xyz, spec.labels, surf, 0.0, 0.04, 1.1, N.PP_RDF, trg, env, [])
    assert np.array_equal(rdf, ref_rdf["bins"])
    ctx.free(cid)


def LANES(bx, by=1, bz=1):
    """Tile code of the centre-per-lane scan: a block of bx x by x bz cells."""
    return ((bx | by << 8 | bz << 12) << 16) | N.PP_TILE_LANES


@pytest.mark.parametrize("block", [(1, 1, 1), (2, 1, 1), (4, 2, 2), (3, 3, 2), (8, 1, 3)])
@pytest.mark.parametrize("ratio", [2.0, 3.5, 5.0])
@pytest.mark.parametrize("symmetric", [1, 0])
def test_lanes_scan(ctx, oracle, block, ratio, symmetric):
    """The centre-per-lane block scan of RDF/RIPK passes against the oracle and
    against the per-centre scan: overlapping target and environment sets, a
    label permutation, a non-zero lower radius, the symmetric and the
    one-sided pair rule."""
    spec = synth.cone_specimen(n=50000, r_apex=8.0, half_angle_deg=10.0, length=18.0, n_clusters=25,
                               members=40, nspecies=4, seed=61, nseg=64, stack=4.0)
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    ctx.tuning(cid, ratio, LANES(*block))
    surf = oracle.surface_distance(spec.xyz, spec.hull, 2.0)
    perm = np.random.default_rng(sum(block) * 7 + int(ratio)).permutation(spec.xyz.shape[0]).astype(np.uint32)
    trg, env = [[1], [2, 3], [4], [1, 2, 3, 4]], [[1, 2], [1, 2, 3], [1], [4]]
    ctx.tasks(trg, env)
    ctx.hist(0.1, 0.02, 1.4)
    flags = N.PP_RDF | N.PP_RIPK
    ctx.set_option("symmetric", symmetric)
    try:
        ctx.run(cid, flags, [], label_perm=perm)
        lanes, st = ctx.fetch(), ctx.stats()
        kernel, tests_lanes = ctx.last_kernel(), ctx.run_tests()
        ctx.set_option("lanes", 0)
        ctx.run(cid, flags, [], label_perm=perm)
        scan, st2 = ctx.fetch(), ctx.stats()
        tests_scan = ctx.run_tests()
    finally:
        ctx.set_option("lanes", 1)
        ctx.set_option("symmetric", 1)
    ctx.free(cid)
    ref = oracle.spatstat(spec.xyz, spec.labels[perm], surf, 0.1, 0.02, 1.4, flags, trg, env, [])
    assert kernel == "k_lanes"
    assert st["pairs"] == ref["pairs"] == st2["pairs"] and st["centres"] == ref["centres"]
    assert tests_lanes >= st["pairs"] // (2 if symmetric else 1) and tests_scan >= st["pairs"] // 2
    assert np.array_equal(lanes, ref["bins"]) and np.array_equal(scan, ref["bins"])


def test_lanes_scan_rdf_bins_in_global_memory(ctx, oracle):
    """Many tasks: the RDF cores do not fit shared memory and the
    centre-per-lane scan adds to the global uint64 bins directly."""
    spec = synth.cone_specimen(n=30000, r_apex=8.0, half_angle_deg=10.0, length=12.0, n_clusters=10,
                               members=30, nspecies=8, seed=67, nseg=64, stack=4.0)
    types = list(range(1, 9))
    trg = [[a] for a in types for b in types]
    env = [[b] for a in types for b in types]
    gpu, st, ref, _ = _run_both(ctx, oracle, spec, 0.0, 0.002, 1.2, N.PP_RDF, trg, env, [])
    assert st["pairs"] == ref["pairs"]
    assert np.array_equal(gpu, ref["bins"])


@pytest.mark.parametrize("block", [(1, 1, 1), (4, 2, 2), (3, 3, 2)])
@pytest.mark.parametrize("ratio", [2.0, 4.0])
@pytest.mark.parametrize("with_rdf", [False, True])
def test_lanes_knn_scan(ctx, oracle, block, ratio, with_rdf):
    """The centre-per-lane block scan of kNN passes (disjoint environment sets,
    k up to 12, 1NN, the miss bin) against the oracle and the per-centre scan,
    under a label permutation; with RDF in the same pass on a cloud tuned to a
    cell block, the RDF and the kNN centre-per-lane passes run one after the
    other and the pairs are counted once."""
    spec = synth.cone_specimen(n=50000, r_apex=8.0, half_angle_deg=10.0, length=18.0, n_clusters=25,
                               members=40, nspecies=4, seed=71, nseg=64, stack=4.0)
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    ctx.tuning(cid, ratio, LANES(*block))
    surf = oracle.surface_distance(spec.xyz, spec.hull, 2.0)
    perm = np.random.default_rng(sum(block) + int(ratio)).permutation(spec.xyz.shape[0]).astype(np.uint32)
    trg = [[1], [1], [2, 3], [4], [1, 2, 3, 4]]
    env = [[1, 2], [3], [1, 2, 3], [4], [4]]
    ks = [12, 5, 1]
    flags = N.PP_1NN | N.PP_MKNN | (N.PP_RDF if with_rdf else 0)
    ctx.tasks(trg, env)
    ctx.hist(0.0, 0.01, 1.3)
    try:
        ctx.run(cid, flags, ks, label_perm=perm)
        lanes, st = ctx.fetch(), ctx.stats()
        kernel = ctx.last_kernel()
        ctx.set_option("lanes", 0)
        ctx.run(cid, flags, ks, label_perm=perm)
        scan = ctx.fetch()
    finally:
        ctx.set_option("lanes", 1)
    ctx.free(cid)
    ref = oracle.spatstat(spec.xyz, spec.labels[perm], surf, 0.0, 0.01, 1.3, flags, trg, env, ks)
    assert st["pairs"] == ref["pairs"] and st["centres"] == ref["centres"]
    assert np.array_equal(lanes, ref["bins"]) and np.array_equal(scan, ref["bins"])
    assert kernel == ("k_lanes+k_lanes_knn" if with_rdf else "k_lanes_knn")


@pytest.mark.parametrize("shift", [0.0, 4096.0])
@pytest.mark.parametrize("block", [(1, 1, 1), (4, 2, 2), (4, 4, 4)])
def test_lanes_box_filter(ctx, oracle, shift, block):
    """The centre-per-lane scans drop candidates beyond R of the bounding box of
    a batch's centres and trim stencil rows to that box: RDF (symmetric and
    one-sided) and kNN bins and pair counts are the same with the filter off,
    and equal the oracle's, on a cloud far from the origin too (coarser float
    spacing); the filter leaves fewer distance tests."""
    spec = synth.cone_specimen(n=40000, r_apex=8.0, half_angle_deg=10.0, length=14.0, n_clusters=20,
                               members=40, nspecies=3, seed=83, nseg=64, stack=4.0)
    off = np.array([shift, -0.5 * shift, 0.25 * shift], dtype=np.float32)
    xyz = (spec.xyz + off).astype(np.float32)
    hull = (spec.hull.reshape(-1, 3) + off).astype(np.float32).reshape(spec.hull.shape)
    cid = ctx.upload(xyz, spec.labels)
    ctx.hull(cid, hull, 2.0)
    ctx.tuning(cid, 4.0, LANES(*block))
    surf = oracle.surface_distance(xyz, hull, 2.0)
    types = [1, 2, 3]
    trg = [[a] for a in types for b in types]
    env = [[b] for a in types for b in types]
    ctx.tasks(trg, env)
    # 0.01 nm bins: every category-table cell holds at most one threshold and
    # the RDF binning takes one step from the table; 0.001 nm bins: the
    # general threshold walk
    cases = [(N.PP_RDF | N.PP_RIPK, [], (0.0, 0.01, 1.2), 1), (N.PP_RDF, [], (0.05, 0.02, 1.1), 0),
             (N.PP_RDF, [], (0.0, 0.001, 1.2), 1), (N.PP_1NN | N.PP_MKNN, [9, 4, 1], (0.0, 0.005, 1.2), 1)]
    try:
        for flags, ks, hist, sym in cases:
            ctx.hist(*hist)
            ctx.set_option("symmetric", sym)
            out = {}
            for box in (1, 0):
                ctx.set_option("box_filter", box)
                ctx.run(cid, flags, ks)
                out[box] = (ctx.fetch(), ctx.stats(), ctx.run_tests(), ctx.last_kernel())
            ref = oracle.spatstat(xyz, spec.labels, surf, *hist, flags, trg, env, ks)
            (b1, s1, t1, k1), (b0, s0, t0, k0) = out[1], out[0]
            assert k1 == k0 and k1.startswith("k_lanes")
            assert s1["pairs"] == s0["pairs"] == ref["pairs"] and s1["centres"] == ref["centres"]
            assert np.array_equal(b1, ref["bins"]) and np.array_equal(b0, ref["bins"])
            assert t1 < t0
    finally:
        ctx.set_option("box_filter", 1)
        ctx.set_option("symmetric", 1)
    ctx.free(cid)


@pytest.mark.parametrize("symmetric", [1, 0])
def test_combined_pass_split_with_overlapping_sets(ctx, oracle, symmetric):
    """RDF/RIPK with kNN on a cloud tuned to a cell block, overlapping
    environment sets: the RDF part takes the centre-per-lane scan, the kNN part
    the per-centre scan; untuned, the whole pass takes the per-centre scan."""
    spec = synth.cone_specimen(n=40000, r_apex=8.0, half_angle_deg=10.0, length=14.0, n_clusters=12,
                               members=30, nspecies=3, seed=79, nseg=64, stack=4.0)
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    surf = oracle.surface_distance(spec.xyz, spec.hull, 2.0)
    trg, env = [[1], [1], [2, 3]], [[1, 2], [2, 3], [1, 2, 3]]
    ks = [7, 3, 1]
    flags = N.PP_RDF | N.PP_RIPK | N.PP_1NN | N.PP_MKNN
    ctx.tasks(trg, env)
    ctx.hist(0.05, 0.01, 1.25)
    ref = oracle.spatstat(spec.xyz, spec.labels, surf, 0.05, 0.01, 1.25, flags, trg, env, ks)
    ctx.set_option("symmetric", symmetric)
    try:
        ctx.run(cid, flags, ks)
        got, st = ctx.fetch(), ctx.stats()
        assert ctx.last_kernel() == "k_scan"
        assert st["pairs"] == ref["pairs"] and np.array_equal(got, ref["bins"])
        ctx.tuning(cid, 4.0, LANES(4, 2, 2))
        ctx.run(cid, flags, ks)
        got, st = ctx.fetch(), ctx.stats()
        assert ctx.last_kernel() == "k_lanes+k_scan"
        assert st["pairs"] == ref["pairs"] and st["centres"] == ref["centres"]
        assert np.array_equal(got, ref["bins"])
    finally:
        ctx.set_option("symmetric", 1)
        ctx.free(cid)


@pytest.mark.parametrize("flags", [N.PP_MKNN, N.PP_MKNN | N.PP_RDF | N.PP_1NN])
def test_lanes_knn_overlapping_sets_fall_back(ctx, oracle, flags):
    """Overlapping environment sets of one centre type take the per-centre scan."""
    spec = synth.cone_specimen(n=30000, r_apex=8.0, half_angle_deg=10.0, length=12.0, n_clusters=10,
                               members=30, nspecies=3, seed=73, nseg=64, stack=4.0)
    trg, env = [[1], [1]], [[1, 2], [2, 3]]
    gpu, st, ref, _ = _run_both(ctx, oracle, spec, 0.0, 0.01, 1.2, flags, trg, env, [6, 1])
    assert ctx.last_kernel() == "k_scan"
    assert st["pairs"] == ref["pairs"] and st["centres"] == ref["centres"]
    assert np.array_equal(gpu, ref["bins"])


@pytest.mark.parametrize("block", [(1, 1, 1), (8, 8, 8), (64, 15, 15)])
def test_lanes_small_and_sparse_clouds(ctx, oracle, block):
    """Centre-per-lane scans on clouds smaller than one cell block, with
    isolated ions (kNN misses) and coincident positions, through explicit block
    shapes: RDF (symmetric and one-sided) and kNN against the oracle."""
    rng = np.random.default_rng(sum(block))
    a = (rng.random((150, 3)) * 2.0).astype(np.float32)           # a dense 2 nm cube
    b = (rng.random((40, 3)) * 2.0 + 9.0).astype(np.float32)      # a far, sparse corner
    c = np.repeat(a[:5], 2, axis=0)                               # coincident pairs
    xyz = np.concatenate([a, b, c]).astype(np.float32)
    labels = (rng.integers(1, 4, size=xyz.shape[0])).astype(np.uint8)
    n = xyz.shape[0]
    surf = np.full(n, 100.0, dtype=np.float32)
    cid = ctx.upload(xyz, labels)
    ctx.surfdist(cid, surf)
    ctx.tuning(cid, 5.0, LANES(*block))
    types = [1, 2, 3]
    trg = [[t] for t in types for _ in types]
    env = [[u] for _ in types for u in types]
    ctx.tasks(trg, env)
    try:
        for flags, ks, sym in ((N.PP_RDF | N.PP_RIPK, [], 1), (N.PP_RDF, [], 0), (N.PP_1NN | N.PP_MKNN, [4, 2], 1),
                               (N.PP_RDF | N.PP_MKNN, [3, 1], 1)):
            ctx.set_option("symmetric", sym)
            ctx.hist(0.0, 0.02, 1.0)
            ctx.run(cid, flags, ks)
            got, st = ctx.fetch(), ctx.stats()
            assert ctx.last_kernel() in ("k_lanes", "k_lanes_knn", "k_lanes+k_lanes_knn")
            ref = oracle.spatstat(xyz, labels, surf, 0.0, 0.02, 1.0, flags, trg, env, ks)
            assert st["pairs"] == ref["pairs"] and st["centres"] == ref["centres"]
            assert np.array_equal(got, ref["bins"])
    finally:
        ctx.set_option("symmetric", 1)
        ctx.free(cid)


def test_freed_cloud_buffers_reused(ctx, oracle):
    """Uploads after pp_cloud_free take the freed clouds' device buffers
    (smaller and larger clouds, with and without a hull); every result still
    equals the oracle's."""
    flags, ks = N.PP_RDF | N.PP_MKNN, [4, 1]
    for i, n in enumerate((40000, 15000, 60000, 25000)):
        spec = synth.cylinder_specimen(n=n, radius=5.0, height=n / 2000.0, seed=300 + i, nseg=64, stack=4.0)
        cid = ctx.upload(spec.xyz, spec.labels)
        hull = i != 3
        if hull:
            ctx.hull(cid, spec.hull, 2.0)
        ctx.tasks([[2], [1]], [[1, 2, 3], [1]])
        ctx.hist(0.0, 0.01, 1.0)
        ctx.run(cid, flags, ks)
        gpu = ctx.fetch()
        surf = (oracle.surface_distance(spec.xyz, spec.hull, 2.0) if hull
                else np.full(n, np.float32(2.0) * np.float32(2.0), dtype=np.float32))
        ref = oracle.spatstat(spec.xyz, spec.labels, surf, 0.0, 0.01, 1.0, flags, [[2], [1]], [[1, 2, 3], [1]], ks)
        assert np.array_equal(gpu, ref["bins"]), n
        ctx.free(cid)


def test_hull_with_non_finite_vertex_is_refused(ctx, oracle):
    """A hull with a NaN vertex is refused with PP_ERR_INVALID and leaves the
    cloud's previous hull (and its ion2surf) in place."""
    spec = synth.cylinder_specimen(n=20000, radius=5.0, height=16.0, seed=21, nseg=64, stack=4.0)
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    ctx.tasks([[1]], [[1, 2, 3]])
    ctx.hist(0.0, 0.01, 1.0)
    ctx.run(cid, N.PP_RDF, [])
    before = ctx.fetch()
    bad = spec.hull.copy()
    bad[7, 4] = np.nan
    with pytest.raises(N.PPError) as err:
        ctx.hull(cid, bad, 2.0)
    assert err.value.code == N.PP_ERR_INVALID
    ctx.run(cid, N.PP_RDF, [])
    assert np.array_equal(ctx.fetch(), before)
    surf = oracle.surface_distance(spec.xyz, spec.hull, 2.0)
    ref = oracle.spatstat(spec.xyz, spec.labels, surf, 0.0, 0.01, 1.0, N.PP_RDF, [[1]], [[1, 2, 3]], [])
    assert np.array_equal(before, ref["bins"])
    ctx.free(cid)


@pytest.mark.parametrize("R", [0.5, 1.0, 2.5])
def test_hull_distance_hull_beyond_the_cloud(ctx, oracle, R):
    """The hull grid covers the ions only: a hull reaching far beyond them (a
    third of the cylinder's ions kept) and one shifted wholly away still give
    ion2surf bit-identical to the oracle, for hull cells of 1 to 10 ion cells."""
    spec = synth.cylinder_specimen(n=30000, radius=5.0, height=24.0, seed=23, nseg=64, stack=4.0)
    keep = spec.xyz[:, 2] < 8.0
    xyz, labels = spec.xyz[keep], spec.labels[keep]
    away = spec.hull.copy()
    away[:, 2::3] += 40.0
    for hull in (spec.hull, away):
        cid = ctx.upload(xyz, labels)
        ctx.hull(cid, hull, 2.0)
        ctx.tasks([[1]], [[1, 2, 3]])
        ctx.hist(0.0, 0.01, R)
        ctx.run(cid, N.PP_RDF, [])
        ctx.fetch()
        gs = ctx.surfdist_fetch(cid, xyz.shape[0])
        rp = max(np.float32(R), np.float32(2.0))
        cs = oracle.surface_distance(xyz, hull, rp)
        assert np.array_equal(gs.view(np.uint32), cs.view(np.uint32))
        ctx.free(cid)
