"""The CUDA path against the oracle at the sizes of the benchmark workloads.

The small seeded clouds of test_gpu_parity.py exercise every kernel, but some
paths only trigger at size (shared-memory bin flushes, chunked pair lists,
long stencil walks).  These tests run the workloads the benchmark measures,
at full size where the oracle finishes in seconds and otherwise at reduced
ion counts with the same geometry, density, species mix, tasks, radii, bin
widths and k lists, and compare every bin exactly:

  * the 1M-ion cylinder (RDF R = 1 nm + kNN k = 1, 5, 10, species-1 centres), full size;
  * a 2M-ion cut of the 20M-ion clustered tip: all 36 pair tasks, RDF
    R = 2/0.01 and kNN k = 1..10 at 0.005 nm, with the default dispatch and
    with the centre-per-lane cell block the autotuner picks for the full tip;
  * 1.5M ions of the 150M-ion tip's kind (8 species, 64 tasks, RDF + kNN
    k = 1..20 at R = 2.5/0.01 in one pass), with the default dispatch and
    forced cell blocks;
  * the 5M-ion batched configuration (R = 1.5, kNN k = 1..8, 36 tasks) with
    the measured labels, label shuffles and spherical regions of interest in
    one batched call, each realisation against the oracle.
"""
import numpy as np
import pytest

from paraprobe_gb300 import native as N
from paraprobe_gb300 import synth

pytestmark = pytest.mark.gpu

RHO_TIP20M = 20_000_000 / synth.cone_volume(30.0, 10.0, 200.0)
RHO_TIP150M = 150_000_000 / synth.cone_volume(50.0, 12.0, 400.0)


def lanes_code(bx, by, bz):
    """pp_cloud_tuning tile code of a centre-per-lane cell block."""
    return ((bx | by << 8 | bz << 12) << 16) | N.PP_TILE_LANES


def tip20m_cut(n, seed):
    """The 20M-ion tip's cone (apex 30 nm, 10 deg), density and cluster
    density, shortened to hold n ions."""
    length = synth.cone_length_for(n, RHO_TIP20M, 30.0, 10.0)
    return synth.cone_specimen(n=n, r_apex=30.0, half_angle_deg=10.0, length=length,
                               n_clusters=max(1, round(2000 * n / 20_000_000)), sigma=1.5, members=50,
                               cluster_p=(0.7, 0.3), iid=(0.02, 0.01, 0.005), nspecies=6, seed=seed), length


def tip150m_cut(n, seed, r_apex=30.0):
    """The 150M-ion tip's half-angle (12 deg), 8 species, density and cluster
    density, with a narrower apex (so that a cut of n ions is longer than it
    is wide and most ions lie R or more from the surface)."""
    length = synth.cone_length_for(n, RHO_TIP150M, r_apex, 12.0)
    return synth.cone_specimen(n=n, r_apex=r_apex, half_angle_deg=12.0, length=length,
                               n_clusters=max(1, round(5000 * n / 150_000_000)), sigma=1.5, members=50,
                               cluster_p=(0.7, 0.3), iid=(0.02, 0.01, 0.005, 0.005, 0.002), nspecies=8,
                               seed=seed)


def all_pairs(nspecies):
    types = list(range(1, nspecies + 1))
    return [[a] for a in types for b in types], [[b] for a in types for b in types]


def _diff(gpu, ref):
    bad = np.nonzero(gpu != ref)[0]
    return f"{bad.size} of {gpu.size} bins differ, first {bad[:8]}"


def test_cyl1m_full(ctx, oracle):
    """The 1M-ion cylinder workload exactly (seed as in the benchmark), whole cloud."""
    spec = synth.cylinder_specimen(n=1_000_000, radius=10.0, height=63.66, fractions=(0.90, 0.08, 0.02),
                                   seed=20261204)
    trg, env = [[2]], [[1, 2, 3]]
    flags, ks, hist = N.PP_RDF | N.PP_MKNN, [10, 5, 1], (0.0, 0.01, 1.0)
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    ctx.tasks(trg, env)
    ctx.hist(*hist)
    surf = oracle.surface_distance(spec.xyz, spec.hull, 2.0)
    ref = oracle.spatstat(spec.xyz, spec.labels, surf, *hist, flags, trg, env, ks)
    for tuning in (None, (4.0, lanes_code(4, 2, 2)), (2.0, 128)):
        if tuning:
            ctx.tuning(cid, *tuning)
        ctx.run(cid, flags, ks)
        gpu = ctx.fetch()
        st = ctx.stats()
        assert st["centres"] == ref["centres"] and st["pairs"] == ref["pairs"], (tuning, ctx.last_kernel())
        assert np.array_equal(gpu, ref["bins"]), f"{tuning} {ctx.last_kernel()}: " + _diff(gpu, ref["bins"])
    gs = ctx.surfdist_fetch(cid, spec.xyz.shape[0])
    assert np.array_equal(gs.view(np.uint32), surf.view(np.uint32))
    ctx.free(cid)


def test_tip20m_cut_2m_both_passes(ctx, oracle):
    """2M ions of the 20M-ion tip, all 36 tasks, both passes of one step."""
    spec, _ = tip20m_cut(2_000_000, seed=20261211)
    trg, env = all_pairs(6)
    passes = [(N.PP_RDF, (0.0, 0.01, 2.0), []), (N.PP_MKNN, (0.0, 0.005, 2.0), list(range(10, 0, -1)))]
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    ctx.tasks(trg, env)
    surf = oracle.surface_distance(spec.xyz, spec.hull, 2.0)
    kernels = set()
    for flags, hist, ks in passes:
        ctx.hist(*hist)
        ref = oracle.spatstat(spec.xyz, spec.labels, surf, *hist, flags, trg, env, ks)
        for tuning, lists, uni in ((None, 0, 1), ((4.0, lanes_code(4, 2, 2)), 0, 1), ((4.0, lanes_code(3, 2, 2)), 0, 1),
                                   ((4.0, lanes_code(4, 2, 2)), 2, 1), ((4.0, lanes_code(4, 2, 2)), 0, 0)):
            if tuning:
                ctx.tuning(cid, *tuning)
            ctx.set_option("knn_lists", lists)
            ctx.set_option("uniform_sets", uni)
            try:
                ctx.run(cid, flags, ks)
                gpu = ctx.fetch()
            finally:
                ctx.set_option("knn_lists", 0)
                ctx.set_option("uniform_sets", 1)
            kernels.add(ctx.last_kernel())
            assert ctx.stats()["pairs"] == ref["pairs"], (flags, tuning)
            assert np.array_equal(gpu, ref["bins"]), (f"{flags} {tuning} lists {lists} uniform {uni} "
                                                      f"{ctx.last_kernel()}: " + _diff(gpu, ref["bins"]))
    assert {"k_lanes", "k_lanes_knn"} <= kernels
    ctx.free(cid)


def test_tip20m_sample_mask(ctx, oracle):
    """A centre mask (as the benchmark samples the 20M-ion tip) gives the
    oracle's bins over the same centres; the unmasked pass equals the sum of
    the pass over the mask and over its complement."""
    spec, _ = tip20m_cut(1_000_000, seed=20261212)
    trg, env = all_pairs(6)
    n = spec.xyz.shape[0]
    mask = (np.random.default_rng(3).random(n) < 0.3).astype(np.uint8)
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    ctx.tasks(trg, env)
    surf = oracle.surface_distance(spec.xyz, spec.hull, 2.0)
    ctx.tuning(cid, 4.0, lanes_code(4, 2, 2))
    for flags, hist, ks in ((N.PP_RDF, (0.0, 0.01, 2.0), []), (N.PP_MKNN, (0.0, 0.005, 2.0), list(range(10, 0, -1)))):
        ctx.hist(*hist)
        ref = oracle.spatstat(spec.xyz, spec.labels, surf, *hist, flags, trg, env, ks, centre_mask=mask)
        ctx.run(cid, flags, ks, centre_mask=mask)
        part = ctx.fetch()
        assert ctx.stats()["centres"] == ref["centres"] and ctx.stats()["pairs"] == ref["pairs"]
        assert np.array_equal(part, ref["bins"]), _diff(part, ref["bins"])
        ctx.run(cid, flags, ks, centre_mask=1 - mask)
        rest = ctx.fetch()
        ctx.run(cid, flags, ks)
        assert np.array_equal(ctx.fetch(), part + rest)
    ctx.free(cid)


def test_tip150m_cut_k20_8_species(ctx, oracle):
    """The 150M-ion tip's analyses (64 tasks, RDF + kNN k = 1..20 at
    R = 2.5/0.01 in one pass) on 1.5M ions of its kind, with the default
    dispatch and with centre-per-lane cell blocks."""
    spec = tip150m_cut(1_500_000, seed=20261213)
    trg, env = all_pairs(8)
    flags, hist, ks = N.PP_RDF | N.PP_MKNN, (0.0, 0.01, 2.5), list(range(20, 0, -1))
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    ctx.tasks(trg, env)
    ctx.hist(*hist)
    surf = oracle.surface_distance(spec.xyz, spec.hull, 2.5)
    ref = oracle.spatstat(spec.xyz, spec.labels, surf, *hist, flags, trg, env, ks)
    assert ref["centres"] > 0.5 * spec.xyz.shape[0]
    # the kNN lane scan's lists: automatic (categories for 8 sets of k = 20),
    # distances (one block per SM) and categories
    for tuning, lists in ((None, 0), ((5.0, lanes_code(4, 2, 2)), 0), ((4.0, lanes_code(3, 2, 2)), 0),
                          ((5.0, lanes_code(4, 2, 2)), 1), ((5.0, lanes_code(4, 2, 2)), 2)):
        if tuning:
            ctx.tuning(cid, *tuning)
        ctx.set_option("knn_lists", lists)
        try:
            ctx.run(cid, flags, ks)
            gpu = ctx.fetch()
        finally:
            ctx.set_option("knn_lists", 0)
        kern = ctx.last_kernel()
        assert ctx.stats()["pairs"] == ref["pairs"], (tuning, kern)
        assert np.array_equal(gpu, ref["bins"]), f"{tuning} lists {lists} {kern}: " + _diff(gpu, ref["bins"])
    ctx.free(cid)


def test_batched_5m_shuffles_and_rois(ctx, oracle):
    """The 5M-ion batched configuration: measured labels, 3 label shuffles and
    4 spherical regions of interest in one batched call (RDF R = 1.5 nm and
    kNN k = 1..8, 0.01 nm bins, 36 tasks); every realisation against the
    oracle, the regions through the oracle's centre mask."""
    spec, length = tip20m_cut(5_000_000, seed=20261206)
    n = spec.xyz.shape[0]
    trg, env = all_pairs(6)
    hist, ks, flags = (0.0, 0.01, 1.5), list(range(8, 0, -1)), N.PP_RDF | N.PP_MKNN
    sets = np.stack([N.shuffle_labels(spec.labels, 1000 + r) for r in range(3)])
    rng = np.random.default_rng(20261207)
    tn = np.tan(np.radians(10.0))
    rois = []
    while len(rois) < 4:
        z = rng.uniform(0, length)
        rz = 30.0 + z * tn
        x, y = rng.uniform(-rz, rz, 2)
        if x * x + y * y <= rz * rz:
            rois.append([x, y, z, float(np.exp(rng.uniform(np.log(5.0), np.log(40.0))))])
    rois = np.asarray(rois, dtype=np.float32)
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    ctx.tasks(trg, env)
    ctx.hist(*hist)
    ctx.run_batched(cid, flags, ks, include_original=True, label_sets=sets, rois=rois)
    assert ctx.batched_count() == 1 + 3 + 4
    outs = [ctx.fetch_batched(r) for r in range(8)]
    surf = oracle.surface_distance(spec.xyz, spec.hull, 2.0)
    ref = oracle.spatstat(spec.xyz, spec.labels, surf, *hist, flags, trg, env, ks)
    assert np.array_equal(outs[0], ref["bins"]), "measured labels: " + _diff(outs[0], ref["bins"])
    for q in range(3):
        refq = oracle.spatstat(spec.xyz, sets[q], surf, *hist, flags, trg, env, ks)
        assert np.array_equal(outs[1 + q], refq["bins"]), f"label set {q}: " + _diff(outs[1 + q], refq["bins"])
    for q in range(4):
        c = rois[q]
        dx = (spec.xyz[:, 0] - c[0]).astype(np.float32)
        dy = (spec.xyz[:, 1] - c[1]).astype(np.float32)
        dz = (spec.xyz[:, 2] - c[2]).astype(np.float32)
        d = np.sqrt((dx * dx + dy * dy) + dz * dz).astype(np.float32)
        mask = ((np.float32(c[3]) - d) >= np.float32(hist[2])).astype(np.uint8)
        refq = oracle.spatstat(spec.xyz, spec.labels, surf, *hist, flags, trg, env, ks, centre_mask=mask)
        assert np.array_equal(outs[4 + q], refq["bins"]), f"roi {q}: " + _diff(outs[4 + q], refq["bins"])
    ctx.free(cid)


def test_masked_edge_cases(ctx, oracle):
    """A mask that selects no centre gives empty bins (every histogram zero,
    no kNN miss either), one that selects a single ion that ion's ball, and a
    mask of ones the unmasked pass."""
    spec, _ = tip20m_cut(200_000, seed=20261214)
    trg, env = all_pairs(6)
    n = spec.xyz.shape[0]
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    ctx.tasks(trg, env)
    flags, hist, ks = N.PP_RDF | N.PP_MKNN, (0.0, 0.01, 2.0), [5, 1]
    ctx.hist(*hist)
    surf = oracle.surface_distance(spec.xyz, spec.hull, 2.0)
    one = np.zeros(n, np.uint8)
    one[int(np.argmax(surf))] = 1  # the ion deepest inside: a centre for sure
    for mask in (np.zeros(n, np.uint8), one, np.ones(n, np.uint8)):
        ctx.run(cid, flags, ks, centre_mask=mask)
        gpu = ctx.fetch()
        ref = oracle.spatstat(spec.xyz, spec.labels, surf, *hist, flags, trg, env, ks, centre_mask=mask)
        assert ctx.stats()["centres"] == ref["centres"]
        assert np.array_equal(gpu, ref["bins"])
        if not mask.any():
            assert ref["centres"] == 0 and not gpu.any()
    ctx.run(cid, flags, ks)
    assert np.array_equal(ctx.fetch(), gpu)
    ctx.free(cid)
