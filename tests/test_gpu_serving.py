"""Serving loop: queries of different clouds, radii, k and species pairs run
concurrently on the worker streams; every result must be identical to the same
query run alone through pp_run."""
import threading

import numpy as np
import pytest

from paraprobe_gb300 import native as N
from paraprobe_gb300 import synth

pytestmark = pytest.mark.gpu


def test_results_same_alone_and_in_the_mix(ctx):
    clouds = []
    for i, n in enumerate((20000, 60000, 120000)):
        spec = synth.cone_specimen(n=n, r_apex=8.0, half_angle_deg=10.0,
                                   length=synth.cone_length_for(n, 13.4, 8.0, 10.0), n_clusters=20,
                                   members=30, nspecies=4, seed=40 + i, nseg=96, stack=4.0)
        cid = ctx.upload(spec.xyz, spec.labels)
        ctx.hull(cid, spec.hull, 2.0)
        ctx.prepare(cid, 0.5, 3.0)
        clouds.append(cid)
    rng = np.random.default_rng(3)
    queries = []
    for q in range(24):
        cid = clouds[rng.integers(0, 3)]
        R = float(np.float32(rng.uniform(0.5, 3.0)))
        k = int(rng.integers(1, 21))
        a, b = (int(x) for x in rng.integers(1, 5, size=2))
        queries.append((cid, N.PP_RDF | N.PP_MKNN, (0.0, 0.01, R), [[a]], [[b]], [k]))
    srv = N.Server(ctx, slots=4, budget_bytes=1 << 30)
    tickets = [srv.submit(c, f, h, t, e, k) for (c, f, h, t, e, k) in queries]
    mixed = [srv.wait(t)[0] for t in tickets]
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(queries) and st["rejected"] == 0
    assert st["p99_ms"] >= st["p50_ms"] > 0
    for (c, f, h, t, e, k), got in zip(queries, mixed):
        ctx.tasks(t, e)
        ctx.hist(*h)
        ctx.run(c, f, k)
        alone = ctx.fetch()
        assert np.array_equal(alone, got)
    for c in clouds:
        ctx.free(c)


def test_admission_rejects_oversized_queries(ctx):
    spec = synth.cylinder_specimen(n=20000, radius=5.0, height=16.0, seed=1, nseg=64, stack=4.0)
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.prepare(cid, 0.5, 3.0)
    srv = N.Server(ctx, slots=2, budget_bytes=1024)
    with pytest.raises(N.PPError):
        srv.submit(cid, N.PP_RDF, (0.0, 0.01, 1.0), [[1]], [[1]])
    assert srv.stats()["rejected"] == 1
    srv.close()
    ctx.free(cid)


def _merge_cloud(ctx, n=80000, seed=77):
    spec = synth.cone_specimen(n=n, r_apex=8.0, half_angle_deg=10.0, length=synth.cone_length_for(n, 13.4, 8.0, 10.0),
                               n_clusters=25, members=30, nspecies=4, seed=seed, nseg=96, stack=4.0)
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    ctx.prepare(cid, 0.5, 3.0)
    return cid


def _merge_queries():
    """Queries that differ in everything a merged pass keeps per query:
    radius (below and above the carving radius), bin width and lower edge,
    analyses, k lists, several tasks with multi-type and overlapping sets."""
    R, M = N.PP_RDF, N.PP_MKNN
    return [
        (R | M, (0.0, 0.01, 2.7), [[1]], [[2]], [20, 3]),
        (R | N.PP_1NN, (0.0, 0.02, 0.9), [[2], [1, 3]], [[1, 2, 3, 4], [3]], []),
        (M, (0.0, 0.005, 1.6), [[3]], [[1]], [7, 1, 12]),
        (N.PP_RIPK | M, (0.3, 0.05, 2.2), [[1], [2]], [[1, 2], [2, 4]], [5]),
        (R, (0.0, 0.01, 3.0), [[4]], [[1]], []),
        (R | N.PP_1NN | N.PP_RIPK | M, (0.0, 0.01, 1.2), [[1, 2]], [[3, 4]], [32, 2]),
        (M, (0.0, 0.01, 2.0), [[2]], [[2]], [1]),
        (R | M, (0.1, 0.01, 2.35), [[1], [1], [4]], [[1], [2, 3], [4]], [9, 4, 1]),
    ]


@pytest.mark.parametrize("batch", [32, 1])
def test_merged_pass_matches_each_query_alone(ctx, batch):
    """Queries queued together on one cloud run as merged passes (one worker,
    so all but the first wait and are merged); every query's bins and pair
    count equal its own pp_run.  With option server_batch = 1 every query runs
    alone, with the same results."""
    cid = _merge_cloud(ctx)
    qs = _merge_queries()
    ctx.set_option("server_batch", batch)
    try:
        srv = N.Server(ctx, slots=1, budget_bytes=4 << 30)
    finally:
        ctx.set_option("server_batch", 32)
    tickets = [srv.submit(cid, f, h, t, e, k) for (f, h, t, e, k) in qs]
    got = [srv.wait(t) for t in tickets]
    passes, nq = srv.passes()
    srv.close()
    assert nq == len(qs)
    if batch == 1:
        assert passes == len(qs)
    else:
        assert passes < len(qs), "no queries were merged"
    for (f, h, t, e, k), (bins, pairs, _) in zip(qs, got):
        ctx.tasks(t, e)
        ctx.hist(*h)
        ctx.run(cid, f, k)
        alone = ctx.fetch()
        assert ctx.stats()["pairs"] == pairs, (f, h)
        assert np.array_equal(alone, bins), (f, h, t, e, k)
    ctx.free(cid)
