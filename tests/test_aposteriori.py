"""Statistics after clustering (clustertask::flag2exclude_guard and
generic_spatstat, src/PARAPROBE_SolverHdl.cpp:4790-4945).

CPU: the oracle against a brute-force numpy restatement on a small cloud and,
with no ion clustered, against the plain statistics that the golden fixtures
pin; its restatement of the reference's guard loop as written against
fixtures the reference's own KD-tree code produced (tests/golden/apost/).
GPU: pp_run_aposteriori against the oracle and, with option
aposteriori_guard = 1, against those fixtures, bit-exact.
"""
import json
import os

import numpy as np
import pytest

import golden_cases as G
from paraprobe_gb300 import synth


def _hist(d, rmin, rincr, rmax):
    """histogram::add (src/PARAPROBE_Histogram.h:53-117) over float distances."""
    s, w, e = (float(np.float32(v)) for v in (rmin, rincr, rmax))
    nb = int((e - s) / w)
    scale = 1.0 / (e - s) * nb
    out = np.zeros(nb + 2, dtype=np.uint64)
    x = np.asarray(d, dtype=np.float32).astype(np.float64)
    inr = (x >= s) & (x <= e)
    b = np.floor(((x[inr] - s) * scale).astype(np.float32)).astype(np.int64)
    np.add.at(out, np.where(b < nb, b + 1, nb + 1), 1)
    out[0] += np.count_nonzero(x < s)
    out[nb + 1] += np.count_nonzero(x > e)
    return out


def _brute(xyz, clus, surf, rmin, rincr, rmax):
    R2 = np.float32(rmax) * np.float32(rmax)
    n = xyz.shape[0]
    dx = xyz[:, None, 0] - xyz[None, :, 0]
    dy = xyz[:, None, 1] - xyz[None, :, 1]
    dz = xyz[:, None, 2] - xyz[None, :, 2]
    d2 = (dx * dx + dy * dy) + dz * dz
    near = (d2 <= R2) & ~np.eye(n, dtype=bool)
    c = clus.astype(bool)
    guard = near[c].any(axis=0) & ~c
    cent = (surf >= R2) & ~c & ~guard
    env = near[cent] & ~c[None, :]
    d = np.sqrt(d2[cent])
    rdf = _hist(d[env], rmin, rincr, rmax)
    dmin = np.where(env, d, np.inf).min(axis=1)
    nn = _hist(dmin[np.isfinite(dmin)], rmin, rincr, rmax)
    return rdf, nn, (int(cent.sum()), int(guard.sum()), int((~np.isfinite(dmin)).sum()))


def test_oracle_aposteriori_matches_brute_force(oracle):
    rng = np.random.default_rng(5)
    n = 1500
    xyz = (rng.random((n, 3)) * 8.0).astype(np.float32)
    clus = (rng.random(n) < 0.03).astype(np.uint8)
    surf = np.full(n, 100.0, dtype=np.float32)
    surf[rng.random(n) < 0.1] = 0.5  # near the hull: never a centre
    rmin, rincr, rmax = 0.0, 0.05, 1.2
    got, st = oracle.aposteriori(xyz, clus, surf, rmin, rincr, rmax, oracle.RDF | oracle.NN1 | oracle.RIPK)
    rdf, nn, bst = _brute(xyz, clus, surf, rmin, rincr, rmax)
    assert st == bst and st[0] > 100 and st[1] > 50
    assert np.array_equal(got["rdf"], rdf) and np.array_equal(got["ripk"], rdf)
    assert np.array_equal(got["1nn"], nn)


def test_oracle_aposteriori_without_clusters_is_plain(oracle):
    """No cluster, no guard: centres and environment are every ion, as in the
    plain pass over all types (pinned by a golden fixture); 1NN then differs
    only by the miss dumps that the plain pass adds."""
    c = G.load("cone_pairs")
    types = sorted(int(t) for t in np.unique(c["labels"]))
    flags = oracle.RDF | oracle.NN1
    got, st = oracle.aposteriori(c["xyz"], np.zeros(c["xyz"].shape[0], np.uint8), c["surf"], c["rmin"], c["rincr"],
                                 c["rmax"], flags)
    ref = oracle.spatstat(c["xyz"], c["labels"], c["surf"], c["rmin"], c["rincr"], c["rmax"], flags, [types],
                          [types], nthreads=2)
    H = ref["nbins"] + 2
    assert st[0] == ref["centres"] and st[1] == 0
    assert np.array_equal(got["rdf"], ref["bins"][:H])
    nn_plain = ref["bins"][H:2 * H].copy()
    nn_plain[-1] -= np.uint64(st[2])
    assert np.array_equal(got["1nn"], nn_plain)


def _case(n=200_000, seed=71):
    spec = synth.cone_specimen(n=n, r_apex=12.0, half_angle_deg=10.0, length=40.0, n_clusters=150, members=60,
                               nspecies=3, seed=seed, nseg=128, stack=3.0)
    clus = (spec.species == 1).astype(np.uint8)
    return spec, clus


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["rdf_1nn", "ripk", "1nn"])
def test_gpu_aposteriori_matches_oracle(ctx, oracle, which):
    from paraprobe_gb300 import native as N
    flags = {"rdf_1nn": N.PP_RDF | N.PP_1NN, "ripk": N.PP_RIPK, "1nn": N.PP_1NN}[which]
    spec, clus = _case()
    rmin, rincr, rmax = 0.0, 0.01, 1.5
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    ctx.tasks([[1, 2]], [[1, 2, 3]])
    ctx.hist(rmin, rincr, rmax)
    ctx.run_aposteriori(cid, clus, flags)
    got = ctx.fetch()
    surf = ctx.surfdist_fetch(cid, spec.xyz.shape[0])
    ctx.free(cid)
    ref, st = oracle.aposteriori(spec.xyz, clus, surf, rmin, rincr, rmax, flags)
    want = np.concatenate([ref[k] for k in ("rdf", "1nn", "ripk") if k in ref])
    assert st[0] > 10_000 and st[1] > 1_000
    assert np.array_equal(np.asarray(got).reshape(-1), want)


@pytest.mark.gpu
def test_gpu_aposteriori_keeps_tasks(ctx):
    """The tasks set with pp_tasks_set survive a pass after clustering."""
    from paraprobe_gb300 import native as N
    spec, clus = _case(n=40_000, seed=73)
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    ctx.tasks([[1], [2]], [[1], [1, 2]])
    ctx.hist(0.0, 0.01, 1.0)
    ctx.run(cid, N.PP_RDF, [])
    before = np.asarray(ctx.fetch()).copy()
    ctx.run_aposteriori(cid, clus, N.PP_RDF)
    one = np.asarray(ctx.fetch())
    assert one.size * 2 == before.size
    ctx.run(cid, N.PP_RDF, [])
    after = np.asarray(ctx.fetch())
    ctx.free(cid)
    assert np.array_equal(before, after)


# ---- the reference's guard loop as written, pinned on reference-generated fixtures
APOST_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "apost")
APOST_FLAG = {"rdf": 1, "1nn": 2, "ripk": 4}


def _apost_names():
    return sorted(f[:-4] for f in os.listdir(APOST_DIR) if f.endswith(".npz")) if os.path.isdir(APOST_DIR) else []


def _apost(name):
    z = np.load(os.path.join(APOST_DIR, name + ".npz"))
    meta = json.loads(str(z["meta"]))
    c = meta["case"]
    order = z["tree_order"].astype(np.int64)
    r = tuple(np.float32(float(v)) for v in c["r"])
    return dict(z=z, c=c, stats=meta["stats"], order=order, r=r, flags=APOST_FLAG[c["what"]])


@pytest.mark.parametrize("name", _apost_names())
def test_oracle_reference_guard_matches_reference(oracle, name):
    """guard_mode 1 of the oracle against the reference's own KD-tree run of
    flag2exclude_guard + generic_spatstat, the cloud in the tree's order."""
    a = _apost(name)
    z, o = a["z"], a["order"]
    got, st = oracle.aposteriori(z["xyz"][o], z["clustered"][o], z["surf"][o], *a["r"], a["flags"], guard_mode=1)
    assert (st[0], st[1], st[2]) == (a["stats"]["centres"], a["stats"]["guarded"], a["stats"]["lost"])
    assert np.array_equal(got[a["c"]["what"]], z["bins"])


def test_apost_fixtures_present():
    assert len(_apost_names()) == 3


@pytest.mark.gpu
@pytest.mark.parametrize("name", _apost_names())
def test_gpu_reference_guard_matches_reference(ctx, name):
    """pp_run_aposteriori with option aposteriori_guard = 1, the cloud
    uploaded in the reference's KD-tree order, against the reference."""
    a = _apost(name)
    z, o = a["z"], a["order"]
    cid = ctx.upload(z["xyz"][o], z["labels"][o])
    ctx.hull(cid, z["hull"], 2.0)
    ctx.hist(*a["r"])
    ctx.set_option("aposteriori_guard", 1)
    try:
        ctx.run_aposteriori(cid, z["clustered"][o], a["flags"])
    finally:
        ctx.set_option("aposteriori_guard", 0)
    got = np.asarray(ctx.fetch()).reshape(-1)
    st = ctx.stats()
    surf = ctx.surfdist_fetch(cid, o.size)
    ctx.free(cid)
    assert np.array_equal(surf.view(np.uint32), z["surf"][o].view(np.uint32))
    assert st["centres"] == a["stats"]["centres"]
    assert np.array_equal(got, z["bins"])


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["rdf_1nn", "ripk"])
def test_gpu_reference_guard_matches_oracle_at_size(ctx, oracle, which):
    """Option aposteriori_guard = 1 on a 200k-ion clustered cone against the
    oracle's restatement of the reference loop (pinned on the fixtures above),
    with the cloud's input order as the positions; and with no clustered ion,
    where both guard rules give the plain statistics over every ion."""
    from paraprobe_gb300 import native as N
    flags = {"rdf_1nn": N.PP_RDF | N.PP_1NN, "ripk": N.PP_RIPK}[which]
    spec, clus = _case()
    rmin, rincr, rmax = 0.0, 0.01, 1.5
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    ctx.hist(rmin, rincr, rmax)
    for c in (clus, np.zeros_like(clus)):
        ctx.set_option("aposteriori_guard", 1)
        try:
            ctx.run_aposteriori(cid, c, flags)
        finally:
            ctx.set_option("aposteriori_guard", 0)
        got = np.asarray(ctx.fetch()).reshape(-1)
        surf = ctx.surfdist_fetch(cid, spec.xyz.shape[0])
        ref, st = oracle.aposteriori(spec.xyz, c, surf, rmin, rincr, rmax, flags, guard_mode=1)
        want = np.concatenate([ref[k] for k in ("rdf", "1nn", "ripk") if k in ref])
        assert np.array_equal(got, want)
        if not c.any():
            ctx.run_aposteriori(cid, c, flags)
            assert np.array_equal(np.asarray(ctx.fetch()).reshape(-1), want)
    ctx.free(cid)
