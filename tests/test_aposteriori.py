"""Statistics after clustering (clustertask::flag2exclude_guard and
generic_spatstat, src/PARAPROBE_SolverHdl.cpp:4790-4945).

CPU: the oracle against a brute-force numpy restatement on a small cloud and,
with no ion clustered, against the plain statistics that the golden fixtures
pin.  GPU: pp_run_aposteriori against the oracle, bit-exact.
"""
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
