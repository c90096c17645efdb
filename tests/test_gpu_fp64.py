"""FP64 audit: the float arithmetic (the reference's) against a double
recomputation of the same pairs; every disagreement is listed and must sit on
a bin edge or on the cut-off radius within float rounding."""
import numpy as np
import pytest

from paraprobe_gb300 import native as N
from paraprobe_gb300 import synth

pytestmark = pytest.mark.gpu


def test_fp64_audit_lists_and_justifies_disagreements(ctx, oracle):
    spec = synth.cone_specimen(n=80000, r_apex=8.0, half_angle_deg=10.0, length=25.0, n_clusters=30,
                               members=40, nspecies=3, seed=77, nseg=96, stack=4.0)
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    trg, env = [[1], [2]], [[1, 2, 3], [1]]
    rmin, rincr, rmax = 0.0, 0.005, 1.2
    ctx.tasks(trg, env)
    ctx.hist(rmin, rincr, rmax)
    audit = ctx.fp64_audit(cid, max_centres=0, cap=1 << 16)
    ctx.run(cid, N.PP_RDF, [])
    st = ctx.stats()
    # pairs on which float and double agree about d <= R, against the float count
    assert abs(audit["pairs"] - st["pairs"]) <= audit["set_disagreements"]
    assert 0 < audit["max_abs_err"] < 1e-6
    assert audit["max_rel_err"] < 1e-6
    nb = oracle.nbins(rmin, rincr, rmax)
    edges = np.float64(np.float32(rmin)) + np.arange(nb + 1) * (
        (np.float64(np.float32(rmax)) - np.float64(np.float32(rmin))) / nb)
    for (i, j), (d32, d64) in zip(audit["listed_ids"], audit["listed_d"]):
        near_edge = np.min(np.abs(edges - d64)) <= 4e-7 * max(d64, 1e-3)
        near_r = abs(d64 - np.float64(np.float32(rmax))) <= 4e-7 * rmax
        assert near_edge or near_r, (i, j, d32, d64)
        assert abs(d32 - d64) <= 1e-6
    ctx.free(cid)
