"""The CPU oracle restatement against outputs of the reference's own compiled
units (golden fixtures made by tests/golden/make_golden.py)."""
import numpy as np
import pytest

import golden_cases as G


@pytest.mark.parametrize("name", G.names())
def test_oracle_matches_reference(oracle, name):
    c = G.load(name)
    rp = max(c["rmax"], np.float32(2.0))
    if c["hull"].shape[0]:
        surf = oracle.surface_distance(c["xyz"], c["hull"], rp)
    else:
        surf = np.full(c["xyz"].shape[0], np.float32(rp) * np.float32(rp), dtype=np.float32)
    assert np.array_equal(surf.view(np.uint32), c["surf"].view(np.uint32))
    L = c["stats"]["cntnb_len"]
    out = oracle.spatstat(c["xyz"], c["labels"], surf, c["rmin"], c["rincr"], c["rmax"], c["flags"], c["trg"],
                          c["env"], c["k"], nthreads=3, cntnb_len=max(L, 1) + 64)
    assert out["centres"] == c["stats"]["centres"]
    assert out["discarded"] == c["stats"]["discarded"]
    assert out["pairs"] == c["stats"]["pairs"]
    assert out["nbins"] == c["stats"]["nbins"]
    assert np.array_equal(out["bins"], c["bins"])
    if L:
        ref = c["cntnb"].reshape(len(c["trg"]), L)
        assert np.array_equal(out["cntnb"][:, :L], ref)
        assert out["cntnb"][:, L:].sum() == 0


def test_oracle_thread_count_invariance(oracle):
    c = G.load("cone_pairs")
    surf = c["surf"]
    outs = [oracle.spatstat(c["xyz"], c["labels"], surf, c["rmin"], c["rincr"], c["rmax"], c["flags"], c["trg"],
                            c["env"], c["k"], nthreads=t)["bins"] for t in (1, 2, 7)]
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])


def test_category_edges(oracle):
    # d == R goes to the upper dump (b == nbins); 0.1-wide bins over [0.3,1.3]
    # hold 9 bins because (1.3f - 0.3f) / 0.1f truncates to 9
    assert oracle.category(0.0, 0.01, 1.0, 1.0) == 101
    assert oracle.category(0.0, 0.01, 1.0, 0.0) == 1
    assert oracle.category(0.3, 0.1, 1.3, 0.29) == 0
    assert oracle.nbins(0.3, 0.1, 1.3) == 9
    assert oracle.nbins(0.0, 0.01, 1.3) == 129
    assert oracle.category(0.0, 0.01, 1.0, np.float32(1.0) + np.float32(1e-6)) == 101


def _voxel_equal(v, ref):
    return (v["nions_inside"] == ref["nions_inside"] and float(v["volume_inside"]) == ref["volume_inside"]
            and v["vacuum"] == ref["vacuum_bins"] and v["surface"] == ref["surface_bins"]
            and v["inside"] == ref["inside_bins"] and (v["nx"], v["ny"], v["nz"]) == (ref["nx"], ref["ny"], ref["nz"]))


@pytest.mark.parametrize("name", G.names())
def test_oracle_voxelizer_matches_reference(oracle, name):
    """NumberOfIonsInside / VolumeInside (and the voxel classes behind them)
    against the reference's occupancy grid and Hoshen-Kopelman unit."""
    c = G.load(name)
    v = oracle.voxelize(c["xyz"], *c["bin_width"])
    assert _voxel_equal(v, c["voxel"]), (v, c["voxel"])


def test_oracle_npcorr_matches_reference(oracle):
    """n-point correlation counts against the reference's npc3d class driven
    by its own KD-tree queries and nth_element (fixture "npcorr")."""
    c = G.load("npcorr")
    out = oracle.npcorr(c["xyz"], c["labels"], c["surf"], c["rincr"], c["rmax"], c["trg"], c["env"],
                        c["npcorr_order"])
    assert c["npcorr"].size == out.size and c["npcorr"].sum() > 0
    assert np.array_equal(out.reshape(-1), c["npcorr"])
