#!/usr/bin/env python3
"""Generate the golden fixtures in tests/golden/ from the REFERENCE itself.

Each case builds a seeded synthetic specimen, writes the PARAPROBE inputs
(POS, RRNG, VTK hull, XML settings), and runs oracle/_ref/ref_spatstat -- the
reference's own KDTree.cpp / Histogram.h / Math.cpp / AABBTree.cpp /
PeriodicTable.cpp / Settings.cpp compiled from the read-only reference tree
by oracle/ref/Makefile, driven by a restatement of the SolverHdl.cpp glue.
The fixture stores the inputs (float32 arrays), the settings text, and the
reference's outputs: raw histogram counts, neighbour-count histograms,
centre/pair statistics, ion-to-hull distances, the occupancy grid's
NumberOfIonsInside / VolumeInside (which head the RDF files) and the CSV
files.

Run where the reference tree is present (its location in
PARAPROBE_REFERENCE_TREE, or the default oracle/ref/Makefile names):
    make -C oracle/ref
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from paraprobe_gb300 import synth  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "ref_spatstat")

CASES = [
    dict(name="cyl_basic", geom="cyl", n=15000, radius=5.0, height=14.0, seed=101, analyses="1234",
         tasks="Sc-Al,Sc,Zr;Al-Sc;Sc,Zr-Zr", r=("0.0", "0.01", "1.0"), mknn="1;5;10", threads=4),
    dict(name="cone_pairs", geom="cone", n=20000, seed=102, nspecies=4, analyses="14",
         tasks=None, r=("0.0", "0.005", "1.5"), mknn="1;3;8", threads=3),
    dict(name="cntnb", geom="cyl", n=12000, radius=4.5, height=14.0, seed=103, analyses="16",
         tasks="Sc-Al,Sc,Zr;Al,Sc-Zr", r=("0.0", "0.02", "1.2"), mknn="", threads=2),
    dict(name="edges", geom="cyl", n=12000, radius=4.5, height=14.0, seed=104, analyses="1234",
         tasks="Al-Al,Sc,Zr;Sc-Al", r=("0.3", "0.1", "1.3"), mknn="2;40", threads=5,
         bin_width=("0.5", "0.6", "0.7")),
    dict(name="shuffled", geom="cyl", n=15000, radius=5.0, height=14.0, seed=105, analyses="12",
         tasks="Sc-Al,Sc,Zr", r=("0.0", "0.01", "1.0"), mknn="", threads=4, shuffle_seed=9001),
    dict(name="nohull", geom="cyl", n=12000, radius=4.5, height=14.0, seed=106, analyses="24",
         tasks="Al,Sc,Zr-Al,Sc,Zr", r=("0.0", "0.01", "0.8"), mknn="1;2;3;4;5", threads=2, hull=False),
    dict(name="bigk", geom="cyl", n=15000, radius=5.0, height=14.0, seed=107, analyses="4",
         tasks="Al-Al,Sc,Zr;Sc-Sc,Zr", r=("0.0", "0.01", "1.3"), mknn="1;33;64;100", threads=3),
    dict(name="rdf_sym", geom="cone", n=20000, seed=108, nspecies=4, analyses="13",
         tasks="Al-Al,Sc;Sc,Zr-Al,Sc,Zr;Si-Al", r=("0.1", "0.02", "1.6"), mknn="", threads=3),
    dict(name="npcorr", geom="cone", n=15000, seed=109, nspecies=3, analyses="125",
         tasks="Al-Al,Sc;Sc-Al,Sc,Zr;Zr-Zr", r=("0.0", "0.05", "1.0"), mknn="", threads=3, knn_order=3),
]


def specimen(c):
    if c["geom"] == "cyl":
        return synth.cylinder_specimen(n=c["n"], radius=c["radius"], height=c["height"], seed=c["seed"],
                                       nseg=64, stack=4.0)
    return synth.cone_specimen(n=c["n"], r_apex=7.0, half_angle_deg=10.0, length=16.0, n_clusters=15,
                               members=40, nspecies=c["nspecies"], seed=c["seed"], nseg=64, stack=4.0)


def make(c, outdir):
    spec = specimen(c)
    with tempfile.TemporaryDirectory() as tmp:
        pos, rrng, vtk = synth.write_inputs(spec, tmp, c["name"])
        tasks = c["tasks"] or synth.all_pairs_tasks(spec.nspecies)
        hull = c.get("hull", True)
        xml = os.path.join(tmp, "settings.xml")
        synth.write_settings_xml(xml, pos, rrng, vtk if hull else None, c["analyses"], tasks, *c["r"],
                                 mknn=c["mknn"], bin_width=c.get("bin_width"), knn_order=c.get("knn_order", 1))
        out = os.path.join(tmp, "out")
        # the harness computes NumberOfIonsInside / VolumeInside with the
        # reference's occupancy grid (its own Hoshen-Kopelman unit)
        cmd = [REF, "7", xml, str(c["threads"]), out, "--dump-surf", "--voxelize"]
        labels = spec.labels
        if "shuffle_seed" in c:
            from paraprobe_gb300 import native
            labels = native.shuffle_labels(spec.labels, c["shuffle_seed"])
            lf = os.path.join(tmp, "labels.u8")
            labels.tofile(lf)
            cmd += ["--labels", lf]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"{c['name']}: reference harness failed\n{r.stderr[-2000:]}")
        _, mq = synth.read_pos(pos)
        voxel = {}
        for line in open(os.path.join(out, "voxel.txt")):
            k, v = line.split()
            voxel[k] = float(v) if k == "volume_inside" else int(v)
        nins, vol = voxel["nions_inside"], voxel["volume_inside"]
        stats = {}
        task_lines, ks = [], []
        for line in open(os.path.join(out, "stats.txt")):
            p = line.split()
            if p[0] == "task":
                task_lines.append(p[1:])
            elif p[0] == "k":
                ks.append(int(p[1]))
            else:
                stats[p[0]] = int(p[1])
        trg = [[int(x[1:]) for x in t[3:] if x.startswith("T")] for t in task_lines]
        env = [[int(x[1:]) for x in t[3:] if x.startswith("E")] for t in task_lines]
        csvs = {}
        for f in sorted(os.listdir(out)):
            if f.endswith(".csv"):
                csvs[f] = open(os.path.join(out, f)).read()
        meta = dict(case=c, tasks_code=tasks, trg=trg, env=env, names=[t[1:3] for t in task_lines], k=ks,
                    stats=stats, nions_inside=nins, volume_inside=vol, voxel=voxel,
                    settings_xml=open(xml).read().replace(tmp + "/", ""),
                    rrng=open(rrng).read())
        np.savez_compressed(
            os.path.join(outdir, c["name"] + ".npz"),
            xyz=spec.xyz, mq=mq, labels=labels, hull=spec.hull if hull else np.zeros((0, 9), np.float32),
            surf=np.fromfile(os.path.join(out, "ion2surf.f32"), dtype=np.float32),
            bins=np.fromfile(os.path.join(out, "raw_bins.u64"), dtype=np.uint64),
            cntnb=np.fromfile(os.path.join(out, "raw_cntnb.u64"), dtype=np.uint64),
            npcorr=(np.fromfile(os.path.join(out, "raw_npcorr.u32"), dtype=np.uint32)
                    if os.path.exists(os.path.join(out, "raw_npcorr.u32")) else np.zeros(0, np.uint32)),
            meta=np.array(json.dumps(meta)), csv=np.array(json.dumps(csvs)))
        return stats


# Statistics after clustering (clustertask::flag2exclude_guard and
# generic_spatstat): the harness builds the clustering task's global KD-tree
# with the reference's own kd_tree and runs the guard loop as written.  The
# fixtures go to tests/golden/apost/ with the tree order, so that a test can
# hand the cloud over in that order.
APOST_CASES = [
    dict(name="apost_rdf", n=20000, seed=201, what="rdf", r=("0.0", "0.01", "1.0"), frac=0.5),
    dict(name="apost_1nn", n=20000, seed=202, what="1nn", r=("0.0", "0.005", "0.8"), frac=0.7),
    dict(name="apost_ripk", n=25000, seed=203, what="ripk", r=("0.1", "0.02", "1.2"), frac=0.3),
]
APOST_DIR = os.path.join(HERE, "apost")


def make_apost(c, outdir):
    spec = synth.cone_specimen(n=c["n"], r_apex=7.0, half_angle_deg=10.0, length=16.0, n_clusters=15,
                               members=40, nspecies=3, seed=c["seed"], nseg=64, stack=4.0)
    # clustered ions: a seeded share of the cluster-forming species
    rng = np.random.default_rng(c["seed"])
    clustered = ((spec.labels == 2) & (rng.random(spec.labels.size) < c["frac"])).astype(np.uint8)
    what_digit = {"rdf": "1", "1nn": "2", "ripk": "3"}[c["what"]]
    with tempfile.TemporaryDirectory() as tmp:
        pos, rrng, vtk = synth.write_inputs(spec, tmp, c["name"])
        xml = os.path.join(tmp, "settings.xml")
        synth.write_settings_xml(xml, pos, rrng, vtk, what_digit, synth.all_pairs_tasks(spec.nspecies), *c["r"],
                                 mknn="")
        cf = os.path.join(tmp, "clustered.u8")
        clustered.tofile(cf)
        out = os.path.join(tmp, "out")
        cmd = [REF, "7", xml, "1", out, "--dump-surf", "--aposteriori", cf, c["what"]]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"{c['name']}: reference harness failed\n{r.stderr[-2000:]}")
        stats = {}
        for line in open(os.path.join(out, "apost_stats.txt")):
            k, v = line.split()
            stats[k] = int(v)
        np.savez_compressed(
            os.path.join(outdir, c["name"] + ".npz"),
            xyz=spec.xyz, labels=spec.labels, clustered=clustered, hull=spec.hull,
            surf=np.fromfile(os.path.join(out, "ion2surf.f32"), dtype=np.float32),
            bins=np.fromfile(os.path.join(out, "raw_apost.u64"), dtype=np.uint64),
            tree_order=np.fromfile(os.path.join(out, "tree_order.u64"), dtype=np.uint64),
            meta=np.array(json.dumps(dict(case=c, stats=stats))))
        return stats


def main():
    if not os.path.exists(REF):
        raise SystemExit(f"{REF} missing: build it with make -C oracle/ref")
    only = set(sys.argv[1:])
    for c in CASES:
        if only and c["name"] not in only:
            continue
        st = make(c, HERE)
        print(c["name"], st)
    os.makedirs(APOST_DIR, exist_ok=True)
    for c in APOST_CASES:
        if only and c["name"] not in only:
            continue
        st = make_apost(c, APOST_DIR)
        print(c["name"], st)


if __name__ == "__main__":
    main()
