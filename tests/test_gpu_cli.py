"""The drop-in CLI (settings -> POS -> device ranging -> hull -> tasks -> C ABI
-> CSV) writes the same CSV files, byte for byte, as the reference harness."""
import os
import subprocess

import numpy as np
import pytest

import golden_cases as G
from host_inputs import write_case

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "paraprobe_gb300", "_lib", "paraprobe_gpu")


@pytest.mark.parametrize("inside", ["given", "computed"])
@pytest.mark.parametrize("name", G.names())
def test_cli_csv_identical(ctx, tmp_path, name, inside):
    """With --inside the header values are passed in; without it the CLI
    computes them with the occupancy grid, as the reference does."""
    c = G.load(name)
    write_case(c, str(tmp_path))
    out = tmp_path / "out"
    out.mkdir()
    cmd = [CLI, "7", "settings.xml", "--outdir", str(out)]
    if inside == "given":
        cmd += ["--inside", str(c["meta"]["nions_inside"]), repr(c["meta"]["volume_inside"])]
    if name == "shuffled":
        np.ascontiguousarray(c["labels"], dtype=np.uint8).tofile(tmp_path / "labels.u8")
        cmd += ["--labels", "labels.u8"]
    r = subprocess.run(cmd, cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr + r.stdout
    produced = sorted(f for f in os.listdir(out) if f.endswith(".csv") and ".FP64Audit." not in f)
    assert produced == sorted(c["csv"].keys())
    # n-point correlations: one raw uint32 file per task, as the reference's counts
    raws = sorted(f for f in os.listdir(out) if ".NPCORR." in f)
    if c["npcorr"].size:
        got = np.concatenate([np.fromfile(out / f, dtype=np.uint32) for f in
                              sorted(raws, key=lambda f: [G.task_index(c, f)])])
        assert len(raws) == len(c["trg"]) and np.array_equal(got, c["npcorr"])
    else:
        assert not raws
    for f in produced:
        assert (out / f).read_text() == c["csv"][f], f
    # the FP64 audit beside the reports: small errors, every listed pair on an edge
    audits = [f for f in os.listdir(out) if ".FP64Audit." in f]
    assert len(audits) == 1 and "FP64 audit" in r.stdout
    lines = (out / audits[0]).read_text().splitlines()
    head = dict(l.split(";", 1) for l in lines[:5])
    assert float(head["MaxAbsError"]) < 1e-6 and int(head["Pairs"]) > 0
    rows = [l.split(";") for l in lines[6:]]
    assert len(rows) == min(int(head["BinDisagreements"]) + int(head["InBallDisagreements"]), 1 << 16)
    for row in rows:
        assert abs(float(row[6])) <= 1e-6 * max(float(row[3]), 1e-3), row


@pytest.mark.parametrize("name", ["cyl_basic", "npcorr"])
def test_cli_epos_input(ctx, tmp_path, name):
    """The same specimen given as an EPOS file (InputFileformat 2, coordinates
    taken as they are: ReconstructionAlgorithm 3) gives the same CSV files."""
    from paraprobe_gb300 import synth
    c = G.load(name)
    write_case(c, str(tmp_path))
    stem = c["meta"]["case"]["name"]
    synth.write_epos(str(tmp_path / (stem + ".epos")), c["xyz"], c["mq"])
    xml = (tmp_path / "settings.xml").read_text()
    xml = xml.replace("<InputFileformat>1<", "<InputFileformat>2<")
    xml = xml.replace("<ReconstructionAlgorithm>2<", "<ReconstructionAlgorithm>3<")
    xml = xml.replace(stem + ".pos<", stem + ".epos<")
    assert "<InputFileformat>2<" in xml and ".epos<" in xml
    (tmp_path / "settings.xml").write_text(xml)
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([CLI, "7", "settings.xml", "--outdir", str(out)], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr + r.stdout
    produced = sorted(f for f in os.listdir(out) if f.endswith(".csv") and ".FP64Audit." not in f)
    assert produced == sorted(c["csv"].keys())
    for f in produced:
        assert (out / f).read_text() == c["csv"][f], f
