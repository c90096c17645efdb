"""Host layer (settings, ranging, tasks, MKNN code) against the reference's own
parsers, through the drop-in CLI's --plan mode; CPU only."""
import json
import os
import subprocess

import numpy as np
import pytest

import golden_cases as G
from host_inputs import write_case

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "paraprobe_gb300", "_lib", "paraprobe_gpu")


@pytest.mark.parametrize("name", G.names())
def test_plan_matches_reference_parsers(native_lib, tmp_path, name):
    c = G.load(name)
    write_case(c, str(tmp_path))
    r = subprocess.run([CLI, "7", "settings.xml", "--plan"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    plan = json.loads(r.stdout.strip().splitlines()[-1])
    assert plan["flags"] == c["flags"]
    assert plan["k"] == c["k"]
    assert plan["max_type_id"] == c["stats"]["maxtypeid"]
    assert [t["trg"] for t in plan["tasks"]] == c["trg"]
    assert [t["env"] for t in plan["tasks"]] == c["env"]
    assert [t["names"] for t in plan["tasks"]] == c["meta"]["names"]
    assert np.float32(plan["rmax"]) == c["rmax"]


def _xml(tmp_path, **kw):
    from paraprobe_gb300 import synth
    synth.write_settings_xml(str(tmp_path / "s.xml"), "x.pos", "x.rrng", None, **kw)
    return "s.xml"


def _plan(tmp_path, xml):
    r = subprocess.run([CLI, "1", xml, "--plan"], cwd=tmp_path, capture_output=True, text=True)
    return r


def test_analysis_digit_rules(native_lib, tmp_path):
    (tmp_path / "x.rrng").write_text("[Ranges]\nRange1=1 2 Vol:0.1 Al:1 Color:0\nRange2=3 4 Vol:0.1 Sc:1 Color:0\n")
    cases = {"1": 1, "14": 9, "1234": 15, "12346": None, "104": None, "6": 32, "26": 34, "5": 16, "125": 19}
    for code, flags in cases.items():
        xml = _xml(tmp_path, analyses=code, tasks="Al-Sc", rmin="0", rincr="0.1", rmax="1", mknn="1;2")
        r = _plan(tmp_path, xml)
        if flags is None:
            assert "No spatial statistics task to do" in r.stdout
        else:
            assert json.loads(r.stdout.strip().splitlines()[-1])["flags"] == flags, code


def test_invalid_settings_rejected(native_lib, tmp_path):
    (tmp_path / "x.rrng").write_text("[Ranges]\nRange1=1 2 Vol:0.1 Al:1 Color:0\n")
    xml = _xml(tmp_path, analyses="1", tasks="Al-Al", rmin="1.0", rincr="0.1", rmax="0.5")
    r = _plan(tmp_path, xml)
    assert r.returncode == 3 and "SpatStatRadiusMin is larger" in r.stderr
    (tmp_path / "bad.xml").write_text("<Parameters><RAWFilenameIn>x</Parameters>")
    r = _plan(tmp_path, "bad.xml")
    assert r.returncode == 3


def test_molecular_and_invalid_tasks(native_lib, tmp_path):
    (tmp_path / "x.rrng").write_text(
        "[Ions]\n[Ranges]\nRange1=1 2 Vol:0.1 Al:1 H:1 Color:0\nRange2=3 4 Vol:0.1 Sc:1 Color:0\n"
        "Range3=5 6 Vol:0.1 S:1 Color:0\nRange4=7 8 Vol:0.1 Al:1 Color:0\n")
    xml = _xml(tmp_path, analyses="4", tasks="AlH-Sc;Sc-S;X-Al;Al-Al-Sc;HAl,Al-Sc,S", rmin="0", rincr="0.1",
               rmax="1", mknn="3;1;-2")
    plan = json.loads(_plan(tmp_path, xml).stdout.strip().splitlines()[-1])
    # AlH and HAl name the same molecular ion; X is unknown and Al-Al-Sc has two '-'
    assert [t["names"] for t in plan["tasks"]] == [["AlH", "Sc"], ["Sc", "S"], ["AlAlH", "SSc"]]
    assert plan["k"] == []  # a '-' anywhere disables the MKNN code
