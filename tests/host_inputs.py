"""Write a golden case's PARAPROBE input files into a directory."""
import os

import numpy as np

from paraprobe_gb300 import synth


def write_case(c, d):
    meta = c["meta"]
    name = meta["case"]["name"]
    synth.write_pos(os.path.join(d, name + ".pos"), c["xyz"], c["mq"])
    with open(os.path.join(d, name + ".rrng"), "w") as f:
        f.write(meta["rrng"])
    if c["hull"].shape[0]:
        synth.write_vtk(os.path.join(d, name + ".vtk"), c["hull"])
    xml = os.path.join(d, "settings.xml")
    with open(xml, "w") as f:
        f.write(meta["settings_xml"])
    return xml
