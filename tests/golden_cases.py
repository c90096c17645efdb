"""Loader for the reference-generated golden fixtures in tests/golden/."""
import glob
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")

FLAG_OF_DIGIT = {"1": 1, "2": 2, "3": 4, "4": 8, "5": 16, "6": 32}


def names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(z["meta"]))
    c = meta["case"]
    flags = 0
    for d in c["analyses"]:
        flags |= FLAG_OF_DIGIT.get(d, 0)
    rmin, rincr, rmax = (np.float32(float(x)) for x in c["r"])
    bw = c.get("bin_width") or ("1.0", "1.0", "1.0")
    return dict(xyz=z["xyz"], mq=z["mq"], labels=z["labels"], hull=z["hull"], surf=z["surf"], bins=z["bins"],
                cntnb=z["cntnb"], meta=meta, csv=json.loads(str(z["csv"])), flags=flags,
                rmin=rmin, rincr=rincr, rmax=rmax, trg=meta["trg"], env=meta["env"], k=meta["k"],
                stats=meta["stats"], voxel=meta["voxel"],
                npcorr=z["npcorr"] if "npcorr" in z.files else np.zeros(0, np.uint32),
                npcorr_order=int(c.get("knn_order", 1)) - 1,
                bin_width=(np.float32(float(bw[0])), np.float32(float(bw[2]))))


def task_index(c, filename):
    """Task of a per-task output file, from the task names in its name."""
    for t, (a, b) in enumerate(c["meta"]["names"]):
        if f".{a}.{b}." in filename:
            return t
    raise KeyError(filename)
