"""Helpers to read the committed golden fixtures (tests/golden/*.npz)."""
import os

import numpy as np

from ima2p_gb300.synth import Genealogy

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name))


def trees(d, prefix=""):
    up0, up1, down = d[prefix + "up0"], d[prefix + "up1"], d[prefix + "down"]
    time, root = d[prefix + "time"], d[prefix + "root"]
    return [Genealogy(up0[i].copy(), up1[i].copy(), down[i].copy(), time[i].copy(), int(root[i]))
            for i in range(len(root))]
