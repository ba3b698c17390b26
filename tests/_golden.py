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


class TwCase:
    """One case of golden_tw.npz: the population model, loci, split times,
    labelled genealogies and the reference's weights and integrals."""

    def __init__(self, d, c):
        from ima2p_gb300 import popmodel
        from ima2p_gb300.synth import LabelledGenealogy
        k = "c%d_" % c
        self.npops, self.nch, self.nl, expo, nomig = (int(v) for v in d[k + "meta"])
        self.expo, self.nomig = bool(expo), bool(nomig)
        self.tree = str(d[k + "tree"])
        self.thetaprior, self.mprior = (float(v) for v in d[k + "priors"])
        loci = d[k + "loci"]
        self.loci = [(int(r[0]), float(r[1]), [int(v) for v in r[2:]]) for r in loci]
        self.tvals = d[k + "tvals"]
        self.pm = popmodel.build(self.tree, self.npops, nomig=self.nomig)
        no, mo = d[k + "node_off"], d[k + "mig_off"]
        self.gens = []
        for i in range(self.nch * self.nl):
            a, b = int(no[i]), int(no[i + 1])
            pop = d[k + "pop"][a:b].copy()
            mig = []
            for j in range(a, b):
                mig.append([(float(d[k + "mig_t"][e]), int(d[k + "mig_p"][e])) for e in range(mo[j], mo[j + 1])])
            root = int(np.flatnonzero(d[k + "down"][a:b] == -1)[0])
            g = Genealogy(d[k + "up0"][a:b].copy(), d[k + "up1"][a:b].copy(), d[k + "down"][a:b].copy(),
                          d[k + "time"][a:b].copy(), root)
            self.gens.append(LabelledGenealogy(g, pop, mig))
        self.ref = {f: d[k + f] for f in ("cc", "hcc", "fc", "mc", "fm", "scal", "pg")}
        self.th_pr, self.mg_pr = d[k + "th_pr"], d[k + "mg_pr"]
        self.th_wp = self._wp(d[k + "th_wp"], len(self.th_pr), 2)
        self.mg_wp = self._wp(d[k + "mg_wp"], len(self.mg_pr), 3)

    @staticmethod
    def _wp(a, n, w):
        lens, rest, out, o = a[:n], a[n:], [], 0
        for ln in lens:
            out.append([tuple(int(v) for v in rest[o + w * j:o + w * j + w]) for j in range(ln)])
            o += w * ln
        return out

    def gen(self, ci, li):
        return self.gens[ci * self.nl + li]


def tw_cases():
    d = load("golden_tw.npz")
    return [TwCase(d, c) for c in range(int(d["ncases"]))]
