"""Shared helpers of the GPU parity tests."""
import numpy as np

from ima2p_gb300 import api, synth


def ctx_with(loci_specs, nruns=1, cpr=1):
    """loci_specs: list of ("is", seq) | ("hky", HKYLocus) | ("sw", n, nlinked)."""
    c = api.Context(0)
    for spec in loci_specs:
        if spec[0] == "is":
            c.add_locus_is(spec[1])
        elif spec[0] == "hky":
            L = spec[1]
            c.add_locus_hky(L.seq, L.mult, L.totsites)
        else:
            c.add_locus_sw(spec[1], spec[2] if len(spec) > 2 else 1)
    c.set_chains(nruns, cpr)
    return c
