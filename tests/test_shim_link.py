"""The link-level drop-in: IMa2p's own sources, compiled where they lie with
the hot-path functions of three files renamed (cpu_*), linked with
ima2p_gb300/shim/ima2p_shims.cpp and libima2p_gb300.so into IMa2p_gb300.
The program must link, its hot-path symbols must be the shim's (the
reference's bodies renamed beside them), and it must start (its command-line
banner needs no GPU).  Needs the IMa2p source tree (oracle.pyoracle.REFERENCE, set by
IMA2P_REFERENCE); skipped where it is absent."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "ima2p_gb300", "shim")
from oracle.pyoracle import REFERENCE as REF
LIB = os.path.join(ROOT, "ima2p_gb300", "libima2p_gb300.so")

pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")) or not os.path.exists(LIB),
                                reason="IMa2p sources or the built library absent")

REPLACED = ["likelihoodIS(int, int, double)", "likelihoodHKY(int, int, double, double, int, int, int, int)",
            "likelihoodSW(int, int, int, double, double)", "copyfraclike(int, int)",
            "storescalefactors(int, int)", "restorescalefactors(int, int)", "swapchains(int, int, int, int)"]


def test_ima2p_links_against_the_library():
    subprocess.run(["make", "-s", "-j8", "-C", SHIM, "IMA2P_REFERENCE=" + REF], check=True)
    exe = os.path.join(SHIM, "_build", "IMa2p_gb300")
    assert os.path.exists(exe)
    syms = subprocess.run(["nm", "-C", exe], capture_output=True, text=True, check=True).stdout
    shim = subprocess.run(["nm", "-C", os.path.join(SHIM, "_build", "ima2p_shims.o")], capture_output=True,
                          text=True, check=True).stdout
    for f in REPLACED:
        assert " T " + f in shim, f                 # defined by the shim
        assert " T cpu_" + f in syms, f             # the reference's body, renamed
        assert sum(1 for l in syms.splitlines() if l.endswith(" " + f)) == 1, f
    dyn = subprocess.run(["ldd", exe], capture_output=True, text=True).stdout
    assert "libima2p_gb300.so" in dyn and "not found" not in dyn.split("libima2p_gb300.so")[1].splitlines()[0]
    out = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert "IMa2p" in out.stdout
