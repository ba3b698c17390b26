"""Saved-genealogy (.ti) files: the library's parser against the format the
reference writes (savegenealogyfile, output.cpp:662-685: "%.6f\\t" per value)
and reads (loadgenealogyvalues, ima_main_mpi.cpp:3216-3440), including its
running-fraction subsampling rule, and the binary side-car.  Host code only:
no device work, so these run on CPU (skipped if the library is not built)."""
import os

import numpy as np
import pytest

from ima2p_gb300 import api

pytestmark = pytest.mark.skipif(not os.path.exists(api.LIB_PATH), reason="library not built here")


def write_ti(path, rows, header_lines=3):
    with open(path, "w") as f:
        for k in range(header_lines):
            f.write("IMa2p header line %d: parameters and priors\n" % k)
        f.write("VALUESSTART\n")
        for r in rows:
            f.write("".join("%.6f\t" % v for v in np.asarray(r, np.float32)) + "\n")


def parsed(rows):
    """What sscanf("%f") makes of each "%.6f" value."""
    return np.array([[np.float32(float("%.6f" % v)) for v in r] for r in np.asarray(rows, np.float32)], np.float32)


def ref_keep(counts, maxload):
    """The reference's kept-line rule in its float arithmetic."""
    tot = sum(counts)
    numtoload = min(tot, maxload) if maxload > 0 else tot
    numtoload = min(numtoload, 300000)
    loadall = numtoload >= tot
    lf = np.float32(numtoload) / np.float32(tot)
    keep, nl, nn = [], 0, 0
    for f, c in enumerate(counts):
        for line in range(c):
            if loadall or nl == 0 or np.float32(nl) / np.float32(nl + nn) <= lf:
                keep.append((f, line))
                nl += 1
            else:
                nn += 1
    return keep


def test_text_files_load_as_the_reference_reads_them(tmp_path):
    rng = np.random.default_rng(4)
    rowlen = 21
    parts = [rng.normal(0, 50, (n, rowlen)).astype(np.float32) for n in (700, 1100, 5)]
    paths = []
    for k, p in enumerate(parts):
        paths.append(str(tmp_path / ("run%d.ti" % k)))
        write_ti(paths[-1], p, header_lines=2 + k)
    rows, total = api.ti_read(paths, rowlen)
    assert total == 1805
    assert np.array_equal(rows, parsed(np.concatenate(parts)))
    # subsampled: 600 of 1805 by the running-fraction rule, across files in order
    rows, total = api.ti_read(paths, rowlen, maxload=600)
    keep = ref_keep([len(p) for p in parts], 600)
    want = parsed(np.stack([parts[f][line] for f, line in keep]))
    assert total == 1805 and np.array_equal(rows, want)


def test_malformed_files_are_rejected(tmp_path):
    rowlen = 5
    good = np.arange(20, dtype=np.float32).reshape(4, 5)
    p = str(tmp_path / "short.ti")
    write_ti(p, good)
    with open(p, "a") as f:
        f.write("1.0\t2.0\t3.0\n")  # too few values
    with pytest.raises(api.ImaError):
        api.ti_read([p], rowlen)
    q = str(tmp_path / "long.ti")
    write_ti(q, np.arange(12, dtype=np.float32).reshape(2, 6))  # too many for rowlen 5
    with pytest.raises(api.ImaError):
        api.ti_read([q], rowlen)
    r = str(tmp_path / "nostart.ti")
    with open(r, "w") as f:
        f.write("no start marker\n1\t2\t3\t4\t5\t\n")
    with pytest.raises(api.ImaError):
        api.ti_read([r], rowlen)


def test_binary_side_car_round_trip(tmp_path):
    rng = np.random.default_rng(5)
    rows = rng.normal(0, 10, (3000, 48)).astype(np.float32)
    p = str(tmp_path / "rows.tib")
    api.ti_write_binary(p, rows)
    back = api.ti_read_binary(p)
    assert back.dtype == np.float32 and np.array_equal(back, rows)


def test_binary_side_car_checks_the_callers_buffer(tmp_path):
    """A buffer sized for another row length, or for fewer rows, is refused
    before anything is read into it."""
    import ctypes as C
    rng = np.random.default_rng(6)
    rows = rng.normal(0, 10, (50, 48)).astype(np.float32)
    p = str(tmp_path / "rows.tib")
    api.ti_write_binary(p, rows)
    lib = api.load_library()
    buf = np.full((100, 21), 7.0, np.float32)
    G, rl = C.c_int(), C.c_int(21)
    rc = lib.ima_ti_read_binary(os.fsencode(p), C.byref(G), C.byref(rl), buf.ctypes.data_as(C.c_void_p), 100)
    assert rc == api.IMA_ERR_DATA and rl.value == 48 and G.value == 50
    assert np.all(buf == 7.0)
    buf = np.full((49, 48), 7.0, np.float32)
    rl = C.c_int(48)
    rc = lib.ima_ti_read_binary(os.fsencode(p), C.byref(G), C.byref(rl), buf.ctypes.data_as(C.c_void_p), 49)
    assert rc != api.IMA_OK and np.all(buf == 7.0)
