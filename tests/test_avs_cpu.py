"""The AVS/Express writers (icep_avs_init, icep_avs_charge_frame,
icep_avs_particles; host code, no GPU) against the reference's own writers
(avs_output.cxx, avs_output_p.cxx): tests/golden/make_golden.py ran those on
the seeded inputs of cases.avs_inputs and recorded the SHA-256 and size of
every file they wrote, binary and ASCII. Every file written here must be
byte-identical."""
import ctypes as C
import hashlib
import json
import os

import numpy as np
import pytest

import cases
from icep_kapsel_gb300 import abi

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def lib():
    from icep_kapsel_gb300 import build
    build.build()
    from icep_kapsel_gb300 import runtime
    return runtime.load_library()


def write(L, d, ascii, fields, parts, n):
    arr = (C.POINTER(C.c_double) * 7)(*[f.ctypes.data_as(C.POINTER(C.c_double)) for f in fields])
    dd, nm = os.fsencode(d), b"data"
    assert L.icep_avs_init(dd, nm, ascii, 16, 16, 16, C.c_double(1.0), 6, n) == 0
    assert L.icep_avs_charge_frame(dd, nm, ascii, 16, 16, 16, 20, C.c_double(0.25), arr) == 0
    assert L.icep_avs_particles(dd, nm, ascii, 20, C.c_double(0.25), parts, n, C.c_double(2.0)) == 0


def listing(d, ascii):
    out = {}
    for root, _, names in os.walk(d):
        for nm in names:
            path = os.path.join(root, nm)
            blob = open(path, "rb").read()
            out["%d/%s" % (ascii, os.path.relpath(path, d))] = [hashlib.sha256(blob).hexdigest(), len(blob)]
    return out


def test_avs_files_match_reference_writers(lib, tmp_path):
    with open(os.path.join(GOLD, "avs16.json")) as fh:
        meta = json.load(fh)
    n = 3
    fields, x, q = cases.avs_inputs(16, 16, 16, n)
    parts = abi.make_particles(x)
    for i in range(n):
        for d in range(4):
            parts[i].q[d] = q[i, d]
    got = {}
    for ascii in (0, 1):
        d = str(tmp_path / ("a%d" % ascii))
        write(lib, d, ascii, fields, parts, n)
        got.update(listing(d, ascii))
        for rel, txt in meta["text"].items():
            if rel.startswith("%d/" % ascii):
                assert open(os.path.join(d, rel[2:])).read() == txt, rel
    assert got == meta["files"]


def test_avs_binary_payload_layout(lib, tmp_path):
    """The binary frame holds the 7 fields as float32, x fastest, in order."""
    n = 3
    fields, x, q = cases.avs_inputs(16, 16, 16, n)
    parts = abi.make_particles(x)
    for i in range(n):
        for d in range(4):
            parts[i].q[d] = q[i, d]
    d = str(tmp_path / "b")
    write(lib, d, 0, fields, parts, n)
    data = np.fromfile(os.path.join(d, "avs", "data_20.dat"), dtype=np.float32).reshape(7, 16, 16, 16)
    for v in range(7):
        assert np.array_equal(data[v], fields[v][:, :, :16].astype(np.float32).transpose(2, 1, 0))
    cod = np.fromfile(os.path.join(d, "avs", "datap_20.cod"), dtype=np.float32).reshape(3, n)
    assert np.array_equal(cod, x[:, ::-1].T.astype(np.float32))


def test_avs_errors(lib, tmp_path):
    bad = os.fsencode(str(tmp_path / "missing" / "deeper"))
    assert lib.icep_avs_init(bad, b"data", 0, 16, 16, 16, C.c_double(1.0), 6, 0) == 6  # ICEP_ERR_IO
    assert lib.icep_avs_init(None, b"data", 0, 16, 16, 16, C.c_double(1.0), 6, 0) == 1  # ICEP_ERR_ARG
