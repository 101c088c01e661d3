"""icep_Calc_f_Lennard_Jones_noalloc (scratch in a fixed device array, no
context) against icep_Calc_f_Lennard_Jones on a context, through the C-ABI.

Both run the same cell-list kernels in FP64, so the forces agree to rounding
(tolerance 1e-12 relative, per component). Two different workloads run back
to back through the shared scratch array, so the second call also shows that
what the first left behind is not used. The file sorts last so that it also
runs after every other GPU test in one session.
"""
import ctypes as C

import numpy as np
import pytest

import cases
from icep_kapsel_gb300 import abi
from icep_kapsel_gb300.runtime import Simulation, load_library

pytestmark = pytest.mark.gpu

RTOL = 1e-12
MAX_PARTICLES = 65536  # ICEP_LJ_NOALLOC_MAX_PARTICLES
ERR_UNSUPPORTED = 3  # ICEP_ERR_UNSUPPORTED


def _lib():
    lib = load_library()
    f = lib.icep_Calc_f_Lennard_Jones_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    f.restype = C.c_int
    lib.icep_Calc_f_Lennard_Jones.argtypes = [C.c_void_p]
    lib.icep_Calc_f_Lennard_Jones.restype = C.c_int
    return lib


def _fr(parts, n):
    return np.array([[parts[q].fr[d] for d in range(3)] for q in range(n)])


def _with_context(lib, p, parts):
    sim = Simulation(p, parts)
    try:
        assert lib.icep_Calc_f_Lennard_Jones(sim.ctx) == 0
        return _fr(sim.particles(), p.n_particles)
    finally:
        sim.close()


def _no_alloc(lib, p, parts):
    torch = pytest.importorskip("torch")
    n = p.n_particles
    raw = bytes(parts)[: n * C.sizeof(abi.Particle)]
    # stale fr values: the entry point must overwrite them
    dev = torch.frombuffer(bytearray(raw), dtype=torch.uint8).to("cuda")
    torch.cuda.synchronize()
    st = lib.icep_Calc_f_Lennard_Jones_noalloc(C.byref(p), C.c_void_p(dev.data_ptr()), n, None)
    assert st == 0
    torch.cuda.synchronize()
    back = (abi.Particle * n).from_buffer_copy(dev.cpu().numpy().tobytes())
    return _fr(back, n)


def _cases():
    pa, xa = cases.lj_dense_case()  # 32^3: two cells per side, repeated visits
    pb, xb = cases.lj_dense_case(n=64, npart=96, seed=11, minsep=7.0)
    for q in range(pb.n_particles):
        xb[q].fr[0] = 123.0  # non-zero fr on input
    return [(pa, xa), (pb, xb)]


def test_no_alloc_matches_context_entry_point_twice():
    lib = _lib()
    for p, parts in _cases():
        ref = _with_context(lib, p, parts)
        got = _no_alloc(lib, p, parts)
        assert np.abs(ref).max() > 0.0
        np.testing.assert_allclose(got, ref, rtol=RTOL, atol=RTOL * np.abs(ref).max())


@pytest.mark.parametrize("truncate", [0, -1])
def test_no_alloc_matches_other_cutoffs(truncate):
    """LJ_truncate OFF (cutoff at half the smallest box edge, at most 2.5
    diameters) and NONE (no Lennard-Jones force: fr comes back zero), both
    entry points deriving the cutoff from the same parameters."""
    lib = _lib()
    p, parts = cases.lj_dense_case()
    p.lj_truncate = truncate
    for q in range(p.n_particles):
        parts[q].fr[1] = -7.0  # stale input
    ref = _with_context(lib, p, parts)
    got = _no_alloc(lib, p, parts)
    if truncate < 0:
        assert np.abs(ref).max() == 0.0 and np.abs(got).max() == 0.0
    else:
        assert np.abs(ref).max() > 0.0
        np.testing.assert_allclose(got, ref, rtol=RTOL, atol=RTOL * np.abs(ref).max())


def test_no_alloc_rejects_oversize():
    lib = _lib()
    p, _ = cases.lj_dense_case()
    st = lib.icep_Calc_f_Lennard_Jones_noalloc(C.byref(p), C.c_void_p(16), MAX_PARTICLES + 1, None)
    assert st == ERR_UNSUPPORTED
    for n in (48, 512):  # not a power of two; more than 16 cells of 16 DX per side
        q, _ = cases.lj_dense_case()
        q.nx = n
        st = lib.icep_Calc_f_Lennard_Jones_noalloc(C.byref(q), C.c_void_p(16), 4, None)
        assert st == ERR_UNSUPPORTED, n
