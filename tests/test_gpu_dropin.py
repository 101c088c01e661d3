"""The drop-in call icep_time_evolution (the reference's Time_evolution
function pointer, sp_3d_ns.cxx:10) on host arrays, one step per call.

* Stepping through the drop-in call continues the device-resident run
  exactly (1e-12 in FP64, 1e-6 in MIXED: scatter atomics): the fields go
  down and come back as FP64 arrays, and in MIXED precision a potential
  handed back unchanged keeps the Poisson solver's float-float state (its
  warm start and time extrapolation).
* A potential changed by the caller is taken as the new state: the solve
  restarts from it and still reaches the tolerance.
"""
import numpy as np
import pytest

import cases
from icep_kapsel_gb300 import abi

pytestmark = pytest.mark.gpu


def rel(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / (nb if nb > 0 else 1.0))


@pytest.fixture(scope="module")
def Sim():
    from icep_kapsel_gb300.build import build
    build()
    from icep_kapsel_gb300.runtime import Simulation
    return Simulation


def case(precision):
    return cases.icep_case(n=32, npart=4, minsep=12.0, seed=2, eps_f=80.0, eps_p=3.0, e_ext=(0.0, 0.0, 0.1),
                           tol=1e-8, solver=abi.SOLVER_SPECTRAL, precision=precision)


@pytest.mark.parametrize("precision,tol", [(abi.FP64, 1e-12), (abi.MIXED, 1e-6)])
def test_dropin_continues_device_run(Sim, precision, tol):
    p, parts = case(precision)
    a = Sim(p, parts)
    a.init_state()
    a.step(2)
    p2, parts2 = case(precision)
    b = Sim(p2, parts2)
    b.init_state()
    b.step(2)
    host = {k: np.ascontiguousarray(b.get(k)) for k in ("zeta0", "zeta1", "c0", "c1", "pot")}
    uk = np.ascontiguousarray(b.uk_dc())
    hp = b.particles()
    for _ in range(3):
        b.time_evolution(host["zeta0"], host["zeta1"], uk, hp, host["c0"], host["c1"], host["pot"], 1)
    a.step(3)
    it_a = a.solver_stats()[0]
    it_b = b.solver_stats()[0]
    assert abs(it_b - it_a) <= 1  # the same warm start (a restart from the FP32 potential takes far more)
    nz = p.nz
    for k in ("zeta0", "zeta1", "c0", "c1"):
        assert rel(host[k], a.get(k)) < tol, k
    x, y = host["pot"][:, :, :nz], a.get("pot")[:, :, :nz]
    assert rel(x - x.mean(), y - y.mean()) < tol
    pa = abi.particles_to_numpy(hp, p.n_particles)
    pb = abi.particles_to_numpy(a.particles(), p.n_particles)
    assert rel(pa["x"], pb["x"]) < tol


def test_dropin_changed_potential_is_taken(Sim):
    p, parts = case(abi.MIXED)
    b = Sim(p, parts)
    b.init_state()
    b.step(2)
    host = {k: np.ascontiguousarray(b.get(k)) for k in ("zeta0", "zeta1", "c0", "c1", "pot")}
    uk = np.ascontiguousarray(b.uk_dc())
    hp = b.particles()
    host["pot"] *= 0.5  # a different initial guess from the caller
    b.time_evolution(host["zeta0"], host["zeta1"], uk, hp, host["c0"], host["c1"], host["pot"], 1)
    _, err, _ = b.solver_stats()
    assert err <= 1e-8


def test_dropin_pinned_host_arrays(Sim):
    """Host arrays pinned through icep_pin_host are read and written by the
    conversion kernels over the CPU-GPU link instead of staging copies: the
    values are the same bits as through the staged path (an I/O-only call),
    and stepping two contexts through either path gives the same run (3e-6:
    the FP32 scatter atomics of two contexts add in different orders)."""
    import ctypes as C
    from icep_kapsel_gb300 import runtime
    lib = runtime.load_library()
    lib.icep_pin_host.argtypes = [C.c_void_p, C.c_size_t]
    lib.icep_unpin_host.argtypes = [C.c_void_p]
    keys = ("zeta0", "zeta1", "c0", "c1", "pot")
    p, parts = case(abi.MIXED)
    a = Sim(p, parts)
    a.init_state()
    a.step(2)
    pinned = {k: np.ascontiguousarray(a.get(k)) for k in keys}
    plain = {k: v.copy() for k, v in pinned.items()}
    for v in pinned.values():
        assert lib.icep_pin_host(v.ctypes.data, v.nbytes) == 0
    try:
        uk, hp = np.ascontiguousarray(a.uk_dc()), a.particles()
        a.time_evolution(pinned["zeta0"], pinned["zeta1"], uk, hp, pinned["c0"], pinned["c1"], pinned["pot"], 0)
        a.time_evolution(plain["zeta0"], plain["zeta1"], uk, hp, plain["c0"], plain["c1"], plain["pot"], 0)
        for k in keys:
            assert np.array_equal(pinned[k], plain[k]), k
        b = Sim(*case(abi.MIXED))
        b.init_state()
        b.step(2)
        ukb, hpb = np.ascontiguousarray(b.uk_dc()), b.particles()
        for _ in range(2):
            a.time_evolution(pinned["zeta0"], pinned["zeta1"], uk, hp, pinned["c0"], pinned["c1"], pinned["pot"], 1)
            b.time_evolution(plain["zeta0"], plain["zeta1"], ukb, hpb, plain["c0"], plain["c1"], plain["pot"], 1)
        for k in ("zeta0", "zeta1", "c0", "c1"):
            assert rel(pinned[k], plain[k]) < 3e-6, k
        x, y = pinned["pot"][:, :, :p.nz], plain["pot"][:, :, :p.nz]
        assert rel(x - x.mean(), y - y.mean()) < 3e-6
    finally:
        for v in pinned.values():
            lib.icep_unpin_host(v.ctypes.data)


def test_failed_pin_leaves_no_error_behind(Sim):
    """icep_pin_host reports a failed registration itself (here: the array is
    registered already) and leaves no CUDA error pending for the context's
    next call, which steps normally."""
    import ctypes as C
    from icep_kapsel_gb300 import runtime
    lib = runtime.load_library()
    lib.icep_pin_host.argtypes = [C.c_void_p, C.c_size_t]
    lib.icep_unpin_host.argtypes = [C.c_void_p]
    p, parts = case(abi.MIXED)
    a = Sim(p, parts)
    a.init_state()
    z = np.ascontiguousarray(a.get("zeta0"))
    assert lib.icep_pin_host(z.ctypes.data, z.nbytes) == 0
    try:
        assert lib.icep_pin_host(z.ctypes.data, z.nbytes) != 0
        keys = ("zeta1", "c0", "c1", "pot")
        h = {k: np.ascontiguousarray(a.get(k)) for k in keys}
        uk, hp = np.ascontiguousarray(a.uk_dc()), a.particles()
        a.time_evolution(z, h["zeta1"], uk, hp, h["c0"], h["c1"], h["pot"], 1)
        assert np.isfinite(z).all()
    finally:
        lib.icep_unpin_host(z.ctypes.data)
    assert lib.icep_unpin_host(z.ctypes.data) != 0  # not registered any more
    a.step(1)
