"""The fused k-space Poisson operator of the MIXED solve and the bounded waits
of its kernels.

test_fused_operator_against_fp64: WORK = B WV1 = A M^-1 WV1 through the three
fused passes (inverse x pass with the gradient multipliers, the plane pass,
forward x pass with the staggered divergence) against an FP64 numpy
restatement of the same operator: the reference's Ax (operate_dielectric.cxx:
485-522: spectral staggered gradient i k exp(i dx k/2), face permittivity
0.5 (eps + eps at the next point), staggered divergence) applied to
M^-1 x, M^-1 = -1/(eps_ref |k|^2), on a random Hermitian-consistent half
spectrum. The 64^3 and 128^3 meshes run the register-resident plane kernel,
32^3 the shared-memory one. Tolerance: 2e-5 relative L2 (FP32 transforms).

test_bounded_wait_*: a kernel launched so that its mbarrier wait runs out
(nothing issued that could complete it) reports ICEP_ERR_TIMEOUT to the host
through its error word, skips its work, and the context then steps normally.
"""
import numpy as np
import pytest

import cases
from icep_kapsel_gb300 import abi

pytestmark = pytest.mark.gpu

ICEP_ERR_TIMEOUT = 7


@pytest.fixture(scope="module")
def Sim():
    from icep_kapsel_gb300.build import build
    build()
    from icep_kapsel_gb300.runtime import Simulation
    return Simulation


def read_weight(n, h):
    """Weights of the half-spectrum modes in a Parseval inner product (2, 1 at
    self-conjugate points, 0 where the inverse transform does not read)."""
    i = np.arange(n)[:, None, None]
    j = np.arange(n)[None, :, None]
    kz = np.arange(h + 1)[None, None, :]
    w = np.full((n, n, h + 1), 2, dtype=np.int8)
    edge = (kz == 0) | (kz == h)
    selfc = (((n - i) % n) == i) & (((n - j) % n) == j)
    kept = np.where((j >= 1) & (j <= n // 2 - 1), True, np.where((j == 0) | (j == n // 2), i <= n // 2, False))
    kept = np.where(kz == h, ~kept, kept)
    w = np.where(edge & selfc, 1, np.where(edge & ~kept, 0, w))
    return np.broadcast_to(w, (n, n, h + 1))


def apply_b_fp64(ph, eps, n):
    h = n // 2
    wave = 2 * np.pi / n
    kint = np.where(np.arange(n) > n // 2, np.arange(n) - n, np.arange(n))
    ks = [kint[:, None, None] * wave, kint[None, :, None] * wave, np.arange(h + 1)[None, None, :] * wave]
    k2 = ks[0] ** 2 + ks[1] ** 2 + ks[2] ** 2
    eref = eps.mean()
    m = np.where(k2 > 0, -1.0 / (eref * np.where(k2 > 0, k2, 1.0)), 0.0)
    out = np.zeros((n, n, h + 1), complex)
    for d in range(3):
        sh = np.exp(0.5j * ks[d])
        w = np.fft.irfftn(m * 1j * ks[d] * sh * ph, s=(n, n, n), axes=(0, 1, 2))
        ef = 0.5 * (eps + np.roll(eps, -1, axis=d))
        out += 1j * ks[d] * np.conj(sh) * np.fft.rfftn(ef * w)
    return out


@pytest.mark.parametrize("n", [32, 64, 128, 256])
def test_fused_operator_against_fp64(Sim, n):
    """The fused operator B = A M^-1 against an FP64 restatement; 256^3 takes
    the split plane step (its x-plane does not fit in shared memory)."""
    p, parts = cases.icep_case(n=n, npart=max(4, n // 8), minsep=10.0, seed=7, eps_f=80.0, eps_p=2.0,
                               e_ext=(0.0, 0.0, 0.1), tol=1e-8, solver=abi.SOLVER_SPECTRAL,
                               precision=abi.MIXED)
    s = Sim(p, parts)
    s.call("dielectric_field")
    eps = s.get("eps")[:, :, :n]
    assert eps.min() < 10 and eps.max() > 70
    rng = np.random.default_rng(n)
    ph = np.fft.rfftn(rng.standard_normal((n, n, n)))
    buf = np.zeros((n, n, n + 2))
    buf[:, :, 0::2] = ph.real
    buf[:, :, 1::2] = ph.imag
    s.set("wv1", buf)
    s.call("apply_bk")
    got = s.get("work")
    gh = got[:, :, 0::2] + 1j * got[:, :, 1::2]
    ref = apply_b_fp64(ph, eps, n)
    wt = read_weight(n, n // 2)
    d2 = np.where(wt == 2, np.abs(gh - ref) ** 2, 0.0) + np.where(wt == 1, (gh.real - ref.real) ** 2, 0.0)
    r2 = np.where(wt == 2, np.abs(ref) ** 2, 0.0) + np.where(wt == 1, ref.real ** 2, 0.0)
    err = float(np.sqrt(d2.sum() / r2.sum()))
    assert err < 2e-5, err
    s.close()


def read_weight3(nx, ny, h):
    """read_weight on an nx x ny x (h+1) half spectrum (NX != NY allowed)."""
    i = np.arange(nx)[:, None, None]
    j = np.arange(ny)[None, :, None]
    kz = np.arange(h + 1)[None, None, :]
    w = np.full((nx, ny, h + 1), 2, dtype=np.int8)
    edge = (kz == 0) | (kz == h)
    selfc = (((nx - i) % nx) == i) & (((ny - j) % ny) == j)
    kept = np.where((j >= 1) & (j <= ny // 2 - 1), True, np.where((j == 0) | (j == ny // 2), i <= nx // 2, False))
    kept = np.where(kz == h, ~kept, kept)
    w = np.where(edge & selfc, 1, np.where(edge & ~kept, 0, w))
    return np.broadcast_to(w, (nx, ny, h + 1))


def apply_b_fp64_3(ph, eps, shape):
    """apply_b_fp64 on an (nx, ny, nz) mesh."""
    ns = shape
    ks = []
    for d, n in enumerate(ns):
        kint = np.arange(n // 2 + 1) if d == 2 else np.where(np.arange(n) > n // 2, np.arange(n) - n, np.arange(n))
        sh = [1, 1, 1]
        sh[d] = -1
        ks.append((kint * 2 * np.pi / n).reshape(sh))
    k2 = ks[0] ** 2 + ks[1] ** 2 + ks[2] ** 2
    m = np.where(k2 > 0, -1.0 / (eps.mean() * np.where(k2 > 0, k2, 1.0)), 0.0)
    out = np.zeros(ph.shape, complex)
    for d in range(3):
        sh = np.exp(0.5j * ks[d])
        w = np.fft.irfftn(m * 1j * ks[d] * sh * ph, s=ns, axes=(0, 1, 2))
        ef = 0.5 * (eps + np.roll(eps, -1, axis=d))
        out += 1j * ks[d] * np.conj(sh) * np.fft.rfftn(ef * w)
    return out


@pytest.mark.parametrize("shape", [(32, 64, 128), (128, 32, 64), (64, 256, 128), (128, 64, 256)])
def test_fused_operator_noncubic(Sim, shape):
    """The fused operator on meshes whose edges differ: the y and z gradient
    and divergence factors of the plane pass index the y and z wavenumbers
    of their own edges (32 x 64 x 128: the register plane kernel, NY = 64,
    NZ/2 = 64; 128 x 32 x 64: the shared-memory one; 64 x 256 x 128 and
    128 x 64 x 256: the split plane step, whose factor kernels index the
    half spectrum's rows and columns). Against the FP64 restatement, 2e-5
    relative L2."""
    nx, ny, nz = shape
    p, parts = cases.icep_case(n=32, npart=4, minsep=10.0, seed=9, eps_f=80.0, eps_p=2.0,
                               e_ext=(0.0, 0.0, 0.1), tol=1e-8, solver=abi.SOLVER_SPECTRAL, precision=abi.MIXED)
    p.nx, p.ny, p.nz = nx, ny, nz
    s = Sim(p, parts)
    s.call("dielectric_field")
    eps = s.get("eps")[:, :, :nz]
    assert eps.min() < 10 and eps.max() > 70
    rng = np.random.default_rng(nx + 3 * ny + 7 * nz)
    ph = np.fft.rfftn(rng.standard_normal((nx, ny, nz)))
    buf = np.zeros((nx, ny, nz + 2))
    buf[:, :, 0::2] = ph.real
    buf[:, :, 1::2] = ph.imag
    s.set("wv1", buf)
    s.call("apply_bk")
    got = s.get("work")
    gh = got[:, :, 0::2] + 1j * got[:, :, 1::2]
    ref = apply_b_fp64_3(ph, eps, shape)
    wt = read_weight3(nx, ny, nz // 2)
    d2 = np.where(wt == 2, np.abs(gh - ref) ** 2, 0.0) + np.where(wt == 1, (gh.real - ref.real) ** 2, 0.0)
    r2 = np.where(wt == 2, np.abs(ref) ** 2, 0.0) + np.where(wt == 1, ref.real ** 2, 0.0)
    err = float(np.sqrt(d2.sum() / r2.sum()))
    assert err < 2e-5, err
    s.close()


def test_bounded_wait_plane_pass(Sim):
    p, parts = cases.icep_case(n=64, npart=8, minsep=10.0, seed=5, eps_f=80.0, eps_p=2.0, e_ext=(0.0, 0.0, 0.1),
                               tol=1e-8, solver=abi.SOLVER_SPECTRAL, precision=abi.MIXED)
    s = Sim(p, parts)
    s.init_state()
    st, msg = s.selftest_wait(1)
    assert st == ICEP_ERR_TIMEOUT, (st, msg)
    assert "bounded wait" in msg
    s.step(2)  # the context stays usable: the next solve converges
    _, err, _ = s.solver_stats()
    assert err <= 1e-8
    assert np.isfinite(s.get("zeta0")).all()
    s.close()


def test_bounded_wait_convolution(Sim):
    p, parts = cases.icep_case(n=32, npart=4, minsep=10.0, seed=6, eps_f=80.0, eps_p=2.0, e_ext=(0.0, 0.0, 0.1),
                               tol=1e-8, solver=abi.SOLVER_LEARNED, precision=abi.MIXED)
    s = Sim(p, parts)
    s.init_state()
    st, msg = s.selftest_wait(2)
    assert st == ICEP_ERR_TIMEOUT, (st, msg)
    s.step(1)
    _, err, _ = s.solver_stats()
    assert err <= 1e-8
    s.close()


def expected_pick(t):
    """The x-pass pick from the times of 8, 16, 32 pencils per block: the
    default 16 unless a candidate is more than 3% faster; then the fastest."""
    b = 1
    for c in range(3):
        if 0 < t[c] < 0.97 * t[1] and t[c] < t[b]:
            b = c
    return (8, 16, 32)[b]


def test_autotune_picks_and_every_tile_shape(Sim, monkeypatch):
    """The tile autotuner times every candidate at context creation and keeps
    the default x tiles unless a candidate is clearly faster, and the faster
    plane kernel; every candidate tile shape computes the same operator
    (ICEP_KOP_TILES sets the tiles for a context)."""
    p, parts = cases.icep_case(n=64, npart=8, minsep=10.0, seed=7, eps_f=80.0, eps_p=2.0, e_ext=(0.0, 0.0, 0.1),
                               tol=1e-8, solver=abi.SOLVER_SPECTRAL, precision=abi.MIXED)
    s = Sim(p, parts)
    picks, us = s.autotune_picks()
    assert picks[0] in (8, 16, 32) and picks[1] in (8, 16, 32) and picks[2] in (0, 1)
    assert np.all(us[:6] > 0) and us[6] > 0 and us[7] > 0
    assert picks[0] == expected_pick(us[0:3]) and picks[1] == expected_pick(us[3:6])
    assert picks[2] == (0 if us[6] <= us[7] else 1)
    s.close()
    rng = np.random.default_rng(3)
    ph = np.fft.rfftn(rng.standard_normal((64, 64, 64)))
    buf = np.zeros((64, 64, 66))
    buf[:, :, 0::2] = ph.real
    buf[:, :, 1::2] = ph.imag
    outs = []
    for tiles in ("8,8,0", "16,16,1", "32,32,0", "16,32,1"):
        monkeypatch.setenv("ICEP_KOP_TILES", tiles)
        q = Sim(p, parts)
        q.call("dielectric_field")
        q.set("wv1", buf)
        q.call("apply_bk")
        outs.append(q.get("work"))
        q.close()
    wt = read_weight(64, 32)
    for o in outs[1:]:
        a = o[:, :, 0::2] + 1j * o[:, :, 1::2]
        b = outs[0][:, :, 0::2] + 1j * outs[0][:, :, 1::2]
        d = np.where(wt > 0, np.abs(a - b), 0.0)
        assert float(np.linalg.norm(d) / np.linalg.norm(np.where(wt > 0, np.abs(b), 0.0))) < 2e-6


@pytest.mark.parametrize("n", [64, 128])
def test_register_plane_fft_against_fp64(Sim, n):
    """The plain FP32 3D transforms of a MIXED context run their plane pass on
    the register-resident kernels (R2C: z rows forward, split, y forward; C2R:
    y inverse with the Hermitian completion, z rows inverse): both against the
    FP64 context's transforms of the same field, to FP32 accuracy, and the
    round trip."""
    pm, xm = cases.icep_case(n=n, npart=4, minsep=12.0, seed=3, precision=abi.MIXED,
                             solver=abi.SOLVER_SPECTRAL)
    pd, xd = cases.icep_case(n=n, npart=4, minsep=12.0, seed=3, precision=abi.FP64,
                             solver=abi.SOLVER_SPECTRAL)
    m, d = Sim(pm, xm), Sim(pd, xd)
    rng = np.random.default_rng(n)
    a = np.zeros((n, n, n + 2))
    a[:, :, :n] = rng.standard_normal((n, n, n))
    fm, fd = m.fft_r2c(a.copy()), d.fft_r2c(a.copy())
    err = np.linalg.norm(fm - fd) / np.linalg.norm(fd)
    assert err < 2e-6, err
    bm, bd = m.fft_c2r(fd.copy()), d.fft_c2r(fd.copy())
    err = np.linalg.norm(bm[:, :, :n] - bd[:, :, :n]) / np.linalg.norm(bd[:, :, :n])
    assert err < 2e-6, err
    assert np.abs(bm[:, :, n:]).max() == 0.0  # the padding of the real rows
    back = m.fft_c2r(m.fft_r2c(a.copy()))
    assert np.linalg.norm(back[:, :, :n] - a[:, :, :n]) / np.linalg.norm(a) < 2e-6
    m.close()
    d.close()
