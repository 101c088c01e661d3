"""The learned Poisson preconditioner on the GPU (solver LEARNED, MIXED).

* The network's forward values and parameter gradients against the CPU
  oracle (oracle/unet_ref.py). The GPU keeps tensor-core weights,
  activations and the gradients fed to convolutions in BF16 (FP32
  accumulation). Against the oracle rounding at the same points: 5e-3
  (relative L2) on the output, 2e-2 per layer on the gradients; against the
  plain FP64 oracle: 3e-2 on the output.
* A solve with the learned preconditioner reaches the same FP64 true
  residual as the plain solver and gives the same fields within the MIXED
  tolerances; the trained correction does not raise the one-step loss of the
  spectral preconditioner. The iteration counts of the flexible
  GMRES with and without the network and of the plain BiCGSTAB are printed
  (run with -s to see them).
"""
import numpy as np
import pytest

import cases
import unet_ref as U
from icep_kapsel_gb300 import abi

pytestmark = pytest.mark.gpu


def rel(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / (nb if nb > 0 else 1.0))


def learned_case(n=32, npart=4, seed=2, solver=abi.SOLVER_LEARNED, tol=1e-8):
    return cases.icep_case(n=n, npart=npart, minsep=12.0, seed=seed, a=4.0, eps_f=80.0, eps_p=3.0,
                           e_ext=(0.0, 0.0, 0.1), tol=tol, maxit=1000, dt=0.01, per_particle_eps=(1.0, 5.0),
                           solver=solver, precision=abi.MIXED)


def test_network_against_oracle():
    from icep_kapsel_gb300.runtime import Simulation
    p, parts = learned_case()
    s = Simulation(p, parts)
    s.init_state()
    nz = p.nz
    eps = s.get("eps")
    rng = np.random.default_rng(7)
    r = np.zeros_like(eps)
    r[:, :, :nz] = rng.standard_normal((p.nx, p.ny, nz))
    eref = float(eps[:, :, :nz].mean())
    params = s.learned_params()
    params += 0.05 * rng.standard_normal(params.size)  # non-zero biases too
    s.set_learned_params(params)
    y = s.learned_forward(eps, r, eref)
    x, _ = U.network_input(eps[:, :, :nz], r[:, :, :nz], eref)
    y64, _ = U.forward(params, x)
    assert rel(y, y64) < 3e-2
    yo, cache = U.forward(params, x, emulate=True)
    assert rel(y, yo) < 5e-3
    gy = rng.standard_normal(y.shape)
    g = s.learned_backward(gy)
    go = U.backward(params, cache, gy)
    go64 = U.backward(params, U.forward(params, x)[1], gy)
    off, _ = U.param_offsets()
    for name, ci, co in U.LAYERS:
        w0, b0, _, _ = off[name]
        # bound: 2e-2, or twice what BF16 rounding alone changes the oracle's
        # own gradient (the first layer's gradient is a long cancelling sum
        # behind every rounded gradient of the backward chain)
        tw = max(2e-2, 2 * rel(go[w0:b0], go64[w0:b0]))
        tb = max(2e-2, 2 * rel(go[b0:b0 + co], go64[b0:b0 + co]))
        assert rel(g[w0:b0], go[w0:b0]) < tw, name
        assert rel(g[b0:b0 + co], go[b0:b0 + co]) < tb, name + " bias"


def test_learned_solve_matches_plain():
    from icep_kapsel_gb300.runtime import Simulation
    p0, parts0 = learned_case(n=64, npart=24, seed=5, solver=abi.SOLVER_SPECTRAL)
    plain = Simulation(p0, parts0)
    plain.init_state()
    p1, parts1 = learned_case(n=64, npart=24, seed=5)
    lrn = Simulation(p1, parts1)
    lrn.init_state()  # flexible GMRES with the spectral preconditioner only (untrained network)
    it_fg0 = lrn.solver_stats()[0]
    ls0, ll0 = lrn.learned_eval(4)
    l0, l1 = lrn.learned_train(configs=6, steps=40, seed=11, lr=1e-3)
    assert np.isfinite(l1)
    ls1, ll1 = lrn.learned_eval(4)
    print("\none-step loss on the context's residuals: spectral %.4f, learned before %.4f after %.4f"
          % (ls1, ll0, ll1))
    # training keeps its parameters only when they lower the one-step loss on
    # these residuals (the context's own, not trained on) below the spectral
    # preconditioner's: the learned preconditioner is never worse here
    assert ll1 <= ls1
    plain.step(3)
    lrn.step(3)
    it_plain, err_plain, _ = plain.solver_stats()
    it_lrn, err_lrn, _ = lrn.solver_stats()
    fb, apps = lrn.learned_stats()
    print("\nplain BiCGSTAB iterations %d (err %.2e); flexible GMRES spectral-only at init %d; "
          "learned %d (err %.2e, %d network applications, %d fallbacks); training loss %.3e -> %.3e"
          % (it_plain, err_plain, it_fg0, it_lrn, err_lrn, apps, fb, l0, l1))
    assert err_lrn <= 1e-8 and err_plain <= 1e-8
    nz = p0.nz
    for name in ("zeta0", "zeta1", "phi"):
        assert rel(lrn.get(name), plain.get(name)) < 2e-5, name
    a, b = lrn.get("pot")[:, :, :nz], plain.get("pot")[:, :, :nz]
    assert rel(a - a.mean(), b - b.mean()) < 2e-5
