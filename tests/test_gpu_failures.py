"""Failure handling through the C-ABI, made on the host (no device fault):
a non-finite input stops the step with ICEP_ERR_NOT_CONVERGED and a message,
the context and the process stay usable; reaching MaxIter keeps the
reference's non-fatal semantics (operate_dielectric.cxx:563-570)."""
import numpy as np
import pytest

import cases
from icep_kapsel_gb300 import abi
from icep_kapsel_gb300.runtime import Simulation

pytestmark = pytest.mark.gpu

ERR_NOT_CONVERGED = 4


def case(**kw):
    args = dict(n=32, npart=4, seed=2, a=4.0, eps_f=80.0, eps_p=3.0, e_ext=(0.0, 0.0, 0.1), tol=1e-8, maxit=1000,
                solver=abi.SOLVER_SPECTRAL, precision=abi.MIXED)
    args.update(kw)
    return cases.icep_case(**args)


@pytest.mark.parametrize("precision", [abi.MIXED, abi.FP64])
def test_non_finite_input_is_reported(precision):
    p, parts = case(precision=precision)
    s = Simulation(p, parts)
    s.init_state()
    c0 = s.get("c0")
    c0[3, 4, 0] = np.nan
    s.set("c0", c0)
    st = s.lib.icep_step(s.ctx, 1)
    assert st == ERR_NOT_CONVERGED
    assert b"non-finite" in s.lib.icep_last_error(s.ctx)
    s.get("phi")  # the context still answers
    s.close()
    q = Simulation(*case(precision=precision))  # and a new one steps normally
    q.init_state()
    q.step(1)
    assert np.isfinite(q.get("zeta0")).all()


def test_max_iterations_is_not_fatal():
    p, parts = case(solver=abi.SOLVER_REF, precision=abi.FP64, maxit=2)
    s = Simulation(p, parts)
    s.init_state()
    s.step(1)  # both attempts stop at MaxIter; the step completes
    it, err, _ = s.solver_stats()
    assert it == 2 and err > 1e-8
