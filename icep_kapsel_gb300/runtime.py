"""Python handle on the GB300 library (ctypes over include/icep_gb300.h).

The host-side mirror of the reference's entry points: a Simulation owns one
icep_ctx (one GPU context, one CUDA stream) and exposes the same calls as the
reference's Time_evolution / phase functions, with fields exchanged as
numpy arrays in the reference layout [NX][NY][NZ_].

There is no CPU fallback: constructing a Simulation without the compiled
library or without a CUDA device raises.
"""
import ctypes as C
import os

import numpy as np

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libicep_gb300.so")

FIELDS = ["zeta0", "zeta1", "u0", "u1", "u2", "up0", "up1", "up2", "phi", "phi_sum",
          "f0", "f1", "f2", "pot", "eps", "ge0", "ge1", "ge2", "c0", "c1", "rho", "work",
          "sn0", "sn1", "sn2", "ns0_0", "ns0_1", "ns1_0", "ns1_1", "crhs0", "crhs1",
          "wv1", "wv3_0", "wv3_1", "wv3_2"]
FIELD_ID = {n: i for i, n in enumerate(FIELDS)}
CALLS = ["zeta_k2u_k", "u_k2zeta_k", "u2advection_k", "solenoidal_u", "ns_slaved_euler",
         "make_phi_sum", "make_u_sum", "f_hydro", "lj", "pos_euler", "pos_ab2", "vel_euler",
         "vel_ab2", "dielectric_field", "build_rhs", "solve_potential", "maxwell",
         "nssolute_euler", "surface_normal", "f_particle_sole", "truncate", "charge_field",
         "init_ion", "zeta_k2u"]
CALL_ID = {n: i + 1 for i, n in enumerate(CALLS)}
CALL_ID["apply_bk"] = 26  # MIXED: WORK = B WV1 through the fused k-space passes (25: the checkers' field output)

_DP = C.POINTER(C.c_double)
_lib = None


class IcepError(RuntimeError):
    pass


def _dp(a):
    return a.ctypes.data_as(_DP)


def load_library(path=None):
    """Load (once) and type the C-ABI library; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise IcepError("GPU library not built: %s (run icep_kapsel_gb300.build)" % path)
    L = C.CDLL(path)
    V = C.c_void_p
    I = C.c_int
    L.icep_create.restype = V
    L.icep_create.argtypes = [V, V, I, C.POINTER(I)]
    L.icep_destroy.argtypes = [V]
    L.icep_last_error.restype = C.c_char_p
    L.icep_last_error.argtypes = [V]
    for fn in ("icep_init_state", "icep_synchronize", "icep_NS_solver_slavedEuler",
               "icep_NSsolute_solver_Euler", "icep_Make_phi_particle_sum", "icep_Make_u_particle_sum",
               "icep_Make_surface_normal", "icep_Calc_f_hydro_correct_precision",
               "icep_Calc_f_Lennard_Jones", "icep_Make_dielectric_field", "icep_Conc_k2charge_field",
               "icep_Build_rhs", "icep_Make_Maxwell_force_x_on_fluid"):
        getattr(L, fn).argtypes = [V]
    L.icep_step.argtypes = [V, I]
    L.icep_call.argtypes = [V, I]
    L.icep_get_field.argtypes = [V, I, _DP]
    L.icep_set_field.argtypes = [V, I, _DP]
    L.icep_get_particles.argtypes = [V, V]
    L.icep_set_particles.argtypes = [V, V]
    L.icep_get_uk_dc.argtypes = [V, _DP]
    L.icep_set_uk_dc.argtypes = [V, _DP]
    L.icep_get_time.argtypes = [V, C.POINTER(I), _DP]
    L.icep_set_time.argtypes = [V, I, C.c_double]
    L.icep_save_checkpoint.argtypes = [V, C.c_char_p]
    L.icep_udf_read.argtypes = [C.c_char_p, V, V, I, C.POINTER(I), C.POINTER(I), C.POINTER(I), C.c_char_p, I]
    L.icep_udf_value.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, I]
    L.icep_load_checkpoint.argtypes = [V, C.c_char_p]
    L.icep_A2a_k.argtypes = [V, _DP]
    L.icep_A_k2a.argtypes = [V, _DP]
    L.icep_Ax.argtypes = [V, _DP, _DP]
    L.icep_lj_pairs.argtypes = [V, C.POINTER(I), I, C.POINTER(I)]
    L.icep_MD_solver_position.argtypes = [V, I]
    L.icep_MD_solver_velocity.argtypes = [V, I]
    L.icep_Charge_field2potential_dielectric.argtypes = [V, C.POINTER(I), _DP]
    L.icep_solver_stats.argtypes = [V, C.POINTER(I), _DP, C.POINTER(C.c_long)]
    L.icep_step_graphs.argtypes = [V, C.POINTER(C.c_long)]
    L.icep_time_evolution.argtypes = [V, _DP, _DP, _DP, _DP, _DP, _DP, V, I]
    L.icep_stream.restype = V
    L.icep_stream.argtypes = [V]
    L.icep_batch_create.restype = V
    L.icep_batch_create.argtypes = [I, V, V, C.POINTER(I)]
    L.icep_batch_destroy.argtypes = [V]
    L.icep_batch_size.argtypes = [V]
    L.icep_batch_context.restype = V
    L.icep_batch_context.argtypes = [V, I]
    L.icep_batch_last_error.restype = C.c_char_p
    L.icep_batch_last_error.argtypes = [V]
    L.icep_batch_init_state.argtypes = [V]
    L.icep_batch_step.argtypes = [V, I]
    L.icep_learned_train.argtypes = [V, I, I, C.c_uint, C.c_double, _DP, _DP]
    L.icep_learned_enable.argtypes = [V, I]
    L.icep_learned_eval.argtypes = [V, I, _DP, _DP]
    L.icep_learned_nparams.restype = C.c_long
    L.icep_learned_nparams.argtypes = [V]
    L.icep_learned_get_params.argtypes = [V, _DP]
    L.icep_learned_set_params.argtypes = [V, _DP]
    L.icep_learned_forward.argtypes = [V, _DP, _DP, C.c_double, _DP]
    L.icep_learned_backward.argtypes = [V, _DP, _DP]
    L.icep_learned_stats.argtypes = [V, C.POINTER(I), C.POINTER(I)]
    L.icep_selftest_wait.argtypes = [V, I]
    L.icep_autotune_picks.argtypes = [V, C.POINTER(I), _DP]
    _lib = L
    return L



def udf_read(path):
    """Parameters, initial particles, GTS and Num_snap of a kapsel input UDF
    file (icep_udf_read; no GPU needed)."""
    L = load_library()
    p = abi.Params()
    n, gts, nsnap = C.c_int(), C.c_int(), C.c_int()
    err = C.create_string_buffer(512)
    st = L.icep_udf_read(os.fsencode(path), C.byref(p), None, 0, C.byref(n), C.byref(gts), C.byref(nsnap), err, 512)
    if st:
        raise IcepError("icep_udf_read failed (%d): %s" % (st, err.value.decode()))
    parts = (abi.Particle * max(n.value, 1))()
    st = L.icep_udf_read(os.fsencode(path), C.byref(p), parts, n.value, C.byref(n), C.byref(gts), C.byref(nsnap),
                         err, 512)
    if st:
        raise IcepError("icep_udf_read failed (%d): %s" % (st, err.value.decode()))
    return p, parts, gts.value, nsnap.value


def udf_value(path, key):
    """The text of one value of a UDF file by its dotted path (icep_udf_value)."""
    L = load_library()
    buf = C.create_string_buffer(4096)
    st = L.icep_udf_value(os.fsencode(path), key.encode(), buf, 4096)
    if st:
        raise IcepError("icep_udf_value failed (%d): %s" % (st, buf.value.decode()))
    return buf.value.decode()

class Simulation:
    """One ICEP simulation on the GPU (see include/icep_gb300.h)."""

    def __init__(self, params, particles):
        self.lib = load_library()
        self.params = params
        self.np = params.n_particles
        st = C.c_int(0)
        self.ctx = self.lib.icep_create(C.byref(params), particles, self.np, C.byref(st))
        if not self.ctx:
            raise IcepError("icep_create failed with status %d" % st.value)

    def close(self):
        if getattr(self, "ctx", None) and getattr(self, "_owned", True):
            self.lib.icep_destroy(self.ctx)
        self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st, what):
        if st != 0:
            msg = self.lib.icep_last_error(self.ctx)
            raise IcepError("%s failed (%d): %s" % (what, st, msg.decode() if msg else ""))

    def _shape(self):
        p = self.params
        return (p.nx, p.ny, 2 * (p.nz // 2 + 1))

    # state
    def init_state(self):
        self._check(self.lib.icep_init_state(self.ctx), "init_state")

    def step(self, n=1):
        self._check(self.lib.icep_step(self.ctx, n), "step")

    def synchronize(self):
        self._check(self.lib.icep_synchronize(self.ctx), "synchronize")

    def get(self, name):
        out = np.zeros(self._shape(), dtype=np.float64)
        self._check(self.lib.icep_get_field(self.ctx, FIELD_ID[name], _dp(out)), "get " + name)
        return out

    def set(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(self._shape())
        self._check(self.lib.icep_set_field(self.ctx, FIELD_ID[name], _dp(a)), "set " + name)

    def call(self, name):
        self._check(self.lib.icep_call(self.ctx, CALL_ID[name]), name)

    def autotune_picks(self):
        """The tile autotuner's picks (xinv pencils per block, xfwd pencils per
        block, plane kernel 0 register / 1 shared memory) and its timings (us
        per launch: xinv 8/16/32, xfwd 8/16/32, plane register/shared)."""
        picks = (C.c_int * 3)()
        us = np.zeros(8)
        self._check(self.lib.icep_autotune_picks(self.ctx, picks, _dp(us)), "autotune_picks")
        return list(picks), us

    def selftest_wait(self, kernel):
        """icep_selftest_wait: the status (ICEP_ERR_TIMEOUT expected) and the
        error text of a kernel launched so that its bounded wait runs out."""
        st = self.lib.icep_selftest_wait(self.ctx, int(kernel))
        msg = self.lib.icep_last_error(self.ctx)
        return st, (msg.decode() if msg else "")

    def particles(self):
        arr = (abi.Particle * max(self.np, 1))()
        self._check(self.lib.icep_get_particles(self.ctx, arr), "get_particles")
        return arr

    def set_particles(self, arr):
        self._check(self.lib.icep_set_particles(self.ctx, arr), "set_particles")

    def uk_dc(self):
        o = np.zeros(3)
        self._check(self.lib.icep_get_uk_dc(self.ctx, _dp(o)), "get_uk_dc")
        return o

    def set_uk_dc(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        self._check(self.lib.icep_set_uk_dc(self.ctx, _dp(v)), "set_uk_dc")

    def set_ts(self, ts, time):
        self._check(self.lib.icep_set_time(self.ctx, ts, time), "set_time")

    def time(self):
        ts, t = C.c_int(), C.c_double()
        self._check(self.lib.icep_get_time(self.ctx, C.byref(ts), C.byref(t)), "get_time")
        return ts.value, t.value

    def save_checkpoint(self, path):
        """Write the step state (Save_Restart_udf + potential) to `path`."""
        self._check(self.lib.icep_save_checkpoint(self.ctx, os.fsencode(path)), "save_checkpoint")

    def load_checkpoint(self, path):
        """Restore the step state written by save_checkpoint."""
        self._check(self.lib.icep_load_checkpoint(self.ctx, os.fsencode(path)), "load_checkpoint")

    OUTPUT_FIELDS = ("u0", "u1", "u2", "phi", "surface_charge", "solute_charge", "potential", "epsilon")

    def charge_field_data(self):
        """The fields of Output_dielectric_charge_field_data (icep_charge_field_data)
        as a dict of [NX][NY][NZ_] arrays."""
        out = {k: np.zeros(self._shape(), dtype=np.float64) for k in self.OUTPUT_FIELDS}
        self._check(self.lib.icep_charge_field_data(self.ctx, *[_dp(out[k]) for k in self.OUTPUT_FIELDS]),
                    "charge_field_data")
        return out

    def output_avs(self, out_dir, name, ascii=False):
        """One AVS frame of the current state (icep_output_avs); call
        avs_init(out_dir, name, ...) once before the first frame."""
        self._check(self.lib.icep_output_avs(self.ctx, os.fsencode(out_dir), os.fsencode(name), int(ascii)),
                    "output_avs")

    def avs_init(self, out_dir, name, nstep, ascii=False):
        """The AVS headers for this context's mesh (icep_avs_init)."""
        p = self.params
        st = self.lib.icep_avs_init(os.fsencode(out_dir), os.fsencode(name), int(ascii), p.nx, p.ny, p.nz,
                                    C.c_double(p.dx), int(nstep), p.n_particles)
        if st:
            raise IcepError("avs_init failed (%d)" % st)

    # reference-named phases
    def fft_r2c(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64).copy()
        self._check(self.lib.icep_A2a_k(self.ctx, _dp(a)), "A2a_k")
        return a

    def fft_c2r(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64).copy()
        self._check(self.lib.icep_A_k2a(self.ctx, _dp(a)), "A_k2a")
        return a

    def apply_A(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        self._check(self.lib.icep_Ax(self.ctx, _dp(x), _dp(y)), "Ax")
        return y

    def solve_potential(self):
        it = C.c_int(0)
        er = C.c_double(0)
        self._check(self.lib.icep_Charge_field2potential_dielectric(self.ctx, C.byref(it), C.byref(er)),
                    "Charge_field2potential_dielectric")
        return it.value, er.value

    def solver_stats(self):
        it = C.c_int(0)
        er = C.c_double(0)
        mv = C.c_long(0)
        self._check(self.lib.icep_solver_stats(self.ctx, C.byref(it), C.byref(er), C.byref(mv)), "stats")
        return it.value, er.value, mv.value

    def step_graphs(self):
        """Steps taken as one CUDA graph so far (icep_step_graphs)."""
        n = C.c_long(0)
        self._check(self.lib.icep_step_graphs(self.ctx, C.byref(n)), "step_graphs")
        return n.value

    def last_iterations(self):
        return self.solver_stats()[0]

    def last_error(self):
        return self.solver_stats()[1]

    # learned preconditioner (solver LEARNED)
    def learned_train(self, configs, steps, seed=1, lr=1e-3):
        l0, l1 = C.c_double(0), C.c_double(0)
        self._check(self.lib.icep_learned_train(self.ctx, configs, steps, seed, lr, C.byref(l0), C.byref(l1)),
                    "learned_train")
        return l0.value, l1.value

    def learned_eval(self, chain=4):
        a, b = C.c_double(0), C.c_double(0)
        self._check(self.lib.icep_learned_eval(self.ctx, chain, C.byref(a), C.byref(b)), "learned_eval")
        return a.value, b.value

    def learned_enable(self, on):
        self._check(self.lib.icep_learned_enable(self.ctx, 1 if on else 0), "learned_enable")

    def learned_params(self):
        out = np.zeros(self.lib.icep_learned_nparams(self.ctx))
        self._check(self.lib.icep_learned_get_params(self.ctx, _dp(out)), "learned_get_params")
        return out

    def set_learned_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float64)
        self._check(self.lib.icep_learned_set_params(self.ctx, _dp(p)), "learned_set_params")

    def learned_forward(self, eps, r, eps_ref):
        """Network output on the half-resolution grid for fine real fields eps, r."""
        n = self.params.nx // 2
        y = np.zeros(n * n * n)
        e = np.ascontiguousarray(eps, dtype=np.float64).reshape(self._shape())
        rr = np.ascontiguousarray(r, dtype=np.float64).reshape(self._shape())
        self._check(self.lib.icep_learned_forward(self.ctx, _dp(e), _dp(rr), eps_ref, _dp(y)), "learned_forward")
        return y.reshape(n, n, n)

    def learned_backward(self, gy):
        g = np.zeros(self.lib.icep_learned_nparams(self.ctx))
        gy = np.ascontiguousarray(gy, dtype=np.float64)
        self._check(self.lib.icep_learned_backward(self.ctx, _dp(gy), _dp(g)), "learned_backward")
        return g

    def learned_stats(self):
        fb, ap = C.c_int(0), C.c_int(0)
        self._check(self.lib.icep_learned_stats(self.ctx, C.byref(fb), C.byref(ap)), "learned_stats")
        return fb.value, ap.value

    def lj_pairs(self, max_pairs=1 << 20):
        buf = np.zeros(2 * max_pairs, dtype=np.int32)
        n = C.c_int(0)
        self._check(self.lib.icep_lj_pairs(self.ctx, buf.ctypes.data_as(C.POINTER(C.c_int)), max_pairs,
                                           C.byref(n)), "lj_pairs")
        return buf[: 2 * min(n.value, max_pairs)].reshape(-1, 2)

    def time_evolution(self, zeta0, zeta1, uk_dc, particles, conc0=None, conc1=None, potential=None, nsteps=1):
        """The drop-in Time_evolution call on host arrays (updated in place)."""
        def ptr(a):
            return _dp(a) if a is not None else None
        self._check(self.lib.icep_time_evolution(self.ctx, _dp(zeta0), _dp(zeta1), _dp(uk_dc), ptr(conc0),
                                                 ptr(conc1), ptr(potential), particles, nsteps),
                    "time_evolution")


class Batch:
    """Independent replicas advanced together (icep_batch_*, include/icep_gb300.h).
    replica(i) gives a Simulation view on replica i's context."""

    def __init__(self, replicas):
        """replicas: list of (params, particles) pairs."""
        self.lib = load_library()
        n = len(replicas)
        self._params = (abi.Params * n)(*[p for p, _ in replicas])
        self._parts = [parts for _, parts in replicas]
        ptrs = (C.c_void_p * n)(*[C.addressof(pp) for pp in self._parts])
        st = C.c_int(0)
        self.handle = self.lib.icep_batch_create(n, self._params, ptrs, C.byref(st))
        if not self.handle:
            raise IcepError("icep_batch_create failed with status %d" % st.value)
        self.n = n

    def _check(self, st, what):
        if st != 0:
            msg = self.lib.icep_batch_last_error(self.handle)
            raise IcepError("%s failed (%d): %s" % (what, st, msg.decode() if msg else ""))

    def init_state(self):
        self._check(self.lib.icep_batch_init_state(self.handle), "batch_init_state")

    def step(self, n=1):
        self._check(self.lib.icep_batch_step(self.handle, n), "batch_step")

    def replica(self, i):
        v = Simulation.__new__(Simulation)
        v.lib = self.lib
        v.params = self._params[i]
        v.np = v.params.n_particles
        v.ctx = self.lib.icep_batch_context(self.handle, i)
        v._owned = False
        return v

    def close(self):
        if getattr(self, "handle", None):
            self.lib.icep_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

