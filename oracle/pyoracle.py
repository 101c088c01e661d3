"""Python handles on the two CPU checkers.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's cpu_baseline / reference legs, never by the product package.

  Oracle     -- oracle/liboracle.so, the C restatement (icep_oracle.c); builds
                anywhere gcc is present.
  RefKapsel  -- oracle/_ref/libkapsel_ref.so, the reference's own sources
                compiled by oracle/ref/Makefile; only where the reference
                tree was available at build time.

Both expose the same calls, so a script can run against either.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libkapsel_ref.so")

FIELDS = ["zeta0", "zeta1", "u0", "u1", "u2", "up0", "up1", "up2", "phi", "phi_sum",
          "f0", "f1", "f2", "pot", "eps", "ge0", "ge1", "ge2", "c0", "c1", "rho", "work",
          "sn0", "sn1", "sn2", "ns0_0", "ns0_1", "ns1_0", "ns1_1"]
FIELD_ID = {n: i for i, n in enumerate(FIELDS)}

CALLS = ["zeta_k2u_k", "u_k2zeta_k", "u2advection_k", "solenoidal_u", "ns_slaved_euler",
         "make_phi_sum", "make_u_sum", "f_hydro", "lj", "pos_euler", "pos_ab2", "vel_euler",
         "vel_ab2", "dielectric_field", "build_rhs", "solve_potential", "maxwell",
         "nssolute_euler", "surface_normal", "f_particle_sole", "truncate", "charge_field",
         "init_ion", "zeta_k2u", "charge_output"]
CALL_ID = {n: i + 1 for i, n in enumerate(CALLS)}

_DP = C.POINTER(C.c_double)


def _dp(a):
    return a.ctypes.data_as(_DP)


def build_oracle(force=False):
    """Compile oracle/liboracle.so with gcc (OpenMP, no FMA contraction)."""
    src = os.path.join(HERE, "icep_oracle.c")
    if not force and os.path.exists(ORACLE_SO) and os.path.getmtime(ORACLE_SO) >= os.path.getmtime(src):
        return ORACLE_SO
    tmp = ORACLE_SO + ".tmp"
    cmd = ["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
           "-o", tmp, src, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, ORACLE_SO)  # atomic: processes that loaded the old file keep it
    return ORACLE_SO


def ref_dir():
    """The reference source tree the checker is compiled from: the
    ICEP_REFERENCE_DIR environment variable, else the tree's location in the
    build container (absent on GPU hosts, where only the committed fixtures
    are used)."""
    return os.environ.get("ICEP_REFERENCE_DIR", "/root/reference")


def build_ref(ref_dir=None):
    """Build oracle/_ref/libkapsel_ref.so from the reference tree if present."""
    ref_dir = ref_dir or globals()["ref_dir"]()
    if not os.path.isdir(ref_dir):
        return None
    subprocess.check_call(["make", "-s", "-j8", "-C", os.path.join(HERE, "ref"), "REF=" + ref_dir])
    return REF_SO


class _Base:
    def _shape(self):
        p = self.params
        return (p.nx, p.ny, 2 * (p.nz // 2 + 1))

    def get(self, name):
        out = np.zeros(self._shape(), dtype=np.float64)
        rc = self._get_field(FIELD_ID[name], out)
        if rc:
            raise KeyError(name)
        return out

    def set(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(self._shape())
        rc = self._set_field(FIELD_ID[name], a)
        if rc:
            raise KeyError(name)

    def call(self, name):
        rc = self._call(CALL_ID[name])
        if rc:
            raise RuntimeError("call failed: " + name)


class Oracle(_Base):
    """The C restatement (one independent context per instance)."""

    def __init__(self, params, particles, so=None):
        self.lib = C.CDLL(so or build_oracle())
        L = self.lib
        L.ko_create.restype = C.c_void_p
        L.ko_create.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        for fn in ("ko_init_state", "ko_destroy"):
            getattr(L, fn).argtypes = [C.c_void_p]
        L.ko_step.argtypes = [C.c_void_p, C.c_int]
        L.ko_set_ts.argtypes = [C.c_void_p, C.c_int, C.c_double]
        L.ko_get_field.argtypes = [C.c_void_p, C.c_int, _DP]
        L.ko_set_field.argtypes = [C.c_void_p, C.c_int, _DP]
        L.ko_call.argtypes = [C.c_void_p, C.c_int]
        L.ko_a2a_k.argtypes = [C.c_void_p, _DP]
        L.ko_a_k2a.argtypes = [C.c_void_p, _DP]
        L.ko_apply_A.argtypes = [C.c_void_p, _DP, _DP]
        L.ko_get_particles.argtypes = [C.c_void_p, C.c_void_p]
        L.ko_set_particles.argtypes = [C.c_void_p, C.c_void_p]
        L.ko_get_uk_dc.argtypes = [C.c_void_p, _DP]
        L.ko_set_uk_dc.argtypes = [C.c_void_p, _DP]
        L.ko_last_iterations.restype = C.c_long
        L.ko_last_iterations.argtypes = [C.c_void_p]
        L.ko_pb_iterations.restype = C.c_long
        L.ko_pb_iterations.argtypes = [C.c_void_p]
        L.ko_last_error.restype = C.c_double
        L.ko_last_error.argtypes = [C.c_void_p]
        L.ko_matvec_count.restype = C.c_long
        L.ko_matvec_count.argtypes = [C.c_void_p]
        L.ko_set_potential_iter.argtypes = [C.c_void_p, C.c_int]
        L.ko_np_domain.argtypes = [C.c_void_p]
        L.ko_sekibun.argtypes = [C.c_void_p, C.POINTER(C.c_int)]
        L.ko_lj_pairs.restype = C.c_long
        L.ko_lj_pairs.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.c_long]
        self.params = params
        self.np = params.n_particles
        self.ctx = L.ko_create(C.byref(params), particles, self.np)
        if not self.ctx:
            raise RuntimeError("ko_create failed")

    def __del__(self):
        try:
            if self.ctx:
                self.lib.ko_destroy(self.ctx)
                self.ctx = None
        except Exception:
            pass

    def _get_field(self, i, out):
        return self.lib.ko_get_field(self.ctx, i, _dp(out))

    def _set_field(self, i, a):
        return self.lib.ko_set_field(self.ctx, i, _dp(a))

    def _call(self, i):
        return self.lib.ko_call(self.ctx, i)

    def init_state(self):
        self.lib.ko_init_state(self.ctx)

    def step(self, n=1):
        self.lib.ko_step(self.ctx, n)

    def set_ts(self, ts, time):
        self.lib.ko_set_ts(self.ctx, ts, time)

    def fft_r2c(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64).copy()
        self.lib.ko_a2a_k(self.ctx, _dp(a))
        return a

    def fft_c2r(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64).copy()
        self.lib.ko_a_k2a(self.ctx, _dp(a))
        return a

    def apply_A(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        self.lib.ko_apply_A(self.ctx, _dp(x), _dp(y))
        return y

    def particles(self):
        from icep_kapsel_gb300 import abi
        arr = (abi.Particle * max(self.np, 1))()
        self.lib.ko_get_particles(self.ctx, arr)
        return arr

    def set_particles(self, arr):
        self.lib.ko_set_particles(self.ctx, arr)

    def uk_dc(self):
        o = np.zeros(3)
        self.lib.ko_get_uk_dc(self.ctx, _dp(o))
        return o

    def set_uk_dc(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        self.lib.ko_set_uk_dc(self.ctx, _dp(v))

    def last_iterations(self):
        return self.lib.ko_last_iterations(self.ctx)

    def last_error(self):
        return self.lib.ko_last_error(self.ctx)

    def matvecs(self):
        return self.lib.ko_matvec_count(self.ctx)

    def pb_iterations(self):
        """Relaxation steps of the last Poisson-Boltzmann initialisation."""
        return self.lib.ko_pb_iterations(self.ctx)

    def set_potential_iter(self, maxit):
        self.lib.ko_set_potential_iter(self.ctx, int(maxit))

    def sekibun(self):
        n = self.lib.ko_np_domain(self.ctx)
        out = np.zeros((n, 3), dtype=np.int32)
        self.lib.ko_sekibun(self.ctx, out.ctypes.data_as(C.POINTER(C.c_int)))
        return out

    def lj_pairs(self, max_pairs=1 << 20):
        buf = np.zeros(2 * max_pairs, dtype=np.int32)
        n = self.lib.ko_lj_pairs(self.ctx, buf.ctypes.data_as(C.POINTER(C.c_int)), max_pairs)
        return buf[: 2 * min(n, max_pairs)].reshape(-1, 2)


class RefKapsel(_Base):
    """The reference's own object code (process-global state: one at a time)."""

    def __init__(self, params, particles, so=REF_SO):
        self.lib = C.CDLL(so)
        L = self.lib
        L.kref_setup.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        L.kref_get_field.argtypes = [C.c_int, _DP]
        L.kref_set_field.argtypes = [C.c_int, _DP]
        L.kref_call.argtypes = [C.c_int]
        L.kref_step.argtypes = [C.c_int]
        L.kref_set_ts.argtypes = [C.c_int, C.c_double]
        L.kref_a2a_k.argtypes = [_DP]
        L.kref_a_k2a.argtypes = [_DP]
        L.kref_apply_A.argtypes = [_DP, _DP]
        L.kref_get_particles.argtypes = [C.c_void_p]
        L.kref_set_particles.argtypes = [C.c_void_p]
        L.kref_get_uk_dc.argtypes = [_DP]
        L.kref_set_uk_dc.argtypes = [_DP]
        L.kref_last_iterations.restype = C.c_long
        L.kref_last_error.restype = C.c_double
        L.kref_matvec_count.restype = C.c_long
        L.kref_sekibun.argtypes = [C.POINTER(C.c_int)]
        if hasattr(L, "kref_avs"):
            L.kref_avs.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.POINTER(_DP)]
        self.params = params
        self.np = params.n_particles
        rc = L.kref_setup(C.byref(params), particles, self.np)
        if rc:
            raise RuntimeError("kref_setup failed")

    def _get_field(self, i, out):
        return self.lib.kref_get_field(i, _dp(out))

    def _set_field(self, i, a):
        return self.lib.kref_set_field(i, _dp(a))

    def _call(self, i):
        return self.lib.kref_call(i)

    def init_state(self):
        self.lib.kref_init_state()

    def step(self, n=1):
        self.lib.kref_step(n)

    def set_ts(self, ts, time):
        self.lib.kref_set_ts(ts, time)

    def fft_r2c(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64).copy()
        self.lib.kref_a2a_k(_dp(a))
        return a

    def fft_c2r(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64).copy()
        self.lib.kref_a_k2a(_dp(a))
        return a

    def apply_A(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        self.lib.kref_apply_A(_dp(x), _dp(y))
        return y

    def particles(self):
        from icep_kapsel_gb300 import abi
        arr = (abi.Particle * max(self.np, 1))()
        self.lib.kref_get_particles(arr)
        return arr

    def set_particles(self, arr):
        self.lib.kref_set_particles(arr)

    def uk_dc(self):
        o = np.zeros(3)
        self.lib.kref_get_uk_dc(_dp(o))
        return o

    def set_uk_dc(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        self.lib.kref_set_uk_dc(_dp(v))

    def last_iterations(self):
        return self.lib.kref_last_iterations()

    def last_error(self):
        return self.lib.kref_last_error()

    def matvecs(self):
        return self.lib.kref_matvec_count()

    def avs(self, out_dir, name, ascii, num_snap, fields):
        """The reference's AVS writers: headers and one frame of `fields`
        (7 arrays [NX][NY][NZ_]) and the particles, at the set ts and time."""
        arrs = [np.ascontiguousarray(f, dtype=np.float64) for f in fields]
        ptrs = (_DP * 7)(*[_dp(a) for a in arrs])
        st = self.lib.kref_avs(os.fsencode(out_dir), os.fsencode(name), int(ascii), int(num_snap), ptrs)
        if st:
            raise RuntimeError("kref_avs failed")

    def sekibun(self):
        n = self.lib.kref_np_domain()
        out = np.zeros((n, 3), dtype=np.int32)
        self.lib.kref_sekibun(out.ctypes.data_as(C.POINTER(C.c_int)))
        return out
