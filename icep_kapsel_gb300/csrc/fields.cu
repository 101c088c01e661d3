// fields.cu -- grid-field kernels (see fields.cuh for the reference mapping).
#include "fields.cuh"

namespace icep {

namespace {

constexpr int TPB = 256;

struct Mode {
  int i, j, kz;
  long im;  // index of the real part
};

// Grids hold at most 2^24 points, so 32-bit index arithmetic suffices.
__device__ __forceinline__ bool mode_of(const Grid &g, long tl, Mode &m) {
  if (tl >= g.nmodes()) return false;
  mode_ijk3(g, (unsigned)tl, m.i, m.j, m.kz);
  m.im = gidx(g, m.i, m.j, 2 * m.kz);
  return true;
}

struct Pt {
  int i, j, k;
  long im;
};

__device__ __forceinline__ bool pt_of(const Grid &g, long tl, Pt &p) {
  if (tl >= g.nreal()) return false;
  real_ijk(g, (unsigned)tl, p.i, p.j, p.k);
  p.im = gidx(g, p.i, p.j, p.k);
  return true;
}

// periodic wrap (mesh sizes are powers of two)
__device__ __forceinline__ long wrapi(const Grid &g, int i, int j, int k) {
  i &= g.nx - 1;
  j &= g.ny - 1;
  k &= g.nz - 1;
  return gidx(g, i, j, k);
}

template <typename R>
__device__ __forceinline__ void kvec(const Grid &g, const Mode &m, R *k) {
  k[0] = wave_of<R>(g, 0) * (R)kx_of(g, m.i);
  k[1] = wave_of<R>(g, 1) * (R)ky_of(g, m.j);
  k[2] = wave_of<R>(g, 2) * (R)m.kz;
}

template <typename R>
__device__ __forceinline__ R k2_of(const R *k) { return k[0] * k[0] + k[1] * k[1] + k[2] * k[2]; }

__device__ __forceinline__ double exp_t(double a) { return exp(a); }
__device__ __forceinline__ float exp_t(float a) { return expf(a); }

#define TID ((long)blockIdx.x * blockDim.x + threadIdx.x)

// three component fields passed by value
template <typename R>
struct V3 {
  R *p[3];
};

// ---------------------------------------------------------------- k-space
template <typename R>
__global__ void k_truncate(FieldBatch<R> fb, Grid g) {
  Mode m;
  if (!mode_of(g, TID, m)) return;
  if (in_two_third(g, m.i, m.j, m.kz)) return;
  R *a = fb.p[blockIdx.y];
  a[m.im] = R(0);
  a[m.im + 1] = R(0);
}

// u(k) of one mode from its two stored vorticity components (a, b):
// v[0..5] = u0 re, im, u1 re, im, u2 re, im
template <typename R>
__device__ __forceinline__ void zeta_mode_to_u(const Grid &g, const Mode &m, R a_r, R a_i, R b_r, R b_i, R *v) {
  const int KX = kx_of(g, m.i), KY = ky_of(g, m.j);
  R kx = wave_of<R>(g, 0) * (R)KX, ky = wave_of<R>(g, 1) * (R)KY, kz = wave_of<R>(g, 2) * (R)m.kz;
  const R k2 = kx * kx + ky * ky + kz * kz;
  const R ik2 = (k2 > R(0)) ? R(1) / k2 : R(0);
  R wr0, wi0, wr1, wi1, wr2, wi2;
  if (KX != 0) {
    const R ikx = R(1) / kx;
    wr0 = -ikx * (ky * a_r + kz * b_r);
    wi0 = -ikx * (ky * a_i + kz * b_i);
    wr1 = a_r; wi1 = a_i;
    wr2 = b_r; wi2 = b_i;
  } else if (KY != 0) {
    const R r = -(kz / ky);
    wr0 = b_r; wi0 = b_i;
    wr1 = r * a_r; wi1 = r * a_i;
    wr2 = a_r; wi2 = a_i;
  } else {
    wr0 = a_r; wi0 = a_i;
    wr1 = b_r; wi1 = b_i;
    wr2 = R(0); wi2 = R(0);
  }
  kx *= ik2; ky *= ik2; kz *= ik2;
  v[0] = -(ky * wi2 - kz * wi1); v[1] = (ky * wr2 - kz * wr1);
  v[2] = -(kz * wi0 - kx * wi2); v[3] = (kz * wr0 - kx * wr2);
  v[4] = -(kx * wi1 - ky * wi0); v[5] = (kx * wr1 - ky * wr0);
}

template <typename R>
__global__ void k_zeta_k2u_k(Grid g, const R *z0, const R *z1, const double *ukdc, R *u0, R *u1, R *u2) {
  Mode m;
  if (!mode_of(g, TID, m)) return;
  R v[6];
  zeta_mode_to_u(g, m, z0[m.im], z0[m.im + 1], z1[m.im], z1[m.im + 1], v);
  // the k = 0 mode takes uk_dc (k_set_k0), written after this kernel so that
  // no warp issues the FP64 conversions under a predicate
  u0[m.im] = v[0]; u0[m.im + 1] = v[1];
  u1[m.im] = v[2]; u1[m.im + 1] = v[3];
  u2[m.im] = v[4]; u2[m.im + 1] = v[5];
}

// u_d(k = 0) = uk_dc[d] (Zeta_k2u_k's mean flow, fft_wrapper.cxx:614-711)
template <typename R>
__global__ void k_set_k0(R *u0, R *u1, R *u2, const double *ukdc) {
  u0[0] = (R)ukdc[0];
  u1[0] = (R)ukdc[1];
  u2[0] = (R)ukdc[2];
}

// Truncate_two_third_rule_k of the vorticity (in place) followed by
// Zeta_k2u_k, in one pass: a mode outside the 2/3 cube is zeroed in zeta and
// u; the k = 0 mode takes uk_dc
template <typename R>
__global__ void k_zeta_k2u_trunc(Grid g, R *z0, R *z1, const double *ukdc, R *u0, R *u1, R *u2) {
  Mode m;
  if (!mode_of(g, TID, m)) return;
  R v[6];
  if (!in_two_third(g, m.i, m.j, m.kz)) {
    z0[m.im] = R(0); z0[m.im + 1] = R(0);
    z1[m.im] = R(0); z1[m.im + 1] = R(0);
#pragma unroll
    for (int c = 0; c < 6; c++) v[c] = R(0);
  } else {
    zeta_mode_to_u(g, m, z0[m.im], z0[m.im + 1], z1[m.im], z1[m.im + 1], v);
    if (m.im == 0) {
      v[0] = (R)ukdc[0];
      v[2] = (R)ukdc[1];
      v[4] = (R)ukdc[2];
    }
  }
  u0[m.im] = v[0]; u0[m.im + 1] = v[1];
  u1[m.im] = v[2]; u1[m.im + 1] = v[3];
  u2[m.im] = v[4]; u2[m.im + 1] = v[5];
}

template <typename R>
__device__ __forceinline__ void u_mode_to_zeta(const Grid &g, const Mode &m, const R *k, const R *v, R *z0, R *z1,
                                               double *ukdc) {
  const R a0r = v[0], a0i = v[1];
  const R a1r = v[2], a1i = v[3];
  const R a2r = v[4], a2i = v[5];
  R wr[3], wi[3];
  wr[0] = -(k[1] * a2i - k[2] * a1i); wi[0] = (k[1] * a2r - k[2] * a1r);
  wr[1] = -(k[2] * a0i - k[0] * a2i); wi[1] = (k[2] * a0r - k[0] * a2r);
  wr[2] = -(k[0] * a1i - k[1] * a0i); wi[2] = (k[0] * a1r - k[1] * a0r);
  int a, b;
  if (kx_of(g, m.i) != 0) { a = 1; b = 2; }
  else if (ky_of(g, m.j) != 0) { a = 2; b = 0; }
  else { a = 0; b = 1; }
  z0[m.im] = wr[a]; z0[m.im + 1] = wi[a];
  z1[m.im] = wr[b]; z1[m.im + 1] = wi[b];
  if (m.im == 0) {
    ukdc[0] = a0r; ukdc[1] = a1r; ukdc[2] = a2r;
  }
}

template <typename R>
__global__ void k_u_k2zeta_k(Grid g, const R *u0, const R *u1, const R *u2, R *z0, R *z1, double *ukdc) {
  Mode m;
  if (!mode_of(g, TID, m)) return;
  R k[3];
  kvec(g, m, k);
  const R v[6] = {u0[m.im], u0[m.im + 1], u1[m.im], u1[m.im + 1], u2[m.im], u2[m.im + 1]};
  u_mode_to_zeta(g, m, k, v, z0, z1, ukdc);
}

// The end of the step in k-space, one pass: the particle force f (spectrum)
// truncated to the 2/3 cube and made solenoidal (Make_f_particle_dt_sole,
// f_particle.h:67-78, through Solenoidal_u, operate_omega.h:109-116) is added
// to u (Add_f_particle, f_particle.h:79-95) and the sum becomes the vorticity
// and mean flow (U2zeta_k, operate_omega.h:212-215).
// u + f is added spectrally rather than in real space: the same sum, since
// the truncated, projected f keeps the Hermitian symmetry of a real field and
// has no Nyquist modes. u keeps the spectrum of the sum, as after U2zeta_k.
template <typename R>
__global__ void k_sole_add_zeta(Grid g, V3<R> f, V3<R> u, R *z0, R *z1, double *ukdc) {
  Mode m;
  if (!mode_of(g, TID, m)) return;
  R k[3];
  kvec(g, m, k);
  R v[6];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    v[2 * c] = u.p[c][m.im];
    v[2 * c + 1] = u.p[c][m.im + 1];
  }
  if (in_two_third(g, m.i, m.j, m.kz)) {
    const R k2 = k2_of(k);
    const R ik2 = (k2 > R(0)) ? R(1) / k2 : R(0);
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const R a = f.p[0][m.im + h], b = f.p[1][m.im + h], d = f.p[2][m.im + h];
      const R r = ik2 * (a * k[0] + b * k[1] + d * k[2]);
      v[h] += a - r * k[0];
      v[2 + h] += b - r * k[1];
      v[4 + h] += d - r * k[2];
    }
  }
#pragma unroll
  for (int c = 0; c < 3; c++) {
    u.p[c][m.im] = v[2 * c];
    u.p[c][m.im + 1] = v[2 * c + 1];
  }
  u_mode_to_zeta(g, m, k, v, z0, z1, ukdc);
}

template <typename R>
__global__ void k_advection_combine(Grid g, R *u0, R *u1, R *u2, R *a0, R *a1) {
  Mode m;
  if (!mode_of(g, TID, m)) return;
  R k[3];
  kvec(g, m, k);
  const R k1 = k[0], k2 = k[1], k3 = k[2];
  const R k1k2 = k1 * k2, k2k3 = k2 * k3, k3k1 = k3 * k1;
  int sa, sb;
  if (kx_of(g, m.i) != 0) { sa = 1; sb = 2; }
  else if (ky_of(g, m.j) != 0) { sa = 2; sb = 0; }
  else { sa = 0; sb = 1; }
#pragma unroll
  for (int c = 0; c < 2; c++) {
    const long im = m.im + c;
    const R u2u3 = u0[im], u3u1 = u1[im], u1u2 = u2[im];
    const R u22_u32 = a0[im], u32_u12 = a1[im];
    const R u12_u22 = -u32_u12 - u22_u32;
    R o[3];
    o[0] = -(k2k3 * u22_u32 + (k3 - k2) * (k3 + k2) * u2u3 + k3k1 * u1u2 - k1k2 * u3u1);
    o[1] = -(k3k1 * u32_u12 + (k1 - k3) * (k1 + k3) * u3u1 + k1k2 * u2u3 - k2k3 * u1u2);
    o[2] = -(k1k2 * u12_u22 + (k2 - k1) * (k2 + k1) * u1u2 + k2k3 * u3u1 - k3k1 * u2u3);
    u0[im] = o[0]; u1[im] = o[1]; u2[im] = o[2];
    a0[im] = o[sa];
    a1[im] = o[sb];
  }
}

template <typename R>
// mnudt = -nu dt and inu = 1/nu come from the host (no FP64 arithmetic per thread)
__global__ void k_ns_slaved(Grid g, R *z0, R *z1, const R *a0, const R *a1, R mnudt, R inu) {
  Mode m;
  if (!mode_of(g, TID, m)) return;
  if (!in_two_third(g, m.i, m.j, m.kz)) return;
  R k[3];
  kvec(g, m, k);
  const R k2 = k2_of(k);
  const R ik2 = (k2 > R(0)) ? R(1) / k2 : R(0);
  const R f = exp_t(mnudt * k2) - R(1);
#pragma unroll
  for (int c = 0; c < 2; c++) {
    const long im = m.im + c;
    const R x0 = z0[im], x1 = z1[im];
    z0[im] = x0 + f * (x0 - inu * ik2 * a0[im]);
    z1[im] = x1 + f * (x1 - inu * ik2 * a1[im]);
  }
}

// Truncate_two_third_rule of each component then Solenoidal_uk, the k-space
// part of Solenoidal_u (operate_omega.h:109-116), in one pass
template <typename R>
__global__ void k_solenoidal(Grid g, R *u0, R *u1, R *u2) {
  Mode m;
  if (!mode_of(g, TID, m)) return;
  if (!in_two_third(g, m.i, m.j, m.kz)) {
    u0[m.im] = R(0); u0[m.im + 1] = R(0);
    u1[m.im] = R(0); u1[m.im + 1] = R(0);
    u2[m.im] = R(0); u2[m.im + 1] = R(0);
    return;
  }
  R k[3];
  kvec(g, m, k);
  const R k2 = k2_of(k);
  const R ik2 = (k2 > R(0)) ? R(1) / k2 : R(0);
#pragma unroll
  for (int c = 0; c < 2; c++) {
    const long im = m.im + c;
    const R a = u0[im], b = u1[im], d = u2[im];
    const R r = ik2 * (a * k[0] + b * k[1] + d * k[2]);
    u0[im] = a - r * k[0];
    u1[im] = b - r * k[1];
    u2[im] = d - r * k[2];
  }
}

template <typename R>
__global__ void k_grad(Grid g, const R *a, R *d0, R *d1, R *d2, R scale, int shift, int ext, R ex0, R ex1, R ex2) {
  Mode m;
  if (!mode_of(g, TID, m)) return;
  R k[3];
  kvec(g, m, k);
  const R re = scale * a[m.im], im = scale * a[m.im + 1];
  const int idx[3] = {m.i, m.j, m.kz};
  R *d[3] = {d0, d1, d2};
#pragma unroll
  for (int c = 0; c < 3; c++) {
    R gr = -k[c] * im, gi = k[c] * re;
    if (shift) {
      R sn, cs;
      shift_of(g, c, idx[c], cs, sn);
      const R tr = gr * cs - gi * sn, ti = gr * sn + gi * cs;
      gr = tr;
      gi = ti;
    }
    if (ext && m.im == 0) gr -= (c == 0) ? ex0 : (c == 1) ? ex1 : ex2;
    d[c][m.im] = gr;
    d[c][m.im + 1] = gi;
  }
}

// Truncate_two_third_rule of a concentration spectrum (in place), its
// unshifted gradient scale i k a and a copy of the truncated spectrum, in one
// pass (the start of each species' flux in Rhs_NS_Nernst_Planck,
// fluid_solver.cxx:246-292)
template <typename R>
__global__ void k_grad_trunc_copy(Grid g, R *a, R *d0, R *d1, R *d2, R *cp, R scale) {
  Mode m;
  if (!mode_of(g, TID, m)) return;
  R *d[3] = {d0, d1, d2};
  if (!in_two_third(g, m.i, m.j, m.kz)) {
    a[m.im] = R(0); a[m.im + 1] = R(0);
    cp[m.im] = R(0); cp[m.im + 1] = R(0);
#pragma unroll
    for (int c = 0; c < 3; c++) {
      d[c][m.im] = R(0);
      d[c][m.im + 1] = R(0);
    }
    return;
  }
  const R ar = a[m.im], ai = a[m.im + 1];
  cp[m.im] = ar;
  cp[m.im + 1] = ai;
  R k[3];
  kvec(g, m, k);
  const R re = scale * ar, im = scale * ai;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    d[c][m.im] = -k[c] * im;
    d[c][m.im + 1] = k[c] * re;
  }
}

template <typename R>
__global__ void k_div(Grid g, const R *u0, const R *u1, const R *u2, R *div, int shift) {
  Mode m;
  if (!mode_of(g, TID, m)) return;
  R k[3];
  kvec(g, m, k);
  const R *u[3] = {u0, u1, u2};
  R sr = R(0), si = R(0);
  if (!shift) {
    R a = R(0), b = R(0);
#pragma unroll
    for (int c = 0; c < 3; c++) {
      a += k[c] * u[c][m.im + 1];
      b += k[c] * u[c][m.im];
    }
    div[m.im] = -a;
    div[m.im + 1] = b;
    return;
  }
  const int idx[3] = {m.i, m.j, m.kz};
#pragma unroll
  for (int c = 0; c < 3; c++) {
    R sn, cs;
    shift_of(g, c, idx[c], cs, sn);
    const R ksr = k[c] * cs, ksi = -k[c] * sn;
    const R ur = u[c][m.im], ui = u[c][m.im + 1];
    sr += ur * ksr - ui * ksi;
    si += ur * ksi + ui * ksr;
  }
  div[m.im] = -si;
  div[m.im + 1] = sr;
}

template <typename R>
__global__ void k_euler(Grid g, R *z0, R *z1, R *r0, R *r1, R *c0, R *c1, const R *cr0, const R *cr1, R nu, R dt) {
  Mode m;
  if (!mode_of(g, TID, m)) return;
  if (!in_two_third(g, m.i, m.j, m.kz)) return;
  R k[3];
  kvec(g, m, k);
  const R k2 = k2_of(k);
  const R nuk2 = nu * k2, rdt = dt;
#pragma unroll
  for (int c = 0; c < 2; c++) {
    const long im = m.im + c;
    const R q0 = r0[im] + -(nuk2 * z0[im]);
    const R q1 = r1[im] + -(nuk2 * z1[im]);
    r0[im] = q0;
    r1[im] = q1;
    z0[im] = z0[im] + rdt * q0;
    z1[im] = z1[im] + rdt * q1;
    c0[im] = c0[im] + rdt * cr0[im];
    c1[im] = c1[im] + rdt * cr1[im];
  }
}

template <typename R>
__global__ void k_inv_laplace(Grid g, R *a, R ieps) {
  Mode m;
  if (!mode_of(g, TID, m)) return;
  R k[3];
  kvec(g, m, k);
  const R k2 = k2_of(k);
  const R f = (k2 > R(0)) ? -ieps / k2 : R(0);
  a[m.im] *= f;
  a[m.im + 1] *= f;
}

template <typename R>
__global__ void k_scale_copy(long n, const R *x, R *y, R a) {
  const long t = TID;
  if (t < n) y[t] = a * x[t];
}

// ------------------------------------------------------------ real space
template <typename R>
__global__ void k_adv_products(Grid g, R *u0, R *u1, R *u2, R *a0, R *a1) {
  Pt p;
  if (!pt_of(g, TID, p)) return;
  const R x = u0[p.im], y = u1[p.im], z = u2[p.im];
  u0[p.im] = y * z;
  u1[p.im] = z * x;
  u2[p.im] = x * y;
  a0[p.im] = (y - z) * (y + z);
  a1[p.im] = (z - x) * (z + x);
}

template <typename R>
__global__ void k_phi_clip(Grid g, const R *phs, R *phi) {
  Pt p;
  if (!pt_of(g, TID, p)) return;
  const R v = phs[p.im];
  phi[p.im] = (v < R(1)) ? v : R(1);
}

template <typename R>
__global__ void k_f_nonsole(Grid g, V3<R> f, V3<R> up, const R *phi, V3<R> u) {
  Pt p;
  if (!pt_of(g, TID, p)) return;
  const R ph = phi[p.im];
#pragma unroll
  for (int d = 0; d < 3; d++) f.p[d][p.im] = up.p[d][p.im] - ph * u.p[d][p.im];
}

template <typename R>
// efdc = eps_f dc, dc, epdc = (eps_p - eps_f) dc from the host
__global__ void k_eps_from_profile(Grid g, R *eps, const R *phis, const R *epsw, R efdc, R dc, R epdc) {
  Pt p;
  if (!pt_of(g, TID, p)) return;
  if (epsw) eps[p.im] = efdc + dc * epsw[p.im];
  else eps[p.im] = efdc + epdc * phis[p.im];
}

// Janus: eps = sum_n phi (eps_ave + eps_delta tanh) + eps_f (1 - phi_p) Dc
// (operate_dielectric.cxx:282-292)
template <typename R>
__global__ void k_eps_janus(Grid g, R *eps, const R *phis, const R *epsj, R ef, R dc) {
  Pt p;
  if (!pt_of(g, TID, p)) return;
  eps[p.im] = epsj[p.im] + ef * (R(1) - phis[p.im]) * dc;
}

template <typename R>
__global__ void k_charge_add(Grid g, R *rho, const R *c, const R *phi, R ze, int first) {
  Pt p;
  if (!pt_of(g, TID, p)) return;
  const R v = ze * c[p.im] * (R(1) - phi[p.im]);
  rho[p.im] = first ? v : rho[p.im] + v;
}

// both species in one pass, the sums in the order of two k_charge_add passes
template <typename R>
__global__ void k_charge_add2(Grid g, R *rho, const R *c0, const R *c1, const R *phi, R ze0, R ze1, int first) {
  Pt p;
  if (!pt_of(g, TID, p)) return;
  const R ph = R(1) - phi[p.im];
  const R v0 = ze0 * c0[p.im] * ph, v1 = ze1 * c1[p.im] * ph;
  rho[p.im] = (first ? v0 : rho[p.im] + v0) + v1;
}

// the solute charge of the field output (output.cxx:286-297):
// (e z_0 c_0 + e z_1 c_1) (1 - phi)
template <typename R>
__global__ void k_solute_charge(Grid g, R *out, const R *c0, const R *c1, const R *phi, R ze0, R ze1) {
  Pt p;
  if (!pt_of(g, TID, p)) return;
  const R q = ze0 * c0[p.im] + ze1 * c1[p.im];
  out[p.im] = q * (R(1) - phi[p.im]);
}

template <typename R>
__global__ void k_eps_face_mul(Grid g, R *w0, R *w1, R *w2, const R *eps) {
  Pt p;
  if (!pt_of(g, TID, p)) return;
  const R e0 = eps[p.im];
  w0[p.im] *= R(0.5) * (eps[wrapi(g, p.i + 1, p.j, p.k)] + e0);
  w1[p.im] *= R(0.5) * (eps[wrapi(g, p.i, p.j + 1, p.k)] + e0);
  w2[p.im] *= R(0.5) * (eps[wrapi(g, p.i, p.j, p.k + 1)] + e0);
}

template <typename R>
__global__ void k_eps_face_E(Grid g, R *w0, R *w1, R *w2, const R *eps, R e0, R e1, R e2) {
  Pt p;
  if (!pt_of(g, TID, p)) return;
  const R s0 = R(0.5) * eps[p.im];
  w0[p.im] = (R(0.5) * eps[wrapi(g, p.i + 1, p.j, p.k)] + s0) * e0;
  w1[p.im] = (R(0.5) * eps[wrapi(g, p.i, p.j + 1, p.k)] + s0) * e1;
  w2[p.im] = (R(0.5) * eps[wrapi(g, p.i, p.j, p.k + 1)] + s0) * e2;
}

template <typename R>
__global__ void k_axpby_real(Grid g, const R *x, R *y, R a, R b) {
  Pt p;
  if (!pt_of(g, TID, p)) return;
  y[p.im] = a * x[p.im] + b * y[p.im];
}

// face values to nodes; the result goes to out and, where given, to out2,
// and acc += a * result where acc is given (null pointers skip a target)
template <typename R>
__global__ void k_interp_normal(Grid g, V3<R> out, V3<R> in, V3<R> out2, V3<R> acc, R a) {
  Pt p;
  if (!pt_of(g, TID, p)) return;
  R t[3];
  t[0] = R(0.5) * in.p[0][p.im] + R(0.5) * in.p[0][wrapi(g, p.i - 1, p.j, p.k)];
  t[1] = R(0.5) * in.p[1][p.im] + R(0.5) * in.p[1][wrapi(g, p.i, p.j - 1, p.k)];
  t[2] = R(0.5) * in.p[2][p.im] + R(0.5) * in.p[2][wrapi(g, p.i, p.j, p.k - 1)];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (out.p[0]) out.p[d][p.im] = t[d];
    if (out2.p[0]) out2.p[d][p.im] = t[d];
    if (acc.p[0]) acc.p[d][p.im] += t[d] * a;
  }
}

template <typename R>
__global__ void k_maxwell_e2(Grid g, const R *f0, const R *f1, const R *f2, R *w1, R e0, R e1, R e2, int ext) {
  Pt p;
  if (!pt_of(g, TID, p)) return;
  R fw0 = -f0[p.im], fw1 = -f1[p.im], fw2 = -f2[p.im];
  R bw0 = -f0[wrapi(g, p.i - 1, p.j, p.k)];
  R bw1 = -f1[wrapi(g, p.i, p.j - 1, p.k)];
  R bw2 = -f2[wrapi(g, p.i, p.j, p.k - 1)];
  if (ext) {
    fw0 += e0; fw1 += e1; fw2 += e2;
    bw0 += e0; bw1 += e1; bw2 += e2;
  }
  const R a = (fw0 + bw0) / R(2), b = (fw1 + bw1) / R(2), c = (fw2 + bw2) / R(2);
  w1[p.im] = a * a + b * b + c * c;
}

template <typename R>
__global__ void k_maxwell_face(Grid g, V3<R> grad_pot, V3<R> out, const R *rho, const R *w1, V3<R> ge, R e0, R e1, R e2,
                               int ext) {
  Pt p;
  if (!pt_of(g, TID, p)) return;
  const R E[3] = {e0, e1, e2};
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const long ip = wrapi(g, p.i + (d == 0), p.j + (d == 1), p.k + (d == 2));
    R efw = -grad_pot.p[d][p.im];
    if (ext) efw += E[d];
    const R rf = R(0.5) * rho[ip] + R(0.5) * rho[p.im];
    const R e2v = R(0.5) * w1[p.im] + R(0.5) * w1[ip];
    out.p[d][p.im] = rf * efw - e2v * ge.p[d][p.im] / R(2);
  }
}

// One species' flux in one pass, the flux held in registers between the
// terms: the diffusion flux (read) plus the electric term L z e c grad(pot)
// (Solute_solver_rhs_nonlinear_x_single, solute_rhs.cxx:150-189), the normal
// component removed where the surface normal is non-zero
// (Solute_impermeability, :42-97), then the advective flux -c u
// (Add_advection_flux, :190-210) when u is given.
template <typename R>
__global__ void k_np_flux(Grid g, V3<R> flux, const R *c, V3<R> gp, R lz, V3<R> sn, V3<R> u) {
  Pt p;
  if (!pt_of(g, TID, p)) return;
  const R cc = c[p.im];
  R f[3];
#pragma unroll
  for (int d = 0; d < 3; d++) f[d] = flux.p[d][p.im] + cc * (gp.p[d][p.im] * lz);
  const R n0 = sn.p[0][p.im], n1 = sn.p[1][p.im], n2 = sn.p[2][p.im];
  const R nn = n0 * n0 + n1 * n1 + n2 * n2;
  if (nn > R(0)) {
    const R dd = (f[0] * n0 + f[1] * n1 + f[2] * n2) / nn;
    f[0] = f[0] - n0 * dd;
    f[1] = f[1] - n1 * dd;
    f[2] = f[2] - n2 * dd;
  }
  if (u.p[0]) {
#pragma unroll
    for (int d = 0; d < 3; d++) f[d] += cc * -u.p[d][p.im];
  }
#pragma unroll
  for (int d = 0; d < 3; d++) flux.p[d][p.im] = f[d];
}

template <typename R>
__global__ void k_fill_real(Grid g, R *a, R v) {
  Pt p;
  if (!pt_of(g, TID, p)) return;
  a[p.im] = v;
}

template <typename R>
V3<R> v3(R *const *p) {
  V3<R> v;
  v.p[0] = p[0]; v.p[1] = p[1]; v.p[2] = p[2];
  return v;
}

inline unsigned nblk_modes(const Grid &g) { return div_up(g.nmodes(), TPB); }
inline unsigned nblk_real(const Grid &g) { return div_up(g.nreal(), TPB); }

}  // namespace

template <typename R> void truncate_23(const Grid &g, const FieldBatch<R> &fb, cudaStream_t s) {
  count_launch(fld<R>(g, 2.0 * fb.n));
  k_truncate<R><<<dim3(nblk_modes(g), fb.n), TPB, 0, s>>>(fb, g);
}
template <typename R> void zeta_k2u_k(const Grid &g, const R *z0, const R *z1, const double *uk_dc, R *u0, R *u1, R *u2, cudaStream_t s) {
  count_launch(fld<R>(g, 5));
  k_zeta_k2u_k<R><<<nblk_modes(g), TPB, 0, s>>>(g, z0, z1, uk_dc, u0, u1, u2);
  count_launch();
  k_set_k0<R><<<1, 1, 0, s>>>(u0, u1, u2, uk_dc);
}
template <typename R> void zeta_k2u_trunc(const Grid &g, R *z0, R *z1, const double *uk_dc, R *u0, R *u1, R *u2, cudaStream_t s) {
  count_launch(fld<R>(g, 7));
  k_zeta_k2u_trunc<R><<<nblk_modes(g), TPB, 0, s>>>(g, z0, z1, uk_dc, u0, u1, u2);
}
template <typename R> void u_k2zeta_k(const Grid &g, const R *u0, const R *u1, const R *u2, R *z0, R *z1, double *uk_dc, cudaStream_t s) {
  count_launch(fld<R>(g, 5));
  k_u_k2zeta_k<R><<<nblk_modes(g), TPB, 0, s>>>(g, u0, u1, u2, z0, z1, uk_dc);
}
template <typename R> void sole_add_zeta(const Grid &g, R *const *f, R *const *u, R *z0, R *z1, double *uk_dc, cudaStream_t s) {
  count_launch(fld<R>(g, 11));
  k_sole_add_zeta<R><<<nblk_modes(g), TPB, 0, s>>>(g, v3(f), v3(u), z0, z1, uk_dc);
}
template <typename R> void advection_combine(const Grid &g, R *u0, R *u1, R *u2, R *a0, R *a1, cudaStream_t s) {
  count_launch(fld<R>(g, 7));
  k_advection_combine<R><<<nblk_modes(g), TPB, 0, s>>>(g, u0, u1, u2, a0, a1);
}
template <typename R> void ns_slaved_update(const Grid &g, R *z0, R *z1, const R *a0, const R *a1, double nu, double dt, cudaStream_t s) {
  count_launch(fld<R>(g, 6));
  k_ns_slaved<R><<<nblk_modes(g), TPB, 0, s>>>(g, z0, z1, a0, a1, (R)(-nu * dt), (R)(1. / nu));
}
template <typename R> void truncate_solenoidal_uk(const Grid &g, R *u0, R *u1, R *u2, cudaStream_t s) {
  count_launch(fld<R>(g, 6));
  k_solenoidal<R><<<nblk_modes(g), TPB, 0, s>>>(g, u0, u1, u2);
}
template <typename R> void grad_k(const Grid &g, const R *a, R *d0, R *d1, R *d2, R scale, bool shift, const double *e_ext_n, cudaStream_t s) {
  const int ext = e_ext_n ? 1 : 0;
  const R ex0 = ext ? (R)e_ext_n[0] : R(0), ex1 = ext ? (R)e_ext_n[1] : R(0), ex2 = ext ? (R)e_ext_n[2] : R(0);
  count_launch(fld<R>(g, 4));
  k_grad<R><<<nblk_modes(g), TPB, 0, s>>>(g, a, d0, d1, d2, scale, shift ? 1 : 0, ext, ex0, ex1, ex2);
}
template <typename R> void grad_trunc_copy(const Grid &g, R *a, R *d0, R *d1, R *d2, R *cp, R scale, cudaStream_t s) {
  count_launch(fld<R>(g, 6));
  k_grad_trunc_copy<R><<<nblk_modes(g), TPB, 0, s>>>(g, a, d0, d1, d2, cp, scale);
}
template <typename R> void div_k(const Grid &g, const R *u0, const R *u1, const R *u2, R *div, bool shift, cudaStream_t s) {
  count_launch(fld<R>(g, 4));
  k_div<R><<<nblk_modes(g), TPB, 0, s>>>(g, u0, u1, u2, div, shift ? 1 : 0);
}
template <typename R> void euler_update(const Grid &g, R *z0, R *z1, R *r0, R *r1, R *c0, R *c1, const R *cr0, const R *cr1, double nu, double dt, cudaStream_t s) {
  count_launch(fld<R>(g, 12));
  k_euler<R><<<nblk_modes(g), TPB, 0, s>>>(g, z0, z1, r0, r1, c0, c1, cr0, cr1, (R)nu, (R)dt);
}
template <typename R> void inv_laplace_k(const Grid &g, R *a, double eps_ref, cudaStream_t s) {
  count_launch(fld<R>(g, 2));
  k_inv_laplace<R><<<nblk_modes(g), TPB, 0, s>>>(g, a, (R)(1.0 / eps_ref));
}
template <typename R> void scale_copy(const Grid &g, const R *x, R *y, R a, cudaStream_t s) {
  count_launch(fld<R>(g, 2));
  k_scale_copy<R><<<div_up(g.nf(), TPB), TPB, 0, s>>>(g.nf(), x, y, a);
}
template <typename R> void advection_products(const Grid &g, R *u0, R *u1, R *u2, R *a0, R *a1, cudaStream_t s) {
  count_launch(fld<R>(g, 8));
  k_adv_products<R><<<nblk_real(g), TPB, 0, s>>>(g, u0, u1, u2, a0, a1);
}
template <typename R> void phi_clip(const Grid &g, const R *phs, R *phi, cudaStream_t s) {
  count_launch(fld<R>(g, 2));
  k_phi_clip<R><<<nblk_real(g), TPB, 0, s>>>(g, phs, phi);
}
template <typename R> void f_nonsole(const Grid &g, R *const *f, R *const *up, const R *phi, R *const *u, cudaStream_t s) {
  count_launch(fld<R>(g, 10));
  k_f_nonsole<R><<<nblk_real(g), TPB, 0, s>>>(g, v3(f), v3(up), phi, v3(u));
}
template <typename R> void eps_from_profile(const Grid &g, R *eps, const R *phi_sin, const R *eps_w, double ef, double ep, double dc, cudaStream_t s) {
  count_launch(fld<R>(g, 3));
  k_eps_from_profile<R><<<nblk_real(g), TPB, 0, s>>>(g, eps, phi_sin, eps_w, (R)(ef * dc), (R)dc, (R)((ep - ef) * dc));
}
template <typename R> void eps_janus(const Grid &g, R *eps, const R *phi_sin, const R *eps_j, double ef, double dc, cudaStream_t s) {
  count_launch(fld<R>(g, 3));
  k_eps_janus<R><<<nblk_real(g), TPB, 0, s>>>(g, eps, phi_sin, eps_j, (R)ef, (R)dc);
}
template <typename R> void charge_add(const Grid &g, R *rho, const R *c, const R *phi, double ze, bool first, cudaStream_t s) {
  count_launch(fld<R>(g, first ? 3.0 : 4.0));
  k_charge_add<R><<<nblk_real(g), TPB, 0, s>>>(g, rho, c, phi, (R)ze, first ? 1 : 0);
}
template <typename R> void charge_add2(const Grid &g, R *rho, const R *c0, const R *c1, const R *phi, double ze0, double ze1, bool first, cudaStream_t s) {
  count_launch(fld<R>(g, first ? 4.0 : 5.0));
  k_charge_add2<R><<<nblk_real(g), TPB, 0, s>>>(g, rho, c0, c1, phi, (R)ze0, (R)ze1, first ? 1 : 0);
}
template <typename R>
void solute_charge(const Grid &g, R *out, const R *c0, const R *c1, const R *phi, double ze0, double ze1, cudaStream_t s) {
  count_launch(fld<R>(g, 4));
  k_solute_charge<R><<<nblk_real(g), TPB, 0, s>>>(g, out, c0, c1, phi, (R)ze0, (R)ze1);
}
template <typename R> void eps_face_mul(const Grid &g, R *w0, R *w1, R *w2, const R *eps, cudaStream_t s) {
  count_launch(fld<R>(g, 7));
  k_eps_face_mul<R><<<nblk_real(g), TPB, 0, s>>>(g, w0, w1, w2, eps);
}
template <typename R> void eps_face_E(const Grid &g, R *w0, R *w1, R *w2, const R *eps, double e0, double e1, double e2, cudaStream_t s) {
  count_launch(fld<R>(g, 4));
  k_eps_face_E<R><<<nblk_real(g), TPB, 0, s>>>(g, w0, w1, w2, eps, (R)e0, (R)e1, (R)e2);
}
template <typename R> void axpby_real(const Grid &g, const R *x, R *y, R a, R b, cudaStream_t s) {
  count_launch(fld<R>(g, 3));
  k_axpby_real<R><<<nblk_real(g), TPB, 0, s>>>(g, x, y, a, b);
}
template <typename R> void interp_normal(const Grid &g, R *const *out, R *const *in, cudaStream_t s) {
  count_launch(fld<R>(g, 6));
  k_interp_normal<R><<<nblk_real(g), TPB, 0, s>>>(g, v3(out), v3(in), V3<R>{}, V3<R>{}, R(0));
}
template <typename R> void interp_normal_to(const Grid &g, R *const *in, R *const *out, R *const *out2, R *const *acc, R a, cudaStream_t s) {
  const V3<R> none{};
  count_launch(fld<R>(g, 3.0 + (out ? 3 : 0) + (out2 ? 3 : 0) + (acc ? 6 : 0)));
  k_interp_normal<R><<<nblk_real(g), TPB, 0, s>>>(g, out ? v3(out) : none, v3(in), out2 ? v3(out2) : none,
                                                   acc ? v3(acc) : none, a);
}
template <typename R> void maxwell_e2(const Grid &g, const R *f0, const R *f1, const R *f2, R *w1, double e0, double e1, double e2, int ext, cudaStream_t s) {
  count_launch(fld<R>(g, 4));
  k_maxwell_e2<R><<<nblk_real(g), TPB, 0, s>>>(g, f0, f1, f2, w1, (R)e0, (R)e1, (R)e2, ext);
}
template <typename R> void maxwell_face(const Grid &g, R *const *grad_pot, R *const *out, const R *rho, const R *w1, R *const *ge, double e0, double e1, double e2, int ext, cudaStream_t s) {
  count_launch(fld<R>(g, 11));
  k_maxwell_face<R><<<nblk_real(g), TPB, 0, s>>>(g, v3(grad_pot), v3(out), rho, w1, v3(ge), (R)e0, (R)e1, (R)e2, ext);
}
template <typename R> void np_flux(const Grid &g, R *const *flux, const R *c, R *const *gp, double L_ze, R *const *sn, R *const *u, cudaStream_t s) {
  count_launch(fld<R>(g, u ? 13.0 : 10.0));
  k_np_flux<R><<<nblk_real(g), TPB, 0, s>>>(g, v3(flux), c, v3(gp), (R)L_ze, v3(sn), u ? v3(u) : V3<R>{});
}
template <typename R> void fill_real(const Grid &g, R *a, R v, cudaStream_t s) {
  count_launch(fld<R>(g, 1));
  k_fill_real<R><<<nblk_real(g), TPB, 0, s>>>(g, a, v);
}

template <typename R>
__global__ void k_pb_energy(Grid g, const R *c0, const R *c1, const R *phi, R *charge, const R *pot, R ze0, R ze1,
                            R ex, R ey, R ez, R dx, int ext, R *ideal, R *es) {
  Pt p;
  if (!pt_of(g, TID, p)) return;
  const R ph = phi[p.im], a = c0[p.im], b = c1[p.im];
  ideal[p.im] = (1. - ph) * a * (log(a) - 1.) + (1. - ph) * b * (log(b) - 1.);
  R q = charge[p.im];
  q += ze0 * a * (1. - ph);
  q += ze1 * b * (1. - ph);
  charge[p.im] = q;
  R pt = 0.5 * pot[p.im];
  if (ext) pt -= (ex * (R)p.i + ey * (R)p.j + ez * (R)p.k) * dx;
  es[p.im] = q * pt;
}
template <typename R>
void pb_energy_terms(const Grid &g, const R *c0, const R *c1, const R *phi, R *charge, const R *pot, double ze0,
                     double ze1, const double *e, double dx, int ext, R *ideal, R *es, cudaStream_t s) {
  count_launch(fld<R>(g, 7));
  k_pb_energy<R><<<nblk_real(g), TPB, 0, s>>>(g, c0, c1, phi, charge, pot, (R)ze0, (R)ze1, (R)e[0], (R)e[1], (R)e[2],
                                              (R)dx, ext, ideal, es);
}

#define ICEP_INST(R)                                                                                                   \
  template void truncate_23<R>(const Grid &, const FieldBatch<R> &, cudaStream_t);                                    \
  template void zeta_k2u_k<R>(const Grid &, const R *, const R *, const double *, R *, R *, R *, cudaStream_t);        \
  template void u_k2zeta_k<R>(const Grid &, const R *, const R *, const R *, R *, R *, double *, cudaStream_t);        \
  template void zeta_k2u_trunc<R>(const Grid &, R *, R *, const double *, R *, R *, R *, cudaStream_t);                \
  template void sole_add_zeta<R>(const Grid &, R *const *, R *const *, R *, R *, double *, cudaStream_t);              \
  template void grad_trunc_copy<R>(const Grid &, R *, R *, R *, R *, R *, R, cudaStream_t);                            \
  template void interp_normal_to<R>(const Grid &, R *const *, R *const *, R *const *, R *const *, R, cudaStream_t);   \
  template void advection_combine<R>(const Grid &, R *, R *, R *, R *, R *, cudaStream_t);                             \
  template void ns_slaved_update<R>(const Grid &, R *, R *, const R *, const R *, double, double, cudaStream_t);       \
  template void truncate_solenoidal_uk<R>(const Grid &, R *, R *, R *, cudaStream_t);                                  \
  template void grad_k<R>(const Grid &, const R *, R *, R *, R *, R, bool, const double *, cudaStream_t);              \
  template void div_k<R>(const Grid &, const R *, const R *, const R *, R *, bool, cudaStream_t);                      \
  template void euler_update<R>(const Grid &, R *, R *, R *, R *, R *, R *, const R *, const R *, double, double,      \
                                cudaStream_t);                                                                         \
  template void scale_copy<R>(const Grid &, const R *, R *, R, cudaStream_t);                                          \
  template void inv_laplace_k<R>(const Grid &, R *, double, cudaStream_t);                                             \
  template void advection_products<R>(const Grid &, R *, R *, R *, R *, R *, cudaStream_t);                            \
  template void phi_clip<R>(const Grid &, const R *, R *, cudaStream_t);                                               \
  template void f_nonsole<R>(const Grid &, R *const *, R *const *, const R *, R *const *, cudaStream_t);               \
  template void eps_from_profile<R>(const Grid &, R *, const R *, const R *, double, double, double, cudaStream_t);    \
  template void eps_janus<R>(const Grid &, R *, const R *, const R *, double, double, cudaStream_t);                   \
  template void charge_add<R>(const Grid &, R *, const R *, const R *, double, bool, cudaStream_t);                    \
  template void charge_add2<R>(const Grid &, R *, const R *, const R *, const R *, double, double, bool, cudaStream_t); \
  template void solute_charge<R>(const Grid &, R *, const R *, const R *, const R *, double, double, cudaStream_t);     \
  template void eps_face_mul<R>(const Grid &, R *, R *, R *, const R *, cudaStream_t);                                 \
  template void eps_face_E<R>(const Grid &, R *, R *, R *, const R *, double, double, double, cudaStream_t);           \
  template void axpby_real<R>(const Grid &, const R *, R *, R, R, cudaStream_t);                                       \
  template void interp_normal<R>(const Grid &, R *const *, R *const *, cudaStream_t);                                  \
  template void maxwell_e2<R>(const Grid &, const R *, const R *, const R *, R *, double, double, double, int,         \
                              cudaStream_t);                                                                           \
  template void maxwell_face<R>(const Grid &, R *const *, R *const *, const R *, const R *, R *const *, double, double, \
                                double,                                                                                \
                                int, cudaStream_t);                                                                    \
  template void np_flux<R>(const Grid &, R *const *, const R *, R *const *, double, R *const *, R *const *,          \
                           cudaStream_t);                                                                              \
  template void fill_real<R>(const Grid &, R *, R, cudaStream_t);                                                    \
  template void pb_energy_terms<R>(const Grid &, const R *, const R *, const R *, R *, const R *, double, double,     \
                                   const double *, double, int, R *, R *, cudaStream_t);

ICEP_INST(double)
ICEP_INST(float)

}  // namespace icep
