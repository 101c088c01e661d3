// particles.cu -- see particles.cuh.
#include <float.h>

#include <type_traits>

#include "particles.cuh"

namespace icep {

namespace {

constexpr int TPB = 256;

__device__ __forceinline__ int nint_d(double a) { return (a >= 0.0) ? (int)(a + .5) : (int)(a - .5); }

// Geometry of stencil point m of a particle at xp: Particle_cell
// (make_phi.h:114-140), Relative_coord (make_phi.h:162-179) and the periodic
// distance of Distance (interaction.h:122-147). Returns the field index.
__device__ __forceinline__ long stencil_point(const PartParams &pp, const double *xp, const int *sek, int m, double *r,
                                              double *dist) {
  const double idx = 1. / pp.dx;
  int rm[3];
  double s = 0.0;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const double v = xp[d] * idx;
    const int xi = (int)v;
    const double res = (v - (double)xi) * pp.dx;
    const int cell = sek[3 * m + d];
    // periodic wrap (N a power of two): unsigned arithmetic keeps the index
    // inside the grid for any coordinate, a non-finite or huge one included
    rm[d] = (int)(((unsigned)xi + (unsigned)cell) & (unsigned)(pp.N[d] - 1));
    r[d] = (double)cell * pp.dx - res;
    double x12 = xp[d] - rm[d] * pp.dx;
    // minimum image: nint(x12/L) is 0 while |x12| < L/2
    if (!(fabs(x12) < 0.5 * pp.L[d])) x12 -= (double)nint_d(x12 / pp.L[d]) * pp.L[d];
    s += x12 * x12;
  }
  *dist = sqrt(s);
  return ((long)rm[0] * pp.N[1] + rm[1]) * pp.nzp + rm[2];
}

// The particle's cell and residue (Particle_cell, make_phi.h:114-140), FP64.
struct PCell {
  int xi[3];
  float res[3];
};
__device__ __forceinline__ void particle_cell(const PartParams &pp, const double *xp, PCell &pc) {
  const double idx = 1. / pp.dx;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const double v = xp[d] * idx;
    pc.xi[d] = (int)v;
    pc.res[d] = (float)((v - (double)pc.xi[d]) * pp.dx);
  }
}
// Stencil point m in the field type R. FP64: stencil_point (the reference's
// rounding). FP32 (MIXED): r = cell dx - residue in FP32 and dist = |r|: the
// minimum image of x_mesh - x_p is -r because the stencil is narrower than
// half the box, so no FP64 arithmetic is needed per point.
template <typename R>
__device__ __forceinline__ long stencil_pt(const PartParams &pp, const double *xp, const PCell &pc, const int *sek,
                                           int m, R *r, R *dist) {
  if constexpr (std::is_same<R, double>::value) {
    return stencil_point(pp, xp, sek, m, r, dist);
  } else {
    int rm[3];
    float s = 0.f;
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const int cell = sek[3 * m + d];
      rm[d] = (int)(((unsigned)pc.xi[d] + (unsigned)cell) & (unsigned)(pp.N[d] - 1));
      r[d] = (float)cell * (float)pp.dx - pc.res[d];
      s = fmaf(r[d], r[d], s);
    }
    *dist = sqrtf(s);
    return ((long)rm[0] * pp.N[1] + rm[1]) * pp.nzp + rm[2];
  }
}

// The scatter kernels run ceil(np_domain / TPB) blocks per particle: block b
// serves particle b / chunks and stencil points (b % chunks) TPB + thread. One
// thread computes the particle's cell (FP64) into shared memory.
__device__ __forceinline__ const PCell &chunk_cell(const PartParams &pp, const icep_particle *p, int &n, int &m) {
  __shared__ PCell spc;
  const int chunks = (pp.np_domain + blockDim.x - 1) / blockDim.x;
  n = (int)(blockIdx.x / chunks);
  m = (int)((blockIdx.x - (unsigned)n * chunks) * blockDim.x + threadIdx.x);
  if (threadIdx.x == 0) particle_cell(pp, p[n].x, spc);
  __syncthreads();
  return spc;
}

template <typename R>
__device__ __forceinline__ R exp_t(R a);
template <>
__device__ __forceinline__ double exp_t<double>(double a) { return exp(a); }
template <>
__device__ __forceinline__ float exp_t<float>(float a) { return expf(a); }
template <typename R>
__device__ __forceinline__ R sin_t(R a);
template <>
__device__ __forceinline__ double sin_t<double>(double a) { return sin(a); }
template <>
__device__ __forceinline__ float sin_t<float>(float a) { return sinf(a); }

// H and Phi (profile.h:29-49)
template <typename R>
__device__ __forceinline__ R prof_h(R dx, R x) {
  return x > R(0) ? exp_t<R>(-(dx / x) * (dx / x)) : R(0);
}
template <typename R>
__device__ __forceinline__ R prof_phi(const PartParams &pp, R x) {
  const R dx = (R)pp.dx, rad = (R)pp.radius, hxi = (R)pp.hxi;
  const R a = prof_h<R>(dx, rad + hxi - x);
  return a / (a + prof_h<R>(dx, x - rad + hxi));
}
// Phi_compact_sin (profile.h:139-152)
template <typename R>
__device__ __forceinline__ R prof_phi_sin(const PartParams &pp, R x) {
  const R d = (R)pp.radius - x, hxi = (R)pp.hxi;
  if (fabs(d) <= hxi) return R(0.5) * sin_t<R>((R)M_PI * d / (R)pp.xi) + R(0.5);
  return (d > hxi) ? R(1) : R(0);
}

template <typename R>
__device__ __forceinline__ R tanh_t(R a);
template <>
__device__ __forceinline__ double tanh_t<double>(double a) { return tanh(a); }
template <>
__device__ __forceinline__ float tanh_t<float>(float a) { return tanhf(a); }

// Janus axis e3 of the particle's species rotated to the space frame and
// normalised (Make_janus_normal_dielectric, operate_dielectric.cxx:173-205;
// BODY2SPACE: q (0, e3) q*, rigid_body.cxx:10-24, quaternion.h:205-213)
// (in the field type R: FP32 arithmetic in MIXED precision)
template <typename R>
__device__ __forceinline__ void janus_normal(const double *qd64, int axis, R *nrm) {
  const R q[4] = {(R)qd64[0], (R)qd64[1], (R)qd64[2], (R)qd64[3]};
  const R e[3] = {R(axis == 0 ? 1 : 0), R(axis == 1 ? 1 : 0), R(axis == 2 ? 1 : 0)};
  const R qs2 = q[0] * q[0] - (q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  const R qd = q[1] * e[0] + q[2] * e[1] + q[3] * e[2];
  R v[3];
  v[0] = qs2 * e[0] + R(2) * (qd * q[1] + q[0] * (q[2] * e[2] - q[3] * e[1]));
  v[1] = qs2 * e[1] + R(2) * (qd * q[2] + q[0] * (q[3] * e[0] - q[1] * e[2]));
  v[2] = qs2 * e[2] + R(2) * (qd * q[3] + q[0] * (q[1] * e[1] - q[2] * e[0]));
  const R in = R(1) / sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  for (int d = 0; d < 3; d++) nrm[d] = v[d] * in;
}

// DPhi_compact_sin (profile.h:168-181)
template <typename R>
__device__ __forceinline__ R prof_dphi_sin(const PartParams &pp, R x) {
  const R hxi = (R)pp.xi * R(.5);
  const R ixi = R(1) / (R)pp.xi;
  const R d = (R)pp.radius - x;
  if (fabs(d) < hxi) return (R)M_PI * R(.5) * ixi * cos((R)M_PI * d * ixi);
  return R(0);
}

template <typename R>
__global__ void k_scatter_profile(PartParams pp, const icep_particle *__restrict__ p, const int *__restrict__ sek, R *out,
                                  R *aux, int kind) {
  int n, m;
  const PCell &pc = chunk_cell(pp, p, n, m);
  if (m >= pp.np_domain) return;
  R r[3], dist;
  const long im = stencil_pt<R>(pp, p[n].x, pc, sek, m, r, &dist);
  if (kind == PROF_PHI) {
    const R v = prof_phi<R>(pp, (R)dist);
    if (v != R(0)) atomicAdd(out + im, v);
  } else if (kind == PROF_QQ) {
    const R v = prof_phi<R>(pp, (R)dist);
    if (v != R(0)) atomicAdd(out + im, v);
    const R sq = (R)pp.qe[p[n].spec] * prof_dphi_sin<R>(pp, (R)dist);
    if (sq != R(0)) atomicAdd(aux + im, sq);
  } else if (kind == PROF_PHI_SIN) {
    const R v = prof_phi_sin<R>(pp, (R)dist);
    if (v != R(0)) {
      atomicAdd(out + im, v);
      if (aux) atomicAdd(aux + im, (R)(p[n].eps_p - pp.eps_f) * v);
    }
  } else {
    const R v = prof_phi_sin<R>(pp, (R)dist);
    if (v != R(0)) {
      R nrm[3];
      janus_normal<R>(p[n].q, pp.janus_axis[p[n].spec], nrm);
      R jr = R(0);
      for (int d = 0; d < 3; d++) jr += r[d] * nrm[d];
      const R th = tanh_t<R>((R)pp.sharp * jr);
      atomicAdd(out + im, v);
      atomicAdd(aux + im, v * ((R)pp.eps_ave + (R)pp.eps_delta * th));
    }
  }
}

template <typename R>
__global__ void k_scatter_up(PartParams pp, const icep_particle *__restrict__ p, const int *__restrict__ sek,
                             const R *__restrict__ phs, R *u0, R *u1, R *u2) {
  int n, m;
  const PCell &pc = chunk_cell(pp, p, n, m);
  if (m >= pp.np_domain) return;
  R r[3], dist;
  const long im = stencil_pt<R>(pp, p[n].x, pc, sek, m, r, &dist);
  const R ps = phs[im];
  const R w = prof_phi<R>(pp, dist) / ((ps > R(1)) ? ps : R(1));
  if (w == R(0)) return;
  R vr[3] = {0, 0, 0};
  if (pp.rotation) {
    const R om[3] = {(R)p[n].omega[0], (R)p[n].omega[1], (R)p[n].omega[2]};
    vr[0] = om[1] * r[2] - om[2] * r[1];
    vr[1] = om[2] * r[0] - om[0] * r[2];
    vr[2] = om[0] * r[1] - om[1] * r[0];
  }
  atomicAdd(u0 + im, ((R)p[n].v[0] + vr[0]) * w);
  atomicAdd(u1 + im, ((R)p[n].v[1] + vr[1]) * w);
  atomicAdd(u2 + im, ((R)p[n].v[2] + vr[2]) * w);
}

template <typename R>
__global__ void k_scatter_normal(PartParams pp, const icep_particle *__restrict__ p, const int *__restrict__ sek, R *s0,
                                 R *s1, R *s2) {
  // the band |r - a| < xi/2 has a sharp edge, which FP32 distances would
  // move: the decision is FP64's for every point near the edge
  int n, m;
  const PCell &pc = chunk_cell(pp, p, n, m);
  if (m >= pp.np_domain) return;
  if constexpr (std::is_same<R, float>::value) {
    // MIXED: FP32 offsets from the particle's cell (distance error < 1e-6)
    // decide the points further than 1e-4 from the band's edges; the normal
    // of a point inside is the FP32 unit vector
    float r[3], dist;
    const long im = stencil_pt<float>(pp, p[n].x, pc, sek, m, r, &dist);
    const float off = fabsf(dist - (float)pp.radius), h = (float)pp.hxi;
    if (off > h + 1e-4f) return;
    if (off < h - 1e-4f) {
      const float ir = 1.f / dist;
      atomicAdd(s0 + im, r[0] * ir);
      atomicAdd(s1 + im, r[1] * ir);
      atomicAdd(s2 + im, r[2] * ir);
      return;
    }
  }
  double r[3], dist;
  const long im = stencil_point(pp, p[n].x, sek, m, r, &dist);
  const double dr2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
  // a conservative test on the squared distance skips the points far from
  // the band before the FP64 square root and division (the exact test below
  // decides every point that passes it)
  if (dr2 < pp.band_lo2 || dr2 > pp.band_hi2) return;
  const double dr = sqrt(dr2);
  if (fabs(dr - pp.radius) < pp.hxi) {
    const double ir = 1. / dr;
    atomicAdd(s0 + im, (R)(r[0] * ir));
    atomicAdd(s1 + im, (R)(r[1] * ir));
    atomicAdd(s2 + im, (R)(r[2] * ir));
  }
}

// One block per particle; force and torque summed per thread in the field
// type (FP64, or FP32 with the FP32 stencil geometry in MIXED precision) and
// across the block in FP64.
template <typename R>
__global__ void k_f_hydro(PartParams pp, icep_particle *p, const int *__restrict__ sek, const R *__restrict__ phs,
                          const R *__restrict__ u0, const R *__restrict__ u1, const R *__restrict__ u2, int copy1) {
  const int n = blockIdx.x;
  if (n >= pp.np) return;
  const icep_particle &q = p[n];
  double xp[3];
  R vp[3], om[3];
  for (int d = 0; d < 3; d++) {
    xp[d] = q.x[d];
    vp[d] = (R)q.v[d];
    om[d] = (R)q.omega[d];
  }
  PCell pc;
  if constexpr (!std::is_same<R, double>::value) particle_cell(pp, xp, pc);
  R acc[6] = {0, 0, 0, 0, 0, 0};
  for (int m = threadIdx.x; m < pp.np_domain; m += blockDim.x) {
    R r[3], dist;
    const long im = stencil_pt<R>(pp, xp, pc, sek, m, r, &dist);
    const R ps = phs[im];
    const R w = prof_phi<R>(pp, dist) / ((ps > R(1)) ? ps : R(1));
    if (w == R(0)) continue;
    R vr[3] = {0, 0, 0};
    if (pp.rotation) {
      vr[0] = om[1] * r[2] - om[2] * r[1];
      vr[1] = om[2] * r[0] - om[0] * r[2];
      vr[2] = om[0] * r[1] - om[1] * r[0];
    }
    const R f0 = ((vp[0] + vr[0]) - u0[im]) * w;
    const R f1 = ((vp[1] + vr[1]) - u1[im]) * w;
    const R f2 = ((vp[2] + vr[2]) - u2[im]) * w;
    acc[0] += f0;
    acc[1] += f1;
    acc[2] += f2;
    acc[3] += r[1] * f2 - r[2] * f1;
    acc[4] += r[2] * f0 - r[0] * f2;
    acc[5] += r[0] * f1 - r[1] * f0;
  }
  __shared__ double red[6][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < 6; c++) {
    R v = acc[c];  // warp sums in the field type, FP64 across warps
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[c][wid] = (double)v;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    double v = 0.0;
    const int nw = (blockDim.x + 31) >> 5;
    for (int w = 0; w < nw; w++) v += red[threadIdx.x][w];
    const double fac = -(pp.dx * pp.dx * pp.dx) * pp.rho / pp.dt;
    const int c = threadIdx.x;
    if (c < 3) {
      p[n].f_hydro[c] = fac * v;
      if (copy1) p[n].f_hydro1[c] = fac * v;
    } else if (pp.rotation) {
      p[n].torque_hydro[c - 3] = fac * v;
      if (copy1) p[n].torque_hydro1[c - 3] = fac * v;
    } else if (copy1) {
      p[n].torque_hydro1[c - 3] = p[n].torque_hydro[c - 3];
    }
  }
}

// Lennard_Jones_f (interaction.h:175-200)
__device__ double lj_f(const PartParams &pp, double x) {
  const double s = pp.lj_dia / x;
  double t;
  if (pp.lj_powers == 0) {
    t = (s * s) * (s * s) * (s * s);
    return 24. * pp.lj_eps / (x * x) * (2.0 * t * t - t);
  } else if (pp.lj_powers == 1) {
    const double s2 = s * s;
    t = s2 * s2 * s2 * s2 * s2 * s2;
    return 48. * pp.lj_eps / (x * x) * (2.0 * t * t - t);
  }
  const double s2 = s * s;
  t = s2 * s2 * s2 * s2 * s2 * s2 * s2 * s2 * s2;
  return 72. * pp.lj_eps / (x * x) * (2.0 * t * t - t);
}

struct CellGeom {
  int lc[3];
  double lcr;
};

__device__ __forceinline__ int cell_coord(const CellGeom &cg, double x, int d) {
  int c = (int)(x / cg.lcr);
  // positions are in [0, L) after PBC; clamp so that a non-finite position
  // cannot index outside the cell arrays
  return c < 0 ? 0 : (c >= cg.lc[d] ? cg.lc[d] - 1 : c);
}

__device__ __forceinline__ int cell_of(const CellGeom &cg, const double *x) {
  int mc[3];
  for (int d = 0; d < 3; d++) mc[d] = cell_coord(cg, x[d], d);
  return (mc[0] * cg.lc[1] + mc[1]) * cg.lc[2] + mc[2];
}

// Counting sort of particles into cells of edge 16*DX (one block).
__global__ void k_lj_cells(PartParams pp, CellGeom cg, const icep_particle *__restrict__ p, int *start, int *fill,
                           int *list, int ncell) {
  for (int c = threadIdx.x; c <= ncell; c += blockDim.x) {
    start[c] = 0;
    fill[c] = 0;
  }
  __syncthreads();
  for (int n = threadIdx.x; n < pp.np; n += blockDim.x) atomicAdd(&start[cell_of(cg, p[n].x) + 1], 1);
  __syncthreads();
  if (threadIdx.x == 0)
    for (int c = 0; c < ncell; c++) start[c + 1] += start[c];
  __syncthreads();
  for (int n = threadIdx.x; n < pp.np; n += blockDim.x) {
    const int c = cell_of(cg, p[n].x);
    const int slot = atomicAdd(&fill[c], 1);
    list[start[c] + slot] = n;
  }
}

// Per-particle gather over the 27-cell scan with the reference's wrap rule
// (md_force.cxx:60-82): with one or two cells along an axis a neighbour cell
// is visited more than once and each visit adds the pair force again.
// One warp per particle: lane l < 27 scans neighbour cell l of the 27-cell
// block (the reference's wrap rule, md_force.cxx:60-82: with one or two cells
// along an axis a neighbour cell is visited more than once and each visit
// adds the pair force again); the FP64 force is reduced over the warp. Pairs
// farther than the cutoff are skipped on the squared distance with a margin
// before any division; for the others the arithmetic is the reference's
// (the minimum-image division can only be non-zero where |dx| >= L/2).
__global__ void k_lj_gather(PartParams pp, CellGeom cg, icep_particle *p, const int *__restrict__ start,
                            const int *__restrict__ list, int *pairs, int max_pairs, int *n_pairs) {
  const int a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (a >= pp.np) return;  // whole warps leave together
  double xa[3];
  for (int d = 0; d < 3; d++) xa[d] = p[a].x[d];
  double f[3] = {0, 0, 0};
  const double rc = pp.r_cutoff, rc2 = rc * rc * (1.0 + 1e-9);
  if (lane < 27) {
    int ic[3];
    for (int d = 0; d < 3; d++) ic[d] = cell_coord(cg, xa[d], d);
    const int o[3] = {lane / 9 - 1, (lane / 3) % 3 - 1, lane % 3 - 1};
    int cl[3];
    for (int d = 0; d < 3; d++) {
      cl[d] = ic[d] + o[d];
      if (cl[d] < 0) cl[d] = cg.lc[d] - 1;
      if (cl[d] > cg.lc[d] - 1) cl[d] = 0;
    }
    const int c = (cl[0] * cg.lc[1] + cl[1]) * cg.lc[2] + cl[2];
    for (int q = start[c]; q < start[c + 1]; q++) {
      const int j = list[q];
      if (j == a) continue;
      double rv[3], s = 0.0;
      for (int d = 0; d < 3; d++) {
        rv[d] = p[j].x[d] - xa[d];
        if (!(fabs(rv[d]) < 0.5 * pp.L[d])) rv[d] -= (double)nint_d(rv[d] / pp.L[d]) * pp.L[d];
        s += rv[d] * rv[d];
      }
      if (s > rc2) continue;
      const double rij = sqrt(s);
      if (rij < rc) {
        const double va = DBL_MAX / rij, vb = lj_f(pp, rij);
        const double fr = (va < vb) ? va : vb;
        for (int d = 0; d < 3; d++) f[d] += fr * (-rv[d]);
        if (pairs && j < a) {
          const int k = atomicAdd(n_pairs, 1);
          if (k < max_pairs) {
            pairs[2 * k] = a;
            pairs[2 * k + 1] = j;
          }
        }
      }
    }
  }
  for (int d = 0; d < 3; d++)
    for (int off = 16; off > 0; off >>= 1) f[d] += __shfl_down_sync(0xffffffffu, f[d], off);
  if (lane == 0)
    for (int d = 0; d < 3; d++) p[a].fr[d] += f[d];
}

// quaternion helpers (quaternion.h:173-213, rigid_body.cxx:10-24)
__device__ void qprod(double *q, const double *a, const double *b, double alpha) {
  q[0] = alpha * (a[0] * b[0] - (a[1] * b[1] + a[2] * b[2] + a[3] * b[3]));
  q[1] = alpha * (a[0] * b[1] + b[0] * a[1] + a[2] * b[3] - a[3] * b[2]);
  q[2] = alpha * (a[0] * b[2] + b[0] * a[2] + a[3] * b[1] - a[1] * b[3]);
  q[3] = alpha * (a[0] * b[3] + b[0] * a[3] + a[1] * b[2] - a[2] * b[1]);
}
__device__ void qrot(double *out, const double *qin, const double *v, bool conj) {
  const double q[4] = {qin[0], conj ? -qin[1] : qin[1], conj ? -qin[2] : qin[2], conj ? -qin[3] : qin[3]};
  const double qs2 = q[0] * q[0] - (q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  const double qd = q[1] * v[0] + q[2] * v[1] + q[3] * v[2];
  out[0] = qs2 * v[0] + 2.0 * (qd * q[1] + q[0] * (q[2] * v[2] - q[3] * v[1]));
  out[1] = qs2 * v[1] + 2.0 * (qd * q[2] + q[0] * (q[3] * v[0] - q[1] * v[2]));
  out[2] = qs2 * v[2] + 2.0 * (qd * q[3] + q[0] * (q[1] * v[1] - q[2] * v[0]));
}

__global__ void k_md_position(PartParams pp, icep_particle *p, int ab2) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= pp.np) return;
  icep_particle &q = p[n];
  const double dt = pp.dt, hdt = 0.5 * pp.dt;
  for (int d = 0; d < 3; d++) {
    const double dx = ab2 ? hdt * (3.0 * q.v[d] - q.v_old[d]) : dt * q.v[d];
    q.x_nopbc[d] += dx;
    q.x[d] += dx;
    q.x[d] = fmod(q.x[d] + pp.L[d], pp.L[d]);  // PBC (periodic_boundary.h:9-14)
  }
  if (pp.rotation) {
    double dq[4], qw[4];
    if (!ab2) {
      for (int a = 0; a < 4; a++) q.q_old[a] = q.q[a];
      qw[0] = 0.0; qw[1] = q.omega[0]; qw[2] = q.omega[1]; qw[3] = q.omega[2];
      qprod(dq, qw, q.q, 0.5);
      for (int a = 0; a < 4; a++) q.q[a] += dq[a] * dt;
    } else {
      double wb[3], wbo[3];
      qrot(wb, q.q, q.omega, true);
      qrot(wbo, q.q_old, q.omega_old, true);
      for (int d = 0; d < 3; d++) wb[d] = 3.0 * wb[d] - wbo[d];
      for (int a = 0; a < 4; a++) q.q_old[a] = q.q[a];
      qw[0] = 0.0; qw[1] = wb[0]; qw[2] = wb[1]; qw[3] = wb[2];
      qprod(dq, q.q, qw, 0.5);
      for (int a = 0; a < 4; a++) q.q[a] += dq[a] * hdt;
    }
    const double nrm = 1.0 / sqrt(q.q[0] * q.q[0] + q.q[1] * q.q[1] + q.q[2] * q.q[2] + q.q[3] * q.q[3]);
    for (int a = 0; a < 4; a++) q.q[a] *= nrm;
  }
}

__global__ void k_md_velocity(PartParams pp, icep_particle *p, int ab2) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= pp.np) return;
  icep_particle &q = p[n];
  const int s = q.spec;
  if (pp.g != 0.0) {  // Add_f_gravity (md_force.cxx:261-280)
    const double gf = pp.g * pp.rho * 4. / 3. * M_PI * (pp.radius * pp.radius) * pp.radius;
    q.fr[pp.g_direction] -= gf * (pp.mass_ratio[s] - 1.0);
  }
  double sf[3] = {0, 0, 0}, st[3] = {0, 0, 0};
  bool motor_on = false;
  for (int k = 0; k < pp.n_species; k++)
    if (pp.motor[k]) motor_on = true;
  if (motor_on && pp.motor[s]) {  // self_propulsion (particle_solver.cxx:94-107)
    qrot(sf, q.q, pp.jforce[s], false);
    qrot(st, q.q, pp.jtorque[s], false);
  }
  for (int d = 0; d < 3; d++) {
    q.v_old[d] = q.v[d];
    q.omega_old[d] = q.omega[d];
    if (!ab2) {
      const double a = pp.dt * pp.imass[s], b = pp.dt * pp.imoi[s];
      q.v[d] += a * (q.f_hydro[d] + q.fr[d] + sf[d]);
      q.omega[d] += b * (q.torque_hydro[d] + q.torque_r[d] + st[d]);
    } else {
      const double a = 0.5 * pp.dt * pp.imass[s], b = 0.5 * pp.dt * pp.imoi[s];
      q.v[d] += a * (2.0 * (q.f_hydro[d] + sf[d]) + q.fr[d] + q.fr_previous[d]);
      q.omega[d] += b * (2.0 * (q.torque_hydro[d] + st[d]) + q.torque_r[d] + q.torque_r_previous[d]);
    }
  }
  // reset_Forces (particle_solver.cxx:11-37)
  for (int d = 0; d < 3; d++) {
    q.fr_previous[d] = q.fr[d];
    q.fr[d] = 0.0;
    q.f_hydro_previous[d] = q.f_hydro[d];
    q.f_hydro[d] = 0.0;
    q.torque_r_previous[d] = q.torque_r[d];
    q.torque_r[d] = 0.0;
    q.torque_hydro_previous[d] = q.torque_hydro[d];
    q.torque_hydro[d] = 0.0;
  }
}

inline unsigned blocks_pts(const PartParams &pp) {
  return (unsigned)pp.np * div_up(pp.np_domain, TPB);
}

}  // namespace

template <typename R>
void scatter_profile(const PartParams &pp, const icep_particle *p, const int *sek, R *out, R *aux, int kind,
                     cudaStream_t s) {
  if (pp.np == 0) return;
  count_launch((double)pp.np * pp.np_domain * sizeof(R) * (aux ? 4.0 : 2.0));
  k_scatter_profile<R><<<blocks_pts(pp), TPB, 0, s>>>(pp, p, sek, out, aux, kind);
}
template <typename R>
void scatter_up(const PartParams &pp, const icep_particle *p, const int *sek, const R *phs, R *u0, R *u1, R *u2,
                cudaStream_t s) {
  if (pp.np == 0) return;
  count_launch((double)pp.np * pp.np_domain * sizeof(R) * 7.0);
  k_scatter_up<R><<<blocks_pts(pp), TPB, 0, s>>>(pp, p, sek, phs, u0, u1, u2);
}
template <typename R>
void scatter_normal(const PartParams &pp, const icep_particle *p, const int *sek, R *s0, R *s1, R *s2,
                    cudaStream_t s) {
  if (pp.np == 0) return;
  count_launch((double)pp.np * pp.np_domain * sizeof(R) * 6.0);
  k_scatter_normal<R><<<blocks_pts(pp), TPB, 0, s>>>(pp, p, sek, s0, s1, s2);
}
template <typename R>
void f_hydro(const PartParams &pp, icep_particle *p, const int *sek, const R *phs, const R *u0, const R *u1,
             const R *u2, bool copy_to_1, cudaStream_t s) {
  if (pp.np == 0) return;
  count_launch((double)pp.np * pp.np_domain * sizeof(R) * 4.0);
  k_f_hydro<R><<<pp.np, 256, 0, s>>>(pp, p, sek, phs, u0, u1, u2, copy_to_1 ? 1 : 0);
}

int lj_force(const PartParams &pp, icep_particle *p, int *work, int work_ints, int *pairs, int max_pairs,
             int *n_pairs, cudaStream_t s) {
  if (pp.np == 0) return ICEP_OK;
  CellGeom cg;
  const int cell_len = 16;
  for (int d = 0; d < 3; d++) cg.lc[d] = pp.N[d] / cell_len;
  cg.lcr = cell_len * pp.dx;
  const int ncell = cg.lc[0] * cg.lc[1] * cg.lc[2];
  if (ncell <= 0) return ICEP_ERR_UNSUPPORTED;
  if (work_ints < 2 * (ncell + 1) + pp.np) return ICEP_ERR_ARG;
  int *start = work, *fill = work + (ncell + 1), *list = work + 2 * (ncell + 1);
  count_launch((double)pp.np * sizeof(icep_particle));
  k_lj_cells<<<1, 1024, 0, s>>>(pp, cg, p, start, fill, list, ncell);
  count_launch(2.0 * pp.np * sizeof(icep_particle));
  k_lj_gather<<<div_up((long)pp.np * 32, 128), 128, 0, s>>>(pp, cg, p, start, list, pairs, max_pairs, n_pairs);
  return ICEP_OK;
}

void md_position(const PartParams &pp, icep_particle *p, bool ab2, cudaStream_t s) {
  if (pp.np == 0) return;
  count_launch(2.0 * pp.np * sizeof(icep_particle));
  k_md_position<<<div_up(pp.np, 128), 128, 0, s>>>(pp, p, ab2 ? 1 : 0);
}
void lj_params_from(const icep_params &p, PartParams &pp) {
  pp.lj_eps = p.lj_epsilon;
  pp.lj_dia = 2.0 * pp.radius;
  pp.lj_powers = p.lj_powers;
  double arc;
  if (p.lj_truncate > 0) {
    arc = (p.lj_powers == 0) ? pow(2., 1. / 6.) : (p.lj_powers == 1) ? pow(2., 1. / 12.) : pow(2., 1. / 18.);
  } else if (p.lj_truncate == 0) {
    int nmin = pp.N[0] < pp.N[1] ? pp.N[0] : pp.N[1];
    nmin = nmin < pp.N[2] ? nmin : pp.N[2];
    arc = nmin * pp.dx * .5 / pp.lj_dia;
    if (arc > 2.5) arc = 2.5;
  } else {
    arc = 0.;
  }
  pp.r_cutoff = arc * pp.lj_dia;
  pp.lj_on = p.lj_truncate >= 0;
}
void md_velocity(const PartParams &pp, icep_particle *p, bool ab2, cudaStream_t s) {
  if (pp.np == 0) return;
  count_launch(2.0 * pp.np * sizeof(icep_particle));
  k_md_velocity<<<div_up(pp.np, 128), 128, 0, s>>>(pp, p, ab2 ? 1 : 0);
}

template void scatter_profile<double>(const PartParams &, const icep_particle *, const int *, double *, double *, int, cudaStream_t);
template void scatter_profile<float>(const PartParams &, const icep_particle *, const int *, float *, float *, int, cudaStream_t);
template void scatter_up<double>(const PartParams &, const icep_particle *, const int *, const double *, double *, double *, double *, cudaStream_t);
template void scatter_up<float>(const PartParams &, const icep_particle *, const int *, const float *, float *, float *, float *, cudaStream_t);
template void scatter_normal<double>(const PartParams &, const icep_particle *, const int *, double *, double *, double *, cudaStream_t);
template void scatter_normal<float>(const PartParams &, const icep_particle *, const int *, float *, float *, float *, cudaStream_t);
template void f_hydro<double>(const PartParams &, icep_particle *, const int *, const double *, const double *, const double *, const double *, bool, cudaStream_t);
template void f_hydro<float>(const PartParams &, icep_particle *, const int *, const float *, const float *, const float *, const float *, bool, cudaStream_t);

}  // namespace icep
