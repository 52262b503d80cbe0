// crg_rods.cu -- one chili step for RodMechanics + RodInteraction<MorsePotential> rods.
//
// The physics: for every candidate rod b in the 3^D neighbourhood of rod a's voxel (keyed
// by centroid, bacterial_rods.rs:550-554) the step builds the two matrices
// RodInteraction::calculate_force_between produces (bacterial_rods.rs:292-336):
//   own_a(b): a's vertices against b's segments, force on a's vertices (a.calc(a, b).0)
//   ext_a(b): b's vertices against a's segments, force distributed on a's vertices
//             with weights (1 - t, t)                                   (b.calc(b, a).1)
// and adds them scaled by one half in chili's order:
//   same voxel, b before a in the voxel: ext then own   (update_mechanics.rs:193-199,
//   same voxel, b after a:                own then ext    a is the first or second cell)
//   neighbour voxel, same subdomain:      own only        (:205-220; the ext half is dropped)
//   neighbour voxel, other subdomain:     own in step 2, after every local term, then ext in
//                                         step 3, summed per voxel first (:285-382)
// Vertex/segment evaluations whose FP32 distance exceeds the cutoff plus margin are zero
// in FP64 as well and are skipped; the rest are evaluated in FP64 in the reference's
// operation order.  RodMechanics::calculate_increment (bacterial_rods.rs:157-213), the
// solver, apply_boundary (:489-534) and the centroid voxel key follow.
//
// The FP64 kernels (both produce identical bits): the default path lists every rod's passes
// (one pass = own_a(b) or ext_a(b)) in chili's order (k_rods_walk), evaluates them one pass
// per lane with the survivors of the warp's 32 passes in full FP64 batches (k_rods_passq),
// computes the curvature forces per angle (k_rods_bend) and adds up each rod's passes in
// order before the mechanics and the solver (k_rods_update); k_rods_step is the same
// evaluation with one rod per thread (CRG_OPT_KERNEL_VARIANT 1, and the fallback when the
// pass list overflows).  With several subdomains the order is that of chili's steps 1, 2
// and 3 (k_rods_step explains it).
#include "crg_internal.cuh"
#include "crg_kernels.h"

namespace crg {

namespace {

// FP64 comparisons evaluated on the bit patterns with integer instructions, leaving the FP64
// pipe (the bottleneck of these kernels) to arithmetic.  Same results as the FP64
// comparisons for every input, NaN, signed zeros and infinities included.
__device__ __forceinline__ bool lt_zero(double x) {  // x < 0.0
  const long long b = __double_as_longlong(x);
  const unsigned long long mag = (unsigned long long)b & 0x7fffffffffffffffull;
  return b < 0 && mag - 1ull < 0x7ff0000000000000ull;  // negative, non-zero, not NaN
}
__device__ __forceinline__ bool gt_one(double x) {  // x > 1.0
  const long long b = __double_as_longlong(x);
  return b > 0x3ff0000000000000ll && b <= 0x7ff0000000000000ll;  // positive, not NaN
}

// nearest_point_from_point_to_line (interaction.rs:497-509): returns q and t.
template <int D>
__device__ __forceinline__ void nearest_point_f64(const double *p, const double *l0,
                                                  const double *l1, double *q, double &t) {
  double ab[D], ap[D];
#pragma unroll
  for (int c = 0; c < D; ++c) {
    ab[c] = dsub(l1[c], l0[c]);
    ap[c] = dsub(p[c], l0[c]);
  }
  double dot = dmul(ab[0], ap[0]);
  double nsq = dmul(ab[0], ab[0]);
#pragma unroll
  for (int c = 1; c < D; ++c) {
    dot = dadd(dot, dmul(ab[c], ap[c]));
    nsq = dadd(nsq, dmul(ab[c], ab[c]));
  }
  t = ddiv(dot, nsq);
  if (lt_zero(t)) t = 0.0;
  if (gt_one(t)) t = 1.0;
  const double omt = dsub(1.0, t);
#pragma unroll
  for (int c = 0; c < D; ++c) q[c] = dadd(dmul(l0[c], omt), dmul(l1[c], t));
}

// nearest_point_f64 for segment sy of rod r with the segment's l1 - l0, squared norm and its
// reciprocal taken from P.seg (k_rods_walk computes them with nearest_point_f64's operations)
// and t = dot / nsq from div_rn_recip: the same q and t, bit for bit, with no division.
template <int D>
__device__ __forceinline__ void nearest_point_seg(const double *p, const double *l0,
                                                  const double *l1, const double *seg,
                                                  int64_t cap, double *q, double &t) {
  double ab[D], ap[D];
#pragma unroll
  for (int c = 0; c < D; ++c) {
    ab[c] = seg[c * cap];
    ap[c] = dsub(p[c], l0[c]);
  }
  double dot = dmul(ab[0], ap[0]);
#pragma unroll
  for (int c = 1; c < D; ++c) dot = dadd(dot, dmul(ab[c], ap[c]));
  t = div_rn_recip(dot, seg[D * cap], seg[(D + 1) * cap]);
  if (lt_zero(t)) t = 0.0;
  if (gt_one(t)) t = 1.0;
  const double omt = dsub(1.0, t);
#pragma unroll
  for (int c = 0; c < D; ++c) q[c] = dadd(dmul(l0[c], omt), dmul(l1[c], t));
}

// Full (unhalved) Morse force on `own` from the point `ext` (interaction.rs:151-182).
template <int D>
__device__ __forceinline__ bool morse_full_f64(const double *own, const double *ext,
                                               const SimDev &S, double *f) {
  double z[D];
#pragma unroll
  for (int c = 0; c < D; ++c) z[c] = dsub(own[c], ext[c]);
  double n2 = dmul(z[0], z[0]);
#pragma unroll
  for (int c = 1; c < D; ++c) n2 = dadd(n2, dmul(z[c], z[c]));
  const double dist = __dsqrt_rn(n2);
  // dist > cutoff || dist == 0.0 (dist is +0, positive or NaN; NaN carries on)
  const long long db = __double_as_longlong(dist);
  const unsigned long long mag = (unsigned long long)db & 0x7fffffffffffffffull;
  if (mag <= 0x7ff0000000000000ull && (mag == 0ull || db > S.cutoff_bits)) return false;
  const double e = exp(dmul(S.mrs_nstiff, dsub(dist, S.mrs_r)));
  const double force = dmul(dmul(S.mrs_k, e), dsub(1.0, e));
  const double y = __drcp_rn(dist);  // z[c] / dist for every c from one reciprocal
#pragma unroll
  for (int c = 0; c < D; ++c) f[c] = dmul(div_rn_recip(z[c], dist, y), force);
  return true;
}

// Squared FP32 distance from p to the segment (l0, l1) (prefilter only).
template <int D>
__device__ __forceinline__ float seg_dist2_f32(const float *p, const float *l0,
                                               const float *l1) {
  float ab[D], ap[D];
  float dot = 0.f, nsq = 0.f;
#pragma unroll
  for (int c = 0; c < D; ++c) {
    ab[c] = l1[c] - l0[c];
    ap[c] = p[c] - l0[c];
    dot = fmaf(ab[c], ap[c], dot);
    nsq = fmaf(ab[c], ab[c], nsq);
  }
  float t = (nsq > 0.f) ? __fdividef(dot, nsq) : 0.f;
  t = fminf(fmaxf(t, 0.f), 1.f);
  float d2 = 0.f;
#pragma unroll
  for (int c = 0; c < D; ++c) {
    const float w = fmaf(-t, ab[c], ap[c]);
    d2 = fmaf(w, w, d2);
  }
  return d2;
}

// One half of the pair interaction.  is_ext = false: own_a(b) (a's vertices X against
// b's segments Y, force on X's rows).  is_ext = true: ext_a(b) (b's vertices against a's
// segments, -f distributed on a's rows j, j+1 with weights 1-t, t).  Per-thread operands
// live in shared memory ([component][thread]) so the loops can run over vertices without
// spilling; the accumulated matrix is left in sT.  Returns whether any term was non-zero.
template <int D, int NV, int B>
__device__ __forceinline__ bool rod_pass(bool is_ext, const double *posb, int64_t cap,
                                         const SimDev &S, float thr2, const double (*sPa)[B],
                                         double (*sT)[B], const float (*sOa)[B],
                                         const float (*sOb)[B], int tid) {
  constexpr int NC = NV * D;
#pragma unroll
  for (int k = 0; k < NC; ++k) sT[k][tid] = 0.0;
  bool any = false;
#pragma unroll 1
  for (int vx = 0; vx < NV; ++vx) {
#pragma unroll 1
    for (int sy = 0; sy + 1 < NV; ++sy) {
      float p32[D], l0f[D], l1f[D];
#pragma unroll
      for (int c = 0; c < D; ++c) {
        p32[c] = is_ext ? sOb[vx * D + c][tid] : sOa[vx * D + c][tid];
        l0f[c] = is_ext ? sOa[sy * D + c][tid] : sOb[sy * D + c][tid];
        l1f[c] = is_ext ? sOa[(sy + 1) * D + c][tid] : sOb[(sy + 1) * D + c][tid];
      }
      if (seg_dist2_f32<D>(p32, l0f, l1f) > thr2) continue;
      double p[D], l0[D], l1[D];
#pragma unroll
      for (int c = 0; c < D; ++c) {
        if (is_ext) {
          p[c] = posb[(vx * D + c) * cap];
          l0[c] = sPa[sy * D + c][tid];
          l1[c] = sPa[(sy + 1) * D + c][tid];
        } else {
          p[c] = sPa[vx * D + c][tid];
          l0[c] = posb[(sy * D + c) * cap];
          l1[c] = posb[((sy + 1) * D + c) * cap];
        }
      }
      double q[D], t, f[D];
      nearest_point_f64<D>(p, l0, l1, q, t);
      if (!morse_full_f64<D>(p, q, S, f)) continue;
      any = true;
      if (!is_ext) {
#pragma unroll
        for (int c = 0; c < D; ++c) sT[vx * D + c][tid] = dadd(sT[vx * D + c][tid], f[c]);
      } else {
        const double omt = dsub(1.0, t);
#pragma unroll
        for (int c = 0; c < D; ++c) {
          const double fe = -f[c];
          sT[sy * D + c][tid] = dadd(sT[sy * D + c][tid], dmul(fe, omt));
          sT[(sy + 1) * D + c][tid] = dadd(sT[(sy + 1) * D + c][tid], dmul(fe, t));
        }
      }
    }
  }
  return any;
}

template <int NC, int B>
__device__ __forceinline__ void add_half(double *acc, const double (*sT)[B], int tid) {
#pragma unroll
  for (int k = 0; k < NC; ++k) acc[k] = dadd(acc[k], dmul(sT[k][tid], 0.5));
}

template <int D>
__device__ __forceinline__ double norm_f64(const double *v) {
  double n2 = dmul(v[0], v[0]);
#pragma unroll
  for (int c = 1; c < D; ++c) n2 = dadd(n2, dmul(v[c], v[c]));
  return __dsqrt_rn(n2);
}

// RodMechanics::calculate_increment (bacterial_rods.rs:157-213), the solver, apply_boundary
// (:489-534) and the next voxel key from the centroid, for rod i with interaction force acc.
// Curvature force of angle s of a rod (RodMechanics::calculate_increment,
// bacterial_rods.rs:185-206): f[c] for the vertices s, s + 1, s + 2 from the segments
// d1 = x_s - x_{s+1} and d2 = x_{s+1} - x_{s+2}.
template <int D>
__device__ __forceinline__ void bend_force(const SimDev &S, const double *c1, const double *c2,
                                           double *f) {
  double prod = dmul(c1[0], c2[0]);
#pragma unroll
  for (int c = 1; c < D; ++c) prod = dadd(prod, dmul(c1[c], c2[c]));
  const double n1 = norm_f64<D>(c1), n2 = norm_f64<D>(c2);
  // zero tests and the clamp to [-1, 1] on the integer pipe (same results, NaN included)
  auto is_zero = [](double x) { return (__double_as_longlong(x) & 0x7fffffffffffffffll) == 0; };
  double angle = 0.0;
  if (!(is_zero(n1) || is_zero(n2))) {
    double cang = ddiv(prod, dmul(n1, n2));
    if (f64_lt_key(cang, -0x3ff0000000000000ll)) cang = -1.0;  // key of -1.0
    if (f64_gt_key(cang, 0x3ff0000000000000ll)) cang = 1.0;    // key of 1.0
    angle = acos(cang);
  }
  double fd[D];
#pragma unroll
  for (int c = 0; c < D; ++c) fd[c] = dsub(c1[c], c2[c]);
  const double fdn = norm_f64<D>(fd);
  const double tn = tan(dmul(0.5, angle));
  const bool fd_zero = is_zero(fdn);
#pragma unroll
  for (int c = 0; c < D; ++c) {
    const double fdir = !fd_zero ? ddiv(fd[c], fdn) : fd[c];
    f[c] = dmul(dmul(dmul(fdir, 2.0), S.rigidity), tn);
  }
}

// Mixed precision: the same curvature force with tan(angle / 2) from the half-angle
// identity tan(theta / 2) = |c1 x c2| / (|c1| |c2| + c1 . c2), still in FP64 but without
// acos and tan (about 40 % of the FP64 work of bend_force).  It agrees with the reference's
// acos / tan to a few FP64 ulps for angles away from 0 and pi; near a straight rod the
// reference's acos of a rounded cosine carries an absolute error up to ~1.5e-8 rad that the
// cross product does not share (far inside the mixed path's error).  A rod folded back
// exactly (zero denominator) takes tan(pi / 2) as the reference's FP64 evaluates it.
template <int D>
__device__ __forceinline__ void bend_force_halfangle(const SimDev &S, const double *c1,
                                                     const double *c2, double *f) {
  double prod = dmul(c1[0], c2[0]);
#pragma unroll
  for (int c = 1; c < D; ++c) prod = dadd(prod, dmul(c1[c], c2[c]));
  const double n1 = norm_f64<D>(c1), n2 = norm_f64<D>(c2);
  double cr;
  if (D == 2) {
    cr = fabs(dsub(dmul(c1[0], c2[1]), dmul(c1[1], c2[0])));
  } else {
    const double x = dsub(dmul(c1[1], c2[2]), dmul(c1[2], c2[1]));
    const double y = dsub(dmul(c1[2], c2[0]), dmul(c1[0], c2[2]));
    const double z = dsub(dmul(c1[0], c2[1]), dmul(c1[1], c2[0]));
    cr = __dsqrt_rn(dadd(dadd(dmul(x, x), dmul(y, y)), dmul(z, z)));
  }
  auto is_zero = [](double v) { return (__double_as_longlong(v) & 0x7fffffffffffffffll) == 0; };
  double tn = 0.0;  // zero-length segments: angle 0
  if (!(is_zero(n1) || is_zero(n2))) {
    const double den = dadd(dmul(n1, n2), prod);
    if (den != den)
      tn = den;  // NaN coordinates stay NaN
    else if (f64_gt_key(den, 0))
      tn = ddiv(cr, den);
    else
      tn = 1.633123935319537e16;  // tan(0.5 * acos(-1.0)) in FP64
  }
  double fd[D];
#pragma unroll
  for (int c = 0; c < D; ++c) fd[c] = dsub(c1[c], c2[c]);
  const double fdn = norm_f64<D>(fd);
  const bool fd_zero = is_zero(fdn);
#pragma unroll
  for (int c = 0; c < D; ++c) {
    const double fdir = !fd_zero ? ddiv(fd[c], fdn) : fd[c];
    f[c] = dmul(dmul(dmul(fdir, 2.0), S.rigidity), tn);
  }
}

// CartesianSubDomainRods::apply_boundary (bacterial_rods.rs:489-534) on a rod's updated
// vertices, then its next voxel key from the centroid row_sum / nrows (:550-554); writes
// the next state at `slot` and counts the key.  `key`: the voxel the rod stays in when the
// new index falls outside the grid; `id`: the identifier a BoundaryError reports.
template <int D, int NV>
__device__ __forceinline__ void rod_finish(const PackArgs &P, const SimDev &S, uint32_t slot,
                                           uint32_t key, uint64_t id, double *np, double *nvl) {
  constexpr int NC = NV * D;
  const int64_t cap = P.cap;
  bool inside = true;
#pragma unroll
  for (int s = 0; s < NV; ++s)
#pragma unroll
    for (int c = 0; c < D; ++c) {
      double &p = np[s * D + c];
      double &u = nvl[s * D + c];
      if (f64_lt_key(p, S.min_key[c])) {  // p < min, on the integer pipe
        p = dsub(dmul(S.min[c], 2.0), p);
        u = fabs(u);
      }
      if (f64_gt_key(p, S.max_key[c])) {  // p > max
        p = dsub(dmul(S.max[c], 2.0), p);
        u = -fabs(u);
      }
    }
#pragma unroll
  for (int k = 0; k < NC; ++k)
    if (f64_lt_key(np[k], S.min_key[k % D]) || f64_gt_key(np[k], S.max_key[k % D]))
      inside = false;
  if (!inside) set_status(P.status, CRG_EBOUNDARY, id, *P.step_ctr + 1, S.sim_index);
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    P.npos[k * cap + slot] = np[k];
    P.nvel[k * cap + slot] = nvl[k];
  }
  double cen[D];
#pragma unroll
  for (int c = 0; c < D; ++c) {
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < NV; ++q) s = dadd(s, np[q * D + c]);
    cen[c] = ddiv(s, (double)NV);
  }
  uint32_t plain;
  uint32_t nk = key;
  if (voxel_of<D>(S, cen, plain) == 0) nk = S.voxel_off + plain;
  if (nk - S.voxel_off >= S.n_vox) {
    invariant_failed(P.status, kSiteNextKey, slot);
    nk = key;
  }
  P.nkey[slot] = nk;
  atomicAdd(&P.count[nk], 1u);
}

// BEND: the curvature forces were computed by k_rods_bend (P.bend), else they are computed
// here.  Same values, same order of additions either way.  CYC: cell cycle off (0), on (1)
// or decided by P.dflag at run time (-1).
template <int D, int NV, bool BEND = false, int CYC = -1>
__device__ __forceinline__ void rod_update(const PackArgs &P, const SimDev &S, uint32_t i,
                                           uint32_t key, const double *pa, const double *acc) {
  const bool cyc = (CYC < 0) ? (P.dflag != nullptr) : (CYC == 1);
  constexpr int NC = NV * D;
  const int64_t cap = P.cap;
  if (P.dbg_force) {
#pragma unroll
    for (int k = 0; k < NC; ++k) P.dbg_force[k * cap + i] = acc[k];
  }
  double va[NC];
#pragma unroll
  for (int k = 0; k < NC; ++k) va[k] = P.vel[k * cap + i];
  const double l0 = cyc ? P.slen[i] : S.spring_length;  // RodMechanics::spring_length
  double tf[NC];
#pragma unroll
  for (int k = 0; k < NC; ++k) tf[k] = acc[k];
  double dist[NV - 1][D];
#pragma unroll
  for (int s = 0; s + 1 < NV; ++s)
#pragma unroll
    for (int c = 0; c < D; ++c) dist[s][c] = dsub(pa[s * D + c], pa[(s + 1) * D + c]);
  // springs
#pragma unroll
  for (int s = 0; s + 1 < NV; ++s) {
    const double nrm = norm_f64<D>(dist[s]);
    if ((__double_as_longlong(nrm) & 0x7fffffffffffffffll) != 0) {  // nrm != 0.0
#pragma unroll
      for (int c = 0; c < D; ++c) {
        const double dir = ddiv(dist[s][c], nrm);
        const double fi = dmul(dmul(-dir, S.spring_tension), dsub(nrm, l0));
        tf[s * D + c] = dadd(tf[s * D + c], half_exact(fi));  // x * 0.5 on the bit pattern
        tf[(s + 1) * D + c] = dadd(tf[(s + 1) * D + c], half_exact(-fi));
      }
    }
  }
  // curvature: Matrix::angle = acos(clamp(dot / (|a| |b|), -1, 1)), 0 for zero length
#pragma unroll
  for (int s = 0; s + 2 < NV; ++s) {
    double fb[D];
    if (BEND) {
#pragma unroll
      for (int c = 0; c < D; ++c) fb[c] = P.bend[(s * D + c) * cap + i];
    } else {
      bend_force<D>(S, dist[s], dist[s + 1], fb);
    }
#pragma unroll
    for (int c = 0; c < D; ++c) {
      const double f = fb[c];
      tf[s * D + c] = dadd(tf[s * D + c], half_exact(-f));
      tf[(s + 1) * D + c] = dadd(tf[(s + 1) * D + c], f);
      tf[(s + 2) * D + c] = dadd(tf[(s + 2) * D + c], half_exact(-f));
    }
  }
  // damping
#pragma unroll
  for (int k = 0; k < NC; ++k) tf[k] = dsub(tf[k], dmul(va[k], S.damping));

  // get_random_contribution times dt (bacterial_rods.rs:215-240): dx_rand = N(0, sqrt(dt))
  // * 2^-2 * D / dt per vertex coordinate, dv_rand = 0; zero when D = 0.
  const double dt = S.dt;
  double rx[NC];
#pragma unroll
  for (int k = 0; k < NC; ++k) rx[k] = 0.0;
  if (S.stochastic) {
    double z[NC];
    stream_normals_ool<NC>(S.rng_seed, (uint64_t)(*P.step_ctr + S.step_base), P.id[i], z);
    const double sd = __dsqrt_rn(dt);
#pragma unroll
    for (int k = 0; k < NC; ++k)
      rx[k] = dmul(ddiv(dmul(dmul(dadd(0.0, dmul(sd, z[k])), 0.25), S.diffusion), dt), dt);
  }
  // solver (dx = v, dv = total force)
  double np[NC], nvl[NC];
  // x + 0.0 (dv_rand, and dx_rand without diffusion) is plus_zero(x) exactly
  if (S.order == 1 && !S.stochastic) {
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      np[k] = plus_zero(dadd(dmul(va[k], dt), pa[k]));
      nvl[k] = plus_zero(dadd(dmul(tf[k], dt), va[k]));
    }
  } else if (S.order == 1) {
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      np[k] = dadd(dadd(dmul(va[k], dt), pa[k]), rx[k]);
      nvl[k] = plus_zero(dadd(dmul(tf[k], dt), va[k]));
    }
  } else {
    const bool ab3 = (S.order == 3) && P.hmeta[i];
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      if (ab3) {
        const double f0 = 23.0 / 12.0, f1 = -16.0 / 12.0, f2 = 5.0 / 12.0;
        const double px = P.hist[k * cap + i], pv = P.hist[(NC + k) * cap + i];
        np[k] = dadd(dadd(dmul(dadd(dmul(va[k], f0), dadd(dmul(px, f1), dmul(va[k], f2))), dt),
                          pa[k]), rx[k]);
        nvl[k] = plus_zero(dadd(dmul(dadd(dmul(tf[k], f0), dadd(dmul(pv, f1), dmul(tf[k], f2))), dt),
                                va[k]));
      } else {
        const double f0 = 3.0 / 2.0, f1 = -1.0 / 2.0;
        np[k] = dadd(dadd(dmul(dadd(dmul(va[k], f0), dmul(va[k], f1)), dt), pa[k]), rx[k]);
        nvl[k] = plus_zero(dadd(dmul(dadd(dmul(tf[k], f0), dmul(tf[k], f1)), dt), va[k]));
      }
      P.nhist[k * cap + i] = va[k];
      P.nhist[(NC + k) * cap + i] = tf[k];
    }
    P.nhmeta[i] = 1;
  }

  // Cell cycle (bacterial_rods/src/main.rs:66-98), run after local_mechanics_update as the
  // macro orders the local functions (run_sim.rs:258-283): react_to_neighbors sets the
  // growth rate from this step's neighbour count, update_cycle grows the spring length and
  // flags a division.  A dividing rod leaves reflection and voxel key to k_rods_divide:
  // chili divides (update_cell_cycle_4) before it applies the boundary.
  if (cyc) {
    const uint32_t nn = P.nsense[i];
    double g = S.cyc_growth;
    if (nn > 0u) {
      const double x = ddiv(dmul(S.cyc_growth, dsub(S.cyc_sat, (double)nn)), S.cyc_sat);
      g = (x > 0.0) ? x : 0.0;  // f64::max(x, 0.0): 0 for NaN and negative rates
    }
    const double l1 = dadd(l0, dmul(g, dt));
    P.ngrate[i] = g;
    P.nslen[i] = l1;
    P.nparent[i] = P.parent[i];
    const bool divides = l1 > S.cyc_div_len;
    P.dflag[i] = divides ? 1u : 0u;
    if (divides) {
#pragma unroll
      for (int k = 0; k < NC; ++k) {
        P.npos[k * cap + i] = np[k];
        P.nvel[k * cap + i] = nvl[k];
      }
      P.nkey[i] = key;
      P.nid[i] = P.id[i];
      return;
    }
  }
  rod_finish<D, NV>(P, S, i, key, P.id[i], np, nvl);
  P.nid[i] = P.id[i];
}

// ---------------------------------------------------------------------------------------
// Mixed precision (CRG_PREC_MIXED).  The pair arithmetic of RodInteraction -- nearest point
// on the segment and the Morse force -- runs in FP32; springs, curvature (through the
// half-angle identity, bend_force_halfangle), damping, the solver, the boundary and the
// state stay FP64 (k_rods_bend, k_rods_update).  FP32 loses
// nothing in the coordinate differences: every coordinate x is carried as hi = (float)x
// and lo = (float)(x - hi), and differences are formed as hi + lo pairs (diff_hl), exact
// to ~2^-48 |x| however far from the origin the rods are.  Whether a
// vertex/segment pair interacts is decided as on the FP64 path (mixed_item), so no pair
// switches on or off.  Sums are FP32 with Kahan compensation: per pass matrix row, over a
// rod's passes in chili's order (the step-3 ext passes of a box summed first, as on the
// FP64 path), and converted to FP64 once per rod.  Every FP32 operation uses an explicit
// rounding intrinsic, so the pass kernel and the rod-level fallback produce the same bits.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void kahan_add_f(float &s, float &c, float x) {
  const float y = __fsub_rn(x, c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
}

// FP32 compensated sums of the NC entries of a force matrix.
template <int NC>
struct KahanRows {
  float s[NC], c[NC];
  __device__ __forceinline__ void set(const float *x, int64_t stride) {
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      s[k] = x[k * stride];
      c[k] = 0.f;
    }
  }
  __device__ __forceinline__ void add(const float *x, int64_t stride) {
#pragma unroll
    for (int k = 0; k < NC; ++k) kahan_add_f(s[k], c[k], x[k * stride]);
  }
  __device__ __forceinline__ float value(int k) const { return __fsub_rn(s[k], c[k]); }
  __device__ __forceinline__ void add(const KahanRows &g) {
#pragma unroll
    for (int k = 0; k < NC; ++k) kahan_add_f(s[k], c[k], g.value(k));
  }
};

// Vertex vx of a rod (FP64 positions pp) against segment sy of another (ps) in FP64, as the
// FP64 path evaluates it: the full force on the vertex and t.  Out of line: rare.
template <int D>
__device__ __noinline__ bool item_f64(int vx, int sy, const double *pp, const double *ps,
                                      int64_t cap, const SimDev &S, double *f, double &t) {
  double p[D], l0[D], l1[D], q[D];
#pragma unroll
  for (int c = 0; c < D; ++c) {
    p[c] = pp[(vx * D + c) * cap];
    l0[c] = ps[(sy * D + c) * cap];
    l1[c] = ps[((sy + 1) * D + c) * cap];
  }
  nearest_point_f64<D>(p, l0, l1, q, t);
  return morse_full_f64<D>(p, q, S, f);
}

// Whether vertex vx and segment sy interact, decided from the FP64 distance exactly as the
// FP64 path decides it (out of line: rare).
template <int D>
__device__ __noinline__ bool interacts_f64(int vx, int sy, const double *pp, const double *ps,
                                           int64_t cap, const SimDev &S) {
  double p[D], l0[D], l1[D], q[D], t;
#pragma unroll
  for (int c = 0; c < D; ++c) {
    p[c] = pp[(vx * D + c) * cap];
    l0[c] = ps[(sy * D + c) * cap];
    l1[c] = ps[((sy + 1) * D + c) * cap];
  }
  nearest_point_f64<D>(p, l0, l1, q, t);
  double n2 = 0.0;
#pragma unroll
  for (int c = 0; c < D; ++c) {
    const double z = dsub(p[c], q[c]);
    n2 = (c == 0) ? dmul(z, z) : dadd(n2, dmul(z, z));
  }
  const double dist = __dsqrt_rn(n2);
  const long long db = __double_as_longlong(dist);
  const unsigned long long mag = (unsigned long long)db & 0x7fffffffffffffffull;
  return !(mag <= 0x7ff0000000000000ull && (mag == 0ull || db > S.cutoff_bits));
}

// (a.x + a.y) - (b.x + b.y) for hi / lo coordinates as an unevaluated sum hi + lo: hi the
// FP32 difference of the hi parts, lo its exact rounding error (Knuth's TwoSum) plus the
// difference of the lo parts, so hi + lo is the difference to ~2^-48 of the coordinates.
__device__ __forceinline__ void diff_hl(float2 a, float2 b, float &hi, float &lo) {
  const float nb = -b.x;
  const float s = __fadd_rn(a.x, nb);
  const float bv = __fsub_rn(s, a.x);
  const float err = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bv)), __fsub_rn(nb, bv));
  hi = s;
  lo = __fadd_rn(err, __fsub_rn(a.y, b.y));
}

// One vertex/segment item in FP32: vertex vx of rod p (hi / lo coordinates hp, FP64 pp)
// against segment sy of rod s (hs, ps).  Returns false when the pair does not interact,
// else the force f on the vertex and t.  nearest_point_from_point_to_line and
// calculate_morse_interaction (interaction.rs:497-509, 151-182).
// The vertex-to-segment vector z must be accurate relative to its own length, which for
// crossing rods is far below the segment length: the differences x - l0 and l1 - l0 are
// carried as hi + lo pairs, z = (x - l0) - t (l1 - l0) is formed from them, and for an
// interior nearest point one projection step removes the along-segment error that the
// FP32 t leaves in z.  Then the direction of the force is accurate to a few FP32 ulps and
// its magnitude to the FP32 distance.  A pair whose FP32 distance lies within mix_band_f of
// the cutoff or mix_zero_f of zero is decided from the FP64 distance; a NaN
// distance (NaN or infinite coordinates, a degenerate segment) or a force beyond the FP32
// range takes the FP64 item.
template <int D>
__device__ __forceinline__ bool mixed_item(int vx, int sy, const float2 *hp, const float2 *hs,
                                           const double *pp, const double *ps, int64_t cap,
                                           const SimDev &S, float *f, float &t) {
  float abh[D], abl[D], aph[D], apl[D], ab[D], dot = 0.f, nsq = 0.f;
#pragma unroll
  for (int c = 0; c < D; ++c) {
    const float2 x = hp[(vx * D + c) * cap];
    const float2 l0 = hs[(sy * D + c) * cap];
    const float2 l1 = hs[((sy + 1) * D + c) * cap];
    diff_hl(l1, l0, abh[c], abl[c]);
    diff_hl(x, l0, aph[c], apl[c]);
    ab[c] = __fadd_rn(abh[c], abl[c]);
    dot = __fmaf_rn(ab[c], __fadd_rn(aph[c], apl[c]), dot);
    nsq = __fmaf_rn(ab[c], ab[c], nsq);
  }
  t = __fdiv_rn(dot, nsq);
  const bool interior = t > 0.f && t < 1.f;  // false for NaN
  t = t < 0.f ? 0.f : t;                      // NaN stays NaN, as in FP64
  t = t > 1.f ? 1.f : t;
  float z[D];
#pragma unroll
  for (int c = 0; c < D; ++c)
    z[c] = __fadd_rn(__fmaf_rn(-t, abh[c], aph[c]), __fmaf_rn(-t, abl[c], apl[c]));
  if (interior) {  // z is then short: its component along the segment is t's error
    float zd = 0.f;
#pragma unroll
    for (int c = 0; c < D; ++c) zd = __fmaf_rn(z[c], ab[c], zd);
    const float dt = __fdiv_rn(zd, nsq);
    t = __fadd_rn(t, dt);
#pragma unroll
    for (int c = 0; c < D; ++c) z[c] = __fmaf_rn(-dt, ab[c], z[c]);
  }
  float d2 = 0.f;
#pragma unroll
  for (int c = 0; c < D; ++c) d2 = __fmaf_rn(z[c], z[c], d2);
  if (d2 == d2) {
    const float dist = __fsqrt_rn(d2);
    if (fabsf(__fsub_rn(dist, S.cutoff_f)) <= S.mix_band_f || dist <= S.mix_zero_f) {
      if (!interacts_f64<D>(vx, sy, pp, ps, cap, S)) return false;
    } else if (dist > S.cutoff_f) {
      return false;
    }
    const float e = expf(__fmul_rn(S.mrs_nstiff_f, __fsub_rn(dist, S.mrs_r_f)));
    const float force = __fmul_rn(__fmul_rn(S.mrs_k_f, e), __fsub_rn(1.f, e));
    if (fabsf(force) <= 3.0e38f && dist > 0.f) {  // finite, and a direction to scale
      const float sc = __fdiv_rn(force, dist);
#pragma unroll
      for (int c = 0; c < D; ++c) f[c] = __fmul_rn(z[c], sc);
      return true;
    }
  }
  double f64[D], t64;
  if (!item_f64<D>(vx, sy, pp, ps, cap, S, f64, t64)) return false;
#pragma unroll
  for (int c = 0; c < D; ++c) f[c] = __double2float_rn(f64[c]);
  t = __double2float_rn(t64);
  return true;
}

// M / 2 of one pass in mixed precision, to out[(row * D + c) * stride].  is_ext = false:
// own_a(b), a's vertices against b's segments, row vx collecting the force of items
// (vx, 0..NV-2); true: ext_a(b), b's vertices against a's segments, row r collecting
// -f (1 - t) of items (vx, r) and -f t of items (vx, r - 1).  The FP32 prefilter on the
// offsets (oa, ob: a's and b's in a's voxel frame) marks the items to evaluate; own and
// ext passes run the same loop (groups of items sharing a row) so a warp with both kinds
// does not split.  ha / hb, pa / pb: hi / lo and FP64 coordinates of a and b (stride cap).
template <int D, int NV>
__device__ __forceinline__ void mixed_pass(bool is_ext, const float *oa, const float *ob,
                                           const float2 *ha, const float2 *hb,
                                           const double *pa, const double *pb, int64_t cap,
                                           const SimDev &S, float thr2, float *out,
                                           int64_t stride) {
  constexpr int NE = NV - 1;
  // survivor bit of item (vx, sy): own vx * NE + sy (groups by vertex), ext sy * NV + vx
  // (groups by segment)
  uint64_t mask = 0;
#pragma unroll
  for (int vx = 0; vx < NV; ++vx)
#pragma unroll
    for (int sy = 0; sy < NE; ++sy) {
      float p32[D], l0[D], l1[D];
#pragma unroll
      for (int c = 0; c < D; ++c) {
        p32[c] = is_ext ? ob[vx * D + c] : oa[vx * D + c];
        l0[c] = is_ext ? oa[sy * D + c] : ob[sy * D + c];
        l1[c] = is_ext ? oa[(sy + 1) * D + c] : ob[(sy + 1) * D + c];
      }
      if (!(seg_dist2_f32<D>(p32, l0, l1) > thr2))
        mask |= 1ull << (is_ext ? sy * NV + vx : vx * NE + sy);
    }
  const float2 *hp = is_ext ? hb : ha, *hs = is_ext ? ha : hb;
  const double *pp = is_ext ? pb : pa, *ps = is_ext ? pa : pb;
  const int n_grp = is_ext ? NE : NV, g_size = is_ext ? NV : NE;
  const uint32_t g_mask = (1u << g_size) - 1u;
  float cs[D], cc[D], ns[D], nc[D];  // row g and (ext) row g + 1
#pragma unroll
  for (int k = 0; k < D; ++k) cs[k] = cc[k] = ns[k] = nc[k] = 0.f;
#pragma unroll 1
  for (int g = 0; g < n_grp; ++g) {
    uint32_t m = (uint32_t)(mask >> (g * g_size)) & g_mask;
    while (m) {
      const int j = __ffs(m) - 1;
      m &= m - 1u;
      float f[D], t;
      if (!mixed_item<D>(is_ext ? j : g, is_ext ? g : j, hp, hs, pp, ps, cap, S, f, t))
        continue;
      const float w0 = is_ext ? -__fsub_rn(1.f, t) : 1.f;
#pragma unroll
      for (int k = 0; k < D; ++k) kahan_add_f(cs[k], cc[k], __fmul_rn(f[k], w0));
      if (is_ext) {
#pragma unroll
        for (int k = 0; k < D; ++k) kahan_add_f(ns[k], nc[k], __fmul_rn(f[k], -t));
      }
    }
#pragma unroll
    for (int k = 0; k < D; ++k) {
      out[(g * D + k) * stride] = __fmul_rn(__fsub_rn(cs[k], cc[k]), 0.5f);
      cs[k] = ns[k];
      cc[k] = nc[k];
      ns[k] = nc[k] = 0.f;
    }
  }
  if (is_ext) {
#pragma unroll
    for (int k = 0; k < D; ++k) out[(NE * D + k) * stride] = __fmul_rn(__fsub_rn(cs[k], cc[k]), 0.5f);
  }
}

// Thread per rod, in the order chili's loop adds rod a's terms into its force accumulator
// (update_mechanics.rs:153-382, determinism = true):
//   phase 0, step 1: the boxes of a's subdomain, ascending: a's own voxel pair by pair
//            (b before a: ext then own; b after a: own then ext), a neighbour voxel own only
//            (the ext half is dropped, :205-220);
//   phase 1, step 2: the boxes of other subdomains, ascending: own_a(b) / 2 for each b
//            (PosInformation received and sorted by sender voxel, :304-330);
//   phase 2, step 3: per box of another subdomain, ascending, one term: the sum over its
//            rods b, in storage order, of ext_a(b) / 2 (the ForceInformation that voxel's
//            subdomain returns, summed with xapy, :87-100, :344-382).
// With CRG_WEIGHTS_PHYSICAL every box takes phase 0 with both halves.  Terms skipped by the
// prefilter are +0 and change no sum.  FALLBACK: the kernel runs after a pass-list overflow
// only (P.rctl[3]) and leaves the force in P.frc for k_rods_update; otherwise it runs the
// update itself.  MIXED (with FALLBACK): the passes in mixed precision (mixed_pass), added
// up with the Kahan sums of k_rods_update's mixed fold, every listed pass included.
template <int D, int NV, int B, bool FALLBACK, bool MIXED = false>
__global__ void __launch_bounds__(B) k_rods_step(const PackArgs P) {
  constexpr int NC = NV * D;
  __shared__ double sPa[NC][B];
  __shared__ double sT[NC][B];
  __shared__ double sG[NC][B];  // phase 2: the current box's ext sum
  __shared__ float sOa[NC][B];
  __shared__ float sOb[NC][B];
  __shared__ float sM[MIXED ? NC : 1][B];  // MIXED: M / 2 of the current pass
  static_assert(FALLBACK || !MIXED, "the mixed rod-level kernel is the fallback only");
  if (FALLBACK && !P.rctl[3]) return;  // the pass list fitted: the pass kernel computed this step
  const int tid = threadIdx.x;
  const uint32_t i = blockIdx.x * B + tid;
  if (i >= P.n_agents) return;
  const uint32_t sim = (P.n_sims == 1) ? 0u : sim_of_agent(P, i);
  const SimDev &S = P.sims[sim];
  const int64_t cap = P.cap;
  uint32_t key = P.key[i];
  if (key - S.voxel_off >= S.n_vox) {
    invariant_failed(P.status, kSiteForceKey, i);
    key = S.voxel_off;
  }
  if (sim_frozen(P, S)) {  // frozen simulation (the fallback leaves it to k_rods_update)
    if (!FALLBACK) frozen_copy(P, i, key, NC);
    return;
  }
  const uint32_t v = key - S.voxel_off;
  int idx[D];
  unravel<D>(S, v, idx);
  double pa[NC];
  float oa[NC];
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    pa[k] = P.pos[k * cap + i];
    oa[k] = P.off[k * cap + i];
    if (!MIXED) {
      sPa[k][tid] = pa[k];
      sOa[k][tid] = oa[k];
    }
  }
  float amin[D], amax[D];
#pragma unroll
  for (int c = 0; c < D; ++c) {
    amin[c] = oa[c];
    amax[c] = oa[c];
  }
#pragma unroll
  for (int k = D; k < NC; ++k) {
    amin[k % D] = fminf(amin[k % D], oa[k]);
    amax[k % D] = fmaxf(amax[k % D], oa[k]);
  }
  bool a_nan = false;  // fminf/fmaxf drop NaNs, so test every offset
#pragma unroll
  for (int k = 0; k < NC; ++k) a_nan |= !(oa[k] == oa[k]);
  const SubRange sub_v = subdomain_range(S, v);
  const bool physical = S.weight_mode == CRG_WEIGHTS_PHYSICAL;
  const float thr2 = P.prefilter ? S.filt_thr2 : __int_as_float(0x7f800000);
  const float thr = P.prefilter ? sqrtf(S.filt_thr2) : __int_as_float(0x7f800000);
  double acc[NC];
#pragma unroll
  for (int k = 0; k < NC; ++k) acc[k] = 0.0;
  KahanRows<NC> macc, mgrp;  // MIXED: the rod's sum and the box's step-3 sum
#pragma unroll
  for (int k = 0; k < NC; ++k) macc.s[k] = macc.c[k] = 0.f;
  int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
#pragma unroll
  for (int c = 0; c < D; ++c) {
    lo[c] = idx[c] > 0 ? idx[c] - 1 : 0;
    hi[c] = idx[c] + 1 < S.nvox[c] ? idx[c] + 1 : S.nvox[c] - 1;
  }
#pragma unroll 1
  for (int phase = 0; phase < 3; ++phase)
    for (int j0 = lo[0]; j0 <= hi[0]; ++j0)
      for (int j1 = lo[1]; j1 <= hi[1]; ++j1)
        for (int j2 = lo[2]; j2 <= hi[2]; ++j2) {
          const uint32_t w = (D == 3) ? ((uint32_t)j0 * S.nvox[1] + j1) * S.nvox[2] + j2
                                      : (uint32_t)j0 * S.nvox[1] + j1;
          const bool same = (w == v);
          const bool local = physical || sub_v.same(w);
          if (local != (phase == 0)) continue;
          // b's offsets in a's voxel frame: off_b + (corner_b - corner_a) = off_b + (j-idx) dx
          float kd[D];
          kd[0] = (float)(j0 - idx[0]) * S.dxf[0];
          kd[1] = (float)(j1 - idx[1]) * S.dxf[1];
          if (D == 3) kd[D - 1] = (float)(j2 - idx[D - 1]) * S.dxf[D - 1];
          uint32_t b0 = P.start[S.voxel_off + w], b1 = P.start[S.voxel_off + w + 1];
          if (b0 > b1 || b1 > P.n_agents) {
            invariant_failed(P.status, kSiteForceRange, S.voxel_off + w);
            b1 = b0;
          }
          bool grp = false;  // phase 2: the box's ext sum holds a term
          for (uint32_t b = b0; b < b1; ++b) {
            if (b == i) continue;
            float ob[NC];
            float bmin[D], bmax[D];
#pragma unroll
            for (int k = 0; k < NC; ++k) ob[k] = P.off[k * cap + b] + kd[k % D];
#pragma unroll
            for (int c = 0; c < D; ++c) {
              bmin[c] = ob[c];
              bmax[c] = ob[c];
            }
#pragma unroll
            for (int k = D; k < NC; ++k) {
              bmin[k % D] = fminf(bmin[k % D], ob[k]);
              bmax[k % D] = fmaxf(bmax[k % D], ob[k]);
            }
            // Bounding boxes farther apart than the threshold on one axis: all 2 x NV x
            // (NV-1) evaluations are beyond the cutoff.  (fminf/fmaxf drop NaNs, so a NaN
            // anywhere disables the box test.)
            bool far = false;
            bool b_nan = false;
#pragma unroll
            for (int k = 0; k < NC; ++k) b_nan |= !(ob[k] == ob[k]);
            if (!a_nan && !b_nan) {
#pragma unroll
              for (int c = 0; c < D; ++c)
                far |= (bmin[c] - amax[c] > thr) || (amin[c] - bmax[c] > thr);
            }
            if (far) continue;
            if constexpr (MIXED) {
              const bool twice = phase == 0 && (same || physical);
              const bool ext_first = same && (b < i);
#pragma unroll 1
              for (int pass = 0; pass < 2; ++pass) {
                const bool is_ext = phase == 2 || ((pass == 0) == ext_first);
                if (phase != 2 && is_ext && !twice) continue;
                if (phase == 2 && pass == 1) break;
                mixed_pass<D, NV>(is_ext, oa, ob, P.hl + i, P.hl + b, P.pos + i, P.pos + b, cap,
                                  S, thr2, &sM[0][tid], B);
                if (phase != 2) {
                  macc.add(&sM[0][tid], B);
                } else if (grp) {  // step 3: ext_a(b) / 2 into the box's sum
                  mgrp.add(&sM[0][tid], B);
                } else {
                  mgrp.set(&sM[0][tid], B);
                  grp = true;
                }
              }
            } else {
#pragma unroll
              for (int k = 0; k < NC; ++k) sOb[k][tid] = ob[k];
              const double *posb = P.pos + b;
              if (phase == 2) {  // step 3: ext_a(b) / 2 into the box's sum
                if (rod_pass<D, NV, B>(true, posb, cap, S, thr2, sPa, sT, sOa, sOb, tid)) {
#pragma unroll
                  for (int k = 0; k < NC; ++k) {
                    const double h = dmul(sT[k][tid], 0.5);
                    sG[k][tid] = grp ? dadd(h, sG[k][tid]) : h;
                  }
                  grp = true;
                }
                continue;
              }
              const bool twice = phase == 0 && (same || physical);
              const bool ext_first = same && (b < i);
#pragma unroll 1
              for (int pass = 0; pass < 2; ++pass) {
                const bool is_ext = (pass == 0) == ext_first;
                if (is_ext && !twice) continue;
                if (rod_pass<D, NV, B>(is_ext, posb, cap, S, thr2, sPa, sT, sOa, sOb, tid))
                  add_half<NC, B>(acc, sT, tid);
              }
            }
          }
          if constexpr (MIXED) {
            if (grp) macc.add(mgrp);
          } else if (grp) {
#pragma unroll
            for (int k = 0; k < NC; ++k) acc[k] = dadd(acc[k], sG[k][tid]);
          }
        }
  if constexpr (MIXED) {
#pragma unroll
    for (int k = 0; k < NC; ++k) P.frc[k * cap + i] = (double)macc.value(k);
  } else if (FALLBACK) {
#pragma unroll
    for (int k = 0; k < NC; ++k) P.frc[k * cap + i] = acc[k];
  } else {
    rod_update<D, NV>(P, S, i, key, pa, acc);
  }
}

// ---------------------------------------------------------------------------------------
// Pass-synchronous evaluation (default FP64 path).  Each round every lane of a warp handles
// exactly one pass -- own_a(b) or ext_a(b) -- so the scan of the NV x (NV-1) vertex/segment
// pairs is a uniform loop that records the FP32 survivors in a bitmask; the warp then
// evaluates all survivors of all lanes in FP64 with every lane busy (results to shared
// memory), and the pass matrix M is folded row by row in (vertex, segment) order.  Same
// items, same per-item arithmetic, same order as k_rods_step: identical bits.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ int nth_set_bit64(uint64_t m, int n) {  // n-th set bit (0-based)
  const uint32_t lo = (uint32_t)m;
  const int clo = __popc(lo);
  if (n < clo) return (int)__fns(lo, 0, n + 1);
  return 32 + (int)__fns((uint32_t)(m >> 32), 0, n - clo + 1);
}


// Items of one chunk of the queue kernel's result buffer.  Every lane's items fit (at most
// NV * (NV - 1) <= 56), so a round needs more than one chunk only when the warp's passes
// together have more survivors.
constexpr int kQueueCap = 256;

// Per-warp scratch of the fold's counting sort (after the accumulators in shared memory).
struct FoldScratch {
  uint64_t mask[32];                    // survivor bitmask of each lane's pass
  int32_t slot0[32];                    // first chunk slot of each lane's items
  int32_t cnt[2 * kMaxVertices + 1];    // units per chain length
  int32_t base[2 * kMaxVertices + 1];   // first sorted position of each chain length
  uint32_t tpass[32];                   // pass index of each lane (pass kernel)
  uint8_t ext[32];                      // lane's pass is ext_a(b)
  uint8_t phys[32];                     // physical lane of each virtual lane
  uint8_t desc[32 * kMaxVertices];      // sorted units: lane << 3 | row
};

template <int D, int NV>
constexpr size_t passq_smem_bytes() {  // k_rods_passq: results, fold scratch
  return sizeof(double) * (size_t)2 * D * kQueueCap + sizeof(FoldScratch);
}

// Bit 2 vx + h set when item (vx, r - 1 + h) of an ext pass survived: the contributions to
// row r of the pass matrix, in the reference's order.
template <int NV>
__device__ __forceinline__ uint32_t ext_row_bits(uint64_t mask, int r) {
  constexpr int NE = NV - 1;
  uint32_t em = 0;
#pragma unroll
  for (int vx = 0; vx < NV; ++vx) {
    if (r >= 1) em |= (uint32_t)((mask >> (vx * NE + r - 1)) & 1ull) << (2 * vx);
    if (r < NE) em |= (uint32_t)((mask >> (vx * NE + r)) & 1ull) << (2 * vx + 1);
  }
  return em;
}

// One warp-wide pass step of k_rods_passq.  Every lane brings one pass (own_a(b) or ext_a(b)
// of its rod a and candidate b; is_ext says which) with the bitmask of its FP32-surviving
// vertex/segment pairs.  The warp evaluates the survivors in FP64 with every lane busy into
// a compacted buffer sRes [2D][kQueueCap], in chunks of whole lanes: an item stores f (own
// pass) or -f*t (ext pass) in the first D entries and -f*(1-t) in the last D, so the weights
// are applied while all lanes evaluate.  Then each non-empty (lane, row) of the pass matrix
// M is one unit that sums its own items in the reference's (vertex, segment) order, and the
// pass's M / 2 goes to its slot of mbuf (rows without items: +0).  sAcc is unused.
template <int D, int NV, bool STORE>
__device__ __forceinline__ void eval_fold_queue(const PackArgs &P, double *sRes, double *sAcc,
                                                FoldScratch &F, int lane, uint64_t mask,
                                                bool is_ext, uint32_t a, uint32_t b,
                                                uint32_t sim, uint32_t t, bool has_pass) {
  constexpr int NE = NV - 1, CAP = kQueueCap;
  const int64_t cap = P.cap;
  if (STORE && has_pass) {
    // rows of the pass matrix no item reaches: M / 2 = +0 (written here, whether or not the
    // round has any survivor; the touched rows are written by the fold below)
#pragma unroll
    for (int r = 0; r < NV; ++r) {
      const uint32_t bits = is_ext ? ext_row_bits<NV>(mask, r)
                                   : (uint32_t)((mask >> (r * NE)) & ((1ull << NE) - 1ull));
      if (!bits) {
#pragma unroll
        for (int c = 0; c < D; ++c) P.mbuf[(r * D + c) * P.pass_cap + t] = 0.0;
      }
    }
  }
  // Virtual lane order: own passes first, then ext passes (each in lane order), so that all
  // evaluation batches but one hold a single kind and own-only batches skip the ext
  // weights.  From here on `lane` indexes virtual lanes; F.phys maps back.
  {
    const uint32_t ext_bal = __ballot_sync(0xffffffffu, is_ext);
    const int n_own = 32 - __popc(ext_bal);
    const int src = lane < n_own ? (int)__fns(~ext_bal, 0, lane + 1)
                                 : (int)__fns(ext_bal, 0, lane - n_own + 1);
    const uint32_t mlo = __shfl_sync(0xffffffffu, (uint32_t)mask, src);
    const uint32_t mhi = __shfl_sync(0xffffffffu, (uint32_t)(mask >> 32), src);
    mask = ((uint64_t)mhi << 32) | mlo;
    is_ext = lane >= n_own;
    a = __shfl_sync(0xffffffffu, a, src);
    b = __shfl_sync(0xffffffffu, b, src);
    sim = __shfl_sync(0xffffffffu, sim, src);
    t = __shfl_sync(0xffffffffu, t, src);
    F.phys[lane] = (uint8_t)src;
  }
  const int cnt = __popcll(mask);
  int incl = cnt;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += y;
  }
  const int excl = incl - cnt;
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  for (int cs = 0; cs < total;) {
    // ---- the lanes of this chunk: whole lanes whose items fit from cs on ----------------
    const bool in = excl >= cs && incl <= cs + CAP;
    const int last = 31 - __clz(__ballot_sync(0xffffffffu, in));
    const int ce = __shfl_sync(0xffffffffu, incl, last);

    // ---- evaluate the items [cs, ce) in FP64, every lane busy ---------------------------
    for (int base = cs; base < ce; base += 32) {
      const int j = base + lane;
      int l = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const int cand = l + step;
        const int e = __shfl_sync(0xffffffffu, excl, cand & 31);
        if (cand < 32 && e <= j) l = cand;
      }
      const int ex_l = __shfl_sync(0xffffffffu, excl, l);
      const uint32_t sim_l = __shfl_sync(0xffffffffu, sim, l);
      const uint32_t b_l = __shfl_sync(0xffffffffu, b, l);
      const uint32_t a_l = __shfl_sync(0xffffffffu, a, l);
      const bool ext_l = __shfl_sync(0xffffffffu, (int)is_ext, l) != 0;
      const uint32_t mlo = __shfl_sync(0xffffffffu, (uint32_t)mask, l);
      const uint32_t mhi = __shfl_sync(0xffffffffu, (uint32_t)(mask >> 32), l);
      const int jj = j - cs;
      double tt = 0.0, f[D];
      if (j < ce) {
        const int vs = nth_set_bit64(((uint64_t)mhi << 32) | mlo, j - ex_l);
        const int vx = vs / NE, sy = vs - vx * NE;
        const uint32_t pr = ext_l ? b_l : a_l, sr = ext_l ? a_l : b_l;
        double p[D], l0[D], l1[D], q[D];
#pragma unroll
        for (int c = 0; c < D; ++c) {
          p[c] = P.pos[(vx * D + c) * cap + pr];
          l0[c] = P.pos[(sy * D + c) * cap + sr];
          l1[c] = P.pos[((sy + 1) * D + c) * cap + sr];
        }
        if (P.seg)  // written by this step's k_rods_walk
          nearest_point_seg<D>(p, l0, l1, P.seg + (int64_t)sy * (D + 2) * cap + sr, cap, q, tt);
        else
          nearest_point_f64<D>(p, l0, l1, q, tt);
        if (!morse_full_f64<D>(p, q, P.sims[sim_l], f)) {
#pragma unroll
          for (int c = 0; c < D; ++c) f[c] = 0.0;  // adding +0 leaves M unchanged
        }
        if (!ext_l) {
#pragma unroll
          for (int c = 0; c < D; ++c) sRes[c * CAP + jj] = f[c];
        }
      }
      // ext items store -f t and -f (1 - t); a batch without ext items skips this
      const bool ext_item = j < ce && ext_l;
      if (__any_sync(0xffffffffu, ext_item)) {
        if (ext_item) {
          const double omt = dsub(1.0, tt);
#pragma unroll
          for (int c = 0; c < D; ++c) {
            const double fe = -f[c];
            sRes[c * CAP + jj] = dmul(fe, tt);
            sRes[(D + c) * CAP + jj] = dmul(fe, omt);
          }
        }
      }
    }
    __syncwarp();

    // ---- fold ---------------------------------------------------------------------------
    // Row r of the pass matrix M collects, in the reference's (vertex, segment) order,
    //   own pass: f of items (r, 0..NE-1);
    //   ext pass: for each vertex vx, -f*t of item (vx, r-1) then -f*(1-t) of item (vx, r).
    // Each non-empty (lane, row) of the chunk is a unit: a chain of L contributions summed in
    // that order, then acc += M / 2, i.e. L FP64 adds per component.  The units are sorted
    // by L (counting sort in shared memory, longest first) and dealt to the lanes in snake
    // order; each lane runs its units as one sequence of adds, so every iteration issues
    // exactly D adds for the lanes that still have work.
    int len[NV];
#pragma unroll
    for (int r = 0; r < NV; ++r) {
      const uint32_t bits = is_ext ? ext_row_bits<NV>(mask, r)
                                   : (uint32_t)((mask >> (r * NE)) & ((1ull << NE) - 1ull));
      len[r] = in ? __popc(bits) : 0;
    }
    if (lane <= 2 * NV) F.cnt[lane] = 0;
    F.mask[lane] = mask;
    F.slot0[lane] = excl - cs;  // the lane's first item in the chunk buffer
    F.ext[lane] = is_ext ? 1 : 0;
    F.tpass[lane] = t;
    __syncwarp();
    int rank[NV];
#pragma unroll
    for (int r = 0; r < NV; ++r) rank[r] = len[r] ? atomicAdd(&F.cnt[len[r]], 1) : 0;
    __syncwarp();
    const int cl = (lane >= 1 && lane <= 2 * NV) ? F.cnt[lane] : 0;  // lane L: units of length L
    int suf = cl;  // units of length >= lane
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const int y = __shfl_down_sync(0xffffffffu, suf, off);
      if (lane + off < 32) suf += y;
    }
    const int n_units = __shfl_sync(0xffffffffu, suf, 0);
    if (lane >= 1 && lane <= 2 * NV) F.base[lane] = suf - cl;  // units longer than lane
    __syncwarp();
#pragma unroll
    for (int r = 0; r < NV; ++r)
      if (len[r]) F.desc[F.base[len[r]] + rank[r]] = (uint8_t)((lane << 3) | r);
    __syncwarp();

    int k_unit = 0, p = lane, l = 0, r = 0, slot0 = 0;
    bool act = p < n_units, ext = false;
    uint64_t m_l = 0;
    uint32_t em = 0;  // contributions of the current unit still to add
    double m[D];
    auto contrib = [&](int &h, int &slot) {  // (h, slot) of the unit's next contribution
      const int k = __ffs(em) - 1;
      em &= em - 1u;
      int vs;
      if (ext) {
        h = k & 1;
        vs = (k >> 1) * NE + r - 1 + h;
      } else {
        h = 0;
        vs = r * NE + k;
      }
      slot = slot0 + __popcll(m_l & ((1ull << vs) - 1ull));
    };
    auto load = [&]() {  // start unit p: M = its first contribution (0 + x)
      const uint32_t d = F.desc[p];
      l = (int)(d >> 3);
      r = (int)(d & 7u);
      ext = F.ext[l] != 0;
      m_l = F.mask[l];
      slot0 = F.slot0[l];
      em = ext ? ext_row_bits<NV>(m_l, r)
               : (uint32_t)((m_l >> (r * NE)) & ((1ull << NE) - 1ull));
      int h, slot;
      contrib(h, slot);
#pragma unroll
      for (int c = 0; c < D; ++c) m[c] = plus_zero(sRes[(h * D + c) * CAP + slot]);
    };
    // unit done: 0 + M / 2 to the pass's slot
    auto finish_unit = [&]() {
      (void)sAcc;
#pragma unroll
      for (int c = 0; c < D; ++c)
        P.mbuf[(r * D + c) * P.pass_cap + F.tpass[l]] = plus_zero(half_exact(m[c]));
      ++k_unit;
      p = 32 * k_unit + ((k_unit & 1) ? 31 - lane : lane);
      act = p < n_units;
      if (act) load();
    };
    if (act) load();
    while (__any_sync(0xffffffffu, act)) {
      if (act) {
        while (act && em == 0u) finish_unit();  // no FP64 adds left in this unit
        if (act) {
          int h, slot;
          contrib(h, slot);
#pragma unroll
          for (int c = 0; c < D; ++c) m[c] = dadd(m[c], sRes[(h * D + c) * CAP + slot]);
        }
      }
    }
    __syncwarp();
    cs = ce;
  }
}

// pass_meta bit 7: an ext pass of chili's step 3, summed with the other such passes of the
// same neighbour box before the sum is added to the rod's force.
constexpr uint32_t kPassGroup = 0x80u;

// ---------------------------------------------------------------------------------------
// Pass list of the default rod path.  For every rod, in the order k_rods_step visits them:
// for every candidate b of the 3^D voxel neighbourhood whose FP32 bounding box comes within
// the prefilter threshold, the passes own_a(b) and -- where the pair weight is 1 -- ext_a(b),
// in chili's order.  A rod's passes are contiguous (one reservation per warp, so a rod's
// index range does not depend on timing within the warp).  A list that would outgrow
// pass_cap sets the overflow flag: the rod-level kernel then computes this step, and the
// largest size asked for goes to status[5] for the host to grow the list.
// ---------------------------------------------------------------------------------------
template <int D, int NV>
__global__ void __launch_bounds__(128) k_rods_walk(const PackArgs P) {
  constexpr int NC = NV * D;
  const int lane = threadIdx.x & 31;
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = i < P.n_agents;
  const uint32_t ii = valid ? i : 0u;
  const int64_t cap = P.cap;
  const uint32_t sim = (P.n_sims == 1) ? 0u : sim_of_agent(P, ii);
  const SimDev &S = P.sims[sim];
  const bool live = valid && !sim_frozen(P, S);  // frozen rods have no passes
  if (P.seg && valid) {
    // FP64: each segment's l1 - l0, squared norm and reciprocal for the pass kernel, with
    // the operations of nearest_point_f64 (the coordinates are read first: a load written
    // after a store would wait for it)
    constexpr int NE = NV - 1;
    double x[NC];
#pragma unroll
    for (int k = 0; k < NC; ++k) x[k] = P.pos[k * cap + i];
#pragma unroll
    for (int sy = 0; sy < NE; ++sy) {
      double ab[D];
#pragma unroll
      for (int c = 0; c < D; ++c) ab[c] = dsub(x[(sy + 1) * D + c], x[sy * D + c]);
      double nsq = dmul(ab[0], ab[0]);
#pragma unroll
      for (int c = 1; c < D; ++c) nsq = dadd(nsq, dmul(ab[c], ab[c]));
      double *sg = P.seg + (int64_t)sy * (D + 2) * cap + i;
#pragma unroll
      for (int c = 0; c < D; ++c) sg[c * cap] = ab[c];
      sg[D * cap] = nsq;
      sg[(D + 1) * cap] = __drcp_rn(nsq);
    }
  }
  if (P.hl && live) {  // mixed precision: the hi / lo split of the rod's coordinates
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      const double x = P.pos[k * cap + i];
      const float hi = __double2float_rn(x);
      P.hl[k * cap + i] = make_float2(hi, __double2float_rn(dsub(x, (double)hi)));
    }
  }
  uint32_t key = P.key[ii];
  if (key - S.voxel_off >= S.n_vox) {
    if (live) invariant_failed(P.status, kSiteForceKey, i);
    key = S.voxel_off;
  }
  const uint32_t v = key - S.voxel_off;
  int idx[D];
  unravel<D>(S, v, idx);
  float amin[D], amax[D];
  bool a_nan = false;
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    const float o = P.off[k * cap + ii];
    a_nan |= !(o == o);
    if (k < D) {
      amin[k] = o;
      amax[k] = o;
    } else {
      amin[k % D] = fminf(amin[k % D], o);
      amax[k % D] = fmaxf(amax[k % D], o);
    }
  }
  const SubRange sub_v = subdomain_range(S, v);
  const float thr = P.prefilter ? sqrtf(S.filt_thr2) : __int_as_float(0x7f800000);
  int lo[3] = {0, 0, 0}, nb[3] = {1, 1, 1};
#pragma unroll
  for (int c = 0; c < D; ++c) {
    lo[c] = idx[c] > 0 ? idx[c] - 1 : 0;
    const int hi = idx[c] + 1 < S.nvox[c] ? idx[c] + 1 : S.nvox[c] - 1;
    nb[c] = hi - lo[c] + 1;
  }
  const int n_box = nb[0] * nb[1] * nb[2];
  const bool physical = S.weight_mode == CRG_WEIGHTS_PHYSICAL;
  // visit(b, meta) for every pass of rod i, in the order of k_rods_step: phase 0 the boxes of
  // the rod's subdomain, phase 1 the own halves of the other boxes, phase 2 their ext halves,
  // which are marked (kPassGroup) so that k_rods_update sums each box's ones before adding
  auto walk = [&](auto &&visit) {
    for (int phase = 0; phase < 3; ++phase)
      for (int o = 0; o < n_box; ++o) {
        const int j2 = lo[2] + o % nb[2];
        const int j1 = lo[1] + (o / nb[2]) % nb[1];
        const int j0 = lo[0] + o / (nb[1] * nb[2]);
        const uint32_t w = (D == 3) ? ((uint32_t)j0 * S.nvox[1] + j1) * S.nvox[2] + j2
                                    : (uint32_t)j0 * S.nvox[1] + j1;
        const bool same = (w == v);
        const bool local = physical || sub_v.same(w);
        if (local != (phase == 0)) continue;
        const bool twice = phase == 0 && (same || physical);
        const int dj[3] = {j0 - idx[0], j1 - idx[1], D == 3 ? j2 - idx[D - 1] : 0};
        float kd[D];
#pragma unroll
        for (int c = 0; c < D; ++c) kd[c] = (float)dj[c] * S.dxf[c];
        const uint32_t box = (uint32_t)((dj[0] + 1) | ((dj[1] + 1) << 2) | ((dj[2] + 1) << 4));
        uint32_t b = P.start[S.voxel_off + w], b_end = P.start[S.voxel_off + w + 1];
        if (b > b_end || b_end > P.n_agents) {
          invariant_failed(P.status, kSiteForceRange, S.voxel_off + w);
          b_end = b;
        }
        for (; b < b_end; ++b) {
          if (b == i) continue;
          float bmin[D], bmax[D];
          bool b_nan = false;
#pragma unroll
          for (int k = 0; k < NC; ++k) {
            const float o2 = P.off[k * cap + b] + kd[k % D];
            b_nan |= !(o2 == o2);
            if (k < D) {
              bmin[k] = o2;
              bmax[k] = o2;
            } else {
              bmin[k % D] = fminf(bmin[k % D], o2);
              bmax[k % D] = fmaxf(bmax[k % D], o2);
            }
          }
          bool far = false;
          if (!a_nan && !b_nan) {
#pragma unroll
            for (int c = 0; c < D; ++c)
              far |= (bmin[c] - amax[c] > thr) || (amin[c] - bmax[c] > thr);
          }
          if (far) continue;
          if (phase == 2) {
            visit(b, (box << 1) | 1u | kPassGroup);  // step 3: ext_a(b), summed per box
          } else if (!twice) {
            visit(b, box << 1);  // own_a(b) only: a neighbour voxel, or step 2
          } else {
            const uint32_t ext_first = (same && b < i) ? 1u : 0u;
            visit(b, (box << 1) | ext_first);
            visit(b, (box << 1) | (ext_first ^ 1u));
          }
        }
      }
  };
  uint32_t count = 0;
  if (live) walk([&](uint32_t, uint32_t) { ++count; });
  // one contiguous range per rod, one reservation per warp
  uint32_t incl = count;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += y;
  }
  const uint32_t wtot = __shfl_sync(0xffffffffu, incl, 31);
  uint32_t base = 0;
  if (lane == 31 && wtot) {
    base = atomicAdd(&P.rctl[0], wtot);
    const uint64_t end = (uint64_t)base + wtot;
    atomicMax(&P.status[5], (int32_t)(end < 0x7fffffffull ? end : 0x7fffffffull));
  }
  base = __shfl_sync(0xffffffffu, base, 31);
  const uint64_t first = (uint64_t)base + (incl - count);
  if (valid) {
    P.npass[i] = count;
    P.pass_off[i] = (uint32_t)first;
  }
  if (!count) return;
  if (first + count > (uint64_t)P.pass_cap) {
    P.rctl[3] = 1u;
    return;
  }
  uint32_t k = (uint32_t)first;
  walk([&](uint32_t b, uint32_t meta) {
    P.pass_a[k] = i;
    P.pass_b[k] = b;
    P.pass_meta[k] = (uint8_t)meta;
    ++k;
  });
}

// Warp-per-rod form of k_rods_walk for small systems, where a thread per rod leaves most
// SMs without a warp (a 2,000-rod colony: 63 warps).  The same side outputs (segment data,
// hi / lo split), the same boxes in the same phases, and per box the lanes test 32
// candidates at a time; a prefix sum over the lanes' pass counts (0, 1 or 2 per candidate)
// puts every pass where k_rods_walk puts it within the rod's range.  One reservation per
// rod; a range's place in the list does not change any result (k_rods_update sums each
// rod's passes in range order).
template <int D, int NV>
__global__ void __launch_bounds__(128) k_rods_walk_warp(const PackArgs P) {
  constexpr int NC = NV * D, NE = NV - 1;
  const int lane = threadIdx.x & 31;
  const uint32_t i = (uint32_t)(((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (i >= P.n_agents) return;  // whole warps
  const int64_t cap = P.cap;
  const uint32_t sim = (P.n_sims == 1) ? 0u : sim_of_agent(P, i);
  const SimDev &S = P.sims[sim];
  const bool live = !sim_frozen(P, S);
  if (P.seg) {  // FP64: segment data, one segment per lane
    for (int sy = lane; sy < NE; sy += 32) {
      double ab[D];
#pragma unroll
      for (int c = 0; c < D; ++c)
        ab[c] = dsub(P.pos[((sy + 1) * D + c) * cap + i], P.pos[(sy * D + c) * cap + i]);
      double nsq = dmul(ab[0], ab[0]);
#pragma unroll
      for (int c = 1; c < D; ++c) nsq = dadd(nsq, dmul(ab[c], ab[c]));
      double *sg = P.seg + (int64_t)sy * (D + 2) * cap + i;
#pragma unroll
      for (int c = 0; c < D; ++c) sg[c * cap] = ab[c];
      sg[D * cap] = nsq;
      sg[(D + 1) * cap] = __drcp_rn(nsq);
    }
  }
  if (P.hl && live) {  // mixed precision: hi / lo split, one coordinate per lane
    for (int k = lane; k < NC; k += 32) {
      const double x = P.pos[k * cap + i];
      const float hi = __double2float_rn(x);
      P.hl[k * cap + i] = make_float2(hi, __double2float_rn(dsub(x, (double)hi)));
    }
  }
  uint32_t key = P.key[i];
  if (key - S.voxel_off >= S.n_vox) {
    if (live && lane == 0) invariant_failed(P.status, kSiteForceKey, i);
    key = S.voxel_off;
  }
  const uint32_t v = key - S.voxel_off;
  int idx[D];
  unravel<D>(S, v, idx);
  float amin[D], amax[D];
  bool a_nan = false;
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    const float o = P.off[k * cap + i];
    a_nan |= !(o == o);
    if (k < D) {
      amin[k] = o;
      amax[k] = o;
    } else {
      amin[k % D] = fminf(amin[k % D], o);
      amax[k % D] = fmaxf(amax[k % D], o);
    }
  }
  const SubRange sub_v = subdomain_range(S, v);
  const float thr = P.prefilter ? sqrtf(S.filt_thr2) : __int_as_float(0x7f800000);
  int lo[3] = {0, 0, 0}, nb[3] = {1, 1, 1};
#pragma unroll
  for (int c = 0; c < D; ++c) {
    lo[c] = idx[c] > 0 ? idx[c] - 1 : 0;
    const int hi = idx[c] + 1 < S.nvox[c] ? idx[c] + 1 : S.nvox[c] - 1;
    nb[c] = hi - lo[c] + 1;
  }
  const int n_box = nb[0] * nb[1] * nb[2];
  const bool physical = S.weight_mode == CRG_WEIGHTS_PHYSICAL;
  // emit(k, b, meta): the rod's k-th pass (k counted from 0 in k_rods_walk's order)
  auto walk = [&](auto &&emit) -> uint32_t {
    uint32_t pos = 0;  // passes before this round (the same on every lane)
    for (int phase = 0; phase < 3; ++phase)
      for (int o = 0; o < n_box; ++o) {
        const int j2 = lo[2] + o % nb[2];
        const int j1 = lo[1] + (o / nb[2]) % nb[1];
        const int j0 = lo[0] + o / (nb[1] * nb[2]);
        const uint32_t w = (D == 3) ? ((uint32_t)j0 * S.nvox[1] + j1) * S.nvox[2] + j2
                                    : (uint32_t)j0 * S.nvox[1] + j1;
        const bool same = (w == v);
        const bool local = physical || sub_v.same(w);
        if (local != (phase == 0)) continue;
        const bool twice = phase == 0 && (same || physical);
        const int dj[3] = {j0 - idx[0], j1 - idx[1], D == 3 ? j2 - idx[D - 1] : 0};
        float kd[D];
#pragma unroll
        for (int c = 0; c < D; ++c) kd[c] = (float)dj[c] * S.dxf[c];
        const uint32_t box = (uint32_t)((dj[0] + 1) | ((dj[1] + 1) << 2) | ((dj[2] + 1) << 4));
        const uint32_t b0 = P.start[S.voxel_off + w];
        uint32_t b_end = P.start[S.voxel_off + w + 1];
        if (b0 > b_end || b_end > P.n_agents) {
          if (lane == 0) invariant_failed(P.status, kSiteForceRange, S.voxel_off + w);
          b_end = b0;
        }
        for (uint32_t base = b0; base < b_end; base += 32) {
          const uint32_t b = base + lane;
          uint32_t np = 0, m0 = 0, m1 = 0;
          if (b < b_end && b != i) {
            float bmin[D], bmax[D];
            bool b_nan = false;
#pragma unroll
            for (int k = 0; k < NC; ++k) {
              const float o2 = P.off[k * cap + b] + kd[k % D];
              b_nan |= !(o2 == o2);
              if (k < D) {
                bmin[k] = o2;
                bmax[k] = o2;
              } else {
                bmin[k % D] = fminf(bmin[k % D], o2);
                bmax[k % D] = fmaxf(bmax[k % D], o2);
              }
            }
            bool far = false;
            if (!a_nan && !b_nan) {
#pragma unroll
              for (int c = 0; c < D; ++c)
                far |= (bmin[c] - amax[c] > thr) || (amin[c] - bmax[c] > thr);
            }
            if (!far) {
              if (phase == 2) {
                np = 1;
                m0 = (box << 1) | 1u | kPassGroup;  // step 3: ext_a(b), summed per box
              } else if (!twice) {
                np = 1;
                m0 = box << 1;  // own_a(b) only: a neighbour voxel, or step 2
              } else {
                const uint32_t ext_first = (same && b < i) ? 1u : 0u;
                np = 2;
                m0 = (box << 1) | ext_first;
                m1 = (box << 1) | (ext_first ^ 1u);
              }
            }
          }
          uint32_t incl = np;
#pragma unroll
          for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, off);
            if (lane >= off) incl += y;
          }
          const uint32_t k = pos + incl - np;
          if (np >= 1) emit(k, b, m0);
          if (np == 2) emit(k + 1, b, m1);
          pos += __shfl_sync(0xffffffffu, incl, 31);
        }
      }
    return pos;
  };
  const uint32_t count = live ? walk([](uint32_t, uint32_t, uint32_t) {}) : 0u;
  uint32_t first = 0;
  if (lane == 0) {
    if (count) {
      first = atomicAdd(&P.rctl[0], count);
      const uint64_t end = (uint64_t)first + count;
      atomicMax(&P.status[5], (int32_t)(end < 0x7fffffffull ? end : 0x7fffffffull));
    }
    P.npass[i] = count;
    P.pass_off[i] = first;
  }
  first = __shfl_sync(0xffffffffu, first, 0);
  if (!count) return;
  if ((uint64_t)first + count > (uint64_t)P.pass_cap) {
    if (lane == 0) P.rctl[3] = 1u;
    return;
  }
  walk([&](uint32_t k, uint32_t b, uint32_t meta) {
    P.pass_a[first + k] = i;
    P.pass_b[first + k] = b;
    P.pass_meta[first + k] = (uint8_t)meta;
  });
}

// The passes of the list, 32 consecutive ones per warp and round: every lane carries a pass
// until the list drains, however the passes are spread over rods.  Per pass: the FP32 scan
// of the vertex/segment pairs, the FP64 evaluation and row folds of eval_fold_queue, and
// the pass's M / 2 stored to mbuf for k_rods_update to add up in pass order.
template <int D, int NV>
__global__ void __launch_bounds__(32, 24) k_rods_passq(const PackArgs P) {
  constexpr int NC = NV * D, NE = NV - 1;
  if (P.rctl[3]) return;  // overflow: the rod-level kernel computes this step
  extern __shared__ double sRes[];  // [2D][kQueueCap]: item results, then the fold scratch
  FoldScratch &F = *reinterpret_cast<FoldScratch *>(sRes + 2 * D * kQueueCap);
  const int lane = threadIdx.x;
  const int64_t cap = P.cap;
  const uint32_t total = P.rctl[0];
  const float inf = __int_as_float(0x7f800000);
  while (true) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(&P.rctl[1], 32u);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= total) break;
    const uint32_t t = base + lane;
    const bool have = t < total;
    uint32_t a = 0, b = 0, sim = 0;
    bool is_ext = false;
    uint64_t mask = 0;
    if (have) {
      a = P.pass_a[t];
      b = P.pass_b[t];
      const uint32_t meta = P.pass_meta[t];
      is_ext = (meta & 1u) != 0u;
      sim = (P.n_sims == 1) ? 0u : sim_of_agent(P, a);
      const SimDev &S = P.sims[sim];
      const float thr2 = P.prefilter ? S.filt_thr2 : inf;
      float kd[D];
#pragma unroll
      for (int c = 0; c < D; ++c) kd[c] = (float)((int)((meta >> (1 + 2 * c)) & 3u) - 1) * S.dxf[c];
      float oa[NC], ob[NC];
#pragma unroll
      for (int k = 0; k < NC; ++k) {
        oa[k] = P.off[k * cap + a];
        ob[k] = P.off[k * cap + b] + kd[k % D];
      }
#pragma unroll
      for (int vx = 0; vx < NV; ++vx)
#pragma unroll
        for (int sy = 0; sy < NE; ++sy) {
          const float *pp = is_ext ? &ob[vx * D] : &oa[vx * D];
          const float *s0 = is_ext ? &oa[sy * D] : &ob[sy * D];
          const float *s1 = is_ext ? &oa[(sy + 1) * D] : &ob[(sy + 1) * D];
          float p32[D], l0[D], l1[D];
#pragma unroll
          for (int c = 0; c < D; ++c) {
            p32[c] = pp[c];
            l0[c] = s0[c];
            l1[c] = s1[c];
          }
          if (!(seg_dist2_f32<D>(p32, l0, l1) > thr2)) mask |= 1ull << (vx * NE + sy);
        }
    }
    eval_fold_queue<D, NV, true>(P, sRes, nullptr, F, lane, mask, is_ext, a, b, sim, t, have);
  }
}

// Mixed precision: the passes of the list, one per thread (grid-stride), each pass's M / 2
// as FP32 to its slot of the pass buffer for k_rods_update's mixed fold.
template <int D, int NV>
__global__ void __launch_bounds__(128) k_rods_passmix(const PackArgs P) {
  constexpr int NC = NV * D;
  if (P.rctl[3]) return;  // overflow: the rod-level kernel computes this step
  const uint32_t total = P.rctl[0];
  const int64_t cap = P.cap;
  float *mb = reinterpret_cast<float *>(P.mbuf);
  const float inf = __int_as_float(0x7f800000);
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += gridDim.x * blockDim.x) {
    const uint32_t a = P.pass_a[t], b = P.pass_b[t], meta = P.pass_meta[t];
    const uint32_t sim = (P.n_sims == 1) ? 0u : sim_of_agent(P, a);
    const SimDev &S = P.sims[sim];
    float kd[D];
#pragma unroll
    for (int c = 0; c < D; ++c) kd[c] = (float)((int)((meta >> (1 + 2 * c)) & 3u) - 1) * S.dxf[c];
    float oa[NC], ob[NC];
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      oa[k] = P.off[k * cap + a];
      ob[k] = P.off[k * cap + b] + kd[k % D];
    }
    mixed_pass<D, NV>((meta & 1u) != 0u, oa, ob, P.hl + a, P.hl + b, P.pos + a, P.pos + b, cap,
                      S, P.prefilter ? S.filt_thr2 : inf, mb + t, P.pass_cap);
  }
}

// Curvature forces of every angle of every live rod, one thread per (angle, rod), into
// P.bend [NV - 2][D][cap] for k_rods_update (the acos / tan work, spread over more threads
// than the per-rod update can keep resident; mixed precision: the half-angle identity).
template <int D, int NV>
__global__ void __launch_bounds__(128) k_rods_bend(const PackArgs P) {
  const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t n = P.n_agents;
  if (g >= (uint64_t)n * (NV - 2)) return;
  const int s = (int)(g / n);
  const uint32_t i = (uint32_t)(g - (uint64_t)s * n);
  const uint32_t sim = (P.n_sims == 1) ? 0u : sim_of_agent(P, i);
  const SimDev &S = P.sims[sim];
  if (sim_frozen(P, S)) return;  // frozen: copied by k_rods_update
  const int64_t cap = P.cap;
  double x[3][D], c1[D], c2[D], f[D];
#pragma unroll
  for (int v = 0; v < 3; ++v)
#pragma unroll
    for (int c = 0; c < D; ++c) x[v][c] = P.pos[((s + v) * D + c) * cap + i];
#pragma unroll
  for (int c = 0; c < D; ++c) {
    c1[c] = dsub(x[0][c], x[1][c]);
    c2[c] = dsub(x[1][c], x[2][c]);
  }
  if (P.hl)  // mixed precision
    bend_force_halfangle<D>(S, c1, c2, f);
  else
    bend_force<D>(S, c1, c2, f);
#pragma unroll
  for (int c = 0; c < D; ++c) P.bend[(s * D + c) * cap + i] = f[c];
}

// Mechanics, solver, boundary and next key of every rod from its interaction force -- the
// in-order sum of its passes' M / 2 in mbuf, or after a pass list overflow the force the
// thread-per-rod kernel stored in frc -- and its curvature forces in bend.  Frozen
// simulations copy their state.  MIX: the pass buffer holds FP32 M / 2 (k_rods_passmix),
// added up with Kahan sums in FP32 and converted to FP64 once.
template <int D, int NV, int CYC, bool MIX = false>
__global__ void __launch_bounds__(128) k_rods_update(const PackArgs P) {
  constexpr int NC = NV * D;
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n_agents) return;
  const int64_t cap = P.cap;
  const uint32_t sim = (P.n_sims == 1) ? 0u : sim_of_agent(P, i);
  const SimDev &S = P.sims[sim];
  uint32_t key = P.key[i];
  if (key - S.voxel_off >= S.n_vox) key = S.voxel_off;  // recorded by the force kernel
  if (sim_frozen(P, S)) {
    frozen_copy(P, i, key, NC);
    return;
  }
  double pa[NC], acc[NC];
#pragma unroll
  for (int k = 0; k < NC; ++k) pa[k] = P.pos[k * cap + i];
  if (P.rctl[3]) {
#pragma unroll
    for (int k = 0; k < NC; ++k) acc[k] = P.frc[k * cap + i];
  } else if constexpr (MIX) {
    // the fold below in FP32 Kahan sums, in the same order, step-3 boxes summed first
    const uint32_t p0 = P.pass_off[i];
    const float *mb = reinterpret_cast<const float *>(P.mbuf) + p0;
    const uint8_t *meta = P.pass_meta + p0;
    const uint32_t n = P.npass[i];
    const int64_t pcap = P.pass_cap;
    KahanRows<NC> sum, g;
#pragma unroll
    for (int k = 0; k < NC; ++k) sum.s[k] = sum.c[k] = 0.f;
    uint32_t gbox = 0xffffffffu;
    for (uint32_t p = 0; p < n; ++p) {
      const uint32_t m = meta[p];
      if (!(m & kPassGroup)) {
        sum.add(mb + p, pcap);
        continue;
      }
      const uint32_t box = (m >> 1) & 0x3fu;
      if (box != gbox) {
        if (gbox != 0xffffffffu) sum.add(g);
        g.set(mb + p, pcap);
        gbox = box;
      } else {
        g.add(mb + p, pcap);
      }
    }
    if (gbox != 0xffffffffu) sum.add(g);
#pragma unroll
    for (int k = 0; k < NC; ++k) acc[k] = (double)sum.value(k);
  } else {
    // the sum, in pass order, of the M / 2 that k_rods_passq stored for its passes (rows a
    // pass does not touch are +0, which leaves the sum unchanged since it is never -0);
    // passes marked kPassGroup (they come last) are summed per neighbour box first, and each
    // box's sum is added as one term, as chili adds a ForceInformation
#pragma unroll
    for (int k = 0; k < NC; ++k) acc[k] = 0.0;
    const uint32_t p0 = P.pass_off[i];
    const double *mb = P.mbuf + p0;
    const uint8_t *meta = P.pass_meta + p0;
    const uint32_t n = P.npass[i];
    const int64_t pcap = P.pass_cap;
    double g[NC];
    uint32_t gbox = 0xffffffffu;  // box of the open group (none)
    for (uint32_t p = 0; p < n; ++p) {
      const uint32_t m = meta[p];
      if (!(m & kPassGroup)) {
#pragma unroll
        for (int k = 0; k < NC; ++k) acc[k] = dadd(acc[k], mb[k * pcap + p]);
        continue;
      }
      const uint32_t box = (m >> 1) & 0x3fu;
      if (box != gbox) {
        if (gbox != 0xffffffffu) {
#pragma unroll
          for (int k = 0; k < NC; ++k) acc[k] = dadd(acc[k], g[k]);
        }
#pragma unroll
        for (int k = 0; k < NC; ++k) g[k] = mb[k * pcap + p];
        gbox = box;
      } else {
#pragma unroll
        for (int k = 0; k < NC; ++k) g[k] = dadd(mb[k * pcap + p], g[k]);
      }
    }
    if (gbox != 0xffffffffu) {
#pragma unroll
      for (int k = 0; k < NC; ++k) acc[k] = dadd(acc[k], g[k]);
    }
  }
  rod_update<D, NV, true, CYC>(P, S, i, key, pa, acc);
}

// Candidate rods of the current cell list, a hash of their ids and the number of in-range
// vertex/segment evaluations of a.calc(a, b) (own perspective, FP64, no prefilter).
template <int D, int NV>
__global__ void k_rod_stats(const PackArgs P, uint32_t *n_cand, uint32_t *n_inter,
                            uint64_t *hash) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n_agents) return;
  const uint32_t sim = (P.n_sims == 1) ? 0u : sim_of_agent(P, i);
  const SimDev &S = P.sims[sim];
  const uint32_t v = P.key[i] - S.voxel_off;
  int idx[D];
  unravel<D>(S, v, idx);
  int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  for (int c = 0; c < D; ++c) {
    lo[c] = idx[c] > 0 ? idx[c] - 1 : 0;
    hi[c] = idx[c] + 1 < S.nvox[c] ? idx[c] + 1 : S.nvox[c] - 1;
  }
  uint32_t nc = 0, ni = 0;
  uint64_t h = 0;
  for (int j0 = lo[0]; j0 <= hi[0]; ++j0)
    for (int j1 = lo[1]; j1 <= hi[1]; ++j1)
      for (int j2 = lo[2]; j2 <= hi[2]; ++j2) {
        const uint32_t w = (D == 3) ? ((uint32_t)j0 * S.nvox[1] + j1) * S.nvox[2] + j2
                                    : (uint32_t)j0 * S.nvox[1] + j1;
        for (uint32_t b = P.start[S.voxel_off + w]; b < P.start[S.voxel_off + w + 1]; ++b) {
          if (b == i) continue;
          ++nc;
          uint64_t x = P.id[b] + 0x9e3779b97f4a7c15ull;
          x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
          x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
          h += x ^ (x >> 31);
          for (int vi = 0; vi < NV; ++vi)
            for (int sj = 0; sj + 1 < NV; ++sj) {
              double p[D], l0[D], l1[D], q[D], t, f[D];
              for (int c = 0; c < D; ++c) {
                p[c] = P.pos[(vi * D + c) * P.cap + i];
                l0[c] = P.pos[(sj * D + c) * P.cap + b];
                l1[c] = P.pos[((sj + 1) * D + c) * P.cap + b];
              }
              nearest_point_f64<D>(p, l0, l1, q, t);
              if (morse_full_f64<D>(p, q, S, f)) ++ni;
            }
        }
      }
  n_cand[i] = nc;
  n_inter[i] = ni;
  hash[i] = h;
}

// ---------------------------------------------------------------------------------------
// Cell cycle of rods (single-simulation handles).
// ---------------------------------------------------------------------------------------

// NeighborSensing::accumulate_information of the bacterial-rods agent (bacterial_rods/src/
// main.rs:49-64) over the partners chili lets a rod meet as "own" in one step
// (update_mechanics.rs:105, 201-202; remote partners through the positions received in
// step 2): every other rod of the 3^D neighbourhood, once.  The count is a sum of
// integers, so the visiting order does not matter.  One thread per rod, FP64 distances as
// nalgebra's norm() forms them; a partner whose bounding box lies farther than the range
// (plus a relative 1e-9 for the roundings) from the rod's on some axis is skipped, since no
// vertex pair of it can then be closer than the range.
template <int D, int NV>
__global__ void __launch_bounds__(128) k_rods_sense(const PackArgs P) {
  // one warp per rod, its candidates shared out over the lanes (the count is an integer
  // sum: the order does not matter)
  constexpr int NC = NV * D;
  const int lane = threadIdx.x & 31;
  const uint32_t i = (uint32_t)(((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (i >= P.n_agents) return;  // whole warps
  const SimDev &S = P.sims[0];
  const int64_t cap = P.cap;
  const uint32_t key = P.key[i];
  if (key - S.voxel_off >= S.n_vox) {
    if (lane == 0) {
      invariant_failed(P.status, kSiteForceKey, i);
      P.nsense[i] = 0u;
    }
    return;
  }
  int idx[D];
  unravel<D>(S, key - S.voxel_off, idx);
  double pa[NC];
#pragma unroll
  for (int k = 0; k < NC; ++k) pa[k] = P.pos[k * cap + i];
  const long long x2 = S.cyc_sense_x2;  // sqrt(n2) < r exactly when bits(n2) <= x2
  float oa[NC], lo_a[D], hi_a[D];  // FP32 offsets and their bounding box
#pragma unroll
  for (int k = 0; k < NC; ++k) oa[k] = P.off[k * cap + i];
#pragma unroll
  for (int c = 0; c < D; ++c) {
    lo_a[c] = hi_a[c] = oa[c];
#pragma unroll
    for (int q = 1; q < NV; ++q) {
      lo_a[c] = fminf(lo_a[c], oa[q * D + c]);
      hi_a[c] = fmaxf(hi_a[c], oa[q * D + c]);
    }
  }
  int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
#pragma unroll
  for (int c = 0; c < D; ++c) {
    lo[c] = idx[c] > 0 ? idx[c] - 1 : 0;
    hi[c] = idx[c] + 1 < S.nvox[c] ? idx[c] + 1 : S.nvox[c] - 1;
  }
  uint32_t cnt = 0;
  for (int j0 = lo[0]; j0 <= hi[0]; ++j0)
    for (int j1 = lo[1]; j1 <= hi[1]; ++j1)
      for (int j2 = lo[2]; j2 <= hi[2]; ++j2) {
        const uint32_t w = (D == 3) ? ((uint32_t)j0 * S.nvox[1] + j1) * S.nvox[2] + j2
                                    : (uint32_t)j0 * S.nvox[1] + j1;
        uint32_t b0 = P.start[S.voxel_off + w], b1 = P.start[S.voxel_off + w + 1];
        if (b0 > b1 || b1 > P.n_agents) {
          if (lane == 0) invariant_failed(P.status, kSiteForceRange, S.voxel_off + w);
          b1 = b0;
        }
        float kd[D];  // b's offsets in a's voxel frame: off_b + (j - idx) dx
        kd[0] = (float)(j0 - idx[0]) * S.dxf[0];
        kd[1] = (float)(j1 - idx[1]) * S.dxf[1];
        if (D == 3) kd[D - 1] = (float)(j2 - idx[D - 1]) * S.dxf[D - 1];
        for (uint32_t b = b0 + lane; b < b1; b += 32) {
          if (b == i) continue;
          float ob[NC];
#pragma unroll
          for (int k = 0; k < NC; ++k) ob[k] = P.off[k * cap + b] + kd[k % D];
          // bounding boxes further apart along an axis than the range plus the offsets'
          // error band: no vertex pair can count (NaN offsets compare false: not skipped)
          bool far = false;
#pragma unroll
          for (int c = 0; c < D; ++c) {
            float lb = ob[c], hb = ob[c];
#pragma unroll
            for (int q = 1; q < NV; ++q) {
              lb = fminf(lb, ob[q * D + c]);
              hb = fmaxf(hb, ob[q * D + c]);
            }
            far |= (lb - hi_a[c] > S.sense_gap_f) || (lo_a[c] - hb > S.sense_gap_f);
          }
          if (far) continue;
#pragma unroll
          for (int u = 0; u < NV; ++u)
#pragma unroll
            for (int q = 0; q < NV; ++q) {
              // FP32 first: clearly inside or outside the range (NaN offsets fall through)
              float d2f = 0.f;
#pragma unroll
              for (int c = 0; c < D; ++c) {
                const float e = oa[u * D + c] - ob[q * D + c];
                d2f = fmaf(e, e, d2f);
              }
              if (d2f < S.sense_in2) {
                ++cnt;
                continue;
              }
              if (d2f > S.sense_out2) continue;
              double n2 = 0.0;
#pragma unroll
              for (int c = 0; c < D; ++c) {
                const double d = dsub(pa[u * D + c], P.pos[(q * D + c) * cap + b]);
                n2 = (c == 0) ? dmul(d, d) : dadd(n2, dmul(d, d));
              }
              // (own_point - ext_point).norm() < r (bacterial_rods/src/main.rs:49-64)
              if (__double_as_longlong(n2) <= x2) ++cnt;
            }
        }
      }
  cnt = __reduce_add_sync(0xffffffffu, cnt);
  if (lane == 0) P.nsense[i] = cnt;
}

// Voxel::update_cell_cycle_4 (chili/update_cycle.rs:10-69) for the rods the update kernel
// flagged, then SubDomainBox::apply_boundary and the next voxel keys of both halves.
// dpre is the exclusive scan of the flags over the cell list, so inside voxel v (cell-list
// range [start[v], start[v+1])) the dividing rods are numbered r = dpre[i] - dpre[start[v]]
// of m = dpre[start[v+1]] - dpre[start[v]] in storage order, as chili visits them:
//   * the parent is renamed Division(v, counter + r + 1) and its daughter, appended to the
//     voxel after every other rod of it, becomes Division(v, counter + m + r + 1);
//   * in chili's pre-sort order (voxels ascending, each voxel's Vec) rod i sits at
//     i + dpre[start[v]] and the daughter at start[v+1] + dpre[i]: the sort ranks them so.
// The daughter's state goes to n_agents + dpre[i] of the next-state arrays, with a fresh
// solver history (default aux storage).  RodMechanics::divide (bacterial_rods.rs:586-663):
// both halves get (1/2 - R / (n spring_length)) spring_length; the first keeps the first
// vertex, the second the last, and the vertices are spread along the old polyline at
// steps of (length - 2 R) / (n - 1) / 2; float sums start at -0.0 as Rust's Sum for f64.
template <int D, int NV>
__global__ void k_rods_divide(const PackArgs P) {
  constexpr int NC = NV * D;
  const uint32_t n = P.n_agents;
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const SimDev &S = P.sims[0];
  const int64_t cap = P.cap;
  const uint32_t key = P.key[i];
  if (key - S.voxel_off >= S.n_vox) {
    invariant_failed(P.status, kSiteForceKey, i);
    P.srank[i] = i;
    return;
  }
  const uint32_t d_lo = P.dpre[P.start[key]];
  const uint32_t di = P.dpre[i];
  P.srank[i] = i + d_lo;
  if (P.dpre[i + 1] == di) return;  // not dividing: k_rods_update finished it
  const uint32_t m = P.dpre[P.start[key + 1]] - d_lo;
  const uint32_t r = di - d_lo;
  const uint32_t j = n + di;
  P.srank[j] = P.start[key + 1] + di;
  const uint64_t c0 = P.vctr[key];
  const uint64_t plain = key - S.voxel_off;
  const uint64_t old = P.id[i];
  const uint64_t pid = CRG_ID_DIVISION | (plain << 32) | ((c0 + r + 1) & 0xffffffffull);
  const uint64_t did = CRG_ID_DIVISION | (plain << 32) | ((c0 + m + r + 1) & 0xffffffffull);

  double pos[NC], v1[NC], v2[NC], c1[NC], c2[NC];
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    pos[k] = P.npos[k * cap + i];
    v1[k] = v2[k] = P.nvel[k * cap + i];
    c1[k] = c2[k] = pos[k];
  }
  const double slen = P.nslen[i];
  const double radius = S.radius;
  const double div_factor = dsub(0.5, ddiv(radius, dmul((double)NV, slen)));
  const double nsl = dmul(div_factor, slen);
  double seg[NV - 1];
#pragma unroll
  for (int q = 0; q + 1 < NV; ++q) {
    double n2 = 0.0;
#pragma unroll
    for (int c = 0; c < D; ++c) {
      const double d = dsub(pos[q * D + c], pos[(q + 1) * D + c]);
      n2 = (c == 0) ? dmul(d, d) : dadd(n2, dmul(d, d));
    }
    seg[q] = __dsqrt_rn(n2);
  }
  double total = -0.0;
#pragma unroll
  for (int q = 0; q + 1 < NV; ++q) total = dadd(total, seg[q]);
  const double seglen = ddiv(ddiv(dsub(total, dmul(2.0, radius)), (double)(NV - 1)), 2.0);
  bool ok = true;
  for (int nvx = 0; nvx < NV; ++nvx) {
    const double target = dmul((double)nvx, seglen);
    int k = -1;
    double pk = 0.0, acc = -0.0;
    for (int q = 0; q < NV - 1; ++q) {  // sums of the first q segments
      if (acc <= target) {
        k = q;
        pk = acc;
      }
      acc = dadd(acc, seg[q]);
    }
    int mm = -1;
    double rm = 0.0;
    acc = -0.0;
    for (int q = 0; q < NV; ++q) {  // sums of the last q segments, last first
      if (acc <= target) {
        mm = q;
        rm = acc;
      }
      if (q < NV - 1) acc = dadd(acc, seg[NV - 2 - q]);
    }
    if (k < 0 || mm < 0 || NV - mm - 2 < 0) {
      ok = false;
      break;
    }
    const double qf = ddiv(dsub(target, pk), seg[k]);
    const double pf = ddiv(dsub(target, rm), seg[NV - mm - 2]);
    const double omq = dsub(1.0, qf), omp = dsub(1.0, pf);
    for (int c = 0; c < D; ++c) {
      c1[nvx * D + c] = dadd(dmul(pos[k * D + c], omq), dmul(pos[(k + 1) * D + c], qf));
      c2[(NV - nvx - 1) * D + c] =
          dadd(dmul(pos[(NV - mm - 1) * D + c], omp), dmul(pos[(NV - mm - 2) * D + c], pf));
    }
  }
  if (!ok) {  // DivisionError: the step reports it; both halves stay copies of the parent
    set_status(P.status, CRG_ECALC, old, *P.step_ctr + 1, S.sim_index);
#pragma unroll
    for (int k = 0; k < NC; ++k) c1[k] = c2[k] = pos[k];
  }
  P.nid[i] = pid;
  P.nid[j] = did;
  P.nparent[i] = old;
  P.nparent[j] = old;
  P.nslen[i] = nsl;
  P.nslen[j] = nsl;
  P.ngrate[j] = P.ngrate[i];
  if (P.nhist) {
    for (int k = 0; k < 2 * NC; ++k) P.nhist[k * cap + j] = 0.0;
    P.nhmeta[j] = 0;
  }
  // the voxel the daughter was appended to: its move class in the sort
  const_cast<uint32_t *>(P.key)[j] = key;
  rod_finish<D, NV>(P, S, i, key, pid, c1, v1);
  rod_finish<D, NV>(P, S, j, key, did, c2, v2);
}

// Voxel::id_counter after insert_initial_cells (chili/datastructures.rs:278-299): one per
// agent inserted into the voxel.
__global__ void k_cycle_init(const PackArgs P) {
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= P.n_vox) return;
  P.vctr[v] = (uint64_t)(P.start[v + 1] - P.start[v]);
}

// Per-agent values given in upload order moved to the cell list: slot s holds the agent
// the upload's sort took from input index tmp[s] (its low 31 bits).
__global__ void k_cycle_permute(double *dst, const double *src, const uint64_t *tmp,
                                uint32_t n) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  dst[s] = src[(uint32_t)(tmp[s] & 0x7fffffffull)];
}

// Voxel::id_counter after the divisions of the step: + 2 per division in the voxel.
__global__ void k_cycle_counters(const PackArgs P) {
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= P.n_vox) return;
  P.vctr[v] += 2ull * (uint64_t)(P.dpre[P.start[v + 1]] - P.dpre[P.start[v]]);
}

// Largest rod count the default walk runs with a warp per rod (below it a thread per rod
// leaves most SMs idle).
constexpr uint32_t kWarpWalkMax = 16384;

// Resident warps of k_rods_passq and resident blocks of k_rods_passmix on the current
// device, [D - 2][NV] (set by prepare_rods).
unsigned g_passq_warps[2][9] = {};
unsigned g_passmix_blocks[2][9] = {};

template <int D, int NV>
void launch_t(const PackArgs &P, int precision, int block, cudaStream_t st, cudaEvent_t k0,
              cudaEvent_t k1, cudaEvent_t k2, cudaEvent_t k3) {
  (void)precision;
  auto rec = [&](cudaEvent_t e) { record_event(e, st); };
  constexpr int B = 64;
  const unsigned rod_grid = (P.n_agents + B - 1) / B;
  const bool mixed = precision != CRG_PREC_F64;
  if (P.variant == 1 && !mixed) {  // FP64 thread-per-rod kernel
    rec(k0);
    k_rods_step<D, NV, B, false><<<rod_grid, B, 0, st>>>(P);
    rec(k1);
    return;
  }
  const unsigned warps = (P.n_agents + 31) / 32;
  const unsigned rblocks = (P.n_agents + 127) / 128;
  cudaMemsetAsync(P.rctl, 0, 4 * sizeof(uint32_t), st);
  // walk: a warp per rod for small systems (block 32, or by default below kWarpWalkMax
  // rods), else a thread per rod (block 128); the same pass list either way
  if (block == 32 || (block != 128 && P.n_agents <= kWarpWalkMax))
    k_rods_walk_warp<D, NV><<<(P.n_agents + 3) / 4, 128, 0, st>>>(P);
  else
    k_rods_walk<D, NV><<<rblocks, 128, 0, st>>>(P);
  rec(k0);
  if (mixed) {  // FP32 pair forces; each launch returns at once unless it is this step's
    const unsigned mgrid = g_passmix_blocks[D - 2][NV] ? g_passmix_blocks[D - 2][NV] : rblocks;
    k_rods_passmix<D, NV><<<mgrid, 128, 0, st>>>(P);
    rec(k1);
    k_rods_step<D, NV, B, true, true><<<rod_grid, B, 0, st>>>(P);
  } else {
    const unsigned pgrid = g_passq_warps[D - 2][NV] ? g_passq_warps[D - 2][NV] : warps;
    k_rods_passq<D, NV><<<pgrid, 32, passq_smem_bytes<D, NV>(), st>>>(P);
    rec(k1);
    k_rods_step<D, NV, B, true><<<rod_grid, B, 0, st>>>(P);
  }
  if (NV > 2) {
    const uint64_t nb = ((uint64_t)P.n_agents * (NV - 2) + 127) / 128;
    k_rods_bend<D, NV><<<(unsigned)nb, 128, 0, st>>>(P);
  }
  rec(k2);
  if (mixed)
    k_rods_update<D, NV, 0, true><<<rblocks, 128, 0, st>>>(P);
  else if (P.dflag)
    k_rods_update<D, NV, 1><<<rblocks, 128, 0, st>>>(P);
  else
    k_rods_update<D, NV, 0><<<rblocks, 128, 0, st>>>(P);
  rec(k3);
}

template <int D, int NV>
cudaError_t prepare_t() {
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int psmem = (int)passq_smem_bytes<D, NV>();
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_rods_passq<D, NV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             psmem);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_rods_passq<D, NV>, 32, psmem);
  if (e == cudaSuccess) g_passq_warps[D - 2][NV] = (unsigned)(sms * per_sm);
  int mix_per_sm = 0;
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&mix_per_sm, k_rods_passmix<D, NV>, 128, 0);
  if (e == cudaSuccess) g_passmix_blocks[D - 2][NV] = (unsigned)(sms * (mix_per_sm > 0 ? mix_per_sm : 1));
  return e;
}

template <int D>
cudaError_t prepare_d(int nv) {
  switch (nv) {
    case 2: return prepare_t<D, 2>();
    case 3: return prepare_t<D, 3>();
    case 4: return prepare_t<D, 4>();
    case 5: return prepare_t<D, 5>();
    case 6: return prepare_t<D, 6>();
    case 7: return prepare_t<D, 7>();
    case 8: return prepare_t<D, 8>();
    default: return cudaErrorInvalidValue;
  }
}

template <int D>
void launch_d(int nv, const PackArgs &P, int precision, int block, cudaStream_t st,
              cudaEvent_t k0, cudaEvent_t k1, cudaEvent_t k2, cudaEvent_t k3) {
  switch (nv) {
    case 2: launch_t<D, 2>(P, precision, block, st, k0, k1, k2, k3); break;
    case 3: launch_t<D, 3>(P, precision, block, st, k0, k1, k2, k3); break;
    case 4: launch_t<D, 4>(P, precision, block, st, k0, k1, k2, k3); break;
    case 5: launch_t<D, 5>(P, precision, block, st, k0, k1, k2, k3); break;
    case 6: launch_t<D, 6>(P, precision, block, st, k0, k1, k2, k3); break;
    case 7: launch_t<D, 7>(P, precision, block, st, k0, k1, k2, k3); break;
    case 8: launch_t<D, 8>(P, precision, block, st, k0, k1, k2, k3); break;
    default: break;
  }
}

}  // namespace

// Kernel attributes that must be set outside any stream capture (once per handle).
int prepare_rods(int dim, int nv) {
  return (dim == 3 ? prepare_d<3>(nv) : prepare_d<2>(nv)) == cudaSuccess ? 0 : -1;
}

void launch_rods_step(int dim, int nv, int precision, const PackArgs &P, int block,
                      cudaStream_t st, cudaEvent_t k0, cudaEvent_t k1, cudaEvent_t k2,
                      cudaEvent_t k3) {
  if (!P.n_agents) return;
  if (block <= 0 || block > 128) block = 64;
  if (dim == 3)
    launch_d<3>(nv, P, precision, block, st, k0, k1, k2, k3);
  else
    launch_d<2>(nv, P, precision, block, st, k0, k1, k2, k3);
}

template <int D>
void launch_stats_d(int nv, const PackArgs &P, uint32_t *n_cand, uint32_t *n_inter,
                    uint64_t *hash, cudaStream_t st) {
  const unsigned grid = (P.n_agents + 127) / 128;
  switch (nv) {
    case 2: k_rod_stats<D, 2><<<grid, 128, 0, st>>>(P, n_cand, n_inter, hash); break;
    case 3: k_rod_stats<D, 3><<<grid, 128, 0, st>>>(P, n_cand, n_inter, hash); break;
    case 4: k_rod_stats<D, 4><<<grid, 128, 0, st>>>(P, n_cand, n_inter, hash); break;
    case 5: k_rod_stats<D, 5><<<grid, 128, 0, st>>>(P, n_cand, n_inter, hash); break;
    case 6: k_rod_stats<D, 6><<<grid, 128, 0, st>>>(P, n_cand, n_inter, hash); break;
    case 7: k_rod_stats<D, 7><<<grid, 128, 0, st>>>(P, n_cand, n_inter, hash); break;
    case 8: k_rod_stats<D, 8><<<grid, 128, 0, st>>>(P, n_cand, n_inter, hash); break;
    default: break;
  }
}

template <int D>
void launch_cycle_d(int nv, const PackArgs &P, bool divide, cudaStream_t st) {
  const unsigned grid = (P.n_agents + 127) / 128;
  const unsigned sgrid = (unsigned)(((uint64_t)P.n_agents * 32 + 127) / 128);  // warp per rod
#define CRG_CYCLE_CASE(NVV)                                        \
  case NVV:                                                        \
    if (divide)                                                    \
      k_rods_divide<D, NVV><<<grid, 128, 0, st>>>(P);              \
    else                                                           \
      k_rods_sense<D, NVV><<<sgrid, 128, 0, st>>>(P);              \
    break;
  switch (nv) {
    CRG_CYCLE_CASE(2)
    CRG_CYCLE_CASE(3)
    CRG_CYCLE_CASE(4)
    CRG_CYCLE_CASE(5)
    CRG_CYCLE_CASE(6)
    CRG_CYCLE_CASE(7)
    CRG_CYCLE_CASE(8)
    default: break;
  }
#undef CRG_CYCLE_CASE
}

void launch_rods_sense(int dim, int nv, const PackArgs &P, cudaStream_t st) {
  if (!P.n_agents) return;
  if (dim == 3)
    launch_cycle_d<3>(nv, P, false, st);
  else
    launch_cycle_d<2>(nv, P, false, st);
}

void launch_rods_divide(int dim, int nv, const PackArgs &P, uint32_t n_div, cudaStream_t st) {
  if (!P.n_agents || !n_div) return;
  if (dim == 3)
    launch_cycle_d<3>(nv, P, true, st);
  else
    launch_cycle_d<2>(nv, P, true, st);
}

void launch_cycle_counters(const PackArgs &P, cudaStream_t st) {
  k_cycle_counters<<<(P.n_vox + 255) / 256, 256, 0, st>>>(P);
}

void launch_cycle_init(const PackArgs &P, cudaStream_t st) {
  k_cycle_init<<<(P.n_vox + 255) / 256, 256, 0, st>>>(P);
}

void launch_cycle_permute(double *dst, const double *src, const uint64_t *tmp, uint32_t n,
                          cudaStream_t st) {
  if (n) k_cycle_permute<<<(n + 255) / 256, 256, 0, st>>>(dst, src, tmp, n);
}

void launch_rod_stats(int dim, int nv, const PackArgs &P, uint32_t *n_cand, uint32_t *n_inter,
                      uint64_t *hash, cudaStream_t st) {
  if (!P.n_agents) return;
  if (dim == 3)
    launch_stats_d<3>(nv, P, n_cand, n_inter, hash, st);
  else
    launch_stats_d<2>(nv, P, n_cand, n_inter, hash, st);
}

}  // namespace crg
