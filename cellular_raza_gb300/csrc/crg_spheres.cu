// crg_spheres.cu -- one chili step for NewtonDamped + MorsePotential spheres.
//
// One thread per agent in cell-list order gathers the forces from the 3^D neighbour
// voxels (cellular_raza-building-blocks/src/domains/cartesian_cuboid_n.rs:641-662), then
// applies the solver, the reflecting boundary and computes its next voxel key.
//
// Summation order.  With one subdomain chili adds, for agent a, the own-perspective
// half-forces F_a(b)/2 voxel by voxel in ascending plain index and, inside a voxel, in the
// voxel's Vec order; a partner in the same voxel contributes its half twice in a row
// (update_mechanics.rs:178-203), a partner in a neighbour voxel once (:205-220, the
// other half is dropped).  A partner in a voxel of another subdomain contributes twice
// (steps 2 and 3, :285-382).  The loop below visits partners in exactly that order and
// adds the same separately rounded half-forces, so with one subdomain it repeats chili's
// sums; with several it adds the same terms in a different order.
//
// Candidate prefilter.  A pair whose FP32 distance (from FP32 offsets to the voxel corner,
// error far below the margin folded into filt_thr2) exceeds the cutoff plus margin has an
// FP64 distance above the cutoff, hence a zero force, and is skipped; everything else is
// evaluated in FP64.  Skipping a zero changes no sum.
#include <type_traits>

#include "crg_internal.cuh"
#include "crg_kernels.h"

namespace crg {

namespace {

// The FP32 offsets of sphere agent i: one float4 (3D) or float2 (2D) per agent.
template <int D>
__device__ __forceinline__ void sphere_off(const float *off, uint32_t i, float *o) {
  if (D == 3) {
    const float4 v = reinterpret_cast<const float4 *>(off)[i];
    o[0] = v.x;
    o[1] = v.y;
    o[2] = v.z;
  } else {
    const float2 v = reinterpret_cast<const float2 *>(off)[i];
    o[0] = v.x;
    o[1] = v.y;
  }
}


template <int D>
struct Neigh {
  int lo[D], hi[D];
};

// Kahan-compensated FP32 accumulation (mixed precision).
__device__ __forceinline__ void kahan_add(float &s, float &c, float x) {
  float y = x - c;
  float t = s + y;
  c = (t - s) - y;
  s = t;
}


// morse_half_f64 evaluated by a batch of lanes `act` together (every lane of act calls it):
// the same operations in the same order, so the same bits, with the warp reconverged after
// the square root, the exp and each division.  Without that, a lane that takes a slow path
// inside one of these library calls can leave the batch split into groups for the rest of
// the evaluation, and every later FP64 instruction runs with a fraction of its lanes.
// Returns whether the pair interacts (h = +0 when it does not).
template <int D>
__device__ __forceinline__ bool morse_half_f64_batch(const double *z, const SimDev &S, double *h,
                                                     unsigned act) {
  double n2 = dmul(z[0], z[0]);
#pragma unroll
  for (int c = 1; c < D; ++c) n2 = dadd(n2, dmul(z[c], z[c]));
  const double dist = __dsqrt_rn(n2);
  __syncwarp(act);
  const bool ok = !beyond_cutoff(dist, S.cutoff_bits);
  const double e = exp(dmul(S.mrs_nstiff, dsub(dist, S.mrs_r)));
  __syncwarp(act);
  const double force = dmul(dmul(S.mrs_k, e), dsub(1.0, e));
#pragma unroll
  for (int c = 0; c < D; ++c) {
    const double q = ddiv(z[c], dist);
    __syncwarp(act);
    h[c] = ok ? half_exact(dmul(q, force)) : 0.0;
  }
  return ok;
}

// Mixed path: FP32 Morse half force of agent a (FP64 position pa) from partner b at FP32
// displacement zf, |zf|^2 = d2 (not NaN).  Whether the pair interacts is decided exactly as
// on the FP64 path: a pair whose FP32 distance lies within a few times its error bound of
// the cutoff (mix_band_f) or of zero (mix_zero_f) is decided from the FP64 distance, so no
// pair switches on or off relative to FP64.  Shared by the mixed kernels so they produce the same bits.
template <int D>
__device__ __forceinline__ bool mixed_half(const PackArgs &P, const SimDev &S, const double *pa,
                                           uint32_t b, const float *zf, float d2, float *h) {
  // one reciprocal square root serves the distance and the direction z / dist
  const float rinv = rsqrtf(d2);
  const float dist = d2 > 0.0f ? __fmul_rn(d2, rinv) : 0.0f;
  bool in;
  if (fabsf(dist - S.cutoff_f) <= S.mix_band_f || dist <= S.mix_zero_f) {
    double n2 = 0.0;
#pragma unroll
    for (int c = 0; c < D; ++c) {
      const double z = dsub(pa[c], P.pos[c * P.cap + b]);
      n2 = (c == 0) ? dmul(z, z) : dadd(n2, dmul(z, z));
    }
    const double d64 = __dsqrt_rn(n2);
    in = !(d64 > S.cutoff || d64 == 0.0);
  } else {
    in = !(dist > S.cutoff_f);
  }
  if (!in) return false;
  const float r = S.radius_f + S.radius_f;
  const float e = expf(-S.stiffness_f * (dist - r));
  const float force = -2.0f * S.strength_f * S.stiffness_f * e * (1.0f - e);
  // a pair that interacts in FP64 at an FP32 distance of 0 has no FP32 direction: the NaN
  // hands the agent to the FP64 fix-up kernel
  const float sc = d2 > 0.0f ? __fmul_rn(__fmul_rn(force, 0.5f), rinv) : __int_as_float(0x7fc00000);
#pragma unroll
  for (int c = 0; c < D; ++c) h[c] = __fmul_rn(zf[c], sc);
  return true;
}

// Mixed path, rare case (a NaN displacement: an agent far outside its voxel, NaN
// positions): agent i's interaction force computed exactly as the FP64 path computes it
// (same candidates, same order, FP64 Morse).
struct Vec3 {
  double x[3];
};
template <int D>
__device__ Vec3 agent_force_f64(const PackArgs &P, const SimDev &S, uint32_t i, uint32_t v,
                                const double *pa) {
  const int64_t cap = P.cap;
  int idx[D];
  unravel<D>(S, v, idx);
  const SubRange sub_v = subdomain_range(S, v);
  int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
#pragma unroll
  for (int c = 0; c < D; ++c) {
    lo[c] = idx[c] > 0 ? idx[c] - 1 : 0;
    hi[c] = idx[c] + 1 < S.nvox[c] ? idx[c] + 1 : S.nvox[c] - 1;
  }
  Vec3 r = {{0.0, 0.0, 0.0}};
  for (int j0 = lo[0]; j0 <= hi[0]; ++j0)
    for (int j1 = lo[1]; j1 <= hi[1]; ++j1)
      for (int j2 = lo[2]; j2 <= hi[2]; ++j2) {
        const uint32_t w = (D == 3) ? ((uint32_t)j0 * S.nvox[1] + j1) * S.nvox[2] + j2
                                    : (uint32_t)j0 * S.nvox[1] + j1;
        const bool twice = (w == v) || S.weight_mode == CRG_WEIGHTS_PHYSICAL ||
                           !sub_v.same(w);
        uint32_t b0 = P.start[S.voxel_off + w], b1 = P.start[S.voxel_off + w + 1];
        if (b0 > b1 || b1 > P.n_agents) b1 = b0;  // recorded by the caller's own scan
        for (uint32_t b = b0; b < b1; ++b) {
          if (b == i) continue;
          double z[D], h[D];
#pragma unroll
          for (int c = 0; c < D; ++c) z[c] = dsub(pa[c], P.pos[c * cap + b]);
          if (morse_half_f64<D>(z, S, h)) {
#pragma unroll
            for (int c = 0; c < D; ++c) {
              r.x[c] = dadd(r.x[c], h[c]);
              if (twice) r.x[c] = dadd(r.x[c], h[c]);
            }
          }
        }
      }
  return r;
}

// NewtonDamped increment, solver, boundary and next voxel key of agent i with interaction
// force acc (shared by the force kernels).
template <int D>
__device__ __forceinline__ void sphere_update(const PackArgs &P, const SimDev &S, uint32_t i,
                                              uint32_t key, const double *pa,
                                              const double *va, const double *acc) {
  const int64_t cap = P.cap;
  if (P.dbg_force) {
#pragma unroll
    for (int c = 0; c < D; ++c) P.dbg_force[c * cap + i] = acc[c];
  }

  // Mechanics::calculate_increment.  NewtonDamped (mechanics.rs:166-173): dx = v,
  // dv = F/m - lambda v.  Brownian (:350-357): dx = D / k_B T * F, dv = 0.  Langevin
  // (:452-463): dx = v, dv = 1 / M * F + (-gamma) * v.
  double dxv[D], dvv[D];
  if (S.mech == 1) {
    const double sb = ddiv(S.diffusion, S.kb_temperature);
#pragma unroll
    for (int c = 0; c < D; ++c) {
      dxv[c] = dmul(sb, acc[c]);
      dvv[c] = 0.0;
    }
  } else if (S.mech == 2) {
    const double im = ddiv(1.0, S.mass);
#pragma unroll
    for (int c = 0; c < D; ++c) {
      dxv[c] = va[c];
      dvv[c] = dadd(dmul(im, acc[c]), dmul(-S.damping, va[c]));
    }
  } else if (__all_sync(__activemask(), __double_as_longlong(S.mass) == 0x3ff0000000000000ll)) {
    // F / 1 is F exactly (every input, NaN and signed zeros included): no division
#pragma unroll
    for (int c = 0; c < D; ++c) {
      dxv[c] = va[c];
      dvv[c] = dsub(acc[c], dmul(S.damping, va[c]));
    }
  } else {
#pragma unroll
    for (int c = 0; c < D; ++c) {
      dxv[c] = va[c];
      dvv[c] = dsub(ddiv(acc[c], S.mass), dmul(S.damping, va[c]));
    }
  }
  // get_random_contribution times dt, as the solvers add it (`.xapy(1, dx_rand * dt)`):
  // zero for NewtonDamped (mechanics.rs:158-164); Brownian dx_rand = sqrt(2 D) *
  // N(0, sqrt(dt)) / dt (:336-348 with wiener_process :211-226); Langevin dv_rand =
  // sqrt(2 gamma k_B T / M) * N(0, sqrt(dt)) / dt (:434-450).  N(0, s) = 0 + s z.
  const double dt = S.dt;
  double rx[D], rv[D];
#pragma unroll
  for (int c = 0; c < D; ++c) rx[c] = rv[c] = 0.0;
  if (S.stochastic) {
    double z[D];
    stream_normals<D>(S.rng_seed, (uint64_t)(*P.step_ctr + S.step_base), P.id[i], z);
    const double sd = __dsqrt_rn(dt);
    const double amp = (S.mech == 1)
                           ? __dsqrt_rn(dmul(2.0, S.diffusion))
                           : __dsqrt_rn(ddiv(dmul(dmul(2.0, S.damping), S.kb_temperature), S.mass));
#pragma unroll
    for (int c = 0; c < D; ++c) {
      const double r = dmul(dmul(amp, ddiv(dadd(0.0, dmul(sd, z[c])), dt)), dt);
      if (S.mech == 1)
        rx[c] = r;
      else
        rv[c] = r;
    }
  }
  // Solvers (chili/solvers.rs:23-55, 156-347).
  double np[D], nvl[D];
  uint8_t meta = 0;
  if (S.order == 1 && !S.stochastic) {  // + rx and + rv add +0.0: plus_zero, exactly
#pragma unroll
    for (int c = 0; c < D; ++c) {
      np[c] = plus_zero(dadd(dmul(dxv[c], dt), pa[c]));
      nvl[c] = plus_zero(dadd(dmul(dvv[c], dt), va[c]));
    }
  } else if (S.order == 1) {
#pragma unroll
    for (int c = 0; c < D; ++c) {
      np[c] = dadd(dadd(dmul(dxv[c], dt), pa[c]), rx[c]);
      nvl[c] = dadd(dadd(dmul(dvv[c], dt), va[c]), rv[c]);
    }
  } else {
    // The history is pushed before it is read (solvers.rs:178-185), so the newest stored
    // increment is the current one: AB2 uses [dx, dx]; AB3 uses [dx, dx] on its first step
    // and [dx, previous, dx] afterwards.
    const uint8_t have_prev = P.hmeta[i];
    const bool ab3 = (S.order == 3) && have_prev;
#pragma unroll
    for (int c = 0; c < D; ++c) {
      if (ab3) {
        const double f0 = 23.0 / 12.0, f1 = -16.0 / 12.0, f2 = 5.0 / 12.0;
        const double px = P.hist[c * cap + i], pv = P.hist[(D + c) * cap + i];
        np[c] = dadd(dadd(dmul(dadd(dmul(dxv[c], f0), dadd(dmul(px, f1), dmul(dxv[c], f2))), dt),
                          pa[c]), rx[c]);
        nvl[c] = dadd(dadd(dmul(dadd(dmul(dvv[c], f0), dadd(dmul(pv, f1), dmul(dvv[c], f2))), dt),
                           va[c]), rv[c]);
      } else {
        const double f0 = 3.0 / 2.0, f1 = -1.0 / 2.0;
        np[c] = dadd(dadd(dmul(dadd(dmul(dxv[c], f0), dmul(dxv[c], f1)), dt), pa[c]), rx[c]);
        nvl[c] = dadd(dadd(dmul(dadd(dmul(dvv[c], f0), dmul(dvv[c], f1)), dt), va[c]), rv[c]);
      }
      P.nhist[c * cap + i] = dxv[c];
      P.nhist[(D + c) * cap + i] = dvv[c];
    }
    meta = 1;
    P.nhmeta[i] = meta;
  }

  // CartesianSubDomain::apply_boundary (cartesian_cuboid_n.rs:594-631), the comparisons
  // with the domain bounds on the integer pipe (same results, NaN included).
  bool inside = true;
#pragma unroll
  for (int c = 0; c < D; ++c) {
    if (f64_lt_key(np[c], S.min_key[c])) {
      np[c] = dsub(dmul(2.0, S.min[c]), np[c]);
      nvl[c] = fabs(nvl[c]);
    }
    if (f64_gt_key(np[c], S.max_key[c])) {
      np[c] = dsub(dmul(2.0, S.max[c]), np[c]);
      nvl[c] = -fabs(nvl[c]);
    }
  }
#pragma unroll
  for (int c = 0; c < D; ++c)
    if (f64_lt_key(np[c], S.min_key[c]) || f64_gt_key(np[c], S.max_key[c])) inside = false;
  if (!inside) set_status(P.status, CRG_EBOUNDARY, P.id[i], *P.step_ctr + 1, S.sim_index);
  if (S.mech == 1) {  // Brownian::set_velocity is a no-op: the velocity stays as it was
#pragma unroll
    for (int c = 0; c < D; ++c) nvl[c] = va[c];
  }
#pragma unroll
  for (int c = 0; c < D; ++c) {
    P.npos[c * cap + i] = np[c];
    P.nvel[c * cap + i] = nvl[c];
  }
  // sort_cells_in_voxels_step_1 (update_mechanics.rs:427-456): a failed or out-of-grid
  // index leaves the agent in its voxel.
  uint32_t plain;
  uint32_t nk = key;
  if (voxel_of<D>(S, np, plain) == 0) nk = S.voxel_off + plain;
  if (nk - S.voxel_off >= S.n_vox) {
    invariant_failed(P.status, kSiteNextKey, i);
    nk = key;
  }
  P.nkey[i] = nk;
  P.nid[i] = P.id[i];
  atomicAdd(&P.count[nk], 1u);
}

// Mixed thread-per-agent kernel: prefilter survivors buffered per thread (candidate index
// and box code in dynamic shared memory, [kSurv][blockDim]) and evaluated in candidate
// order once kSurv are buffered and at the end.  The scan itself is cheap, and a warp then
// runs the FP32 Morse over buffered survivors with most lanes busy instead of once per scan
// position with the few lanes whose candidate survived.
constexpr int kSurv = 16;
constexpr size_t mixed_step_smem(int block) { return (size_t)kSurv * block * 5; }

// The force and update of agent i (thread per agent; sSurv: the block's survivor buffer).
template <int D, int PREC>
__device__ __forceinline__ void sphere_agent(const PackArgs &P, const uint32_t i,
                                             uint32_t *sSurv) {
  const uint32_t sim = (P.n_sims == 1) ? 0u : sim_of_agent(P, i);
  const SimDev &S = P.sims[sim];
  const int64_t cap = P.cap;
  uint32_t key = P.key[i];
  if (key - S.voxel_off >= S.n_vox) {
    invariant_failed(P.status, kSiteForceKey, i);
    key = S.voxel_off;
  }
  if (sim_frozen(P, S)) {  // frozen simulation
    frozen_copy(P, i, key, D);
    return;
  }
  const uint32_t v = key - S.voxel_off;
  int idx[D];
  unravel<D>(S, v, idx);
  double pa[D], va[D];
  float oa[D];
#pragma unroll
  for (int c = 0; c < D; ++c) {
    pa[c] = P.pos[c * cap + i];
    va[c] = P.vel[c * cap + i];
  }
  sphere_off<D>(P.off, i, oa);
  const SubRange sub_v = subdomain_range(S, v);
  const float thr2 = P.prefilter ? S.filt_thr2 : __int_as_float(0x7f800000);
  double acc[D];
  float fs[D], fcmp[D];
  bool nan_seen = false;  // mixed path: a NaN displacement met (see k_spheres_fix)
#pragma unroll
  for (int c = 0; c < D; ++c) {
    acc[c] = 0.0;
    fs[c] = 0.0f;
    fcmp[c] = 0.0f;
  }
  int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
#pragma unroll
  for (int c = 0; c < D; ++c) {
    lo[c] = idx[c] > 0 ? idx[c] - 1 : 0;
    hi[c] = idx[c] + 1 < S.nvox[c] ? idx[c] + 1 : S.nvox[c] - 1;
  }
  // MIXED: the buffered survivors, evaluated in order (the scan's own arithmetic for zf)
  const uint32_t bd = blockDim.x, tid = threadIdx.x;
  uint32_t *sB = sSurv;
  uint8_t *sM = reinterpret_cast<uint8_t *>(sSurv + kSurv * bd);
  int ns = 0;
  auto flush = [&]() {
    for (int q = 0; q < ns; ++q) {
      const uint32_t b = sB[q * bd + tid], m = sM[q * bd + tid];
      float kd[D], zf[D], ob[D], d2 = 0.0f;
      sphere_off<D>(P.off, b, ob);
#pragma unroll
      for (int c = 0; c < D; ++c) {
        kd[c] = (float)((int)((m >> (2 * c)) & 3u) - 1) * S.dxf[c];
        zf[c] = (oa[c] - ob[c]) - kd[c];
        d2 = fmaf(zf[c], zf[c], d2);
      }
      float h[D];
      if (mixed_half<D>(P, S, pa, b, zf, d2, h)) {
        const bool twice = (m >> 6) & 1u;
#pragma unroll
        for (int c = 0; c < D; ++c) {
          nan_seen |= h[c] != h[c];
          kahan_add(fs[c], fcmp[c], h[c]);
          if (twice) kahan_add(fs[c], fcmp[c], h[c]);
        }
      }
    }
    ns = 0;
  };
  // Candidates in chili's visiting order: boxes j0, j1 (, j2) ascending, each box's agents
  // in cell-list order.  The up to three boxes along the last axis are consecutive voxels,
  // so each row of them is one contiguous candidate range; a candidate's box (its offset kd
  // on the last axis and its pair weight) follows from two compares with the box bounds.
  constexpr int L = D - 1;  // last axis
  const int nb = hi[L] - lo[L] + 1;  // boxes per row (1..3)
  // The scan's distance takes the box shift into the agent's own offset once per row (and
  // per box on the last axis): (oa - kd) - ob, the same bound on its error as the survivors'
  // (oa - ob) - kd (within the prefilter margin), so the scan keeps the same survivors up to
  // pairs far beyond the cutoff, which the exact decision rejects anyway.
  float oal[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) oal[q] = oa[L] - (float)(lo[L] + q - idx[L]) * S.dxf[L];
  const int n1 = (D == 3) ? hi[1] - lo[1] + 1 : 1;
  const int n_rows = (hi[0] - lo[0] + 1) * n1;
  for (int row = 0; row < n_rows; ++row) {
    const int j0 = lo[0] + row / n1;
    const int j1 = (D == 3) ? lo[1] + row % n1 : 0;
    float oak[D];  // the agent's offsets less the row's box shift (last axis: per box)
    oak[0] = oa[0] - (float)(j0 - idx[0]) * S.dxf[0];
    if (D == 3) oak[1] = oa[1] - (float)(j1 - idx[1]) * S.dxf[1];
    const uint32_t w0 = ((D == 3) ? ((uint32_t)j0 * S.nvox[1] + j1) * S.nvox[2]
                                  : (uint32_t)j0 * S.nvox[1]) + lo[L];
    // box bounds s[0..nb]; a box whose range is not valid is reported and left empty
    uint32_t sb[4];
    sb[0] = P.start[S.voxel_off + w0];
    uint32_t tw_bits = 0;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      if (q < nb) {
        uint32_t e = P.start[S.voxel_off + w0 + q + 1];
        if (sb[q] > e || e > P.n_agents) {
          invariant_failed(P.status, kSiteForceRange, S.voxel_off + w0 + q);
          e = sb[q];
        }
        sb[q + 1] = e;
        const uint32_t w = w0 + q;
        if ((w == v) || S.weight_mode == CRG_WEIGHTS_PHYSICAL || !sub_v.same(w))
          tw_bits |= 1u << q;
      } else {
        sb[q + 1] = sb[q];
      }
    }
    // the bounds are non-decreasing (an invalid box was left empty), so [sb[0], sb[nb]) is
    // the row's candidates box after box (in a cell list that failed its checks, a box left
    // empty may hand its range to the next one: the step reports CRG_EINTERNAL and rolls back)
    {
      for (uint32_t b = sb[0]; b < sb[nb]; ++b) {
        const int q = (int)(b >= sb[1]) + (int)(b >= sb[2]);
        oak[L] = (q == 0) ? oal[0] : (q == 1) ? oal[1] : oal[2];
        const bool twice = (tw_bits >> q) & 1u;
        float ob[D];
        float d2 = 0.0f;
        sphere_off<D>(P.off, b, ob);
#pragma unroll
        for (int c = 0; c < D; ++c) {
          const float z = oak[c] - ob[c];
          d2 = fmaf(z, z, d2);
        }
        // the agent itself and pairs beyond the prefilter threshold are skipped (one branch;
        // a NaN distance falls through to the exact path)
        if (b == i || d2 > thr2) continue;
        if (PREC == CRG_PREC_F64) {
          double z[D], h[D];
#pragma unroll
          for (int c = 0; c < D; ++c) z[c] = dsub(pa[c], P.pos[c * cap + b]);
          if (morse_half_f64<D>(z, S, h)) {
#pragma unroll
            for (int c = 0; c < D; ++c) {
              acc[c] = dadd(acc[c], h[c]);
              if (twice) acc[c] = dadd(acc[c], h[c]);
            }
          }
        } else {
          // FP32 Morse on the FP32 displacement (offsets from the voxel centres, accurate
          // to 2^-25 dx).  Whether the pair interacts is decided exactly as on the FP64
          // path: pairs whose FP32 distance lies within the prefilter margin of the cutoff
          // or of zero are decided from the FP64 distance, so no pair switches on or off
          // relative to FP64.  A NaN displacement (an offset marked NaN because its agent
          // is far outside its voxel, or NaN positions) hands the whole agent to the FP64
          // fix-up kernel.
          if (d2 != d2) {
            nan_seen = true;
            continue;
          }
          const int dl = lo[L] + q - idx[L];
          const int d1 = (D == 3) ? j1 - idx[1] : dl;
          sB[ns * bd + tid] = b;
          sM[ns * bd + tid] = (uint8_t)((j0 - idx[0] + 1) | ((d1 + 1) << 2) |
                                        (((D == 3) ? dl : 0) + 1) << 4 | (twice ? 0x40 : 0));
          if (++ns == kSurv) flush();
        }
      }
    }
  }
  if (PREC != CRG_PREC_F64) {
    flush();
    if (nan_seen) {  // k_spheres_fix computes this agent's force and update in FP64
      P.fix_list[atomicAdd(&P.rctl[0], 1u)] = i;
      return;
    }
#pragma unroll
    for (int c = 0; c < D; ++c) acc[c] = (double)__fsub_rn(fs[c], fcmp[c]);  // the compensated sum, rounded once
  }
  sphere_update<D>(P, S, i, key, pa, va, acc);
}

template <int D, int PREC>
__global__ void __launch_bounds__(256, (PREC == CRG_PREC_F64) ? 3 : 4) k_spheres_step(const PackArgs P) {
  extern __shared__ uint32_t sSurv[];  // MIXED: [kSurv][blockDim] candidates, then box codes
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n_agents) return;
  sphere_agent<D, PREC>(P, i, sSurv);
}

// Persistent form of k_spheres_step (P.tile > 0): a grid of as many blocks as the SMs hold
// at once, each claiming tiles of blockDim * P.tile consecutive agents of the cell list (a
// run of voxels along the last axis and their neighbours' rows) from the counter rctl[2]
// (zeroed before the launch) until none is left.  Thread t of a block takes agents
// base + t, base + t + blockDim, ... of its tile: the same per-agent work as k_spheres_step,
// so the results are identical whatever the tile size and claim order.
template <int D, int PREC>
__global__ void __launch_bounds__(256, (PREC == CRG_PREC_F64) ? 3 : 4) k_spheres_tiles(const PackArgs P) {
  extern __shared__ uint32_t sSurv[];
  __shared__ uint32_t sTile;
  const uint32_t per = (uint32_t)P.tile, tile_agents = blockDim.x * per;
  const uint32_t n_tiles = (P.n_agents + tile_agents - 1) / tile_agents;
  for (;;) {
    if (threadIdx.x == 0) sTile = atomicAdd(&P.rctl[2], 1u);
    __syncthreads();
    const uint32_t t = sTile;
    __syncthreads();  // every thread has read sTile before thread 0 claims again
    if (t >= n_tiles) break;
    const uint32_t base = t * tile_agents;
    for (uint32_t j = 0; j < per; ++j) {
      const uint32_t i = base + j * blockDim.x + threadIdx.x;
      if (i < P.n_agents) sphere_agent<D, PREC>(P, i, sSurv);
    }
  }
}

// Resident blocks of k_spheres_tiles on the whole device for [dim - 2][precision == MIXED]
// [block / 64 - 1], set by prepare_spheres when a handle is created (an occupancy query
// inside a stream capture could load the module, which a capture does not allow); 0: unknown.
unsigned g_tile_grid[2][2][4] = {};

template <int D, int PREC>
cudaError_t prepare_tiles() {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  for (int q = 0; q < 4 && e == cudaSuccess; ++q) {
    const int block = 64 * (q + 1);
    const size_t smem = (PREC == CRG_PREC_F64) ? 0 : mixed_step_smem(block);
    int n = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_spheres_tiles<D, PREC>, block, smem);
    if (e == cudaSuccess) g_tile_grid[D - 2][PREC == CRG_PREC_F64 ? 0 : 1][q] = (unsigned)(sms * n);
  }
  return e;
}

template <int D, int PREC>
void launch_tiles(const PackArgs &P, int block, cudaStream_t st) {
  const uint32_t tile_agents = (uint32_t)block * (uint32_t)P.tile;
  const unsigned n_tiles = (P.n_agents + tile_agents - 1) / tile_agents;
  unsigned grid = g_tile_grid[D - 2][PREC == CRG_PREC_F64 ? 0 : 1][block / 64 - 1];
  if (!grid || grid > n_tiles) grid = n_tiles;
  const size_t smem = (PREC == CRG_PREC_F64) ? 0 : mixed_step_smem(block);
  k_spheres_tiles<D, PREC><<<grid, block, smem, st>>>(P);
}

// Largest system the FP64 default runs with agent groups (k_spheres_groups); above it the
// lane-per-agent kernel has warps enough to fill the SMs.
constexpr uint32_t kSphereGroupsMax = 38912;
constexpr int kGrpCap = 64;  // survivor list of an agent between evaluations

// ---------------------------------------------------------------------------------------
// Agent groups (FP64, small systems).  With a few thousand agents the lane-per-agent kernel
// leaves most SMs without a warp, and a warp per agent wastes the FP64 lanes of the agent's
// few survivors.  Here a warp carries 32 / L agents with L lanes each (L = 8 by default;
// 16 and 32 give small systems more warps):
//   * each group numbers its agent's candidates consecutively -- the 3^D neighbourhood
//     boxes in visiting order, each box's agents in cell-list order, itself skipped -- and
//     scans L per round through the FP32 prefilter, appending survivors in order to the
//     agent's list in shared memory;
//   * the survivors of the warp's agents are evaluated in FP64 in full 32-lane batches;
//   * lanes 0..D-1 of each group add the agent's half-forces in list (= candidate) order,
//     one component each; at the end one thread per agent of the block updates it.
// Same terms, same order of additions as k_spheres_step: identical bits.
// ---------------------------------------------------------------------------------------
template <int D, int L>
__global__ void __launch_bounds__(128) k_spheres_groups(const PackArgs P) {
  constexpr int kGrpL = L;       // lanes per agent
  constexpr int kGrpA = 32 / L;  // agents per warp
  constexpr uint32_t kGrpMask = (L == 32) ? 0xffffffffu : ((1u << L) - 1u);
  __shared__ uint32_t sB0[4][kGrpA][27], sPre[4][kGrpA][28];
  __shared__ float sKd[4][kGrpA][27][D];
  __shared__ uint8_t sTw[4][kGrpA][27];
  __shared__ uint32_t sPart[4][kGrpA][kGrpCap];
  __shared__ uint8_t sWt[4][kGrpA][kGrpCap];
  __shared__ double sH[4][kGrpA][kGrpCap][D];
  __shared__ uint8_t sOk[4][kGrpA][kGrpCap];
  __shared__ double sAcc[4][kGrpA][D];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int g = lane / kGrpL, k = lane % kGrpL;
  const uint32_t agent0 = (blockIdx.x * 4 + w) * kGrpA;
  const uint32_t i = agent0 + g;
  const bool valid = i < P.n_agents;
  const uint32_t ii = valid ? i : 0u;
  const int64_t cap = P.cap;
  const uint32_t sim = (P.n_sims == 1) ? 0u : sim_of_agent(P, ii);
  const SimDev &S = P.sims[sim];
  uint32_t key = P.key[ii];
  if (key - S.voxel_off >= S.n_vox) {
    if (valid && k == 0) invariant_failed(P.status, kSiteForceKey, i);
    key = S.voxel_off;
  }
  const bool live = valid && !sim_frozen(P, S);
  if (valid && !live && k == 0) frozen_copy(P, i, key, D);
  const uint32_t v = key - S.voxel_off;
  int idx[D];
  unravel<D>(S, v, idx);
  float oa[D];
  sphere_off<D>(P.off, ii, oa);
  const SubRange sub_v = subdomain_range(S, v);
  const float thr2 = P.prefilter ? S.filt_thr2 : __int_as_float(0x7f800000);
  int lo[3] = {0, 0, 0}, nb[3] = {1, 1, 1};
#pragma unroll
  for (int c = 0; c < D; ++c) {
    lo[c] = idx[c] > 0 ? idx[c] - 1 : 0;
    const int hi = idx[c] + 1 < S.nvox[c] ? idx[c] + 1 : S.nvox[c] - 1;
    nb[c] = hi - lo[c] + 1;
  }
  const int n_box = live ? nb[0] * nb[1] * nb[2] : 0;  // <= 27
  // ---- the agent's boxes: first agent, count (-> prefix), weight, centre shift --------
  for (int q = k; q < n_box; q += kGrpL) {
    const int j2 = lo[2] + q % nb[2];
    const int j1 = lo[1] + (q / nb[2]) % nb[1];
    const int j0 = lo[0] + q / (nb[1] * nb[2]);
    const uint32_t wv = (D == 3) ? ((uint32_t)j0 * S.nvox[1] + j1) * S.nvox[2] + j2
                                 : (uint32_t)j0 * S.nvox[1] + j1;
    sTw[w][g][q] = ((wv == v) || S.weight_mode == CRG_WEIGHTS_PHYSICAL ||
                    !sub_v.same(wv)) ? 2 : 1;
    const int dj[3] = {j0 - idx[0], j1 - idx[1], D == 3 ? j2 - idx[D - 1] : 0};
#pragma unroll
    for (int c = 0; c < D; ++c) sKd[w][g][q][c] = (float)dj[c] * S.dxf[c];
    const uint32_t b0 = P.start[S.voxel_off + wv], b1 = P.start[S.voxel_off + wv + 1];
    uint32_t cnt = 0;
    if (b0 > b1 || b1 > P.n_agents)
      invariant_failed(P.status, kSiteForceRange, S.voxel_off + wv);
    else
      cnt = b1 - b0;
    sB0[w][g][q] = b0;
    sPre[w][g][q + 1] = cnt;
  }
  __syncwarp();
  if (k == 0) {
    sPre[w][g][0] = 0;
    for (int q = 0; q < n_box; ++q) sPre[w][g][q + 1] += sPre[w][g][q];
  }
  __syncwarp();
  const uint32_t total = sPre[w][g][n_box];

  double acc[D], acc_k = 0.0;  // acc_k: component k of the force (lanes k < D)
  uint32_t j_next = 0;  // the group's next candidate
  while (__any_sync(0xffffffffu, j_next < total)) {
    // ---- scan rounds until the candidates are done or a list could overflow ----------
    int n_list = 0;
    while (true) {
      const bool can = j_next < total && n_list + kGrpL <= kGrpCap;
      if (!__any_sync(0xffffffffu, can)) break;
      const uint32_t j = j_next + k;
      bool surv = false;
      uint32_t b = 0;
      uint8_t wt = 0;
      if (can && j < total) {
        int q = 0, qh = n_box;  // last box whose prefix is <= j
        while (qh - q > 1) {
          const int m = (q + qh) >> 1;
          if (sPre[w][g][m] <= j) q = m; else qh = m;
        }
        b = sB0[w][g][q] + (j - sPre[w][g][q]);
        if (b != i) {
          float d2 = 0.0f, ob[D];
          sphere_off<D>(P.off, b, ob);
#pragma unroll
          for (int c = 0; c < D; ++c) {
            const float z = (oa[c] - ob[c]) - sKd[w][g][q][c];
            d2 = fmaf(z, z, d2);
          }
          surv = !(d2 > thr2);  // NaN falls through to the exact path
          wt = sTw[w][g][q];
        }
      }
      const uint32_t gm = (__ballot_sync(0xffffffffu, surv) >> (g * kGrpL)) & kGrpMask;
      if (surv) {
        const int pos = n_list + __popc(gm & ((1u << k) - 1u));
        sPart[w][g][pos] = b;
        sWt[w][g][pos] = wt;
      }
      if (can) {
        n_list += __popc(gm);
        j_next += kGrpL;
      }
    }
    __syncwarp();
    // ---- FP64 Morse for the listed survivors of the warp's agents, full batches -------
    int st[kGrpA + 1];
    st[0] = 0;
#pragma unroll
    for (int gg = 0; gg < kGrpA; ++gg)
      st[gg + 1] = st[gg] + __shfl_sync(0xffffffffu, n_list, gg * kGrpL);
    for (int t0 = 0; t0 < st[kGrpA]; t0 += 32) {
      const int t = t0 + lane;
      if (t < st[kGrpA]) {
        int gg = 0;
#pragma unroll
        for (int q = 1; q < kGrpA; ++q) gg += (t >= st[q]);
        const int m = t - st[gg];
        const uint32_t a = agent0 + gg, b = sPart[w][gg][m];
        const uint32_t sim_a = (P.n_sims == 1) ? 0u : sim_of_agent(P, a);
        double z[D], h[D];
#pragma unroll
        for (int c = 0; c < D; ++c) z[c] = dsub(P.pos[c * cap + a], P.pos[c * cap + b]);
        // no reconvergence points here: this kernel runs with few warps per SM, where
        // overlapping the three divisions matters more than full lanes
        const bool ok = morse_half_f64<D>(z, P.sims[sim_a], h);
        sOk[w][gg][m] = ok ? 1 : 0;
#pragma unroll
        for (int c = 0; c < D; ++c) sH[w][gg][m][c] = h[c];
      }
    }
    __syncwarp();
    // ---- each agent's half-forces in candidate order: lane k of the group folds
    // component k (the components' sums are independent chains) ------------------------
    if (k < D) {
      for (int m = 0; m < n_list; ++m) {
        if (!sOk[w][g][m]) continue;
        const double h = sH[w][g][m][k];
        acc_k = dadd(acc_k, h);
        if (sWt[w][g][m] == 2) acc_k = dadd(acc_k, h);
      }
    }
    __syncwarp();
  }
  // ---- updates: the block's 4 * kGrpA agents, one thread each (thread t: warp t / kGrpA,
  // group t % kGrpA), so the update's instructions run on a quarter of the warps ---------
  if (k < D) sAcc[w][g][k] = acc_k;
  __syncthreads();
  if (threadIdx.x < 4 * kGrpA) {
    const int wu = threadIdx.x / kGrpA, gu = threadIdx.x % kGrpA;
    const uint32_t iu = (blockIdx.x * 4 + wu) * kGrpA + gu;
    if (iu < P.n_agents) {
      const uint32_t simu = (P.n_sims == 1) ? 0u : sim_of_agent(P, iu);
      const SimDev &Su = P.sims[simu];
      uint32_t keyu = P.key[iu];
      if (keyu - Su.voxel_off >= Su.n_vox) keyu = Su.voxel_off;  // reported above
      if (!sim_frozen(P, Su)) {
        double pu[D], vu[D];
#pragma unroll
        for (int c = 0; c < D; ++c) {
          pu[c] = P.pos[c * cap + iu];
          vu[c] = P.vel[c * cap + iu];
          acc[c] = sAcc[wu][gu][c];
        }
        sphere_update<D>(P, Su, iu, keyu, pu, vu, acc);
      }
    }
  }
}

// The agents the mixed kernel handed over (rctl[0] of them in fix_list): FP64 force and
// update, exactly as the FP64 path would compute them.
template <int D>
__global__ void __launch_bounds__(128) k_spheres_fix(const PackArgs P) {
  const uint32_t n = P.rctl[0];
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const uint32_t i = P.fix_list[t];
    const uint32_t sim = (P.n_sims == 1) ? 0u : sim_of_agent(P, i);
    const SimDev &S = P.sims[sim];
    const uint32_t key = P.key[i];  // checked by the mixed kernel
    const int64_t cap = P.cap;
    double pa[D], va[D], acc[D];
#pragma unroll
    for (int c = 0; c < D; ++c) {
      pa[c] = P.pos[c * cap + i];
      va[c] = P.vel[c * cap + i];
    }
    const Vec3 f = agent_force_f64<D>(P, S, i, key - S.voxel_off, pa);
#pragma unroll
    for (int c = 0; c < D; ++c) acc[c] = f.x[c];
    sphere_update<D>(P, S, i, key, pa, va, acc);
  }
}

// ---------------------------------------------------------------------------------------
// Warp-packed variant (lane per agent; the FP64 default for large systems).  Lane l owns
// agent a_l.  Each round every lane scans the next G positions of its candidate stream
// (neighbour voxels ascending, cell-list order inside a voxel, itself skipped) through the
// FP32 prefilter and records its survivors (partner, neighbour box).  The warp's survivors,
// numbered lane by lane, are evaluated in chunks of kSphereCap with every lane busy
// (half-forces to shared memory); after each chunk every lane adds the half-forces of its
// own survivors in that chunk in stream order, twice for a partner whose pair weight is 1.
// FP64: morse_half_f64 and dadd; mixed: mixed_half and compensated FP32 sums.  Same terms,
// same order of additions as k_spheres_step: identical bits.  Shared memory per warp is
// bounded by the chunk rather than by the worst case of 32 x G survivors, so an SM holds
// enough warps to hide the latency of the scan's loads.
// ---------------------------------------------------------------------------------------
constexpr int kSphereG = 32;  // stream positions a lane scans per round (default shape)

template <int D, int G, int PREC>
__global__ void __launch_bounds__(32) k_spheres_pass(const PackArgs P) {
  static_assert(G <= 64, "survivor weights are a 64-bit mask");
  constexpr bool MIX = PREC != CRG_PREC_F64;
  constexpr int kSphereCap = 4 * G;  // survivors evaluated per chunk
  using Mask = typename std::conditional<(G > 32), uint64_t, uint32_t>::type;
  __shared__ double sH[MIX ? 1 : D][kSphereCap];  // FP64: half-forces of the current chunk
  __shared__ float sF[MIX ? D : 1][kSphereCap];   // mixed: half-forces of the current chunk
  __shared__ uint32_t sOk[kSphereCap / 32];       // mixed: bit set = the pair interacts
  __shared__ uint32_t sB[G][32];                  // survivor k of lane l: partner index
  __shared__ uint8_t sK[MIX ? G : 1][32];         // mixed: neighbour box, 2 bits per axis
  const int lane = threadIdx.x;
  const uint32_t warp_base = blockIdx.x * 32;
  const uint32_t i = warp_base + lane;
  const bool valid = i < P.n_agents;
  const int64_t cap = P.cap;
  const uint32_t ii = valid ? i : 0u;
  const uint32_t sim = (P.n_sims == 1) ? 0u : sim_of_agent(P, ii);
  const SimDev &S = P.sims[sim];
  uint32_t key = P.key[ii];
  if (key - S.voxel_off >= S.n_vox) {
    if (valid) invariant_failed(P.status, kSiteForceKey, i);
    key = S.voxel_off;
  }
  const uint32_t v = key - S.voxel_off;
  int idx[D];
  unravel<D>(S, v, idx);
  double pa[D], va[D];
  float oa[D];
#pragma unroll
  for (int c = 0; c < D; ++c) {
    pa[c] = P.pos[c * cap + ii];
    va[c] = P.vel[c * cap + ii];
  }
  sphere_off<D>(P.off, ii, oa);
  const SubRange sub_v = subdomain_range(S, v);
  const float thr2 = P.prefilter ? S.filt_thr2 : __int_as_float(0x7f800000);
  int lo[3] = {0, 0, 0}, nb[3] = {1, 1, 1};
#pragma unroll
  for (int c = 0; c < D; ++c) {
    lo[c] = idx[c] > 0 ? idx[c] - 1 : 0;
    const int hi = idx[c] + 1 < S.nvox[c] ? idx[c] + 1 : S.nvox[c] - 1;
    nb[c] = hi - lo[c] + 1;
  }
  const bool frozen = valid && sim_frozen(P, S);
  bool done = !valid || frozen;
  int c0 = lo[0], c1 = lo[1], c2 = lo[2];  // next neighbour box; c0 past the end: none left
  uint32_t b_next = 0, b_end = 0;
  bool twice = false;
  uint32_t kcode = 0;
  float kd[D];
#pragma unroll
  for (int c = 0; c < D; ++c) kd[c] = 0.f;
  double acc[D];
  float fs[D], fcmp[D];  // mixed: compensated FP32 sums
  bool nan_seen = false;
#pragma unroll
  for (int c = 0; c < D; ++c) {
    acc[c] = 0.0;
    fs[c] = fcmp[c] = 0.0f;
  }

  while (__any_sync(0xffffffffu, !done)) {
    // ---- scan the next G stream positions ------------------------------------------
    int cnt = 0;
    Mask twice_mask = 0;
    int g = 0;
    while (!done && g < G) {
      if (b_next >= b_end) {
        if (c0 >= lo[0] + nb[0]) {
          done = true;
          break;
        }
        const int j0 = c0, j1 = c1, j2 = c2;  // boxes in the order of k_spheres_step's loops
        if (++c2 >= lo[2] + nb[2]) {
          c2 = lo[2];
          if (++c1 >= lo[1] + nb[1]) {
            c1 = lo[1];
            ++c0;
          }
        }
        const uint32_t w = (D == 3) ? ((uint32_t)j0 * S.nvox[1] + j1) * S.nvox[2] + j2
                                    : (uint32_t)j0 * S.nvox[1] + j1;
        twice = (w == v) || S.weight_mode == CRG_WEIGHTS_PHYSICAL || !sub_v.same(w);
        // centre(a) - centre(b) = -(j - idx) * dx
        kd[0] = (float)(j0 - idx[0]) * S.dxf[0];
        kd[1] = (float)(j1 - idx[1]) * S.dxf[1];
        if (D == 3) kd[D - 1] = (float)(j2 - idx[D - 1]) * S.dxf[D - 1];
        kcode = (uint32_t)(j0 - idx[0] + 1) | ((uint32_t)(j1 - idx[1] + 1) << 2);
        if (D == 3) kcode |= (uint32_t)(j2 - idx[D - 1] + 1) << 4;
        b_next = P.start[S.voxel_off + w];
        b_end = P.start[S.voxel_off + w + 1];
        if (b_next > b_end || b_end > P.n_agents) {
          invariant_failed(P.status, kSiteForceRange, S.voxel_off + w);
          b_end = b_next;
        }
        continue;
      }
      const uint32_t b = b_next++;
      ++g;
      if (b == i) continue;
      float d2 = 0.0f, ob[D];
      sphere_off<D>(P.off, b, ob);
#pragma unroll
      for (int c = 0; c < D; ++c) {
        const float z = (oa[c] - ob[c]) - kd[c];
        d2 = fmaf(z, z, d2);
      }
      if (d2 > thr2) continue;  // NaN falls through to the exact path
      sB[cnt][lane] = b;
      if (MIX) sK[cnt][lane] = (uint8_t)kcode;
      if (twice) twice_mask |= (Mask)1 << cnt;
      ++cnt;
    }

    // ---- number the warp's survivors lane by lane ----------------------------------
    int incl = cnt;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, off);
      if (lane >= off) incl += y;
    }
    const int excl = incl - cnt;
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    __syncwarp();
    for (int base = 0; base < total; base += kSphereCap) {
      const int lim = min(total, base + kSphereCap);
      // ---- evaluate survivors [base, lim) with every lane busy ---------------------
      for (int jb = base; jb < lim; jb += 32) {
        const int j = jb + lane;
        int l = 0;  // owner: the last lane whose first survivor is <= j
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
          const int cand = l + step;
          const int e = __shfl_sync(0xffffffffu, excl, cand & 31);
          if (cand < 32 && e <= j) l = cand;
        }
        const int ex_l = __shfl_sync(0xffffffffu, excl, l);
        const uint32_t sim_l = __shfl_sync(0xffffffffu, sim, l);
        const uint32_t act = __ballot_sync(0xffffffffu, j < lim);
        bool ok = false;
        if (j < lim) {
          const int k = j - ex_l;
          const uint32_t b = sB[k][l];
          const uint32_t a = warp_base + l;
          const SimDev &So = P.sims[sim_l];
          if (!MIX) {
            double z[D], h[D];
#pragma unroll
            for (int c = 0; c < D; ++c) z[c] = dsub(P.pos[c * cap + a], P.pos[c * cap + b]);
            morse_half_f64_batch<D>(z, So, h, act);  // +0 when out of range: adds nothing
#pragma unroll
            for (int c = 0; c < D; ++c) sH[c][j - base] = h[c];
          } else {
            // the scan's FP32 displacement, recomputed with the same operations
            const uint32_t code = sK[k][l];
            float zf[D], hf[D];
            float d2 = 0.0f;
            float oa_l[D], ob_l[D];
            sphere_off<D>(P.off, a, oa_l);
            sphere_off<D>(P.off, b, ob_l);
#pragma unroll
            for (int c = 0; c < D; ++c) {
              const float kdc = (float)((int)((code >> (2 * c)) & 3u) - 1) * So.dxf[c];
              zf[c] = (oa_l[c] - ob_l[c]) - kdc;
              d2 = fmaf(zf[c], zf[c], d2);
            }
            double pa_l[D];
#pragma unroll
            for (int c = 0; c < D; ++c) pa_l[c] = P.pos[c * cap + a];
            // a NaN displacement reaches the owner as a NaN half-force (its agent goes to
            // the fix-up); a pair out of range is left out of the sum altogether
            const bool nan = d2 != d2;
            ok = nan || mixed_half<D>(P, So, pa_l, b, zf, d2, hf);
            __syncwarp(act);
#pragma unroll
            for (int c = 0; c < D; ++c) sF[c][j - base] = nan ? d2 : hf[c];
          }
        }
        if (MIX) {
          const uint32_t okm = __ballot_sync(0xffffffffu, ok);
          if (lane == 0) sOk[(jb - base) >> 5] = okm;
        }
      }
      __syncwarp();
      // ---- each lane adds its own survivors of the chunk in stream order -----------
      const int f0 = max(excl, base), f1 = min(incl, lim);
      for (int j = f0; j < f1; ++j) {
        const bool tw = (twice_mask >> (j - excl)) & 1u;  // j - excl < G
        if (!MIX) {
#pragma unroll
          for (int c = 0; c < D; ++c) {
            const double h = sH[c][j - base];
            acc[c] = dadd(acc[c], h);
            if (tw) acc[c] = dadd(acc[c], h);
          }
        } else {
          if (!((sOk[(j - base) >> 5] >> ((j - base) & 31)) & 1u)) continue;
#pragma unroll
          for (int c = 0; c < D; ++c) {
            const float h = sF[c][j - base];
            nan_seen |= h != h;
            kahan_add(fs[c], fcmp[c], h);
            if (tw) kahan_add(fs[c], fcmp[c], h);
          }
        }
      }
      __syncwarp();
    }
  }
  if (!valid) return;
  if (frozen) {
    frozen_copy(P, i, key, D);
    return;
  }
  if (MIX) {
    if (nan_seen) {  // k_spheres_fix computes this agent's force and update in FP64
      P.fix_list[atomicAdd(&P.rctl[0], 1u)] = i;
      return;
    }
#pragma unroll
    for (int c = 0; c < D; ++c) acc[c] = (double)__fsub_rn(fs[c], fcmp[c]);  // the compensated sum, rounded once
  }
  sphere_update<D>(P, S, i, key, pa, va, acc);
}

template <int D>
__global__ void k_sphere_stats(const PackArgs P, uint32_t *n_cand, uint32_t *n_inter,
                               uint64_t *hash) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n_agents) return;
  const uint32_t sim = (P.n_sims == 1) ? 0u : sim_of_agent(P, i);
  const SimDev &S = P.sims[sim];
  const int64_t cap = P.cap;
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
          double z[D], hf[D];
          for (int c = 0; c < D; ++c) z[c] = dsub(P.pos[c * cap + i], P.pos[c * cap + b]);
          if (morse_half_f64<D>(z, S, hf)) ++ni;
        }
      }
  n_cand[i] = nc;
  n_inter[i] = ni;
  hash[i] = h;
}

}  // namespace

void launch_spheres_step(int dim, int precision, const PackArgs &P, int block, cudaStream_t st) {
  if (!P.n_agents) return;
  // FP64 default: agent groups while there are too few agents to give every SM several
  // warps of the lane-per-agent form (variant 2), the lane-per-agent kernel above that
  const bool small = P.n_agents <= kSphereGroupsMax;
  if (precision == CRG_PREC_F64 && (P.variant == 2 || (P.variant == 0 && small))) {
    // lanes per agent: block 16 or 32 (autotuned shapes), else 8 (four agents per warp)
    const int lanes = (block == 16 || block == 32) ? block : 8;
    const unsigned per_block = 4 * (32 / lanes);  // agents per block of four warps
    const unsigned grid = (P.n_agents + per_block - 1) / per_block;
    if (dim == 3) {
      if (lanes == 32) k_spheres_groups<3, 32><<<grid, 128, 0, st>>>(P);
      else if (lanes == 16) k_spheres_groups<3, 16><<<grid, 128, 0, st>>>(P);
      else k_spheres_groups<3, 8><<<grid, 128, 0, st>>>(P);
    } else {
      if (lanes == 32) k_spheres_groups<2, 32><<<grid, 128, 0, st>>>(P);
      else if (lanes == 16) k_spheres_groups<2, 16><<<grid, 128, 0, st>>>(P);
      else k_spheres_groups<2, 8><<<grid, 128, 0, st>>>(P);
    }
    return;
  }
  if (precision == CRG_PREC_F64 && P.variant != 1) {
    // block (autotuned shape): 64 scans 64 stream positions per round into 256-survivor
    // chunks, any other value 32 into 128.  Default: 64 above 2^21 agents, where its fuller
    // folds outweigh the lower occupancy (larger shared memory per warp); 32 below.
    const unsigned grid = (P.n_agents + 31) / 32;
    if (block == 64 || (block == 0 && P.n_agents > (1u << 21))) {
      if (dim == 3)
        k_spheres_pass<3, 64, CRG_PREC_F64><<<grid, 32, 0, st>>>(P);
      else
        k_spheres_pass<2, 64, CRG_PREC_F64><<<grid, 32, 0, st>>>(P);
    } else {
      if (dim == 3)
        k_spheres_pass<3, kSphereG, CRG_PREC_F64><<<grid, 32, 0, st>>>(P);
      else
        k_spheres_pass<2, kSphereG, CRG_PREC_F64><<<grid, 32, 0, st>>>(P);
    }
    return;
  }
  if (block <= 0 || block > 256) block = 128;
  // persistent form (thread per agent); its tile counter is rctl[2]
  const bool tiles = P.tile > 0 && block % 64 == 0 && P.rctl != nullptr;
  if (precision != CRG_PREC_F64 || tiles)  // fix-up count; tile counter
    cudaMemsetAsync(P.rctl, 0, 3 * sizeof(uint32_t), st);
  if (precision != CRG_PREC_F64 && P.variant == 3) {  // warp-packed mixed kernel
    const unsigned grid = (P.n_agents + 31) / 32;
    if (dim == 3) {
      k_spheres_pass<3, kSphereG, CRG_PREC_MIXED><<<grid, 32, 0, st>>>(P);
      k_spheres_fix<3><<<32, 128, 0, st>>>(P);
    } else {
      k_spheres_pass<2, kSphereG, CRG_PREC_MIXED><<<grid, 32, 0, st>>>(P);
      k_spheres_fix<2><<<32, 128, 0, st>>>(P);
    }
    return;
  }
  if (tiles) {
    if (dim == 3) {
      if (precision == CRG_PREC_F64) {
        launch_tiles<3, CRG_PREC_F64>(P, block, st);
      } else {
        launch_tiles<3, CRG_PREC_MIXED>(P, block, st);
        k_spheres_fix<3><<<32, 128, 0, st>>>(P);
      }
    } else {
      if (precision == CRG_PREC_F64) {
        launch_tiles<2, CRG_PREC_F64>(P, block, st);
      } else {
        launch_tiles<2, CRG_PREC_MIXED>(P, block, st);
        k_spheres_fix<2><<<32, 128, 0, st>>>(P);
      }
    }
    return;
  }
  const unsigned grid = (P.n_agents + block - 1) / block;
  if (dim == 3) {
    if (precision == CRG_PREC_F64) {
      k_spheres_step<3, CRG_PREC_F64><<<grid, block, 0, st>>>(P);
    } else {
      k_spheres_step<3, CRG_PREC_MIXED><<<grid, block, mixed_step_smem(block), st>>>(P);
      k_spheres_fix<3><<<32, 128, 0, st>>>(P);  // returns at once when nothing was handed over
    }
  } else {
    if (precision == CRG_PREC_F64) {
      k_spheres_step<2, CRG_PREC_F64><<<grid, block, 0, st>>>(P);
    } else {
      k_spheres_step<2, CRG_PREC_MIXED><<<grid, block, mixed_step_smem(block), st>>>(P);
      k_spheres_fix<2><<<32, 128, 0, st>>>(P);
    }
  }
}

int prepare_spheres(int dim, int precision) {
  cudaError_t e;
  if (dim == 3)
    e = precision == CRG_PREC_F64 ? prepare_tiles<3, CRG_PREC_F64>() : prepare_tiles<3, CRG_PREC_MIXED>();
  else
    e = precision == CRG_PREC_F64 ? prepare_tiles<2, CRG_PREC_F64>() : prepare_tiles<2, CRG_PREC_MIXED>();
  return e == cudaSuccess ? 0 : 1;
}

void launch_sphere_stats(int dim, const PackArgs &P, uint32_t *n_cand, uint32_t *n_inter,
                         uint64_t *hash, cudaStream_t st) {
  if (!P.n_agents) return;
  const unsigned grid = (P.n_agents + 127) / 128;
  if (dim == 3)
    k_sphere_stats<3><<<grid, 128, 0, st>>>(P, n_cand, n_inter, hash);
  else
    k_sphere_stats<2><<<grid, 128, 0, st>>>(P, n_cand, n_inter, hash);
}

}  // namespace crg
