// crg_internal.cuh -- device-side descriptors and helpers shared by the crg kernels.
//
// Layout in HBM (one "pack" = one or more independent simulations of the same agent kind,
// dimension and precision, concatenated):
//   * agents are kept physically sorted by global voxel index (the cell list); every
//     per-agent array is component-major SoA: x[c * cap + i] for component c of agent i,
//     where a component is (vertex, axis) for rods and the axis for spheres;
//   * voxels of simulation s occupy the global index range [voxel_off, voxel_off + n_vox);
//     the agents of s occupy [agent_off, agent_off + n_agents) because the sort is global;
//   * start[v] .. start[v+1] is the agent range of global voxel v after each re-sort.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/crg.h"

namespace crg {

constexpr int kMaxVertices = 8;

// Per-simulation descriptor (device copy).  Geometry follows CartesianCuboid
// (cellular_raza-building-blocks/src/domains/cartesian_cuboid_n.rs:65-72).
struct SimDev {
  int32_t dim;
  int32_t nvox[3];
  double min[3], max[3], dx[3];
  long long min_key[3], max_key[3];  // f64_order_key of min and max (boundary compares)
  uint32_t cen_off[3];  // first entry of each axis's voxel centres in the pack's table
  float dxf[3];
  float inv_dxf[3];  // (float)(1 / dx): the FP32 voxel-index estimate (voxel_of)
  uint32_t voxel_off, n_vox;
  uint32_t agent_off, n_agents;
  // Subdomain chunking of get_decomp_res/create_subdomains (cartesian_cuboid_n.rs:19-59,
  // 493-584): voxel i belongs to i/avg if i < switcher, else (i-switcher)/div2 + n.
  uint32_t sd_switch, sd_avg, sd_div2, sd_n;
  int32_t weight_mode;  // CRG_WEIGHTS_CHILI or CRG_WEIGHTS_PHYSICAL
  // Mechanics / interaction parameters.
  double mass, damping;
  double spring_tension, rigidity, spring_length;
  double radius, stiffness, cutoff, strength;
  // Morse terms that do not depend on the pair, each rounded exactly as the per-pair
  // expression rounds them: radius + radius, (-2 * strength) * stiffness, -stiffness.
  double mrs_r, mrs_k, mrs_nstiff;
  float mrs_r_f, mrs_k_f, mrs_nstiff_f;  // the same terms in FP32 (mixed-precision rods)
  // Mechanics of point agents: 0 NewtonDamped, 1 Brownian, 2 Langevin; stochastic terms.
  int32_t mech;
  int32_t stochastic;  // Brownian, Langevin, or RodMechanics with diffusion != 0
  double diffusion, kb_temperature;
  uint64_t rng_seed;
  // cutoff as an integer threshold on the bit pattern of a distance d >= 0 (not NaN):
  // d > cutoff exactly when bits(d) > cutoff_bits.
  int64_t cutoff_bits;
  double dt;
  float radius_f, stiffness_f, cutoff_f, strength_f;
  float filt_thr2;  // squared FP32 prefilter threshold (cutoff + conservative margin)^2
  float off_lim;    // |FP32 offset| bound the prefilter margin was derived for
  // mixed precision: FP32 distances closer than mix_band_f to the cutoff, or than
  // mix_zero_f to 0, are decided from the FP64 distance (each a few times the FP32
  // distance's error bound, far below the prefilter margin)
  float mix_band_f, mix_zero_f;
  int32_t order;    // 1 Euler, 2 AB2, 3 AB3
  int32_t sim_index;
  int64_t stop_step;  // the simulation is frozen once the pack's step counter reaches this
  int64_t step_base;  // steps the simulation ran before this pack's counter started (repack):
                      // its own step = pack step + step_base (indexes the random stream)
  // cell cycle (rods): base growth rate, division length, sensing range and saturation
  int32_t cycle;
  double cyc_growth, cyc_div_len, cyc_sense, cyc_sat;
  // bits of the largest squared distance x with RN(sqrt(x)) < cyc_sense (RN o sqrt is
  // monotone, so the sensing test is one integer compare of the bits of x >= 0), -1 if none
  long long cyc_sense_x2;
  // FP32 squared-distance bounds from the offsets: below sense_in2 a vertex pair is surely
  // closer than cyc_sense, above sense_out2 surely not; in between the FP64 test decides
  float sense_in2, sense_out2;
  float sense_gap_f;  // bounding boxes of two rods' FP32 offsets further apart than this
                      // along an axis hold no vertex pair closer than cyc_sense
};

// Arguments shared by the per-step kernels of a pack.
struct PackArgs {
  const SimDev *sims;
  const uint32_t *sim_agent_off;  // [n_sims + 1] prefix of agent counts
  int32_t n_sims;
  int64_t cap;      // component stride
  uint32_t n_agents;
  uint32_t n_vox;   // total voxels of the pack
  // current (sorted) state
  const double *pos;
  const double *vel;
  const uint64_t *id;
  const uint32_t *key;
  const float *off;  // FP32 offsets from the voxel centre (prefilter / mixed precision):
                     // spheres one float4 (3D) or float2 (2D) per agent (sphere_off), rods
                     // component-major [nc][cap]
  const double *hist;     // AB history [2 slots][2 (dx,dv)][nc][cap] or null
  const uint8_t *hmeta;   // ring buffer (first | size << 4) or null
  const uint32_t *start;  // [n_vox + 1]
  // next (updated, unsorted) state
  double *npos;
  double *nvel;
  uint64_t *nid;    // ids in the pre-step order (copied by the force kernel)
  uint32_t *nkey;
  double *nhist;
  uint8_t *nhmeta;
  uint32_t *count;  // histogram of nkey (atomic)
  // status word: [0] code, [1] agent id lo, [2] agent id hi, [3] step
  int32_t *status;
  const int64_t *step_ctr;
  double *dbg_force;  // optional [nc][cap]: interaction force of this step
  // rods: pass list of the default force path (one pass = own_a(b) or ext_a(b))
  uint32_t *npass, *pass_off;  // [cap] number of passes of each rod, index of its first
  uint32_t *pass_a, *pass_b;   // [pass_cap] rod and candidate of each pass
  uint8_t *pass_meta;          // [pass_cap] bit 0: ext pass; bits 1-6: voxel of b - voxel of
                               // a + 1 per axis, 2 bits each; bit 7: a step-3 pass, summed
                               // per neighbour box before it is added
  double *mbuf;                // [nc][pass_cap] M / 2 of each pass, rows in vertex order
  int64_t pass_cap;
  uint32_t *rctl;  // [0] passes reserved, [1] pass queue, [3] pass list overflow (all
                   // zeroed before each step)
  double *frc;     // rods: [nc][cap] interaction force of the rod-level fallback kernel
  double *bend;    // rods: [nv - 2][dim][cap] curvature forces (k_rods_bend)
  float2 *hl;      // mixed-precision rods: [nc][cap] each coordinate x as FP32 hi = (float)x
                   // and lo = (float)(x - hi), written by k_rods_walk (null on FP64)
  double *seg;     // FP64 rods: [nv - 1][dim + 2][cap] per segment l1 - l0 (dim), its squared
                   // norm n and RN(1 / n), written by k_rods_walk (null on mixed)
  uint32_t *fix_list;  // mixed spheres: agents whose force the FP64 fix-up kernel computes
                       // (count in rctl[0])
  int32_t prefilter;  // 0 disables the FP32 candidate prefilter (testing)
  int32_t variant;    // force kernel: 0 default, 1 thread per agent (CRG_OPT_KERNEL_VARIANT)
  int32_t tile;       // spheres, thread per agent: 0 one thread per agent in a grid over all
                      // agents; k > 0 the persistent tile kernel, blockDim * k agents a tile
  // cell cycle (rods; all null when off)
  const double *slen;       // [cap] spring length of each rod (current order)
  const double *grate;      // [cap] growth rate of each rod (current order)
  const uint64_t *parent;   // [cap] identifier the rod divided from (CRG_NO_PARENT if none)
  double *nslen, *ngrate;   // [cap] next spring length and growth rate (pre-step order;
                            // daughters of this step at n_agents + their rank)
  uint64_t *nparent;        // [cap]
  uint32_t *nsense;         // [cap] neighbour count of this step (k_rods_sense)
  uint32_t *dflag;          // [cap + 1] 1 where the rod divides this step (update kernel);
                            // the exclusive scan of it (dpre) numbers the daughters
  const uint32_t *dpre;     // [cap + 1]
  uint64_t *vctr;           // [n_vox] Voxel::id_counter
  uint32_t *srank;          // [cap] position in chili's pre-sort order, daughters included
};

// Records e on st: as an external event node while st is being captured into a graph (so the
// graph records it each time it runs), as a plain record otherwise (the external flag is for
// capture only).
inline void record_event(cudaEvent_t e, cudaStream_t st) {
  if (!e) return;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusActive)
    cudaEventRecordWithFlags(e, st, cudaEventRecordExternal);
  else
    cudaEventRecord(e, st);
}

// ---- IEEE FP64 helpers that are never contracted into fused multiply-adds ----------
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// a / b rounded to nearest -- the bits of ddiv(a, b) -- from y = RN(1 / b), b's correctly
// rounded reciprocal, with one multiply and four FMAs (no division) when a and b are finite,
// non-zero and of binary exponent in [-400, 400]; otherwise ddiv itself.  q = RN(a y) lies
// within 2 ulp of a / b.  One residual step, q + (a - b q) y with the residual from an FMA,
// leaves q within 2^-51 ulp of a / b before rounding: faithful.  For a faithful q and
// y = RN(1 / b) the residual a - b q is exact in an FMA and RN(q + (a - b q) y) = RN(a / b)
// (Markstein's theorem: P. W. Markstein, "Computation of elementary functions on the IBM
// RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990; J.-M. Muller et al., Handbook
// of Floating-Point Arithmetic, division with a fused multiply-add).  The exponent range
// keeps every intermediate (q within 2^+-801, the residual's granularity above 2^-505) in
// the normal range, where the theorem holds.
__device__ __forceinline__ double div_rn_recip(double a, double b, double y) {
  const unsigned long long ea = ((unsigned long long)__double_as_longlong(a) >> 52) & 0x7ffull;
  const unsigned long long eb = ((unsigned long long)__double_as_longlong(b) >> 52) & 0x7ffull;
  if (ea - 623ull > 800ull || eb - 623ull > 800ull) return ddiv(a, b);  // biased 623..1423
  double q = __dmul_rn(a, y);
  double r = __fma_rn(-b, q, a);
  q = __fma_rn(r, y, q);
  r = __fma_rn(-b, q, a);
  return __fma_rn(r, y, q);
}

// 0.0 + x, exactly: x itself except that -0.0 becomes +0.0 (integer instructions only).
__device__ __forceinline__ double plus_zero(double x) {
  return __double_as_longlong(x) == (long long)0x8000000000000000ull ? 0.0 : x;
}

// Comparisons of an FP64 value with a finite bound on the integer pipe, leaving the FP64
// pipe to arithmetic.  f64_order_key maps every non-NaN double to an int64 in the same
// order (both zeros to 0); a NaN compares false, as in IEEE.
__host__ __device__ __forceinline__ long long f64_order_key_bits(long long b) {
  return b >= 0 ? b : -(b & 0x7fffffffffffffffll);
}
__device__ __forceinline__ bool f64_is_nan(long long b) {
  return (unsigned long long)(b & 0x7fffffffffffffffll) > 0x7ff0000000000000ull;
}
__device__ __forceinline__ bool f64_lt_key(double x, long long bound_key) {  // x < bound
  const long long b = __double_as_longlong(x);
  return !f64_is_nan(b) && f64_order_key_bits(b) < bound_key;
}
__device__ __forceinline__ bool f64_gt_key(double x, long long bound_key) {  // x > bound
  const long long b = __double_as_longlong(x);
  return !f64_is_nan(b) && f64_order_key_bits(b) > bound_key;
}

// ---- random stream of the stochastic mechanics --------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3",
// SC'11): ten rounds of two 32x32->64 multiplies with the round keys bumped by the Weyl
// constants.
__device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t lo0 = 0xD2511F53u * c[0], hi0 = __umulhi(0xD2511F53u, c[0]);
    const uint32_t lo1 = 0xCD9E8D57u * c[2], hi1 = __umulhi(0xCD9E8D57u, c[2]);
    const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

// The standard normals z[0..N) of agent `id` at pack step `step`: block j (counter
// {j, step, id_lo, id_hi}) gives u1 in (0, 1] and u2 in [0, 1) with 53 bits each, then
// Box-Muller sqrt(-2 ln u1) (cos, sin)(2 pi u2).  The CPU oracle draws the same stream.
template <int N>
__device__ __forceinline__ void stream_normals(uint64_t seed, uint64_t step, uint64_t id,
                                               double *z) {
  const double two_pi = 6.283185307179586;
  const double inv53 = 1.0 / 9007199254740992.0;  // 2^-53
#pragma unroll
  for (int j = 0; 2 * j < N; ++j) {
    uint32_t w[4] = {(uint32_t)j, (uint32_t)step, (uint32_t)id, (uint32_t)(id >> 32)};
    philox4x32_10(w, (uint32_t)seed, (uint32_t)(seed >> 32));
    const double u1 = (double)((((uint64_t)w[0] << 21) | (w[1] >> 11)) + 1) * inv53;
    const double u2 = (double)(((uint64_t)w[2] << 21) | (w[3] >> 11)) * inv53;
    const double r = __dsqrt_rn(__dmul_rn(-2.0, log(u1)));
    const double th = __dmul_rn(two_pi, u2);
    z[2 * j] = __dmul_rn(r, cos(th));
    if (2 * j + 1 < N) z[2 * j + 1] = __dmul_rn(r, sin(th));
  }
}

// Out of line, for callers whose register budget the unrolled stream would set (rods).
template <int N>
__device__ __noinline__ void stream_normals_ool(uint64_t seed, uint64_t step, uint64_t id,
                                                double *z) {
  stream_normals<N>(seed, step, id, z);
}

// num::ToPrimitive::to_usize for f64: truncation toward zero on the open interval
// (-1, 2^64); everything else (NaN included) has no value.
__device__ __forceinline__ bool to_usize(double x, uint64_t &out) {
  if (x > -1.0 && x < 18446744073709551616.0) {
    out = (x < 1.0) ? 0ull : (uint64_t)x;
    return true;
  }
  return false;
}

__device__ __forceinline__ uint32_t subdomain_of(const SimDev &S, uint32_t v) {
  return v < S.sd_switch ? v / S.sd_avg : (v - S.sd_switch) / S.sd_div2 + S.sd_n;
}

// The voxels of one subdomain are a contiguous range of plain indices (the chunks above):
// the subdomain holding voxel v, as the range [lo, hi) that another voxel w shares with it
// exactly when subdomain_of(w) == subdomain_of(v).  One division per agent instead of one per
// neighbour box.
struct SubRange {
  uint32_t lo, hi;
  __device__ __forceinline__ bool same(uint32_t w) const { return w - lo < hi - lo; }
};
__device__ __forceinline__ SubRange subdomain_range(const SimDev &S, uint32_t v) {
  SubRange r;
  if (v < S.sd_switch) {
    r.lo = (v / S.sd_avg) * S.sd_avg;
    r.hi = r.lo + S.sd_avg;
  } else {
    r.lo = S.sd_switch + ((v - S.sd_switch) / S.sd_div2) * S.sd_div2;
    r.hi = r.lo + S.sd_div2;
  }
  return r;
}

// CartesianSubDomain::get_index_of (cartesian_cuboid_n.rs:469-490) + plain-index lookup.
// Returns 0 ok, 1 conversion failure, 2 index outside the voxel grid.
//
// The index is trunc((p - min) / dx) of the FP64 quotient.  An FP32 estimate q of the
// quotient (one rounding of p - min to FP32, one of 1/dx, one of the product: relative error
// below 3 * 2^-24) decides it when q lies farther than twice that error from every integer:
// the FP64 quotient then truncates to the same integer.  Only quotients that close to a
// voxel face, or outside [0, 2^23), take the FP64 division.
template <int D>
__device__ __forceinline__ int voxel_of(const SimDev &S, const double *p, uint32_t &plain) {
  uint64_t idx[D];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    // p - (+-0.0) is p itself except for p = -0.0 with min = -0.0, whose index is 0 either way
    const double d = S.min_key[i] == 0 ? p[i] : dsub(p[i], S.min[i]);
    const float q = __fmul_rn(__double2float_rn(d), S.inv_dxf[i]);
    const float fl = floorf(q), fr = q - fl;  // exact for 0 <= q < 2^23
    const float eps = __fmaf_rn(q, 4.0e-7f, 1.0e-6f);
    if (q >= 0.0f && q < 8388608.0f && fr > eps && fr < 1.0f - eps) {
      idx[i] = (uint64_t)fl;
    } else {
      const double n_vox = ddiv(d, S.dx[i]);
      if (!to_usize(n_vox, idx[i])) return 1;
    }
  }
#pragma unroll
  for (int i = 0; i < D; ++i)
    if (idx[i] >= (uint64_t)S.nvox[i]) return 2;
  uint64_t q = 0;
#pragma unroll
  for (int i = 0; i < D; ++i) q = q * (uint64_t)S.nvox[i] + idx[i];
  plain = (uint32_t)q;
  return 0;
}

template <int D>
__device__ __forceinline__ void unravel(const SimDev &S, uint32_t v, int *idx) {
#pragma unroll
  for (int i = D - 1; i >= 0; --i) {
    idx[i] = (int)(v % (uint32_t)S.nvox[i]);
    v /= (uint32_t)S.nvox[i];
  }
}

// Centre of voxel idx in FP64: min + (idx + 1/2) dx (one rounding, as an FMA; the sort reads
// the same values from the pack's table, built on the host with std::fma).  The FP32 offsets are taken from it
// (|offset| <= dx / 2 inside the voxel, so their rounding is half that of corner offsets);
// only differences of offsets and of centres, (j - idx) dx, enter the kernels.
__device__ __forceinline__ double voxel_centre(const SimDev &S, int axis, int idx) {
  return S.min[axis] + ((double)idx + 0.5) * S.dx[axis];
}

__device__ __forceinline__ uint32_t sim_of_agent(const PackArgs &P, uint32_t i) {
  int lo = 0, hi = P.n_sims;  // invariant: off[lo] <= i < off[hi]
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (__ldg(&P.sim_agent_off[mid]) <= i)
      lo = mid;
    else
      hi = mid;
  }
  return (uint32_t)lo;
}

// status word: [0] code, [1] agent id lo, [2] agent id hi, [3] step (or check site),
// [4] simulation index within the pack, [5] largest pass list a rod step asked for since
// the status was last cleared (read by the host to size the pass list), [6] the failed
// simulation as of the end of the previous step (0 none, s + 1 simulation s, -1 all), which
// the force and update kernels read instead of [0] because [0] can change during them
__device__ __forceinline__ void set_status(int32_t *status, int32_t code, uint64_t agent,
                                           int64_t step, int32_t sim = 0) {
  if (atomicCAS(&status[0], 0, code) == 0) {
    status[1] = (int32_t)(agent & 0xffffffffu);
    status[2] = (int32_t)(agent >> 32);
    status[3] = (int32_t)step;
    status[4] = sim;
  }
}

// A simulation is frozen (carried through a step unchanged) once its requested number of
// steps is done or once one of its earlier steps failed: chili stops a simulation at its
// first error (chili/errors.rs:73-122), so no later step may change its state.
__device__ __forceinline__ bool sim_frozen(const PackArgs &P, const SimDev &S) {
  const int32_t failed = P.status[6];
  return *P.step_ctr >= S.stop_step || failed == -1 || failed == S.sim_index + 1;
}

// The simulation whose step failed in the force or update kernels (a code other than
// CRG_EINTERNAL in status[0], its index in status[4]), or -1.  Read by the sort kernels that
// follow those kernels: the failing step is not committed for that simulation, so the
// handle keeps the state after the last step that succeeded.  Only invariant checks of the
// sort kernels themselves write the status during a sort, and they write CRG_EINTERNAL
// into a clear word only, so every sort kernel of a step reads the same answer.
__device__ __forceinline__ int32_t failed_sim(const int32_t *status) {
  const int32_t code = status[0];
  return (code != 0 && code != CRG_EINTERNAL) ? status[4] : -1;
}

// A frozen simulation (its requested number of steps is done) is carried through the step
// unchanged: same state, same voxel, same cell-list position.
__device__ __forceinline__ void frozen_copy(const PackArgs &P, uint32_t i, uint32_t key, int nc) {
  const int64_t cap = P.cap;
  for (int c = 0; c < nc; ++c) {
    P.npos[c * cap + i] = P.pos[c * cap + i];
    P.nvel[c * cap + i] = P.vel[c * cap + i];
  }
  if (P.hist) {
    for (int c = 0; c < 2 * nc; ++c) P.nhist[c * cap + i] = P.hist[c * cap + i];
    P.nhmeta[i] = P.hmeta[i];
  }
  if (P.dflag) {  // cell cycle: a frozen rod keeps its state and does not divide
    P.nslen[i] = P.slen[i];
    P.ngrate[i] = P.grate[i];
    P.nparent[i] = P.parent[i];
    P.dflag[i] = 0u;
  }
  P.nkey[i] = key;
  P.nid[i] = P.id[i];
  atomicAdd(&P.count[key], 1u);
}

// Invariant checks of the cell list.  A violation records CRG_EINTERNAL with the index and
// the check site (in the step slot of the status word); the caller skips the access.
enum CheckSite : int32_t {
  kSiteForceKey = 1,    // key of an agent outside the pack's voxels
  kSiteForceRange = 2,  // voxel agent range outside [0, n_agents]
  kSiteNextKey = 3,     // next key outside the pack's voxels
  kSiteScatterKey = 4,
  kSiteScatterSlot = 5,
  kSiteSegRange = 6,
  kSiteGatherSrc = 7,
  kSiteGatherKey = 8,
};

__device__ __forceinline__ void invariant_failed(int32_t *status, int32_t site, uint64_t index) {
  if (atomicCAS(&status[0], 0, CRG_EINTERNAL) == 0) {
    status[1] = (int32_t)(index & 0xffffffffu);
    status[2] = (int32_t)(index >> 32);
    status[3] = site;
  }
}

// x * 0.5 with the IEEE result of the FP64 multiply (round to nearest even), computed on
// the bit pattern with integer instructions.
__device__ __forceinline__ double half_exact(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned long long sign = u & 0x8000000000000000ull, mag = u ^ sign;
  const unsigned long long e = mag >> 52;
  // lowest binade and subnormals: the value is mag * 2^-1074, so halving is a shift of mag
  // rounded to nearest, ties to even (the result is subnormal or zero)
  unsigned long long q = mag >> 1;
  q += (mag & q & 1ull);
  unsigned long long h = sign | q;
  if (e >= 2) h = u - (1ull << 52);  // normal result: exponent - 1, exact
  if (e == 0x7ffull) h = u;          // infinities and NaN are their own half
  return __longlong_as_double((long long)h);
}

// dist > cutoff || dist == 0.0 for a distance taken as the square root of a sum of squares
// (+0, positive, +inf or NaN; NaN carries on as in the reference), compared on the bit
// patterns with integer instructions.  cutoff_bits: the cutoff's bits, INT64_MAX for a NaN
// cutoff (never exceeded), -1 for a cutoff <= 0 (always exceeded).
__device__ __forceinline__ bool beyond_cutoff(double dist, long long cutoff_bits) {
  const long long db = __double_as_longlong(dist);
  const unsigned long long mag = (unsigned long long)db & 0x7fffffffffffffffull;
  return mag <= 0x7ff0000000000000ull && (mag == 0ull || db > cutoff_bits);
}

// calculate_morse_interaction (cellular_raza-building-blocks/src/cell_building_blocks/
// interaction.rs:151-182) in FP64, returning the own-perspective force already scaled by
// one half (chili adds f.xa(1/2), update_mechanics.rs:98,194-199).  Each operation is
// separately rounded in the reference's order; the pair-independent terms (radius + radius,
// -stiffness, -2 strength stiffness) come precomputed per simulation with the same
// roundings, and the halving is done on the bit pattern (half_exact).  Returns false for a
// zero force (dist > cutoff or dist == 0).
template <int D>
__device__ __forceinline__ bool morse_half_f64(const double *z, const SimDev &S, double *h) {
  double n2 = dmul(z[0], z[0]);
#pragma unroll
  for (int c = 1; c < D; ++c) n2 = dadd(n2, dmul(z[c], z[c]));
  const double dist = __dsqrt_rn(n2);
  if (beyond_cutoff(dist, S.cutoff_bits)) return false;
  const double e = exp(dmul(S.mrs_nstiff, dsub(dist, S.mrs_r)));
  const double force = dmul(dmul(S.mrs_k, e), dsub(1.0, e));
  const double y = __drcp_rn(dist);  // z[c] / dist for every c from one reciprocal
#pragma unroll
  for (int c = 0; c < D; ++c) h[c] = half_exact(dmul(div_rn_recip(z[c], dist, y), force));
  return true;
}

}  // namespace crg
