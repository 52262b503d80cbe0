// crg_api.cu -- the C ABI (include/crg.h): handles, upload/step/download, graphs.
//
// A handle owns one "pack": one or more simulations of the same agent kind, dimension,
// precision and solver order, stored back to back in component-major SoA buffers and
// advanced by the same kernel launches.  One step is
//   force+update kernel  (crg_spheres.cu / crg_rods.cu: forces, solver, boundary, next key,
//                         histogram of next keys)
//   sort                 (crg_sort.cu: scan, scatter, per-voxel order, gather)
// and runs on the handle's stream; steps are captured into CUDA graphs in chunks.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <limits>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "crg_host.h"
#include "crg_internal.cuh"
#include "crg_kernels.h"

using crg::PackArgs;
using crg::SimDev;
using crg::SortArgs;

struct crg_ctx {
  int dim = 3, kind = CRG_KIND_SPHERE, nv = 1, nc = 3, precision = CRG_PREC_F64, order = 1;
  int n_sims = 1;
  std::vector<SimDev> sims_h;
  std::vector<int64_t> caps;
  std::vector<uint32_t> agent_off_h;  // [n_sims + 1]
  int64_t cap = 0;
  uint32_t n_agents = 0;
  uint32_t n_vox = 0;
  // device memory
  SimDev *d_sims = nullptr;
  uint32_t *d_agent_off = nullptr, *d_sim_of_voxel = nullptr;
  double *pos = nullptr, *vel = nullptr, *npos = nullptr, *nvel = nullptr;
  uint64_t *id = nullptr, *nid = nullptr;
  uint32_t *key = nullptr, *nkey = nullptr;
  float *off = nullptr;
  double *hist = nullptr, *nhist = nullptr;
  uint8_t *hmeta = nullptr, *nhmeta = nullptr;
  uint32_t *count = nullptr, *start = nullptr, *bsum = nullptr;
  uint64_t *tmp = nullptr;
  int32_t *status = nullptr;
  int64_t *step_ctr = nullptr;
  double *dbg_force = nullptr;
  // rods: pass list of the default force path and the fallback's force buffer
  uint32_t *npass = nullptr, *pass_off = nullptr, *pass_a = nullptr, *pass_b = nullptr;
  uint8_t *pass_meta = nullptr;
  double *mbuf = nullptr;
  int64_t pass_cap = 0;
  uint32_t *rctl = nullptr;
  double *seg = nullptr;  // FP64 rods: per-segment l1 - l0, squared norm, reciprocal
  uint32_t *fix_list = nullptr;  // mixed spheres: agents for the FP64 fix-up kernel
  double *bend = nullptr;        // rods: curvature forces between the bend and update kernels
  // cell cycle (rods, single simulation): per-agent state (current / next), neighbour
  // counts, division flags and their scan, voxel id counters, pre-sort ranks
  int cycle = 0;
  double *slen = nullptr, *nslen = nullptr, *grate = nullptr, *ngrate = nullptr;
  uint64_t *parent = nullptr, *nparent = nullptr, *vctr = nullptr;
  uint32_t *nsense = nullptr, *dflag = nullptr, *dpre = nullptr, *dbsum = nullptr;
  uint32_t *srank = nullptr;
  uint32_t *h_ndiv = nullptr;  // pinned
  double *frc = nullptr;
  float2 *hl = nullptr;  // mixed-precision rods: hi / lo split of the positions
  double *vcen = nullptr;  // voxel centres of every simulation and axis (SimDev::cen_off)
  double *fbuf = nullptr;  // crg_forces: the interaction force of every slot
  double *staging = nullptr;
  char *snap = nullptr;  // crg_snapshot buffer
  uint32_t snap_agents = 0;
  int64_t snap_steps = 0;
  int32_t *h_status = nullptr;  // pinned
  cudaStream_t stream = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int gexec_steps = 0;
  int graph_chunk = 32;
  int prefilter = 1;
  int variant = 0;
  int tile = 0;  // CRG_OPT_TILE
  // set while the library itself loads a checkpoint of this handle taken at another
  // capacity (growth of a cell-cycle handle, the autotuner's trials after a growth)
  bool ckpt_any_capacity = false;
  int block = 0;
  int profile = 0;
  double prof_ms[5] = {0, 0, 0, 0, 0};
  std::vector<cudaEvent_t> pev;  // CRG_OPT_PROFILE: kProfEvents per step of a chunk
  int32_t err_code = CRG_OK;
  int64_t err_agent = -1, err_step = -1;
  int64_t steps_done = 0;
  int32_t err_sim = -1;
  std::vector<crg_domain> doms;  // as given at creation (for crg_repack)
  std::vector<crg_model> mods;
};

namespace {

#define CUDA_TRY(expr)                                  \
  do {                                                  \
    cudaError_t e_ = (expr);                            \
    if (e_ != cudaSuccess) {                            \
      return e_ == cudaErrorMemoryAllocation ? CRG_ENOMEM : CRG_ECUDA; \
    }                                                   \
  } while (0)

bool to_usize_h(double x, uint64_t &out) {
  if (x > -1.0 && x < 18446744073709551616.0) {
    out = (uint64_t)x;
    return true;
  }
  return false;
}

// get_decomp_res (cellular_raza-building-blocks/src/domains/cartesian_cuboid_n.rs:19-59).
bool decomp_res(uint64_t n_voxel, uint64_t n_regions, uint64_t &n_out, uint64_t &m_out,
                uint64_t &avg_out) {
  int64_t average_len = (int64_t)std::ceil((double)n_voxel / (double)n_regions);
  int64_t n = (int64_t)n_regions, m = 0;
  for (uint64_t it = 0; it < n_regions; ++it) {
    int64_t r = (int64_t)n_voxel - average_len * n - (average_len - 1) * m;
    if (r == 0) {
      n_out = (uint64_t)n;
      m_out = (uint64_t)m;
      avg_out = (uint64_t)average_len;
      return true;
    } else if (r > 0) {
      if (n == (int64_t)n_regions) {
        average_len += 1;
        n = (int64_t)n_regions;
        m = 0;
      }
    } else {
      n -= 1;
      m += 1;
    }
  }
  return false;
}

// Fills the geometry and parameters of one simulation descriptor.
// Bits of the largest x >= 0 with sqrt(x) < r in round-to-nearest (-1 when there is none):
// sqrt is correctly rounded on host and device alike and monotone, so sqrt(x) < r holds
// exactly for the x at or below this one.
long long sense_threshold_bits(double r) {
  if (!(r > 0.0)) return -1;  // sqrt(x) >= 0 is never below r <= 0 (or NaN)
  if (std::isinf(r)) {
    const double big = std::numeric_limits<double>::max();
    long long b;
    std::memcpy(&b, &big, sizeof(b));
    return b;
  }
  double x = r * r;
  while (x > 0.0 && !(std::sqrt(x) < r)) x = std::nextafter(x, 0.0);
  while (std::isfinite(std::nextafter(x, INFINITY)) &&
         std::sqrt(std::nextafter(x, INFINITY)) < r)
    x = std::nextafter(x, INFINITY);
  if (!(std::sqrt(x) < r)) return -1;
  long long b;
  std::memcpy(&b, &x, sizeof(b));
  return b;
}

int32_t fill_sim(const crg_domain &d, const crg_model &m, SimDev &S) {
  std::memset(&S, 0, sizeof(S));
  if (d.dim != 2 && d.dim != 3) return CRG_EINVAL;
  S.dim = d.dim;
  uint64_t total = 1;
  for (int i = 0; i < 3; ++i) S.nvox[i] = 1;
  for (int i = 0; i < d.dim; ++i) {
    if (!(d.min[i] < d.max[i])) return CRG_EBOUNDARY;  // check_min_max (:149-162)
    S.min[i] = d.min[i];
    S.max[i] = d.max[i];
    long long bmin, bmax;
    std::memcpy(&bmin, &d.min[i], sizeof(bmin));
    std::memcpy(&bmax, &d.max[i], sizeof(bmax));
    S.min_key[i] = crg::f64_order_key_bits(bmin);
    S.max_key[i] = crg::f64_order_key_bits(bmax);
    uint64_t nvox;
    if (d.voxel_mode == 0) {
      // from_boundaries_and_interaction_range (cartesian_cuboid_n.rs:183-222)
      if (!(d.interaction_range > 0.0)) return CRG_EINVAL;
      double n = std::floor((d.max[i] - d.min[i]) / d.interaction_range);
      uint64_t mm;
      if (!to_usize_h(n, mm)) return CRG_EBOUNDARY;
      nvox = std::max<uint64_t>(mm, 1);
      S.dx[i] = (d.max[i] - d.min[i]) / n;
    } else {
      // from_boundaries_and_n_voxels (cartesian_cuboid_n.rs:226-256)
      if (d.n_voxels[i] <= 0) return CRG_EINVAL;
      nvox = (uint64_t)d.n_voxels[i];
      S.dx[i] = (d.max[i] - d.min[i]) / (double)nvox;
    }
    if (nvox > (1u << 30)) return CRG_ENOTSUP;
    S.nvox[i] = (int32_t)nvox;
    total *= nvox;
    if (total > 0xffffffffull / 2) return CRG_ENOTSUP;
  }
  S.n_vox = (uint32_t)total;
  if (d.n_subdomains < 1) return CRG_EINVAL;
  uint64_t n, mm, avg;
  if ((uint64_t)d.n_subdomains > total || !decomp_res(total, (uint64_t)d.n_subdomains, n, mm, avg))
    return CRG_EDECOMPOSE;
  S.sd_switch = (uint32_t)(n * avg);
  S.sd_avg = (uint32_t)avg;
  S.sd_div2 = (uint32_t)std::max<uint64_t>(avg - 1, 1);
  S.sd_n = (uint32_t)n;
  S.weight_mode = d.weight_mode;
  S.mass = m.mass;
  S.damping = m.damping;
  S.spring_tension = m.spring_tension;
  S.rigidity = m.rigidity;
  S.spring_length = m.spring_length;
  S.radius = m.radius;
  S.stiffness = m.stiffness;
  S.cutoff = m.cutoff;
  S.strength = m.strength;
  S.mech = m.kind == CRG_KIND_BROWNIAN ? 1 : m.kind == CRG_KIND_LANGEVIN ? 2 : 0;
  S.diffusion = m.diffusion;
  S.kb_temperature = m.kb_temperature;
  S.rng_seed = m.rng_seed;
  S.stochastic = (m.kind == CRG_KIND_BROWNIAN || m.kind == CRG_KIND_LANGEVIN ||
                  (m.kind == CRG_KIND_ROD && m.diffusion != 0.0)) ? 1 : 0;
  S.cycle = m.cycle ? 1 : 0;
  S.cyc_growth = m.growth_rate;
  S.cyc_div_len = m.division_length;
  S.cyc_sense = m.sense_range;
  S.cyc_sense_x2 = sense_threshold_bits(m.sense_range);
  S.cyc_sat = m.sense_saturation;
  S.mrs_r = m.radius + m.radius;
  S.mrs_k = (-2.0 * m.strength) * m.stiffness;
  S.mrs_nstiff = -m.stiffness;
  S.mrs_r_f = (float)S.mrs_r;
  S.mrs_k_f = (float)S.mrs_k;
  S.mrs_nstiff_f = (float)S.mrs_nstiff;
  if (std::isnan(m.cutoff))
    S.cutoff_bits = INT64_MAX;  // d > NaN never holds
  else if (!(m.cutoff > 0.0))
    S.cutoff_bits = -1;  // every d > 0 exceeds a cutoff <= 0
  else
    std::memcpy(&S.cutoff_bits, &m.cutoff, sizeof(double));
  S.dt = m.dt;
  S.order = m.solver_order;
  S.stop_step = INT64_MAX;
  S.step_base = 0;
  S.radius_f = (float)m.radius;
  S.stiffness_f = (float)m.stiffness;
  S.cutoff_f = (float)m.cutoff;
  S.strength_f = (float)m.strength;
  double dxmax = 0.0;
  for (int i = 0; i < d.dim; ++i) {
    S.dxf[i] = (float)S.dx[i];
    S.inv_dxf[i] = (float)(1.0 / S.dx[i]);
    if (std::isfinite(S.dx[i])) dxmax = std::max(dxmax, S.dx[i]);
  }
  // FP32 offsets are trusted while |off| <= off_lim.  Every FP32 quantity entering the
  // prefilter distance is then within a few ulps of off_lim (offset roundings, the corner
  // shift, the differences), so its absolute error is bounded by 16 * off_lim * 2^-24 per
  // axis.  The margin below is more than 100 times that bound.
  // a growing rod reaches the division length before it divides
  const double longest = m.cycle ? std::max(std::fabs(m.spring_length), std::fabs(m.division_length))
                                 : std::fabs(m.spring_length);
  double ext = (m.kind == CRG_KIND_ROD) ? 4.0 * (m.n_vertices - 1) * longest : 0.0;
  double off_lim = 4.0 * dxmax + ext + 1.0;
  double err = 16.0 * off_lim * std::ldexp(1.0, -24) * std::sqrt((double)d.dim);
  double margin = 128.0 * err + 1e-4 * std::fabs(m.cutoff) + 1e-6;
  double thr = std::fabs(m.cutoff) + margin;
  S.off_lim = (float)off_lim;
  {
    // sensing (cell cycle): FP32 offset distances are within err per axis of the FP64
    // ones, so pairs farther than 4 err * sqrt(dim) from the range are decided in FP32
    const double r = m.sense_range, band = 4.0 * err;
    const double lo = (r > band) ? r - band : 0.0, hi = r + band;
    S.sense_in2 = (r > band) ? (float)(lo * lo) * (1.0f - 1e-6f) : -1.0f;
    S.sense_out2 = std::isfinite(hi) ? (float)(hi * hi) * (1.0f + 1e-6f) : __builtin_inff();
    if (!(r > 0.0)) S.sense_in2 = -1.0f;
    // per-axis gap of the bounding boxes, rounded up (NaN stays NaN: nothing is skipped)
    S.sense_gap_f = std::isfinite(hi) ? (float)hi + std::fabs((float)hi) * 1e-6f : (float)hi;
  }
  if (m.kind == CRG_KIND_ROD) {
    // mixed rods take their distances from hi / lo coordinates (relative error ~1e-6,
    // absolute ~2^-47 of the largest coordinate): 1e-5 of the cutoff, and 64 x 2^-47 of the
    // largest coordinate near zero
    double xmax = 0.0;
    for (int i = 0; i < d.dim; ++i)
      xmax = std::max(xmax, std::max(std::fabs(d.min[i]), std::fabs(d.max[i])));
    const double zero = 64.0 * std::ldexp(xmax + ext, -47) + 1e-30;
    S.mix_zero_f = (float)zero;
    S.mix_band_f = (float)(1e-5 * std::fabs(m.cutoff) + zero);
  } else {
    // mixed spheres take their displacements from the FP32 offsets, within err per axis
    S.mix_zero_f = (float)(4.0 * err);
    S.mix_band_f = (float)(4.0 * err + std::ldexp(std::fabs(m.cutoff), -20));
  }
  S.filt_thr2 = (float)(thr * thr);
  if (!std::isfinite(S.filt_thr2)) S.filt_thr2 = __builtin_inff();
  return CRG_OK;
}

int32_t check_model(const crg_model &m) {
  if (m.kind < CRG_KIND_SPHERE || m.kind > CRG_KIND_LANGEVIN) return CRG_EINVAL;
  if (m.kind != CRG_KIND_ROD && m.n_vertices != 1) return CRG_EINVAL;
  if (m.kind == CRG_KIND_ROD && (m.n_vertices < 2 || m.n_vertices > crg::kMaxVertices))
    return CRG_ENOTSUP;
  if (m.solver_order < 1 || m.solver_order > 3) return CRG_EINVAL;
  if (m.precision != CRG_PREC_F64 && m.precision != CRG_PREC_MIXED) return CRG_EINVAL;
  // mixed-precision rods: the cell cycle's sensing and division run on FP64 rods only
  if (m.kind == CRG_KIND_ROD && m.precision != CRG_PREC_F64 && m.cycle) return CRG_ENOTSUP;
  // NewtonDamped has no diffusion; Brownian divides by k_B T (mechanics.rs:354)
  if (m.kind == CRG_KIND_SPHERE && m.diffusion != 0.0) return CRG_EINVAL;
  if (m.kind == CRG_KIND_BROWNIAN && !(m.kb_temperature != 0.0)) return CRG_EINVAL;
  if (!(m.dt > 0.0)) return CRG_EINVAL;
  if (m.cycle) {
    if (m.kind != CRG_KIND_ROD) return CRG_ENOTSUP;
    if (!(m.sense_saturation != 0.0)) return CRG_EINVAL;  // the growth law divides by it
  }
  return CRG_OK;
}

template <class T>
int32_t dalloc(T **p, size_t n) {
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    return e == cudaErrorMemoryAllocation ? CRG_ENOMEM : CRG_ECUDA;
  }
  return CRG_OK;
}

void free_pass_list(crg_ctx *c) {
  void *ptrs[] = {c->pass_a, c->pass_b, c->pass_meta, c->mbuf};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  c->pass_a = c->pass_b = nullptr;
  c->pass_meta = nullptr;
  c->mbuf = nullptr;
  c->pass_cap = 0;
}

// (Re)allocates the rod pass list for n passes.  On failure the list stays empty and every
// step takes the rod-level fallback kernel.
int32_t alloc_pass_list(crg_ctx *c, int64_t n) {
  free_pass_list(c);
  if (n < 1024) n = 1024;
  if (dalloc(&c->pass_a, (size_t)n) != CRG_OK || dalloc(&c->pass_b, (size_t)n) != CRG_OK ||
      dalloc(&c->pass_meta, (size_t)n) != CRG_OK || dalloc(&c->mbuf, (size_t)n * c->nc) != CRG_OK) {
    free_pass_list(c);
    return CRG_ENOMEM;
  }
  // poison: an entry a step forgot to write reads as NaN instead of a stale force
  if (cudaMemset(c->mbuf, 0xff, sizeof(double) * (size_t)n * c->nc) != cudaSuccess) {
    free_pass_list(c);
    return CRG_ECUDA;
  }
  c->pass_cap = n;
  return CRG_OK;
}

void free_events(crg_ctx *c) {
  for (cudaEvent_t e : c->pev)
    if (e) cudaEventDestroy(e);
  c->pev.clear();
}

void free_all(crg_ctx *c) {
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  free_events(c);
  void *ptrs[] = {c->d_sims, c->d_agent_off, c->d_sim_of_voxel, c->pos, c->vel, c->npos,
                  c->nvel, c->id, c->nid, c->key, c->nkey, c->off, c->hist, c->nhist,
                  c->hmeta, c->nhmeta, c->count, c->start, c->bsum, c->tmp, c->status,
                  c->step_ctr, c->dbg_force, c->frc, c->hl, c->vcen, c->fbuf, c->bend, c->rctl, c->fix_list, c->npass, c->pass_off, c->seg,
                  c->staging, c->snap, c->slen, c->nslen, c->grate, c->ngrate, c->parent,
                  c->nparent, c->vctr, c->nsense, c->dflag, c->dpre, c->dbsum, c->srank};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  free_pass_list(c);
  if (c->h_status) cudaFreeHost(c->h_status);
  if (c->h_ndiv) cudaFreeHost(c->h_ndiv);
  if (c->stream) cudaStreamDestroy(c->stream);
}

// Floats per agent of the interleaved sphere offsets (one 16- or 8-byte load per agent);
// 0 for the component-major rod offsets.
int off_aos(const crg_ctx *c) { return c->kind == CRG_KIND_ROD ? 0 : (c->dim == 3 ? 4 : 2); }

int32_t allocate(crg_ctx *c) {
  const int64_t cap = c->cap;
  const int nc = c->nc;
  int32_t r;
#define A(ptr, n)                                              \
  do {                                                         \
    if ((r = dalloc(&c->ptr, (size_t)(n))) != CRG_OK) return r; \
  } while (0)
  A(d_sims, c->n_sims);
  A(d_agent_off, c->n_sims + 1);
  A(pos, cap * nc);
  A(vel, cap * nc);
  A(npos, cap * nc);
  A(nvel, cap * nc);
  A(id, cap);
  A(nid, cap);
  A(key, cap);
  A(nkey, cap);
  A(off, cap * (off_aos(c) ? off_aos(c) : nc));
  A(tmp, cap);
  A(count, (size_t)c->n_vox + 1);
  A(start, (size_t)c->n_vox + 1);
  A(bsum, (size_t)c->n_vox / 4096 + 2);
  A(status, 8);
  A(step_ctr, 1);
  A(staging, cap * nc);
  if (c->kind != CRG_KIND_ROD) A(rctl, 4);  // [0] mixed fix-up count, [2] tile counter
  if (c->kind == CRG_KIND_SPHERE && c->precision != CRG_PREC_F64) A(fix_list, cap);
  if (c->kind == CRG_KIND_ROD) {
    A(frc, cap * nc);
    A(bend, cap * (c->nv > 2 ? c->nv - 2 : 1) * c->dim);
    if (c->precision != CRG_PREC_F64) {
      A(hl, cap * nc);
    } else {
      A(seg, cap * (size_t)(c->nv - 1) * (c->dim + 2));
    }
    A(rctl, 4);
    A(npass, cap);
    A(pass_off, cap);
    alloc_pass_list(c, 12 * cap);  // grown after a step that needed more (read_status)
  }
  if (c->order > 1) {
    A(hist, cap * nc * 2);
    A(nhist, cap * nc * 2);
    A(hmeta, cap);
    A(nhmeta, cap);
  }
  if (c->n_sims > 1) A(d_sim_of_voxel, c->n_vox);
  if (c->cycle) {
    A(slen, cap);
    A(nslen, cap);
    A(grate, cap);
    A(ngrate, cap);
    A(parent, cap);
    A(nparent, cap);
    A(nsense, cap);
    A(dflag, cap + 1);
    A(dpre, cap + 1);
    A(dbsum, cap / 4096 + 2);
    A(srank, cap);
    A(vctr, c->n_vox);
  }
#undef A
  if (c->cycle) {
    CUDA_TRY(cudaMallocHost((void **)&c->h_ndiv, 2 * sizeof(uint32_t)));
  }
  CUDA_TRY(cudaMallocHost((void **)&c->h_status, 8 * sizeof(int32_t)));
  CUDA_TRY(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  CUDA_TRY(cudaMemsetAsync(c->count, 0, sizeof(uint32_t) * ((size_t)c->n_vox + 1), c->stream));
  CUDA_TRY(cudaMemsetAsync(c->status, 0, sizeof(int32_t) * 8, c->stream));
  CUDA_TRY(cudaMemsetAsync(c->step_ctr, 0, sizeof(int64_t), c->stream));
  if (c->n_sims > 1) {
    std::vector<uint32_t> sov(c->n_vox);
    for (int s = 0; s < c->n_sims; ++s)
      for (uint32_t v = 0; v < c->sims_h[s].n_vox; ++v) sov[c->sims_h[s].voxel_off + v] = s;
    CUDA_TRY(cudaMemcpy(c->d_sim_of_voxel, sov.data(), sizeof(uint32_t) * c->n_vox,
                        cudaMemcpyHostToDevice));
  }
  return CRG_OK;
}

int32_t create_impl(int32_t n_sims, const crg_domain *domains, const crg_model *models,
                    const int64_t *capacities, crg_ctx **out) {
  if (!out || n_sims < 1 || !domains || !models || !capacities) return CRG_EINVAL;
  *out = nullptr;
  crg_ctx *c = new (std::nothrow) crg_ctx();
  if (!c) return CRG_ENOMEM;
  const crg_model &m0 = models[0];
  c->dim = domains[0].dim;
  c->kind = m0.kind == CRG_KIND_ROD ? CRG_KIND_ROD : CRG_KIND_SPHERE;  // point agents
  c->nv = m0.kind == CRG_KIND_ROD ? m0.n_vertices : 1;
  c->nc = c->nv * c->dim;
  c->precision = m0.precision;
  c->order = m0.solver_order;
  c->cycle = m0.cycle ? 1 : 0;
  if (c->cycle && n_sims > 1) {  // the cell cycle runs on single-simulation handles
    delete c;
    return CRG_ENOTSUP;
  }
  c->n_sims = n_sims;
  c->sims_h.resize(n_sims);
  c->doms.assign(domains, domains + n_sims);
  c->mods.assign(models, models + n_sims);
  c->caps.assign(capacities, capacities + n_sims);
  uint64_t vox = 0;
  int64_t cap = 0;
  for (int s = 0; s < n_sims; ++s) {
    const crg_model &m = models[s];
    int32_t r = check_model(m);
    if (r == CRG_OK && (m.kind != m0.kind || m.n_vertices != m0.n_vertices ||
                        m.precision != m0.precision || m.solver_order != m0.solver_order ||
                        domains[s].dim != c->dim))
      r = CRG_EINVAL;
    if (r == CRG_OK && capacities[s] < 0) r = CRG_EINVAL;
    if (r == CRG_OK) r = fill_sim(domains[s], m, c->sims_h[s]);
    if (r != CRG_OK) {
      delete c;
      return r;
    }
    c->sims_h[s].voxel_off = (uint32_t)vox;
    c->sims_h[s].sim_index = s;
    vox += c->sims_h[s].n_vox;
    cap += capacities[s];
    if (vox > 0x7fffffffull || cap > 0x7fffffffll) {
      delete c;
      return CRG_ENOTSUP;
    }
  }
  c->n_vox = (uint32_t)vox;
  c->cap = std::max<int64_t>(cap, 1);
  c->agent_off_h.assign(n_sims + 1, 0);
  // voxel centres min + (idx + 1/2) dx, per simulation and axis, rounded once (fma) as the
  // device expression voxel_centre rounds them; the sort reads them for the FP32 offsets
  std::vector<double> cen;
  for (int s = 0; s < n_sims; ++s)
    for (int a = 0; a < 3; ++a) {
      const SimDev &S = c->sims_h[s];
      c->sims_h[s].cen_off[a] = (uint32_t)cen.size();
      if (a < c->dim)
        for (int32_t k = 0; k < S.nvox[a]; ++k)
          cen.push_back(std::fma((double)k + 0.5, S.dx[a], S.min[a]));
    }
  int32_t r = allocate(c);
  if (r == CRG_OK) r = dalloc(&c->vcen, cen.size());
  if (r == CRG_OK && cudaMemcpy(c->vcen, cen.data(), sizeof(double) * cen.size(),
                                cudaMemcpyHostToDevice) != cudaSuccess)
    r = CRG_ECUDA;
  if (r == CRG_OK && c->kind == CRG_KIND_ROD && crg::prepare_rods(c->dim, c->nv) != 0)
    r = CRG_ECUDA;
  if (r == CRG_OK && c->kind != CRG_KIND_ROD && crg::prepare_spheres(c->dim, c->precision) != 0)
    r = CRG_ECUDA;
  if (r != CRG_OK) {
    free_all(c);
    delete c;
    return r;
  }
  *out = c;
  return CRG_OK;
}

PackArgs pack_args(crg_ctx *c) {
  PackArgs P;
  std::memset(&P, 0, sizeof(P));
  P.sims = c->d_sims;
  P.sim_agent_off = c->d_agent_off;
  P.n_sims = c->n_sims;
  P.cap = c->cap;
  P.n_agents = c->n_agents;
  P.n_vox = c->n_vox;
  P.pos = c->pos;
  P.vel = c->vel;
  P.id = c->id;
  P.key = c->key;
  P.off = c->off;
  P.hist = c->hist;
  P.hmeta = c->hmeta;
  P.start = c->start;
  P.npos = c->npos;
  P.nvel = c->nvel;
  P.nid = c->nid;
  P.nkey = c->nkey;
  P.nhist = c->nhist;
  P.nhmeta = c->nhmeta;
  P.count = c->count;
  P.status = c->status;
  P.step_ctr = c->step_ctr;
  P.dbg_force = c->dbg_force;
  P.frc = c->frc;
  P.rctl = c->rctl;
  P.fix_list = c->fix_list;
  P.bend = c->bend;
  P.hl = c->hl;
  P.seg = c->seg;
  P.npass = c->npass;
  P.pass_off = c->pass_off;
  P.pass_a = c->pass_a;
  P.pass_b = c->pass_b;
  P.pass_meta = c->pass_meta;
  P.mbuf = c->mbuf;
  P.pass_cap = c->pass_cap;
  P.prefilter = c->prefilter;
  P.variant = c->variant;
  P.tile = c->tile;
  if (c->cycle) {
    P.slen = c->slen;
    P.grate = c->grate;
    P.parent = c->parent;
    P.nslen = c->nslen;
    P.ngrate = c->ngrate;
    P.nparent = c->nparent;
    P.nsense = c->nsense;
    P.dflag = c->dflag;
    P.dpre = c->dpre;
    P.vctr = c->vctr;
    P.srank = c->srank;
  }
  return P;
}

SortArgs sort_args(crg_ctx *c, int initial) {
  SortArgs A;
  std::memset(&A, 0, sizeof(A));
  A.sims = c->d_sims;
  A.vcen = c->vcen;
  A.sim_agent_off = c->d_agent_off;
  A.sim_of_voxel = c->d_sim_of_voxel;
  A.n_sims = c->n_sims;
  A.nc = c->nc;
  A.initial = initial;
  A.cap = c->cap;
  A.n_agents = c->n_agents;
  A.n_vox = c->n_vox;
  A.pos = c->pos;
  A.vel = c->vel;
  A.id = c->id;
  A.key = c->key;
  A.off = c->off;
  A.off_aos = off_aos(c);
  A.hist = c->hist;
  A.hmeta = c->hmeta;
  A.npos = c->npos;
  A.nvel = c->nvel;
  A.nid = c->nid;
  A.nkey = c->nkey;
  A.nhist = c->nhist;
  A.nhmeta = c->nhmeta;
  A.count = c->count;
  A.start = c->start;
  A.tmp = c->tmp;
  A.status = c->status;
  A.step_ctr = initial ? nullptr : c->step_ctr;
  if (c->cycle) {
    A.slen = c->slen;
    A.grate = c->grate;
    A.parent = c->parent;
    A.nslen = c->nslen;
    A.ngrate = c->ngrate;
    A.nparent = c->nparent;
  }
  return A;
}

// Kernels one launch_force issues: the default rod path runs the pass walk, the pass kernel,
// the rod-level fallback (returns at once unless the pass list overflowed) and the update.
// Rods: the pass-list path (walk, pass kernel, overflow fallback, bend, update) runs unless
// the FP64 thread-per-rod variant was chosen; mixed precision always takes it.
bool rod_pass_list(const crg_ctx *c) {
  return c->kind == CRG_KIND_ROD && (c->variant != 1 || c->precision != CRG_PREC_F64);
}

int force_kernel_count(const crg_ctx *c) {
  if (c->kind == CRG_KIND_ROD) return rod_pass_list(c) ? (c->nv > 2 ? 5 : 4) : 1;
  return c->precision == CRG_PREC_F64 ? 1 : 2;
}

// k0 / k1 (optional): events recorded around the dominant force kernel; k2 / k3 around the
// rod update kernel.
void launch_force(crg_ctx *c, cudaEvent_t k0 = nullptr, cudaEvent_t k1 = nullptr,
                  cudaEvent_t k2 = nullptr, cudaEvent_t k3 = nullptr) {
  PackArgs P = pack_args(c);
  if (c->kind == CRG_KIND_SPHERE) {
    crg::record_event(k0, c->stream);
    crg::launch_spheres_step(c->dim, c->precision, P, c->block, c->stream);
    crg::record_event(k1, c->stream);
  } else {
    crg::launch_rods_step(c->dim, c->nv, c->precision, P, c->block, c->stream, k0, k1, k2, k3);
  }
}

// Steps per profiled chunk, and the events of each of its steps (CRG_OPT_PROFILE): before
// the force stage, around the dominant force kernel, between the force stage and the sort,
// after the sort, around the rod update kernel.
constexpr int kProfChunk = 32;
constexpr int kProfEvents = 7;

// One step.  With prof_step >= 0 (profiling) the step's events are recorded around its
// phases (as event nodes when the step is being captured into a graph, so the kernels can
// be timed as they run from the graph).
void launch_one_step(crg_ctx *c, int prof_step = -1) {
  cudaEvent_t *e = (prof_step >= 0 && !c->pev.empty()) ? &c->pev[kProfEvents * prof_step] : nullptr;
  if (e) crg::record_event(e[0], c->stream);
  launch_force(c, e ? e[1] : nullptr, e ? e[2] : nullptr, e ? e[5] : nullptr,
               e ? e[6] : nullptr);
  if (e) crg::record_event(e[3], c->stream);
  crg::launch_sort(sort_args(c, 0), c->bsum, c->stream);
  if (e) crg::record_event(e[4], c->stream);
}

// Waits for the handle's stream and reads the device status word.  A CUDA failure is
// recorded as the handle's error (so every later call reports it too).
void invalidate_graph(crg_ctx *c);

int32_t read_status(crg_ctx *c) {
  cudaError_t e = cudaMemcpyAsync(c->h_status, c->status, 8 * sizeof(int32_t),
                                  cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    c->err_code = (e == cudaErrorMemoryAllocation) ? CRG_ENOMEM : CRG_ECUDA;
    c->err_agent = -1;
    c->err_step = c->steps_done;
    return c->err_code;
  }
  if (c->kind == CRG_KIND_ROD && (int64_t)(uint32_t)c->h_status[5] > c->pass_cap) {
    // a step outgrew the pass list and took the rod-level kernel: make room for next time
    const int64_t need = (int64_t)(uint32_t)c->h_status[5];
    invalidate_graph(c);  // captured launches hold the old buffers
    alloc_pass_list(c, need + need / 4 + 1024);
  }
  if (c->h_status[0] != CRG_OK) {
    c->err_code = c->h_status[0];
    c->err_agent = (int64_t)(((uint64_t)(uint32_t)c->h_status[2] << 32) | (uint32_t)c->h_status[1]);
    c->err_step = c->h_status[3];
    c->err_sim = c->h_status[4];
    return c->err_code;
  }
  return CRG_OK;
}

int32_t ensure_graph(crg_ctx *c, int steps) {
  if (c->gexec && c->gexec_steps == steps) return CRG_OK;
  if (c->gexec) {
    cudaGraphExecDestroy(c->gexec);
    c->gexec = nullptr;
  }
  cudaGraph_t g;
  CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  for (int k = 0; k < steps; ++k) launch_one_step(c, c->profile ? k : -1);
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  if (e != cudaSuccess) return CRG_ECUDA;
  e = cudaGraphInstantiate(&c->gexec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    c->gexec = nullptr;
    return CRG_ECUDA;
  }
  c->gexec_steps = steps;
  return CRG_OK;
}

void invalidate_graph(crg_ctx *c) {
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  c->gexec = nullptr;
  c->gexec_steps = 0;
}

// Cell-cycle handles whose divisions would outgrow the capacity: the handle's state (the
// state before the step, which nothing of the step has changed yet) moves to a new handle of
// at least `need` and twice the capacity, through a checkpoint, and the new handle's
// resources replace the old ones behind the same pointer (the stream stays the caller's).
int32_t grow_capacity(crg_ctx *c, int64_t need) {
  int64_t new_cap = std::max<int64_t>(need, 2 * c->cap);
  new_cap = std::min<int64_t>(new_cap, 0x7fffffffll);
  if (new_cap < need) return CRG_ENOMEM;
  int64_t bytes = 0;
  int32_t r = crg_checkpoint_size(c, &bytes);
  if (r != CRG_OK) return r;
  std::vector<char> blob((size_t)bytes);
  r = crg_checkpoint_save(c, blob.data(), bytes);
  if (r != CRG_OK) return r;
  crg_ctx *g = nullptr;
  r = create_impl(1, c->doms.data(), c->mods.data(), &new_cap, &g);
  if (r != CRG_OK) return r;
  g->ckpt_any_capacity = true;
  g->graph_chunk = c->graph_chunk;
  g->prefilter = c->prefilter;
  g->variant = c->variant;
  g->tile = c->tile;
  g->block = c->block;
  g->profile = c->profile;
  if (c->dbg_force) r = crg_set_option(g, CRG_OPT_DEBUG_FORCES, 1);
  if (r == CRG_OK && c->pass_cap > g->pass_cap) r = alloc_pass_list(g, c->pass_cap);
  if (r == CRG_OK) r = crg_checkpoint_load(g, blob.data(), bytes);
  g->ckpt_any_capacity = false;
  if (r != CRG_OK) {
    crg_destroy(g);
    return r;
  }
  cudaStreamSynchronize(c->stream);
  std::swap(*c, *g);
  std::swap(c->stream, g->stream);  // the caller keeps its stream; g's own is destroyed
  crg_destroy(g);
  return CRG_OK;
}

// Cell-cycle handles run one step at a time: divisions change the agent count that every
// launch is sized by.  Per step: neighbour counts (k_rods_sense), forces and the update
// (growth, division flags), the scan of the flags, a read of the division count, the
// divisions (k_rods_divide), the voxel counters and the sort of the grown list.  A step
// whose divisions would exceed the handle's capacity stops before dividing with CRG_ENOMEM;
// a step that fails stops before its sort, so the handle keeps the previous step's state.
int32_t step_cycle(crg_ctx *c, int64_t n_steps) {
  cudaStream_t st = c->stream;
  int64_t done = 0;
  for (; done < n_steps; ++done) {
    const uint32_t n = c->n_agents;
    PackArgs P = pack_args(c);
    crg::launch_rods_sense(c->dim, c->nv, P, st);
    launch_force(c);
    crg::launch_scan(c->dflag, n, c->dpre, c->dbsum, st);
    if (cudaMemcpyAsync(c->h_ndiv, c->dpre + n, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                        st) != cudaSuccess) {
      c->err_code = CRG_ECUDA;
      c->err_step = c->steps_done + done;
      break;
    }
    if (read_status(c) != CRG_OK) break;
    const uint32_t n_div = c->h_ndiv[0];
    if ((int64_t)n + (int64_t)n_div > c->cap) {
      // nothing of this step is committed yet: grow the handle and take the step again
      const int32_t r = grow_capacity(c, (int64_t)n + (int64_t)n_div);
      if (r != CRG_OK) {
        c->err_code = r;
        c->err_agent = -1;
        c->err_step = c->steps_done + done + 1;
        break;
      }
      --done;
      continue;
    }
    if (n_div) {
      crg::launch_rods_divide(c->dim, c->nv, P, n_div, st);
      // a DivisionError stops the step before anything of it is committed
      if (read_status(c) != CRG_OK) break;
      crg::launch_cycle_counters(P, st);
    }
    SortArgs A = sort_args(c, 0);
    A.n_agents = n + n_div;
    A.srank = n_div ? c->srank : nullptr;
    crg::launch_sort(A, c->bsum, st);
    if (n_div) {
      c->n_agents = n + n_div;
      c->agent_off_h[1] = c->n_agents;
      c->sims_h[0].n_agents = c->n_agents;
      if (cudaMemcpyAsync(c->d_sims, c->sims_h.data(), sizeof(SimDev), cudaMemcpyHostToDevice,
                          st) != cudaSuccess ||
          cudaMemcpyAsync(c->d_agent_off, c->agent_off_h.data(), 2 * sizeof(uint32_t),
                          cudaMemcpyHostToDevice, st) != cudaSuccess) {
        c->err_code = CRG_ECUDA;
        c->err_step = c->steps_done + done + 1;
        ++done;
        break;
      }
    }
    if (cudaGetLastError() != cudaSuccess) {
      c->err_code = CRG_ECUDA;
      c->err_step = c->steps_done + done + 1;
      ++done;
      break;
    }
  }
  if (c->err_code == CRG_OK) read_status(c);
  c->steps_done += done;
  return c->err_code;
}

}  // namespace

extern "C" {

const char *crg_strerror(int32_t code) {
  switch (code) {
    case CRG_OK: return "ok";
    case CRG_ECALC: return "calculation error (CalcError)";
    case CRG_EBOUNDARY: return "agent outside the domain (BoundaryError)";
    case CRG_EINDEX: return "agent outside every voxel (IndexError)";
    case CRG_EDECOMPOSE: return "cannot decompose the domain (DecomposeError)";
    case CRG_EINVAL: return "invalid argument";
    case CRG_ENOMEM: return "out of device memory";
    case CRG_ECUDA: return "CUDA runtime error";
    case CRG_ETIMEDOUT: return "device wait timed out";
    case CRG_ENOTSUP: return "not supported";
    case CRG_EINTERNAL: return "device-side invariant check failed";
    default: return "unknown status";
  }
}

int32_t crg_create(const crg_domain *domain, const crg_model *model, int64_t capacity,
                   crg_ctx **out) {
  if (!domain || !model) return CRG_EINVAL;
  return create_impl(1, domain, model, &capacity, out);
}

int32_t crg_create_batch(int32_t n_sims, const crg_domain *domains, const crg_model *models,
                         const int64_t *capacities, crg_ctx **out) {
  return create_impl(n_sims, domains, models, capacities, out);
}

int32_t crg_destroy(crg_ctx *c) {
  if (!c) return CRG_EINVAL;
  if (c->stream) cudaStreamSynchronize(c->stream);
  free_all(c);
  delete c;
  return CRG_OK;
}

// crg_upload; vel = nullptr gives every agent zero velocity.
static int32_t upload_impl(crg_ctx *c, int64_t n, const int64_t *counts, const double *pos,
                           const double *vel, const uint64_t *ids) {
  if (!c || n < 0 || (n > 0 && !pos)) return CRG_EINVAL;
  std::vector<int64_t> cnt(c->n_sims);
  if (c->n_sims == 1) {
    cnt[0] = counts ? counts[0] : n;
  } else {
    if (!counts) return CRG_EINVAL;
    cnt.assign(counts, counts + c->n_sims);
  }
  int64_t tot = 0;
  for (int s = 0; s < c->n_sims; ++s) {
    if (cnt[s] < 0 || cnt[s] > c->caps[s]) return CRG_EINVAL;
    tot += cnt[s];
  }
  if (tot != n) return CRG_EINVAL;
  c->n_agents = (uint32_t)n;
  c->agent_off_h.assign(c->n_sims + 1, 0);
  for (int s = 0; s < c->n_sims; ++s) {
    c->agent_off_h[s + 1] = c->agent_off_h[s] + (uint32_t)cnt[s];
    c->sims_h[s].agent_off = c->agent_off_h[s];
    c->sims_h[s].n_agents = (uint32_t)cnt[s];
    c->sims_h[s].step_base = 0;
  }
  invalidate_graph(c);
  c->err_code = CRG_OK;
  c->err_agent = c->err_step = -1;
  c->steps_done = 0;
  cudaStream_t st = c->stream;
  CUDA_TRY(cudaMemcpyAsync(c->d_sims, c->sims_h.data(), sizeof(SimDev) * c->n_sims,
                           cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(c->d_agent_off, c->agent_off_h.data(),
                           sizeof(uint32_t) * (c->n_sims + 1), cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemsetAsync(c->status, 0, sizeof(int32_t) * 8, st));
  CUDA_TRY(cudaMemsetAsync(c->step_ctr, 0, sizeof(int64_t), st));
  CUDA_TRY(cudaMemsetAsync(c->count, 0, sizeof(uint32_t) * ((size_t)c->n_vox + 1), st));
  const size_t bytes = sizeof(double) * (size_t)n * c->nc;
  if (n > 0) {
    CUDA_TRY(cudaMemcpyAsync(c->staging, pos, bytes, cudaMemcpyHostToDevice, st));
    crg::launch_transpose_in(c->staging, c->npos, (uint32_t)n, c->nc, c->cap, st);
    if (vel) {
      CUDA_TRY(cudaMemcpyAsync(c->staging, vel, bytes, cudaMemcpyHostToDevice, st));
      crg::launch_transpose_in(c->staging, c->nvel, (uint32_t)n, c->nc, c->cap, st);
    } else {
      CUDA_TRY(cudaMemsetAsync(c->nvel, 0, sizeof(double) * (size_t)c->cap * c->nc, st));
    }
    if (ids) {
      CUDA_TRY(cudaMemcpyAsync(c->nid, ids, sizeof(uint64_t) * n, cudaMemcpyHostToDevice, st));
    } else {
      std::vector<uint64_t> iota(n);
      int64_t k = 0;
      for (int s = 0; s < c->n_sims; ++s)
        for (int64_t j = 0; j < cnt[s]; ++j) iota[k++] = (uint64_t)j;
      CUDA_TRY(cudaMemcpyAsync(c->nid, iota.data(), sizeof(uint64_t) * n, cudaMemcpyHostToDevice, st));
      CUDA_TRY(cudaStreamSynchronize(st));
    }
  }
  if (c->order > 1) {
    CUDA_TRY(cudaMemsetAsync(c->nhmeta, 0, (size_t)c->cap, st));
    CUDA_TRY(cudaMemsetAsync(c->nhist, 0, sizeof(double) * (size_t)c->cap * c->nc * 2, st));
  }
  if (c->cycle && n > 0) {  // every rod starts at the model's spring length, no parent
    std::vector<double> sl((size_t)n, c->mods[0].spring_length);
    std::vector<double> gr((size_t)n, c->mods[0].growth_rate);
    CUDA_TRY(cudaMemcpyAsync(c->nslen, sl.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(c->ngrate, gr.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemsetAsync(c->nparent, 0xff, sizeof(uint64_t) * n, st));
    CUDA_TRY(cudaStreamSynchronize(st));
  }
  SortArgs A = sort_args(c, 1);
  crg::launch_init_keys(A, c->nv, st);
  crg::launch_sort(A, c->bsum, st);
  if (c->cycle) crg::launch_cycle_init(pack_args(c), st);
  CUDA_TRY(cudaGetLastError());
  int32_t r = read_status(c);
  if (r != CRG_OK) {
    c->err_step = 0;
    return r;
  }
  return CRG_OK;
}

int32_t crg_upload(crg_ctx *c, int64_t n, const int64_t *counts, const double *pos,
                   const double *vel, const uint64_t *ids) {
  if (n > 0 && !vel) return CRG_EINVAL;
  return upload_impl(c, n, counts, pos, vel, ids);
}

int32_t crg_forces(crg_ctx *c, int64_t n, const double *pos, double *force) {
  if (!c || n < 0 || (n > 0 && (!pos || !force))) return CRG_EINVAL;
  if (c->n_sims != 1 || c->cycle) return CRG_ENOTSUP;
  int32_t r = upload_impl(c, n, nullptr, pos, nullptr, nullptr);
  if (r != CRG_OK || n == 0) return r;
  if (!c->fbuf && (r = dalloc(&c->fbuf, (size_t)c->cap * c->nc)) != CRG_OK) return r;
  cudaStream_t st = c->stream;
  // One force evaluation of the uploaded cell list.  The kernels also compute the state a
  // step would reach from these forces; it stays in the "next" arrays and is dropped, and a
  // BoundaryError raised by it concerns a step that is not taken.
  crg::PackArgs P = pack_args(c);
  P.dbg_force = c->fbuf;
  if (c->kind == CRG_KIND_SPHERE)
    crg::launch_spheres_step(c->dim, c->precision, P, c->block, st);
  else
    crg::launch_rods_step(c->dim, c->nv, c->precision, P, c->block, st);
  CUDA_TRY(cudaGetLastError());
  r = read_status(c);
  if (r == CRG_EBOUNDARY) {
    c->err_code = CRG_OK;
    c->err_agent = c->err_step = -1;
    c->err_sim = -1;
    r = CRG_OK;
  }
  if (r != CRG_OK) return r;
  CUDA_TRY(cudaMemsetAsync(c->status, 0, sizeof(int32_t) * 8, st));
  // the histogram of the dropped next keys
  CUDA_TRY(cudaMemsetAsync(c->count, 0, sizeof(uint32_t) * ((size_t)c->n_vox + 1), st));
  crg::launch_unsort_out(c->fbuf, c->tmp, c->staging, (uint32_t)n, c->nc, c->cap, c->status, st);
  CUDA_TRY(cudaMemcpyAsync(force, c->staging, sizeof(double) * (size_t)n * c->nc,
                           cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaGetLastError());
  return read_status(c);
}

int32_t crg_step(crg_ctx *c, int64_t n_steps) {
  if (!c || n_steps < 0) return CRG_EINVAL;
  if (c->err_code != CRG_OK) return c->err_code;
  if (n_steps == 0 || c->n_agents == 0) {
    c->steps_done += n_steps;
    return CRG_OK;
  }
  if (c->cycle) return step_cycle(c, n_steps);
  if (c->profile) {
    if (c->pev.empty()) {
      c->pev.assign(kProfEvents * kProfChunk, nullptr);
      for (auto &e : c->pev) CUDA_TRY(cudaEventCreate(&e));
    }
    for (double &x : c->prof_ms) x = 0.0;
  }
  int64_t left = n_steps;
  const int chunk = c->graph_chunk;
  while (left > 0) {
    if (c->profile) {
      // the steps run as they run unprofiled (from a captured graph when chunks are on),
      // with event nodes between the phases; the chunk's times are read after it
      const int k = (int)std::min<int64_t>(left, kProfChunk);
      if (chunk > 0 && k == kProfChunk) {
        int32_t r = ensure_graph(c, k);
        if (r != CRG_OK) return r;
        CUDA_TRY(cudaGraphLaunch(c->gexec, c->stream));
      } else {
        for (int s = 0; s < k; ++s) launch_one_step(c, s);
      }
      CUDA_TRY(cudaStreamSynchronize(c->stream));
      for (int s = 0; s < k; ++s) {
        const cudaEvent_t *e = &c->pev[kProfEvents * s];
        float a = 0.f, b = 0.f, d = 0.f, u = 0.f;
        cudaEventElapsedTime(&a, e[0], e[3]);
        cudaEventElapsedTime(&b, e[3], e[4]);
        cudaEventElapsedTime(&d, e[1], e[2]);
        if (rod_pass_list(c))
          cudaEventElapsedTime(&u, e[5], e[6]);  // recorded by the pass-list rod path only
        c->prof_ms[0] += a;
        c->prof_ms[1] += b;
        c->prof_ms[3] += d;
        c->prof_ms[4] += u;
        c->prof_ms[2] += force_kernel_count(c) + crg::sort_kernel_count(c->n_vox);
      }
      left -= k;
    } else if (chunk > 0 && left >= chunk) {
      int32_t r = ensure_graph(c, chunk);
      if (r != CRG_OK) return r;
      const int64_t reps = std::min<int64_t>(left / chunk, std::max(1, 256 / chunk));
      for (int64_t k = 0; k < reps; ++k) CUDA_TRY(cudaGraphLaunch(c->gexec, c->stream));
      left -= reps * chunk;
    } else {
      const int k = (int)std::min<int64_t>(left, 256);
      for (int s = 0; s < k; ++s) launch_one_step(c);
      left -= k;
    }
    if (cudaGetLastError() != cudaSuccess) {
      c->err_code = CRG_ECUDA;
      c->err_step = c->steps_done;
      break;
    }
    int32_t r = read_status(c);
    if (r != CRG_OK) break;
  }
  c->steps_done += n_steps - std::max<int64_t>(left, 0);
  // The failing step of a simulation is not committed and its later steps leave it frozen
  // (sim_frozen, failed_sim): a single simulation holds the state after its last good step.
  if (c->n_sims == 1 && c->err_code != CRG_OK && c->err_code != CRG_ECUDA &&
      c->err_code != CRG_EINTERNAL && c->err_step >= 1)
    c->steps_done = std::min(c->steps_done, c->err_step - 1);
  return c->err_code;
}

}  // extern "C"

namespace crg {

int32_t step_launch(crg_ctx *c, int64_t n_steps) {
  if (!c || n_steps < 0 || n_steps > 256 || c->cycle || c->profile) return CRG_EINVAL;
  if (c->err_code != CRG_OK) return c->err_code;
  if (n_steps == 0 || c->n_agents == 0) return CRG_OK;
  int64_t left = n_steps;
  const int chunk = c->graph_chunk;
  if (chunk > 0 && left >= chunk) {
    int32_t r = ensure_graph(c, chunk);
    if (r != CRG_OK) return r;
    for (; left >= chunk; left -= chunk) CUDA_TRY(cudaGraphLaunch(c->gexec, c->stream));
  }
  for (; left > 0; --left) launch_one_step(c);
  CUDA_TRY(cudaGetLastError());
  return CRG_OK;
}

int32_t step_wait(crg_ctx *c, int64_t n_steps) {
  if (!c) return CRG_EINVAL;
  if (c->err_code != CRG_OK) return c->err_code;
  if (n_steps == 0 || c->n_agents == 0) {
    c->steps_done += n_steps;
    return CRG_OK;
  }
  read_status(c);
  c->steps_done += n_steps;
  if (c->n_sims == 1 && c->err_code != CRG_OK && c->err_code != CRG_ECUDA &&
      c->err_code != CRG_EINTERNAL && c->err_step >= 1)
    c->steps_done = std::min(c->steps_done, c->err_step - 1);
  return c->err_code;
}

}  // namespace crg

extern "C" {

int32_t crg_download(crg_ctx *c, double *pos, double *vel, uint64_t *ids, uint32_t *voxel) {
  if (!c) return CRG_EINVAL;
  const uint32_t n = c->n_agents;
  if (n == 0) return CRG_OK;
  cudaStream_t st = c->stream;
  const size_t bytes = sizeof(double) * (size_t)n * c->nc;
  if (pos) {
    crg::launch_transpose_out(c->pos, c->staging, n, c->nc, c->cap, st);
    CUDA_TRY(cudaMemcpyAsync(pos, c->staging, bytes, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
  }
  if (vel) {
    crg::launch_transpose_out(c->vel, c->staging, n, c->nc, c->cap, st);
    CUDA_TRY(cudaMemcpyAsync(vel, c->staging, bytes, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
  }
  if (ids) CUDA_TRY(cudaMemcpyAsync(ids, c->id, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost, st));
  if (voxel) {
    CUDA_TRY(cudaMemcpyAsync(voxel, c->key, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    for (int s = 0; s < c->n_sims; ++s)
      for (uint32_t i = c->agent_off_h[s]; i < c->agent_off_h[s + 1]; ++i)
        voxel[i] -= c->sims_h[s].voxel_off;
  }
  CUDA_TRY(cudaStreamSynchronize(st));
  return CRG_OK;
}

int32_t crg_snapshot(crg_ctx *c, int32_t op) {
  if (!c || (op != CRG_SNAPSHOT_SAVE && op != CRG_SNAPSHOT_RESTORE)) return CRG_EINVAL;
  if (c->cycle) return CRG_ENOTSUP;  // the cycle state is not part of snapshots
  const size_t cap = (size_t)c->cap, nc = (size_t)c->nc;
  struct Part {
    void *p;
    size_t bytes;
  };
  std::vector<Part> parts = {
      {c->pos, sizeof(double) * cap * nc}, {c->vel, sizeof(double) * cap * nc},
      {c->id, sizeof(uint64_t) * cap},     {c->key, sizeof(uint32_t) * cap},
      {c->off, sizeof(float) * cap * (off_aos(c) ? off_aos(c) : nc)},
      {c->start, sizeof(uint32_t) * ((size_t)c->n_vox + 1)},
      {c->step_ctr, sizeof(int64_t)}};
  if (c->order > 1) {
    parts.push_back({c->hist, sizeof(double) * cap * nc * 2});
    parts.push_back({c->hmeta, cap});
  }
  size_t total = 0;
  for (auto &p : parts) total += (p.bytes + 255) & ~size_t(255);
  if (op == CRG_SNAPSHOT_SAVE && !c->snap) {
    int32_t r = dalloc(&c->snap, total);
    if (r != CRG_OK) return r;
  }
  if (!c->snap) return CRG_EINVAL;
  size_t off = 0;
  for (auto &p : parts) {
    char *s = c->snap + off;
    if (op == CRG_SNAPSHOT_SAVE)
      CUDA_TRY(cudaMemcpyAsync(s, p.p, p.bytes, cudaMemcpyDeviceToDevice, c->stream));
    else
      CUDA_TRY(cudaMemcpyAsync(p.p, s, p.bytes, cudaMemcpyDeviceToDevice, c->stream));
    off += (p.bytes + 255) & ~size_t(255);
  }
  if (op == CRG_SNAPSHOT_SAVE) {
    c->snap_agents = c->n_agents;
    c->snap_steps = c->steps_done;
  } else {
    if (c->snap_agents != c->n_agents) return CRG_EINVAL;
    c->steps_done = c->snap_steps;
    c->err_code = CRG_OK;
    c->err_agent = c->err_step = -1;
    CUDA_TRY(cudaMemsetAsync(c->status, 0, sizeof(int32_t) * 8, c->stream));
  }
  return CRG_OK;
}

namespace {

struct CkptHeader {
  char magic[8];
  int32_t version, n_sims, nc, dim, kind, order;
  uint32_t n_agents, n_vox;
  int64_t steps_done;
  uint64_t params;  // params_hash of the handle's domains and models
};
constexpr char kCkptMagic[8] = {'C', 'R', 'G', 'C', 'K', 'P', 'T', '1'};
constexpr int32_t kCkptVersion = 4;

// FNV-1a over every field of the handle's domains, models and capacities (field by field:
// crg_model has padding bytes), so a checkpoint loads only into a handle that steps the same
// simulations.
uint64_t params_hash(const crg_ctx *c) {
  uint64_t h = 1469598103934665603ull;
  auto mix = [&h](const void *p, size_t n) {
    const unsigned char *b = static_cast<const unsigned char *>(p);
    for (size_t k = 0; k < n; ++k) h = (h ^ b[k]) * 1099511628211ull;
  };
  for (int s = 0; s < c->n_sims; ++s) {
    const crg_domain &d = c->doms[s];
    const crg_model &m = c->mods[s];
    mix(&d.dim, 4), mix(&d.voxel_mode, 4), mix(d.min, 24), mix(d.max, 24);
    mix(&d.interaction_range, 8), mix(d.n_voxels, 24), mix(&d.n_subdomains, 4);
    mix(&d.weight_mode, 4);
    mix(&m.kind, 4), mix(&m.n_vertices, 4), mix(&m.solver_order, 4), mix(&m.precision, 4);
    const double *dv[] = {&m.mass, &m.damping, &m.spring_tension, &m.rigidity,
                          &m.spring_length, &m.diffusion, &m.radius, &m.stiffness,
                          &m.cutoff, &m.strength, &m.dt, &m.kb_temperature,
                          &m.growth_rate, &m.division_length, &m.sense_range,
                          &m.sense_saturation};
    for (const double *x : dv) mix(x, 8);
    mix(&m.rng_seed, 8), mix(&m.cycle, 4);
    mix(&c->caps[s], 8);
  }
  return h;
}

// The checkpoint's device slices, in blob order: per array, its first n_agents entries of
// each component (arrays are component-major with stride cap).
struct CkptSlice {
  char *dev;
  size_t elem, comps;
};
std::vector<CkptSlice> ckpt_slices(crg_ctx *c) {
  const size_t nc = (size_t)c->nc;
  std::vector<CkptSlice> v = {{(char *)c->pos, sizeof(double), nc},
                              {(char *)c->vel, sizeof(double), nc},
                              {(char *)c->id, sizeof(uint64_t), 1},
                              {(char *)c->key, sizeof(uint32_t), 1}};
  if (off_aos(c))  // interleaved sphere offsets: one record of off_aos floats per agent
    v.push_back({(char *)c->off, sizeof(float) * (size_t)off_aos(c), 1});
  else
    v.push_back({(char *)c->off, sizeof(float), nc});
  if (c->order > 1) {
    v.push_back({(char *)c->hist, sizeof(double), 2 * nc});
    v.push_back({(char *)c->hmeta, 1, 1});
  }
  if (c->cycle) {  // spring length, growth rate and parent of every rod
    v.push_back({(char *)c->slen, sizeof(double), 1});
    v.push_back({(char *)c->grate, sizeof(double), 1});
    v.push_back({(char *)c->parent, sizeof(uint64_t), 1});
  }
  return v;
}

// header, agent offsets, stop steps and step bases, the slices, the cell starts, the step
// counter and (cell cycle) every voxel's id counter
size_t ckpt_bytes(crg_ctx *c, uint32_t n_agents) {
  size_t b = sizeof(CkptHeader) + sizeof(uint32_t) * (c->n_sims + 1) +
             2 * sizeof(int64_t) * c->n_sims;
  for (const CkptSlice &s : ckpt_slices(c)) b += s.elem * s.comps * n_agents;
  b += sizeof(uint32_t) * ((size_t)c->n_vox + 1) + sizeof(int64_t);
  if (c->cycle) b += sizeof(uint64_t) * (size_t)c->n_vox;
  return b;
}

}  // namespace

int32_t crg_checkpoint_size(crg_ctx *c, int64_t *bytes) {
  if (!c || !bytes) return CRG_EINVAL;
  *bytes = (int64_t)ckpt_bytes(c, c->n_agents);
  return CRG_OK;
}

int32_t crg_checkpoint_save(crg_ctx *c, void *buf, int64_t bytes) {
  if (!c || !buf || bytes < (int64_t)ckpt_bytes(c, c->n_agents)) return CRG_EINVAL;
  if (c->err_code != CRG_OK) return c->err_code;
  char *p = (char *)buf;
  CkptHeader h;
  std::memset(&h, 0, sizeof(h));
  std::memcpy(h.magic, kCkptMagic, 8);
  h.version = kCkptVersion;
  h.params = params_hash(c);
  h.n_sims = c->n_sims;
  h.nc = c->nc;
  h.dim = c->dim;
  h.kind = c->kind;
  h.order = c->order;
  h.n_agents = c->n_agents;
  h.n_vox = c->n_vox;
  h.steps_done = c->steps_done;
  std::memcpy(p, &h, sizeof(h));
  p += sizeof(h);
  std::memcpy(p, c->agent_off_h.data(), sizeof(uint32_t) * (c->n_sims + 1));
  p += sizeof(uint32_t) * (c->n_sims + 1);
  for (int s = 0; s < c->n_sims; ++s, p += 2 * sizeof(int64_t)) {
    std::memcpy(p, &c->sims_h[s].stop_step, sizeof(int64_t));
    std::memcpy(p + sizeof(int64_t), &c->sims_h[s].step_base, sizeof(int64_t));
  }
  cudaStream_t st = c->stream;
  const size_t n = c->n_agents;
  for (const CkptSlice &s : ckpt_slices(c))
    for (size_t k = 0; k < s.comps; ++k, p += s.elem * n)
      if (n) CUDA_TRY(cudaMemcpyAsync(p, s.dev + s.elem * k * (size_t)c->cap, s.elem * n,
                                      cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(p, c->start, sizeof(uint32_t) * ((size_t)c->n_vox + 1),
                           cudaMemcpyDeviceToHost, st));
  p += sizeof(uint32_t) * ((size_t)c->n_vox + 1);
  CUDA_TRY(cudaMemcpyAsync(p, c->step_ctr, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  p += sizeof(int64_t);
  if (c->cycle)
    CUDA_TRY(cudaMemcpyAsync(p, c->vctr, sizeof(uint64_t) * (size_t)c->n_vox,
                             cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  return CRG_OK;
}

int32_t crg_checkpoint_load(crg_ctx *c, const void *buf, int64_t bytes) {
  if (!c || !buf || bytes < (int64_t)sizeof(CkptHeader)) return CRG_EINVAL;
  // the library's own loads of a checkpoint of this simulation at another capacity, whose
  // parameter hash differs in that field (the domains and models are the same)
  const bool check_params = !c->ckpt_any_capacity;
  const char *p = (const char *)buf;
  CkptHeader h;
  std::memcpy(&h, p, sizeof(h));
  if (std::memcmp(h.magic, kCkptMagic, 8) != 0 || h.version != kCkptVersion ||
      h.n_sims != c->n_sims || h.nc != c->nc || h.dim != c->dim || h.kind != c->kind ||
      h.order != c->order || h.n_vox != c->n_vox ||
      (check_params && h.params != params_hash(c)) ||
      h.n_agents > (uint64_t)c->cap || bytes < (int64_t)ckpt_bytes(c, h.n_agents))
    return CRG_EINVAL;
  p += sizeof(h);
  std::vector<uint32_t> aoff(c->n_sims + 1);
  std::memcpy(aoff.data(), p, sizeof(uint32_t) * (c->n_sims + 1));
  p += sizeof(uint32_t) * (c->n_sims + 1);
  if (aoff[0] != 0 || aoff[c->n_sims] != h.n_agents) return CRG_EINVAL;
  for (int s = 0; s < c->n_sims; ++s)
    if (aoff[s + 1] < aoff[s] || (int64_t)(aoff[s + 1] - aoff[s]) > c->caps[s]) return CRG_EINVAL;
  std::vector<int64_t> stops(c->n_sims), bases(c->n_sims);
  for (int s = 0; s < c->n_sims; ++s, p += 2 * sizeof(int64_t)) {
    std::memcpy(&stops[s], p, sizeof(int64_t));
    std::memcpy(&bases[s], p + sizeof(int64_t), sizeof(int64_t));
  }
  // The cell starts (after the per-agent slices): they index every per-agent array, so a
  // damaged blob must not reach the device.  start[0] = 0, non-decreasing, start[n_vox] =
  // n_agents, and each simulation's first voxel starts at its first agent.
  {
    size_t slice_bytes = 0;
    for (const CkptSlice &sl : ckpt_slices(c)) slice_bytes += sl.elem * sl.comps * h.n_agents;
    std::vector<uint32_t> st((size_t)c->n_vox + 1);
    std::memcpy(st.data(), p + slice_bytes, sizeof(uint32_t) * st.size());
    if (st[0] != 0 || st[c->n_vox] != h.n_agents) return CRG_EINVAL;
    for (uint32_t v = 0; v < c->n_vox; ++v)
      if (st[v + 1] < st[v]) return CRG_EINVAL;
    for (int s = 0; s < c->n_sims; ++s)
      if (st[c->sims_h[s].voxel_off] != aoff[s]) return CRG_EINVAL;
  }
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  invalidate_graph(c);
  c->n_agents = h.n_agents;
  c->agent_off_h = aoff;
  for (int s = 0; s < c->n_sims; ++s) {
    c->sims_h[s].agent_off = aoff[s];
    c->sims_h[s].n_agents = aoff[s + 1] - aoff[s];
    c->sims_h[s].stop_step = stops[s];
    c->sims_h[s].step_base = bases[s];
  }
  c->steps_done = h.steps_done;
  c->err_code = CRG_OK;
  c->err_agent = c->err_step = -1;
  cudaStream_t st = c->stream;
  CUDA_TRY(cudaMemcpyAsync(c->d_sims, c->sims_h.data(), sizeof(SimDev) * c->n_sims,
                           cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(c->d_agent_off, c->agent_off_h.data(),
                           sizeof(uint32_t) * (c->n_sims + 1), cudaMemcpyHostToDevice, st));
  const size_t n = c->n_agents;
  for (const CkptSlice &s : ckpt_slices(c))
    for (size_t k = 0; k < s.comps; ++k, p += s.elem * n)
      if (n) CUDA_TRY(cudaMemcpyAsync(s.dev + s.elem * k * (size_t)c->cap, p, s.elem * n,
                                      cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(c->start, p, sizeof(uint32_t) * ((size_t)c->n_vox + 1),
                           cudaMemcpyHostToDevice, st));
  p += sizeof(uint32_t) * ((size_t)c->n_vox + 1);
  CUDA_TRY(cudaMemcpyAsync(c->step_ctr, p, sizeof(int64_t), cudaMemcpyHostToDevice, st));
  p += sizeof(int64_t);
  if (c->cycle)
    CUDA_TRY(cudaMemcpyAsync(c->vctr, p, sizeof(uint64_t) * (size_t)c->n_vox,
                             cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemsetAsync(c->status, 0, sizeof(int32_t) * 8, st));
  CUDA_TRY(cudaMemsetAsync(c->count, 0, sizeof(uint32_t) * ((size_t)c->n_vox + 1), st));
  CUDA_TRY(cudaStreamSynchronize(st));
  return CRG_OK;
}


namespace {

// Cell-cycle handles: every shape's trial starts from a host checkpoint (device snapshots
// hold no cycle state) and is timed on the host clock (the cycle step reads its division
// count every step).  The checkpoint loads with any capacity, so a trial that grew the
// handle does not keep the next one from starting where the first did.
int32_t autotune_cycle(crg_ctx *c, int64_t steps, int64_t *variant, int64_t *block,
                       double *ms_per_step) {
  const int shapes[4][2] = {{0, 0}, {0, 32}, {0, 128}, {1, 64}};
  int64_t bytes = 0;
  int32_t r = crg_checkpoint_size(c, &bytes);
  if (r != CRG_OK) return r;
  std::vector<char> blob((size_t)bytes);
  if ((r = crg_checkpoint_save(c, blob.data(), bytes)) != CRG_OK) return r;
  const int saved_variant = c->variant, saved_block = c->block;
  int best_v = saved_variant, best_b = saved_block;
  double best_ms = 1e300;
  auto restore = [&]() {
    c->ckpt_any_capacity = true;
    const int32_t rr = crg_checkpoint_load(c, blob.data(), bytes);
    c->ckpt_any_capacity = false;
    return rr;
  };
  for (const auto &sh : shapes) {
    c->variant = sh[0];
    c->block = sh[1];
    if ((r = restore()) != CRG_OK) break;
    const auto t0 = std::chrono::steady_clock::now();
    const int32_t rs = crg_step(c, steps);
    const auto t1 = std::chrono::steady_clock::now();
    if (rs != CRG_OK) {  // a failing trial (the state's own error): keep the others
      c->err_code = CRG_OK;
      continue;
    }
    const double ms = std::chrono::duration<double, std::milli>(t1 - t0).count() / steps;
    if (ms < best_ms) {
      best_ms = ms;
      best_v = sh[0];
      best_b = sh[1];
    }
  }
  c->variant = best_v;
  c->block = best_b;
  const int32_t r2 = restore();
  if (r != CRG_OK) return r;
  if (variant) *variant = best_v;
  if (block) *block = best_b;
  if (ms_per_step) *ms_per_step = best_ms;
  return r2;
}

}  // namespace

int32_t crg_autotune(crg_ctx *c, int64_t steps, int64_t *variant, int64_t *block,
                     double *ms_per_step) {
  if (!c || steps <= 0) return CRG_EINVAL;
  if (c->err_code != CRG_OK) return c->err_code;
  if (c->cycle) return autotune_cycle(c, steps, variant, block, ms_per_step);
  struct Shape {
    int variant, block, tile;
  };
  std::vector<Shape> shapes;
  if (c->kind == CRG_KIND_ROD && c->precision != CRG_PREC_F64) {
    shapes = {{0, 0, 0}, {0, 32, 0}, {0, 128, 0}};  // one pass kernel, either walk
  } else if (c->kind == CRG_KIND_ROD) {
    // pass list walked by size, with a warp or with a thread per rod; the rod-level kernel
    shapes = {{0, 0, 0}, {0, 32, 0}, {0, 128, 0}, {1, 64, 0}};
  } else if (c->precision == CRG_PREC_F64) {
    // agent groups with 8 (block 0), 16 or 32 lanes per agent; lane per agent; thread per
    // agent, one-shot and persistent
    shapes = {{0, 0, 0},   {2, 0, 0},   {2, 16, 0},  {2, 32, 0},  {3, 0, 0},
              {3, 64, 0},  {1, 64, 0},  {1, 128, 0}, {1, 256, 0}, {1, 128, 1},
              {1, 128, 4}, {1, 256, 2}};
  } else {
    // thread per agent: one-shot grids, and the persistent tile kernel with tiles of
    // block x 1, 2, 4 agents; the warp-packed kernel
    shapes = {{1, 64, 0},  {1, 128, 0}, {1, 256, 0}, {1, 64, 2},  {1, 128, 1},
              {1, 128, 2}, {1, 128, 4}, {1, 256, 1}, {1, 256, 2}, {3, 0, 0}};
  }
  int32_t r = crg_snapshot(c, CRG_SNAPSHOT_SAVE);
  if (r != CRG_OK) return r;
  const int saved_variant = c->variant, saved_block = c->block, saved_profile = c->profile;
  const int saved_tile = c->tile;
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0));
  CUDA_TRY(cudaEventCreate(&e1));
  double best_ms = 1e300;
  Shape best = {saved_variant, saved_block, saved_tile};
  c->profile = 0;
  for (const Shape &s : shapes) {
    c->variant = s.variant;
    c->block = s.block;
    c->tile = s.tile;
    if ((r = crg_snapshot(c, CRG_SNAPSHOT_RESTORE)) != CRG_OK) break;
    launch_one_step(c);  // warm-up (first launch of this shape)
    if ((r = crg_snapshot(c, CRG_SNAPSHOT_RESTORE)) != CRG_OK) break;
    cudaEventRecord(e0, c->stream);
    for (int64_t k = 0; k < steps; ++k) launch_one_step(c);
    cudaEventRecord(e1, c->stream);
    if ((r = read_status(c)) != CRG_OK) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms / steps < best_ms) {
      best_ms = ms / steps;
      best = s;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  c->variant = best.variant;
  c->block = best.block;
  c->tile = best.tile;
  c->profile = saved_profile;
  invalidate_graph(c);
  int32_t r2 = crg_snapshot(c, CRG_SNAPSHOT_RESTORE);
  if (r != CRG_OK) return r;
  if (variant) *variant = best.variant;
  if (block) *block = best.block;
  if (ms_per_step) *ms_per_step = best_ms;
  return r2;
}

int32_t crg_get_stream(crg_ctx *c, void **stream) {
  if (!c || !stream) return CRG_EINVAL;
  *stream = (void *)c->stream;
  return CRG_OK;
}

int32_t crg_step_count(crg_ctx *c, int64_t *steps) {
  if (!c || !steps) return CRG_EINVAL;
  *steps = c->steps_done;
  return CRG_OK;
}

int32_t crg_set_sim_stop(crg_ctx *c, int32_t sim, int64_t stop_step) {
  if (!c || sim < 0 || sim >= c->n_sims) return CRG_EINVAL;
  c->sims_h[sim].stop_step = stop_step < 0 ? 0 : stop_step;
  CUDA_TRY(cudaMemcpyAsync(&c->d_sims[sim], &c->sims_h[sim], sizeof(SimDev),
                           cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  return CRG_OK;
}

int32_t crg_sim_download(crg_ctx *c, int32_t sim, int64_t *n, double *pos, double *vel,
                         uint64_t *ids) {
  if (!c || sim < 0 || sim >= c->n_sims) return CRG_EINVAL;
  const uint32_t off = c->agent_off_h[sim], cnt = c->agent_off_h[sim + 1] - off;
  if (n) *n = cnt;
  if (cnt == 0) return CRG_OK;
  cudaStream_t st = c->stream;
  const size_t bytes = sizeof(double) * (size_t)cnt * c->nc;
  if (pos) {
    crg::launch_transpose_out(c->pos + off, c->staging, cnt, c->nc, c->cap, st);
    CUDA_TRY(cudaMemcpyAsync(pos, c->staging, bytes, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
  }
  if (vel) {
    crg::launch_transpose_out(c->vel + off, c->staging, cnt, c->nc, c->cap, st);
    CUDA_TRY(cudaMemcpyAsync(vel, c->staging, bytes, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
  }
  if (ids)
    CUDA_TRY(cudaMemcpyAsync(ids, c->id + off, sizeof(uint64_t) * cnt, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  return CRG_OK;
}

int32_t crg_clear_error(crg_ctx *c, int32_t *sim) {
  if (!c) return CRG_EINVAL;
  if (sim) *sim = c->err_sim;
  const int32_t code = c->err_code;
  c->err_code = CRG_OK;
  c->err_agent = c->err_step = -1;
  c->err_sim = -1;
  CUDA_TRY(cudaMemsetAsync(c->status, 0, sizeof(int32_t) * 8, c->stream));
  // a cell-cycle step stops before its sort, leaving the voxel histogram filled
  CUDA_TRY(cudaMemsetAsync(c->count, 0, sizeof(uint32_t) * ((size_t)c->n_vox + 1), c->stream));
  if (c->n_sims == 1)  // the frozen steps advanced the device counter past the kept state
    CUDA_TRY(cudaMemcpyAsync(c->step_ctr, &c->steps_done, sizeof(int64_t),
                             cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  return code;
}

int32_t crg_repack(crg_ctx *src, int32_t n_keep, const int32_t *keep, int32_t n_new,
                   const crg_domain *new_domains, const crg_model *new_models,
                   const int64_t *new_caps, const int64_t *new_counts, const double *new_pos,
                   const double *new_vel, crg_ctx **out) {
  if (!out || n_keep < 0 || n_new < 0 || n_keep + n_new < 1) return CRG_EINVAL;
  if (n_keep > 0 && (!src || !keep)) return CRG_EINVAL;
  if (n_new > 0 && (!new_domains || !new_models || !new_caps || !new_counts)) return CRG_EINVAL;
  if (n_keep > 0 && src->cycle) return CRG_ENOTSUP;  // packs hold no cell cycle
  for (int32_t k = 0; k < n_new; ++k)
    if (new_models[k].cycle) return CRG_ENOTSUP;
  *out = nullptr;
  const int n_total = n_keep + n_new;
  std::vector<crg_domain> doms;
  std::vector<crg_model> mods;
  std::vector<int64_t> caps, counts;
  int64_t n_new_agents = 0;
  for (int s = 0; s < n_new; ++s) {
    if (new_counts[s] < 0 || new_counts[s] > new_caps[s]) return CRG_EINVAL;
    doms.push_back(new_domains[s]);
    mods.push_back(new_models[s]);
    caps.push_back(new_caps[s]);
    counts.push_back(new_counts[s]);
    n_new_agents += new_counts[s];
  }
  if (n_new_agents > 0 && (!new_pos || !new_vel)) return CRG_EINVAL;
  std::vector<char> seen(src ? src->n_sims : 0, 0);
  for (int k = 0; k < n_keep; ++k) {
    const int s = keep[k];
    if (s < 0 || s >= src->n_sims || seen[s]) return CRG_EINVAL;
    seen[s] = 1;
    doms.push_back(src->doms[s]);
    mods.push_back(src->mods[s]);
    const int64_t cnt = src->agent_off_h[s + 1] - src->agent_off_h[s];
    caps.push_back(std::max<int64_t>(src->caps[s], cnt));
    counts.push_back(cnt);
  }
  crg_ctx *c = nullptr;
  int32_t r = create_impl(n_total, doms.data(), mods.data(), caps.data(), &c);
  if (r != CRG_OK) return r;
  if (src) {
    c->variant = src->variant;
    c->tile = src->tile;
    c->block = src->block;
    c->prefilter = src->prefilter;
    c->graph_chunk = src->graph_chunk;
  }
  // a kept simulation's own step count continues from the source pack (random stream)
  for (int k = 0; k < n_keep; ++k)
    c->sims_h[n_new + k].step_base = src->sims_h[keep[k]].step_base + src->steps_done;
  // agent layout: new simulations first (input order), then the kept ones
  c->agent_off_h.assign(n_total + 1, 0);
  for (int s = 0; s < n_total; ++s) {
    c->agent_off_h[s + 1] = c->agent_off_h[s] + (uint32_t)counts[s];
    c->sims_h[s].agent_off = c->agent_off_h[s];
    c->sims_h[s].n_agents = (uint32_t)counts[s];
  }
  c->n_agents = c->agent_off_h[n_total];
  cudaStream_t st = c->stream;
  auto fail = [&](int32_t code) {
    crg_destroy(c);
    return code;
  };
  if (cudaMemcpyAsync(c->d_sims, c->sims_h.data(), sizeof(SimDev) * n_total,
                      cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(c->d_agent_off, c->agent_off_h.data(), sizeof(uint32_t) * (n_total + 1),
                      cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemsetAsync(c->count, 0, sizeof(uint32_t) * ((size_t)c->n_vox + 1), st) != cudaSuccess)
    return fail(CRG_ECUDA);
  if (c->order > 1) {
    if (cudaMemsetAsync(c->nhmeta, 0, (size_t)c->cap, st) != cudaSuccess ||
        cudaMemsetAsync(c->nhist, 0, sizeof(double) * (size_t)c->cap * c->nc * 2, st) != cudaSuccess)
      return fail(CRG_ECUDA);
  }
  // new simulations: host data into the "next" arrays
  if (n_new_agents > 0) {
    const size_t bytes = sizeof(double) * (size_t)n_new_agents * c->nc;
    if (cudaMemcpyAsync(c->staging, new_pos, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess)
      return fail(CRG_ECUDA);
    crg::launch_transpose_in(c->staging, c->npos, (uint32_t)n_new_agents, c->nc, c->cap, st);
    if (cudaMemcpyAsync(c->staging, new_vel, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess)
      return fail(CRG_ECUDA);
    crg::launch_transpose_in(c->staging, c->nvel, (uint32_t)n_new_agents, c->nc, c->cap, st);
    std::vector<uint64_t> iota((size_t)n_new_agents);
    size_t q = 0;
    for (int s = 0; s < n_new; ++s)
      for (int64_t j = 0; j < counts[s]; ++j) iota[q++] = (uint64_t)j;
    if (cudaMemcpyAsync(c->nid, iota.data(), sizeof(uint64_t) * iota.size(),
                        cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return fail(CRG_ECUDA);
    SortArgs A = sort_args(c, 1);
    A.n_agents = (uint32_t)n_new_agents;
    crg::launch_init_keys(A, c->nv, st);
  }
  // kept simulations: device-resident state, cell-list order preserved
  if (n_keep > 0) {
    std::vector<uint32_t> dst_off(n_keep + 1), src_off(n_keep);
    std::vector<int64_t> shift(n_keep);
    for (int k = 0; k < n_keep; ++k) {
      dst_off[k] = c->agent_off_h[n_new + k];
      src_off[k] = src->agent_off_h[keep[k]];
      shift[k] = (int64_t)c->sims_h[n_new + k].voxel_off - (int64_t)src->sims_h[keep[k]].voxel_off;
    }
    dst_off[n_keep] = c->n_agents;
    uint32_t *d_dst = nullptr, *d_src = nullptr;
    int64_t *d_shift = nullptr;
    if (dalloc(&d_dst, n_keep + 1) || dalloc(&d_src, n_keep) || dalloc(&d_shift, n_keep)) {
      cudaFree(d_dst);
      cudaFree(d_src);
      return fail(CRG_ENOMEM);
    }
    // the source pack's last launches must be complete before its state is read
    cudaStreamSynchronize(src->stream);
    cudaMemcpyAsync(d_dst, dst_off.data(), sizeof(uint32_t) * (n_keep + 1), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_src, src_off.data(), sizeof(uint32_t) * n_keep, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_shift, shift.data(), sizeof(int64_t) * n_keep, cudaMemcpyHostToDevice, st);
    crg::RepackArgs R;
    std::memset(&R, 0, sizeof(R));
    R.spos = src->pos;
    R.svel = src->vel;
    R.shist = src->hist;
    R.sid = src->id;
    R.skey = src->key;
    R.shmeta = src->hmeta;
    R.scap = src->cap;
    R.dpos = c->npos;
    R.dvel = c->nvel;
    R.dhist = c->nhist;
    R.did = c->nid;
    R.dkey = c->nkey;
    R.dhmeta = c->nhmeta;
    R.dcount = c->count;
    R.dcap = c->cap;
    R.nc = c->nc;
    R.has_hist = c->order > 1 && src->order > 1;
    R.n_keep = n_keep;
    R.dst_off = d_dst;
    R.src_off = d_src;
    R.key_shift = d_shift;
    R.first = c->agent_off_h[n_new];
    R.last = c->n_agents;
    crg::launch_repack(R, st);
    cudaError_t e = cudaStreamSynchronize(st);
    cudaFree(d_dst);
    cudaFree(d_src);
    cudaFree(d_shift);
    if (e != cudaSuccess) return fail(CRG_ECUDA);
  }
  crg::launch_sort(sort_args(c, 1), c->bsum, st);
  if (cudaGetLastError() != cudaSuccess) return fail(CRG_ECUDA);
  r = read_status(c);
  if (r != CRG_OK) return fail(r);
  *out = c;
  return CRG_OK;
}

int32_t crg_set_spring_lengths(crg_ctx *c, const double *spring_length) {
  if (!c || !spring_length) return CRG_EINVAL;
  if (!c->cycle) return CRG_ENOTSUP;
  // the slot table of the upload's sort (tmp) is overwritten by the first step
  if (c->steps_done != 0 || c->err_code != CRG_OK) return CRG_EINVAL;
  const uint32_t n = c->n_agents;
  if (n == 0) return CRG_OK;
  cudaStream_t st = c->stream;
  CUDA_TRY(cudaMemcpyAsync(c->staging, spring_length, sizeof(double) * n,
                           cudaMemcpyHostToDevice, st));
  crg::launch_cycle_permute(c->slen, c->staging, c->tmp, n, st);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaStreamSynchronize(st));
  return CRG_OK;
}

int32_t crg_download_cycle(crg_ctx *c, double *spring_length, double *growth_rate,
                           uint64_t *parent) {
  if (!c) return CRG_EINVAL;
  if (!c->cycle) return CRG_ENOTSUP;
  const uint32_t n = c->n_agents;
  if (n == 0) return CRG_OK;
  cudaStream_t st = c->stream;
  if (spring_length)
    CUDA_TRY(cudaMemcpyAsync(spring_length, c->slen, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
  if (growth_rate)
    CUDA_TRY(cudaMemcpyAsync(growth_rate, c->grate, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
  if (parent)
    CUDA_TRY(cudaMemcpyAsync(parent, c->parent, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  return CRG_OK;
}

int32_t crg_agent_count(crg_ctx *c, int64_t *n) {
  if (!c || !n) return CRG_EINVAL;
  *n = c->n_agents;
  return CRG_OK;
}

int32_t crg_last_error(crg_ctx *c, int64_t *agent, int64_t *step) {
  if (!c) return CRG_EINVAL;
  if (agent) *agent = c->err_agent;
  if (step) *step = c->err_step;
  return c->err_code;
}

int32_t crg_get_option(crg_ctx *c, int32_t option, int64_t *value) {
  if (!c || !value) return CRG_EINVAL;
  switch (option) {
    case CRG_OPT_PREFILTER: *value = c->prefilter; break;
    case CRG_OPT_GRAPH_CHUNK: *value = c->graph_chunk; break;
    case CRG_OPT_BLOCK: *value = c->block; break;
    case CRG_OPT_PROFILE: *value = c->profile; break;
    case CRG_OPT_DEBUG_FORCES: *value = c->dbg_force ? 1 : 0; break;
    case CRG_OPT_KERNEL_VARIANT: *value = c->variant; break;
    case CRG_OPT_PASS_LIST: *value = c->pass_cap; break;
    case CRG_OPT_TILE: *value = c->tile; break;
    default: return CRG_EINVAL;
  }
  return CRG_OK;
}

int32_t crg_set_option(crg_ctx *c, int32_t option, int64_t value) {
  if (!c) return CRG_EINVAL;
  switch (option) {
    case CRG_OPT_PREFILTER: c->prefilter = value ? 1 : 0; break;
    case CRG_OPT_GRAPH_CHUNK:
      if (value < 0 || value > 4096) return CRG_EINVAL;
      c->graph_chunk = (int)value;
      break;
    case CRG_OPT_BLOCK:
      if (value < 0 || value > 1024) return CRG_EINVAL;
      c->block = (int)value;
      break;
    case CRG_OPT_PROFILE:
      c->profile = value ? 1 : 0;
      invalidate_graph(c);  // a captured graph may hold the events
      if (!c->profile) {
        CUDA_TRY(cudaStreamSynchronize(c->stream));
        free_events(c);
      }
      break;
    case CRG_OPT_KERNEL_VARIANT:
      if (value < 0 || value > 3) return CRG_EINVAL;
      c->variant = (int)value;
      break;
    case CRG_OPT_TILE:
      if (value < 0 || value > 16) return CRG_EINVAL;
      c->tile = (int)value;
      break;
    case CRG_OPT_PASS_LIST: {
      if (c->kind != CRG_KIND_ROD || value < 0) return CRG_EINVAL;
      CUDA_TRY(cudaStreamSynchronize(c->stream));
      const int32_t r = alloc_pass_list(c, value);
      if (r != CRG_OK) return r;
      break;
    }
    case CRG_OPT_DEBUG_FORCES:
      if (value && !c->dbg_force) {
        int32_t r = dalloc(&c->dbg_force, (size_t)c->cap * c->nc);
        if (r != CRG_OK) return r;
        CUDA_TRY(cudaMemset(c->dbg_force, 0, sizeof(double) * (size_t)c->cap * c->nc));
      } else if (!value && c->dbg_force) {
        cudaStreamSynchronize(c->stream);
        cudaFree(c->dbg_force);
        c->dbg_force = nullptr;
      }
      break;
    default: return CRG_EINVAL;
  }
  invalidate_graph(c);
  return CRG_OK;
}

int32_t crg_profile(crg_ctx *c, double *out5) {
  if (!c || !out5) return CRG_EINVAL;
  for (int k = 0; k < 5; ++k) out5[k] = c->prof_ms[k];
  return CRG_OK;
}

int32_t crg_debug_forces(crg_ctx *c, double *force, uint64_t *ids) {
  if (!c || !c->dbg_force) return CRG_EINVAL;
  const uint32_t n = c->n_agents;
  cudaStream_t st = c->stream;
  if (force) {
    crg::launch_transpose_out(c->dbg_force, c->staging, n, c->nc, c->cap, st);
    CUDA_TRY(cudaMemcpyAsync(force, c->staging, sizeof(double) * (size_t)n * c->nc,
                             cudaMemcpyDeviceToHost, st));
  }
  if (ids) CUDA_TRY(cudaMemcpyAsync(ids, c->nid, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  return CRG_OK;
}

int32_t crg_debug_neighbor_stats(crg_ctx *c, uint32_t *n_cand, uint32_t *n_inter,
                                 uint64_t *cand_hash, uint64_t *ids) {
  if (!c) return CRG_EINVAL;
  const uint32_t n = c->n_agents;
  if (n == 0) return CRG_OK;
  uint32_t *d_nc = nullptr, *d_ni = nullptr;
  uint64_t *d_h = nullptr;
  int32_t r;
  if ((r = dalloc(&d_nc, n)) || (r = dalloc(&d_ni, n)) || (r = dalloc(&d_h, n))) {
    cudaFree(d_nc);
    cudaFree(d_ni);
    cudaFree(d_h);
    return r;
  }
  crg::launch_neighbor_stats(c->dim, c->kind == CRG_KIND_ROD ? c->nv : 1, pack_args(c), d_nc,
                             d_ni, d_h, c->stream);
  cudaStream_t st = c->stream;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && n_cand) e = cudaMemcpyAsync(n_cand, d_nc, 4ull * n, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && n_inter) e = cudaMemcpyAsync(n_inter, d_ni, 4ull * n, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && cand_hash) e = cudaMemcpyAsync(cand_hash, d_h, 8ull * n, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && ids) e = cudaMemcpyAsync(ids, c->id, 8ull * n, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d_nc);
  cudaFree(d_ni);
  cudaFree(d_h);
  return e == cudaSuccess ? CRG_OK : CRG_ECUDA;
}

int32_t crg_measure_fma_peaks(double *fp64_tflops, double *fp32_tflops) {
  if (!fp64_tflops || !fp32_tflops) return CRG_EINVAL;
  return crg::measure_fma_peaks(fp64_tflops, fp32_tflops);
}

int32_t crg_check_division(int64_t n, uint64_t seed, int64_t *mismatches, int64_t *fast) {
  if (n < 0 || !mismatches || !fast) return CRG_EINVAL;
  return crg::check_division(n, seed, mismatches, fast);
}

}  // extern "C"

namespace crg {
void launch_sphere_stats(int dim, const PackArgs &P, uint32_t *n_cand, uint32_t *n_inter,
                         uint64_t *hash, cudaStream_t st);
void launch_rod_stats(int dim, int nv, const PackArgs &P, uint32_t *n_cand, uint32_t *n_inter,
                      uint64_t *hash, cudaStream_t st);

void launch_neighbor_stats(int dim, int nv, const PackArgs &P, uint32_t *n_cand,
                           uint32_t *n_inter, uint64_t *hash, cudaStream_t st) {
  if (nv == 1)
    launch_sphere_stats(dim, P, n_cand, n_inter, hash, st);
  else
    launch_rod_stats(dim, nv, P, n_cand, n_inter, hash, st);
}
}  // namespace crg
