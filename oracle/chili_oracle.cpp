// chili_oracle.cpp -- CPU restatement of cellular_raza's chili mechanics/interaction step.
//
// TEST INFRASTRUCTURE ONLY (the oracle).  Used by tests/ as the parity checker and by
// bench.py as the timed CPU baseline; never linked into the product library.
//
// Every function cites the reference file:line it restates (paths relative to the
// cellular_raza repository).  Arithmetic is written in the Rust expression order and the
// file is compiled with -ffp-contract=off so no multiply-add is fused, matching rustc.
// Third-party arithmetic the reference calls (not present in the reference tree):
//   nalgebra 0.34: dot/norm_squared are left folds for D<=3, norm = sqrt(norm_squared),
//     normalize = v / norm, Vector / scalar divides each component, Matrix::angle =
//     acos(clamp(dot / (|a| |b|), -1, 1)) with 0 for a zero-length operand.
//   num 0.4: ToPrimitive::to_usize for f64 truncates toward zero and is defined on the
//     open interval (-1, 2^64); NaN and everything else is None.
//   circ_buffer 0.1.8: RingBuffer<T,N>::push appends and overwrites the oldest element
//     once N are stored; iter() yields the stored elements from oldest to newest.
//   f64::{exp, sqrt, tan, acos}: the platform libm (glibc here).
#include "chili_oracle.h"

#ifndef ORACLE_PART
#define ORACLE_PART -1  // -1: whole oracle in one unit; 0: API + spheres; 2/3: rods
#endif

#include <algorithm>
#include <atomic>
#include <barrier>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

namespace oracle_impl {

// ---------------------------------------------------------------------------------
// Domain: CartesianCuboid / CartesianSubDomain
// ---------------------------------------------------------------------------------

// num::ToPrimitive::to_usize for f64 (truncation toward zero on (-1, 2^64)).
inline bool to_usize(double x, uint64_t &out) {
  if (x > -1.0 && x < 18446744073709551616.0) {
    out = (uint64_t)x;
    return true;
  }
  return false;
}

struct Domain {
  int dim = 3;
  double min[3] = {0, 0, 0}, max[3] = {0, 0, 0}, dx[3] = {0, 0, 0};
  uint64_t nvox[3] = {1, 1, 1};
  uint64_t n_total = 1;

  uint64_t plain(const uint64_t *idx) const {  // lexicographic, last axis fastest
    uint64_t p = 0;
    for (int i = 0; i < dim; ++i) p = p * nvox[i] + idx[i];
    return p;
  }
  void unravel(uint64_t p, uint64_t *idx) const {
    for (int i = dim - 1; i >= 0; --i) {
      idx[i] = p % nvox[i];
      p /= nvox[i];
    }
  }
  // CartesianSubDomain::get_index_of (cartesian_cuboid_n.rs:469-490) followed by the
  // voxel_index_to_plain_index lookup of sort_cells_in_voxels_step_1
  // (update_mechanics.rs:433-452).  Returns 0 ok, 1 conversion error, 2 index not found.
  int index_of(const double *pos, uint64_t &plain_out) const {
    uint64_t idx[3];
    for (int i = 0; i < dim; ++i) {
      double n_vox = (pos[i] - min[i]) / dx[i];
      if (!to_usize(n_vox, idx[i])) return 1;
    }
    for (int i = 0; i < dim; ++i)
      if (idx[i] >= nvox[i]) return 2;
    plain_out = plain(idx);
    return 0;
  }
  // CartesianCuboid::get_voxel_index_of_raw (cartesian_cuboid_n.rs:320-337): adds the
  // check_min_max(min, pos) test (min[i] >= pos[i] is a BoundaryError).
  int index_of_raw(const double *pos, uint64_t &plain_out) const {
    for (int i = 0; i < dim; ++i)
      if (min[i] >= pos[i]) return 1;
    return index_of(pos, plain_out);
  }
};

// CartesianCuboid::check_min_max (cartesian_cuboid_n.rs:149-162).
inline bool check_min_max(int dim, const double *min, const double *max) {
  for (int i = 0; i < dim; ++i)
    if (min[i] >= max[i]) return false;
  return true;
}

inline int make_domain(const or_config &c, Domain &d) {
  if (c.dim != 2 && c.dim != 3) return OR_EINVAL;
  d.dim = c.dim;
  for (int i = 0; i < 3; ++i) {
    d.min[i] = c.min[i];
    d.max[i] = c.max[i];
  }
  if (!check_min_max(c.dim, c.min, c.max)) return OR_EBOUNDARY;
  d.n_total = 1;
  for (int i = 0; i < c.dim; ++i) {
    if (c.voxel_mode == 0) {
      // from_boundaries_and_interaction_range (cartesian_cuboid_n.rs:183-222)
      double n = std::floor((c.max[i] - c.min[i]) / c.interaction_range);
      uint64_t m;
      if (!to_usize(n, m)) return OR_EBOUNDARY;
      d.nvox[i] = std::max<uint64_t>(m, 1);
      d.dx[i] = (c.max[i] - c.min[i]) / n;
    } else {
      // from_boundaries_and_n_voxels (cartesian_cuboid_n.rs:226-256)
      if (c.n_voxels[i] <= 0) return OR_EINVAL;
      d.nvox[i] = (uint64_t)c.n_voxels[i];
      d.dx[i] = (c.max[i] - c.min[i]) / (double)d.nvox[i];
    }
    d.n_total *= d.nvox[i];
  }
  return OR_OK;
}

// get_decomp_res (cartesian_cuboid_n.rs:19-59).
inline bool get_decomp_res(uint64_t n_voxel, uint64_t n_regions, uint64_t &n_out, uint64_t &m_out,
                    uint64_t &avg_out) {
  int64_t average_len = (int64_t)std::ceil((double)n_voxel / (double)n_regions);
  auto residue = [&](int64_t n, int64_t m, int64_t avg) {
    return (int64_t)n_voxel - avg * n - (avg - 1) * m;
  };
  int64_t n = (int64_t)n_regions, m = 0;
  for (uint64_t it = 0; it < n_regions; ++it) {
    int64_t r = residue(n, m, average_len);
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

// create_subdomains (cartesian_cuboid_n.rs:493-584): chunk_by over the lexicographic voxel
// enumeration; the first n chunks hold average_len voxels, the rest average_len-1.
inline int subdomain_map(const Domain &d, uint64_t n_sub, std::vector<uint32_t> &map) {
  uint64_t n, m, avg;
  if (n_sub == 0 || n_sub > d.n_total) return OR_EDECOMPOSE;
  if (!get_decomp_res(d.n_total, n_sub, n, m, avg)) return OR_EDECOMPOSE;
  map.resize(d.n_total);
  uint64_t switcher = n * avg;
  uint64_t div2 = std::max<uint64_t>(avg - 1, 1);
  for (uint64_t i = 0; i < d.n_total; ++i)
    map[i] = (uint32_t)(i < switcher ? i / avg : (i - switcher) / div2 + n);
  return OR_OK;
}

// CartesianSubDomain::get_neighbor_voxel_indices (cartesian_cuboid_n.rs:641-662) collected
// into a BTreeSet of plain indices (datastructures.rs:148-161): ascending, self excluded.
inline void neighbors_of(const Domain &d, uint64_t p, std::vector<uint64_t> &out) {
  out.clear();
  uint64_t idx[3] = {0, 0, 0}, lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
  d.unravel(p, idx);
  for (int i = 0; i < d.dim; ++i) {
    lo[i] = idx[i] >= 1 ? idx[i] - 1 : 0;
    hi[i] = std::min(idx[i] + 2, d.nvox[i]);
  }
  uint64_t j[3];
  for (j[0] = lo[0]; j[0] < hi[0]; ++j[0])
    for (j[1] = lo[1]; j[1] < hi[1]; ++j[1])
      for (j[2] = (d.dim == 3 ? lo[2] : 0); j[2] < (d.dim == 3 ? hi[2] : 1); ++j[2]) {
        uint64_t q = d.plain(j);
        if (q != p) out.push_back(q);
      }
  // multi_cartesian_product with the first axis outermost is already ascending.
}

inline uint64_t mix64(uint64_t x) {  // splitmix64 finaliser, used for order-free id hashes
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

// ---------------------------------------------------------------------------------
// Building blocks
// ---------------------------------------------------------------------------------

// calculate_morse_interaction (building-blocks/src/cell_building_blocks/interaction.rs:151-182).
template <int D>
inline bool morse(const double *own, const double *ext, double own_radius, double ext_radius,
                  double cutoff, double strength, double stiffness, double *f_own,
                  double *f_ext) {
  double z[D];
  for (int c = 0; c < D; ++c) z[c] = own[c] - ext[c];
  double n2 = z[0] * z[0];
  for (int c = 1; c < D; ++c) n2 = n2 + z[c] * z[c];
  double dist = std::sqrt(n2);
  if (dist > cutoff || dist == 0.0) {
    for (int c = 0; c < D; ++c) f_own[c] = f_ext[c] = 0.0;
    return false;
  }
  double dir[D];
  for (int c = 0; c < D; ++c) dir[c] = z[c] / dist;
  double r = own_radius + ext_radius;
  double s = strength, a = stiffness;
  double two = 1.0 + 1.0;
  double e = std::exp(-a * (dist - r));
  double force = -two * s * a * e * (1.0 - e);
  for (int c = 0; c < D; ++c) {
    f_own[c] = dir[c] * force;
    f_ext[c] = -dir[c] * force;
  }
  return true;
}

// nearest_point_from_point_to_line (interaction.rs:497-509).
template <int D>
inline double nearest_point(const double *p, const double *l0, const double *l1,
                            double *nearest, double &t_out) {
  double ab[D], ap[D];
  for (int c = 0; c < D; ++c) {
    ab[c] = l1[c] - l0[c];
    ap[c] = p[c] - l0[c];
  }
  double dot = ab[0] * ap[0];
  double nsq = ab[0] * ab[0];
  for (int c = 1; c < D; ++c) {
    dot = dot + ab[c] * ap[c];
    nsq = nsq + ab[c] * ab[c];
  }
  double t = dot / nsq;
  if (t < 0.0) t = 0.0;
  if (t > 1.0) t = 1.0;
  for (int c = 0; c < D; ++c) nearest[c] = l0[c] * (1.0 - t) + l1[c] * t;
  double d2 = 0.0;
  for (int c = 0; c < D; ++c) {
    double q = p[c] - nearest[c];
    d2 = (c == 0) ? q * q : d2 + q * q;
  }
  t_out = t;
  return std::sqrt(d2);
}

struct Params {
  double mass, damping, spring_tension, rigidity, spring_length;
  double radius, stiffness, cutoff, strength, dt;
  int order;
  int kind;  // OR_KIND_*
  double diffusion, kb_temperature;
  uint64_t seed;
};

// ---------------------------------------------------------------------------------
// Random stream of the stochastic mechanics.  The reference draws from per-voxel
// ChaCha8Rng streams (chili/datastructures.rs:180-182) through rand_distr::Normal; those
// crates are not available here, so the oracle and the GPU path share a counter-based
// stream instead: Philox4x32-10 keyed by the seed, counter (draw, step, agent id), and
// Box-Muller normals.  Parity with the reference is statistical (diffusion constant,
// equipartition); with the GPU path it is exact up to libm rounding.
// ---------------------------------------------------------------------------------
inline void philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

// n standard normals for agent id at step: block j (counter {j, step, id_lo, id_hi}) gives
// u1 in (0, 1] and u2 in [0, 1) with 53 bits each, then sqrt(-2 ln u1) (cos, sin)(2 pi u2).
inline void normals(uint64_t seed, uint64_t step, uint64_t id, int n, double *out) {
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  const double two_pi = 6.283185307179586;
  const double inv53 = 1.0 / 9007199254740992.0;  // 2^-53
  for (int j = 0; 2 * j < n; ++j) {
    const uint32_t ctr[4] = {(uint32_t)j, (uint32_t)step, (uint32_t)id, (uint32_t)(id >> 32)};
    uint32_t w[4];
    philox4x32_10(ctr, key, w);
    const double u1 = (double)((((uint64_t)w[0] << 21) | (w[1] >> 11)) + 1) * inv53;
    const double u2 = (double)(((uint64_t)w[2] << 21) | (w[3] >> 11)) * inv53;
    const double r = std::sqrt(-2.0 * std::log(u1));
    const double th = two_pi * u2;
    out[2 * j] = r * std::cos(th);
    if (2 * j + 1 < n) out[2 * j + 1] = r * std::sin(th);
  }
}

// ---------------------------------------------------------------------------------
// Simulation (chili SubDomainBox machinery)
// ---------------------------------------------------------------------------------
template <int D, int NV>
struct Sim {
  static constexpr int NC = D * NV;
  struct Cell {
    uint64_t id;
    double pos[NC];
    double vel[NC];
    // cell cycle (rods): RodMechanics::spring_length, the agent's growth_rate and the
    // identifier of the agent it divided from
    double slen = 0.0, grate = 0.0;
    uint64_t parent = OR_NO_PARENT;
  };
  // AuxStorageMechanics (chili/aux_storage.rs:41-130) with RingBuffer<_, order-1>.
  struct Aux {
    double force[NC];
    double hx[2][NC];
    double hv[2][NC];
    int first = 0, size = 0;
    uint32_t nsense = 0;   // AuxStorageInteraction's NeighborSensing accumulator
    bool divide = false;   // CycleEvent::Division pending
  };
  struct Entry {
    Cell c;
    Aux a;
  };
  struct Voxel {
    uint64_t plain;
    std::vector<uint64_t> nbrs;
    std::vector<Entry> cells;
    uint64_t id_counter = 0;  // Voxel::id_counter (chili/datastructures.rs:42)
  };
  // Cell cycle parameters (or_cycle).
  struct CycleP {
    bool on = false;
    double growth = 0.0, div_len = 0.0, sense = 0.0, sat = 0.0;
  };
  // PosInformation / ForceInformation / SendCell (chili/update_mechanics.rs:19-61).
  struct PosInfo {
    double pos[NC];
    double info;
    uint64_t cell_index, sender, receiver;
  };
  struct ForceInfo {
    double force[NC];
    uint64_t cell_index, sender;
  };
  struct SendCell {
    uint64_t source;
    Entry e;
  };
  struct Box {
    uint64_t lo, hi;
    std::vector<Voxel> voxels;
    int error = OR_OK;
    int64_t err_agent = -1;
  };

  Domain dom;
  Params prm;
  CycleP cyc;
  std::vector<uint32_t> sub_of;  // voxel plain -> subdomain
  std::vector<Box> boxes;
  int S = 1;
  int cap = 0;  // ring-buffer capacity = solver order - 1
  // mailboxes[sender][receiver]
  std::vector<std::vector<std::vector<PosInfo>>> mb_pos;
  std::vector<std::vector<std::vector<ForceInfo>>> mb_force;
  std::vector<std::vector<std::vector<SendCell>>> mb_cell;
  std::atomic<int> got_error{0};
  // debug capture of the last step
  bool want_debug = false;
  std::vector<double> dbg_force;  // indexed by id
  int64_t step_base = 0;          // steps run by earlier calls (random stream index)
  int64_t n_agents = 0;
  const double *slen_in = nullptr;  // cell cycle: initial spring lengths (input order)

  static void zero(double *x) {
    for (int k = 0; k < NC; ++k) x[k] = 0.0;
  }

  Voxel *voxel_local(Box &b, uint64_t p) {
    if (p < b.lo || p >= b.hi) return nullptr;
    return &b.voxels[p - b.lo];
  }

  // Interaction::calculate_force_between for the agent kinds in scope.
  // Spheres: MorsePotential (interaction.rs:234-254).  Rods: RodInteraction
  // (bacterial_rods.rs:292-336).  f_own/f_ext are written (not accumulated).
  void calc(const double *own, const double *ext, double ext_info, double *f_own,
            double *f_ext) const {
    if constexpr (NV == 1) {
      morse<D>(own, ext, prm.radius, ext_info, prm.cutoff, prm.strength, prm.stiffness, f_own,
               f_ext);
    } else {
      zero(f_own);
      zero(f_ext);
      for (int i = 0; i < NV; ++i) {
        const double *p1 = own + i * D;
        for (int j = 0; j + 1 < NV; ++j) {
          double q[D], t;
          nearest_point<D>(p1, ext + j * D, ext + (j + 1) * D, q, t);
          double fo[D], fe[D];
          morse<D>(p1, q, prm.radius, ext_info, prm.cutoff, prm.strength, prm.stiffness, fo,
                   fe);
          for (int c = 0; c < D; ++c) f_own[i * D + c] += fo[c];
          for (int c = 0; c < D; ++c) f_ext[j * D + c] += fe[c] * (1.0 - t);
          int j1 = (j + 1) % NV;
          for (int c = 0; c < D; ++c) f_ext[j1 * D + c] += fe[c] * t;
        }
      }
    }
  }

  static void add_half(double *acc, const double *f) {  // aux.add_force(f.xa(one_half))
    const double one_half = 1.0 / (1.0 + 1.0);
    for (int k = 0; k < NC; ++k) acc[k] += f[k] * one_half;
  }

  void set_error(Box &b, int code, int64_t agent) {
    if (b.error == OR_OK) {
      b.error = code;
      b.err_agent = agent;
    }
    got_error.store(1);
  }

  // neighbor_sensing_single (update_mechanics.rs:578-591) with the bacterial-rods agent's
  // NeighborSensing::accumulate_information (bacterial_rods/src/main.rs:49-64): every pair
  // of an own vertex and an ext vertex closer than the sensing range counts once.
  void sense(Aux &a, const double *own, const double *ext) const {
    if (!cyc.on) return;
    for (int i = 0; i < NV; ++i)
      for (int j = 0; j < NV; ++j) {
        double d[D];
        for (int c = 0; c < D; ++c) d[c] = own[i * D + c] - ext[j * D + c];
        double n2 = d[0] * d[0];
        for (int c = 1; c < D; ++c) n2 = n2 + d[c] * d[c];
        if (std::sqrt(n2) < cyc.sense) a.nsense += 1;
      }
  }

  // Voxel::calculate_force_between_cells_external (update_mechanics.rs:65-108).
  // Returns false when the voxel holds no cells (force is None).
  bool force_external(Voxel &vox, const double *ext_pos, double ext_info, double *force) {
    const double one_half = 1.0 / (1.0 + 1.0);
    bool some = false;
    for (Entry &e : vox.cells) {
      double f1[NC], f2[NC];
      calc(e.c.pos, ext_pos, ext_info, f1, f2);
      add_half(e.a.force, f1);
      sense(e.a, e.c.pos, ext_pos);  // update_mechanics.rs:105
      if (some) {
        for (int k = 0; k < NC; ++k) force[k] = f2[k] * one_half + force[k];
      } else {
        for (int k = 0; k < NC; ++k) force[k] = f2[k] * one_half;
        some = true;
      }
    }
    return some;
  }

  // update_mechanics_interaction_step_1 (update_mechanics.rs:153-238).
  void step1(int s) {
    Box &b = boxes[s];
    for (Voxel &vox0 : b.voxels) {
      size_t n_cells = vox0.cells.size();
      for (size_t n = 0; n < n_cells; ++n) {
        Voxel &vox = vox0;
        Cell c1 = vox.cells[n].c;  // p1, v1 (copies, like cell.pos())
        double i1 = prm.radius;
        for (size_t m = n + 1; m < n_cells; ++m) {
          Entry &e1 = vox.cells[n];
          Entry &e2 = vox.cells[m];
          double f1[NC], f2[NC];
          calc(c1.pos, e2.c.pos, prm.radius, f1, f2);
          add_half(e1.a.force, f1);
          add_half(e2.a.force, f2);
          double g2[NC], g1[NC];
          calc(e2.c.pos, c1.pos, i1, g2, g1);
          add_half(e1.a.force, g1);
          add_half(e2.a.force, g2);
          sense(e1.a, c1.pos, e2.c.pos);  // update_mechanics.rs:201-202
          sense(e2.a, e2.c.pos, c1.pos);
        }
        for (uint64_t nb : vox.nbrs) {
          Voxel *nv = voxel_local(b, nb);
          if (nv) {
            double dropped[NC];
            force_external(*nv, c1.pos, i1, dropped);  // the returned force is never used
          } else {
            PosInfo pi;
            std::memcpy(pi.pos, c1.pos, sizeof(pi.pos));
            pi.info = i1;
            pi.cell_index = n;
            pi.sender = vox.plain;
            pi.receiver = nb;
            mb_pos[s][sub_of[nb]].push_back(pi);
          }
        }
      }
    }
  }

  // update_mechanics_interaction_step_2 (update_mechanics.rs:285-340), determinism = true.
  void step2(int s) {
    Box &b = boxes[s];
    std::vector<PosInfo> rec;
    for (int t = 0; t < S; ++t) {
      auto &q = mb_pos[t][s];
      rec.insert(rec.end(), q.begin(), q.end());
      q.clear();
    }
    std::stable_sort(rec.begin(), rec.end(),
                     [](const PosInfo &x, const PosInfo &y) { return x.sender < y.sender; });
    for (const PosInfo &pi : rec) {
      Voxel *vox = voxel_local(b, pi.receiver);
      if (!vox) {
        set_error(b, OR_EINDEX, -1);
        return;
      }
      ForceInfo fi;
      if (force_external(*vox, pi.pos, pi.info, fi.force)) {
        fi.cell_index = pi.cell_index;
        fi.sender = pi.sender;
        mb_force[s][sub_of[pi.sender]].push_back(fi);
      }
    }
  }

  // update_mechanics_interaction_step_3 (update_mechanics.rs:344-382), determinism = true.
  void step3(int s) {
    Box &b = boxes[s];
    std::vector<ForceInfo> rec;
    for (int t = 0; t < S; ++t) {
      auto &q = mb_force[t][s];
      rec.insert(rec.end(), q.begin(), q.end());
      q.clear();
    }
    std::stable_sort(rec.begin(), rec.end(), [](const ForceInfo &x, const ForceInfo &y) {
      return x.sender < y.sender;
    });
    for (const ForceInfo &fi : rec) {
      Voxel *vox = voxel_local(b, fi.sender);
      if (!vox || fi.cell_index >= vox->cells.size()) {
        set_error(b, OR_EINDEX, -1);
        return;
      }
      double *acc = vox->cells[fi.cell_index].a.force;
      for (int k = 0; k < NC; ++k) acc[k] += fi.force[k];
    }
  }

  // Mechanics::calculate_increment.  Spheres: NewtonDamped (mechanics.rs:166-173).
  // Rods: RodMechanics (bacterial_rods.rs:157-213).
  void increment(const Cell &c, const double *force, double *dx, double *dv) const {
    if constexpr (NV == 1) {
      if (prm.kind == OR_KIND_BROWNIAN) {
        // Brownian: dx = D / k_B T * F, dv = 0 (mechanics.rs:350-357)
        const double s = prm.diffusion / prm.kb_temperature;
        for (int k = 0; k < NC; ++k) {
          dx[k] = s * force[k];
          dv[k] = 0.0;
        }
      } else if (prm.kind == OR_KIND_LANGEVIN) {
        // Langevin: dx = v, dv = 1 / M * F + (-gamma) * v (mechanics.rs:452-463)
        const double im = 1.0 / prm.mass;
        for (int k = 0; k < NC; ++k) {
          dx[k] = c.vel[k];
          dv[k] = im * force[k] + (-prm.damping) * c.vel[k];
        }
      } else {
        for (int k = 0; k < NC; ++k) {
          dx[k] = c.vel[k];
          dv[k] = force[k] / prm.mass - prm.damping * c.vel[k];
        }
      }
    } else {
      const double one_half = 1.0 / (1.0 + 1.0);
      const double two = 1.0 + 1.0;
      double tf[NC];
      for (int k = 0; k < NC; ++k) tf[k] = force[k];
      double dist[NV - 1][D];
      for (int i = 0; i + 1 < NV; ++i)
        for (int c2 = 0; c2 < D; ++c2) dist[i][c2] = c.pos[i * D + c2] - c.pos[(i + 1) * D + c2];
      auto norm = [](const double *v) {
        double n2 = v[0] * v[0];
        for (int c2 = 1; c2 < D; ++c2) n2 = n2 + v[c2] * v[c2];
        return std::sqrt(n2);
      };
      for (int i = 0; i + 1 < NV; ++i) {
        double nrm = norm(dist[i]);
        if (nrm != 0.0) {
          double fi[D];
          for (int c2 = 0; c2 < D; ++c2) {
            double dir = dist[i][c2] / nrm;
            fi[c2] = -dir * prm.spring_tension * (nrm - c.slen);
          }
          for (int c2 = 0; c2 < D; ++c2) tf[i * D + c2] += fi[c2] * one_half;
          for (int c2 = 0; c2 < D; ++c2) tf[(i + 1) * D + c2] += -fi[c2] * one_half;
        }
      }
      for (int i = 0; i + 2 < NV; ++i) {
        const double *c1 = dist[i];
        const double *c2v = dist[i + 1];
        // Matrix::angle
        double prod = c1[0] * c2v[0];
        for (int c2 = 1; c2 < D; ++c2) prod = prod + c1[c2] * c2v[c2];
        double n1 = norm(c1), n2 = norm(c2v);
        double angle;
        if (n1 == 0.0 || n2 == 0.0) {
          angle = 0.0;
        } else {
          double cang = prod / (n1 * n2);
          if (cang < -1.0) cang = -1.0;
          if (cang > 1.0) cang = 1.0;
          angle = std::acos(cang);
        }
        double fd[D];
        for (int c2 = 0; c2 < D; ++c2) fd[c2] = c1[c2] - c2v[c2];
        double fdn = norm(fd);
        double fdir[D];
        for (int c2 = 0; c2 < D; ++c2) fdir[c2] = (fdn != 0.0) ? fd[c2] / fdn : fd[c2];
        double tn = std::tan(one_half * angle);
        double f[D];
        for (int c2 = 0; c2 < D; ++c2) f[c2] = fdir[c2] * two * prm.rigidity * tn;
        for (int c2 = 0; c2 < D; ++c2) tf[i * D + c2] += -f[c2] * one_half;
        for (int c2 = 0; c2 < D; ++c2) tf[(i + 1) * D + c2] += f[c2];
        for (int c2 = 0; c2 < D; ++c2) tf[(i + 2) * D + c2] += -f[c2] * one_half;
      }
      for (int k = 0; k < NC; ++k) tf[k] -= c.vel[k] * prm.damping;
      for (int k = 0; k < NC; ++k) {
        dx[k] = c.vel[k];
        dv[k] = tf[k];
      }
    }
  }

  // RingBuffer (circ_buffer 0.1.8) push / iteration from oldest to newest.
  static void ring_push(Aux &a, int cap, const double *dx, const double *dv) {
    if (cap == 0) return;
    int slot;
    if (a.size < cap) {
      slot = (a.first + a.size) % cap;
      a.size += 1;
    } else {
      slot = a.first;
      a.first = (a.first + 1) % cap;
    }
    std::memcpy(a.hx[slot], dx, sizeof(double) * NC);
    std::memcpy(a.hv[slot], dv, sizeof(double) * NC);
  }

  // Mechanics::get_random_contribution, times dt as the solvers add it (x' = (dx dt + x) 1
  // + dx_rand dt).  NewtonDamped: zero (mechanics.rs:158-164).  Brownian: dx_rand =
  // sqrt(2 D) * N(0, sqrt(dt)) / dt (:336-348, wiener_process :211-226).  Langevin: dv_rand
  // = sqrt(2 gamma k_B T / M) * N(0, sqrt(dt)) / dt (:434-450).  RodMechanics: dx_rand =
  // N(0, sqrt(dt)) * 2^-2 * D / dt per vertex (bacterial_rods.rs:215-240).  A normal draw
  // N(0, sigma) is 0 + sigma * z (rand_distr::Normal).
  void random_terms(const Cell &c, int64_t step, double *rx, double *rv) const {
    const double dt = prm.dt;
    for (int k = 0; k < NC; ++k) rx[k] = rv[k] = 0.0 * dt;
    const bool rod_diffusion = NV > 1 && prm.diffusion != 0.0;
    if (!(prm.kind == OR_KIND_BROWNIAN || prm.kind == OR_KIND_LANGEVIN || rod_diffusion)) return;
    double z[NC];
    normals(prm.seed, (uint64_t)step, c.id, NC, z);
    const double sd = std::sqrt(dt);
    for (int k = 0; k < NC; ++k) {
      const double w = 0.0 + sd * z[k];
      if (prm.kind == OR_KIND_BROWNIAN) {
        rx[k] = (std::sqrt(2.0 * prm.diffusion) * (w / dt)) * dt;
      } else if (prm.kind == OR_KIND_LANGEVIN) {
        const double s = std::sqrt(2.0 * prm.damping * prm.kb_temperature / prm.mass);
        rv[k] = (s * (w / dt)) * dt;
      } else {
        rx[k] = (w * 0.25 * prm.diffusion / dt) * dt;
      }
    }
  }

  // local_mechanics_update (update_mechanics.rs:530-559) -> mechanics_euler /
  // mechanics_adams_bashforth_2 / _3 (chili/solvers.rs:23-55, 156-300) with the
  // euler / adams_bashforth_{2,3} kernels (solvers.rs:303-347).
  void mechanics_update(Entry &e, int64_t step, int64_t *dbg_slot) {
    double force[NC];
    std::memcpy(force, e.a.force, sizeof(force));
    zero(e.a.force);  // get_current_force_and_reset
    if (dbg_slot) std::memcpy(&dbg_force[(size_t)e.c.id * NC], force, sizeof(force));
    double dx[NC], dv[NC];
    increment(e.c, force, dx, dv);
    const double dt = prm.dt;
    const double one = 1.0;
    double rx[NC], rv[NC];  // dx_rand.xa(dt), dv_rand.xa(dt)
    random_terms(e.c, step, rx, rv);
    // set_last_position/velocity run BEFORE the history is read, so the newest stored
    // increment is the current one: AB2 always sees [dx, dx]; AB3 sees [dx, dx] on its
    // first step and [dx, oldest, newest(=dx)] afterwards.
    ring_push(e.a, cap, dx, dv);
    int n_prev = e.a.size;
    double np[NC], nv[NC];
    if (cap == 2 && n_prev == 2) {
      const double f0 = 23.0 / 12.0, f1 = -16.0 / 12.0, f2 = 5.0 / 12.0;
      const double *ox1 = e.a.hx[e.a.first], *ox2 = e.a.hx[(e.a.first + 1) % 2];
      const double *ov1 = e.a.hv[e.a.first], *ov2 = e.a.hv[(e.a.first + 1) % 2];
      for (int k = 0; k < NC; ++k) {
        np[k] = (dx[k] * f0 + (ox1[k] * f1 + ox2[k] * f2)) * dt + e.c.pos[k];
        np[k] = np[k] * one + rx[k];
        nv[k] = (dv[k] * f0 + (ov1[k] * f1 + ov2[k] * f2)) * dt + e.c.vel[k];
        nv[k] = nv[k] * one + rv[k];
      }
    } else if (cap >= 1 && n_prev == 1) {
      const double f0 = 3.0 / 2.0, f1 = -1.0 / 2.0;
      const double *ox = e.a.hx[e.a.first], *ov = e.a.hv[e.a.first];
      for (int k = 0; k < NC; ++k) {
        np[k] = (dx[k] * f0 + ox[k] * f1) * dt + e.c.pos[k];
        np[k] = np[k] * one + rx[k];
        nv[k] = (dv[k] * f0 + ov[k] * f1) * dt + e.c.vel[k];
        nv[k] = nv[k] * one + rv[k];
      }
    } else {
      for (int k = 0; k < NC; ++k) {
        np[k] = (dx[k] * dt + e.c.pos[k]) * one + rx[k];
        nv[k] = (dv[k] * dt + e.c.vel[k]) * one + rv[k];
      }
    }
    std::memcpy(e.c.pos, np, sizeof(np));
    // Brownian::set_velocity is a no-op: the velocity stays zero
    if (!(NV == 1 && prm.kind == OR_KIND_BROWNIAN)) std::memcpy(e.c.vel, nv, sizeof(nv));
  }

  // The local cell functions in the macro's order (run_sim.rs:258-283):
  // local_mechanics_update, local_interaction_react_to_neighbors, local_cycle_update.
  void update_local(int s, bool last, int64_t step) {
    Box &b = boxes[s];
    int64_t dummy = 0;
    for (Voxel &v : b.voxels)
      for (Entry &e : v.cells) {
        mechanics_update(e, step, (last && want_debug) ? &dummy : nullptr);
        if (cyc.on) {
          react(e);
          cycle_update(e);
        }
      }
  }

  // NeighborSensing::react_to_neighbors + clear_accumulator (bacterial_rods/src/
  // main.rs:66-78): rate * (K - n) / K, at least 0, for n > 0 neighbours, else the base
  // rate.  f64::max(x, 0.0) is written x > 0 ? x : 0 (it returns 0 for NaN as Rust's does;
  // the two may differ only in the sign of a zero rate, which adds nothing to the length).
  void react(Entry &e) const {
    const uint32_t n = e.a.nsense;
    if (n > 0) {
      const double v = cyc.growth * (cyc.sat - (double)n) / cyc.sat;
      e.c.grate = (v > 0.0) ? v : 0.0;
    } else {
      e.c.grate = cyc.growth;
    }
    e.a.nsense = 0;
  }

  // local_cycle_update (chili/update_cycle.rs:111-131) with the agent's Cycle::update_cycle
  // (bacterial_rods/src/main.rs:87-98): grow, and divide past the threshold length.
  void cycle_update(Entry &e) const {
    e.c.slen = e.c.slen + e.c.grate * prm.dt;
    if (e.c.slen > cyc.div_len) e.a.divide = true;
  }

  static uint64_t division_id(uint64_t plain, uint64_t counter) {
    return OR_ID_DIVISION | (plain << 32) | (counter & 0xffffffffull);
  }

  // RodMechanics::divide (bacterial_rods.rs:586-663): c1 keeps the first vertex and c2 the
  // last; both get div_factor * spring_length; the vertices are re-spread along the old
  // polyline.  Float sums start at -0.0 as Rust's Sum for f64 does.  Returns false for a
  // DivisionError (no segment index satisfies the search, or the index leaves the range).
  bool divide(Cell &c1, Cell &c2) const {
    if constexpr (NV < 2) {
      return false;
    } else {
      const double two = 1.0 + 1.0, one_half = 1.0 / two;
      const double radius = prm.radius;
      double pos[NC];
      std::memcpy(pos, c1.pos, sizeof(pos));
      c2 = c1;
      const double div_factor = one_half - radius / ((double)NV * c1.slen);
      const double nsl = div_factor * c1.slen;
      c1.slen = nsl;
      c2.slen = nsl;
      double seg[NV - 1];
      for (int q = 0; q + 1 < NV; ++q) {
        double d[D];
        for (int c = 0; c < D; ++c) d[c] = pos[q * D + c] - pos[(q + 1) * D + c];
        double n2 = d[0] * d[0];
        for (int c = 1; c < D; ++c) n2 = n2 + d[c] * d[c];
        seg[q] = std::sqrt(n2);
      }
      double total = -0.0;
      for (int q = 0; q + 1 < NV; ++q) total = total + seg[q];
      const double seglen = (total - two * radius) / (double)(NV - 1) / two;
      for (int nvx = 0; nvx < NV; ++nvx) {
        const double target = (double)nvx * seglen;
        int k = -1;
        double pk = 0.0, acc = -0.0;
        for (int n = 0; n < NV - 1; ++n) {  // sum of the first n segments
          if (acc <= target) {
            k = n;
            pk = acc;
          }
          acc = acc + seg[n];
        }
        if (k < 0) return false;
        const double q = (target - pk) / seg[k];
        for (int c = 0; c < D; ++c)
          c1.pos[nvx * D + c] = pos[k * D + c] * (1.0 - q) + pos[(k + 1) * D + c] * q;
        int m = -1;
        double rm = 0.0;
        acc = -0.0;
        for (int n = 0; n < NV; ++n) {  // sum of the last n segments, last first
          if (acc <= target) {
            m = n;
            rm = acc;
          }
          if (n < NV - 1) acc = acc + seg[NV - 2 - n];
        }
        if (m < 0 || NV - m - 2 < 0) return false;
        const double p = (target - rm) / seg[NV - m - 2];
        for (int c = 0; c < D; ++c)
          c2.pos[(NV - nvx - 1) * D + c] =
              pos[(NV - m - 1) * D + c] * (1.0 - p) + pos[(NV - m - 2) * D + c] * p;
      }
      return true;
    }
  }

  // SubDomainBox::update_cell_cycle_4 -> Voxel::update_cell_cycle_4 (chili/update_cycle.rs:
  // 10-69): per voxel, dividing agents in storage order get the identifier Division(voxel,
  // ++counter) and their daughters are collected; the daughters are appended to the voxel
  // with Division(voxel, ++counter) each and a fresh AuxStorage (no solver history).
  void cycle4(int s) {
    Box &b = boxes[s];
    for (Voxel &v : b.voxels) {
      std::vector<Entry> born;
      for (Entry &e : v.cells) {
        if (!e.a.divide) continue;
        e.a.divide = false;
        Cell c2;
        const uint64_t old = e.c.id;
        if (!divide(e.c, c2)) {
          set_error(b, OR_ECALC, (int64_t)old);
          return;
        }
        v.id_counter += 1;
        e.c.id = division_id(v.plain, v.id_counter);
        e.c.parent = old;
        Entry ne;
        ne.c = c2;
        ne.c.parent = old;
        zero(ne.a.force);
        born.push_back(ne);
      }
      for (Entry &ne : born) {
        v.id_counter += 1;
        ne.c.id = division_id(v.plain, v.id_counter);
        v.cells.push_back(ne);
      }
    }
  }

  // SubDomainMechanics::apply_boundary (cartesian_cuboid_n.rs:594-631; rods:
  // bacterial_rods.rs:489-534), called from SubDomainBox::apply_boundary
  // (update_mechanics.rs:387-406).
  bool reflect(Cell &c) const {
    const double two = 1.0 + 1.0;
    // Brownian::set_velocity is a no-op, so the reflection leaves its velocity alone
    const bool keep_vel = NV == 1 && prm.kind == OR_KIND_BROWNIAN;
    for (int v = 0; v < NV; ++v) {
      double *p = c.pos + v * D;
      double *u = c.vel + v * D;
      for (int i = 0; i < D; ++i) {
        if (p[i] < dom.min[i]) {
          p[i] = (NV == 1) ? two * dom.min[i] - p[i] : dom.min[i] * two - p[i];
          if (!keep_vel) u[i] = std::fabs(u[i]);
        }
        if (p[i] > dom.max[i]) {
          p[i] = (NV == 1) ? two * dom.max[i] - p[i] : dom.max[i] * two - p[i];
          if (!keep_vel) u[i] = -std::fabs(u[i]);
        }
      }
    }
    for (int v = 0; v < NV; ++v)
      for (int i = 0; i < D; ++i)
        if (c.pos[v * D + i] < dom.min[i] || c.pos[v * D + i] > dom.max[i]) return false;
    return true;
  }

  void boundary(int s) {
    Box &b = boxes[s];
    for (Voxel &v : b.voxels)
      for (Entry &e : v.cells)
        if (!reflect(e.c)) {
          set_error(b, OR_EBOUNDARY, (int64_t)e.c.id);
          return;
        }
  }

  // Position used for voxel keys: the point itself (spheres) or the rod centroid
  // row_sum / nrows (bacterial_rods.rs:368-372, 550-554).
  static void key_point(const Cell &c, double *out) {
    if constexpr (NV == 1) {
      for (int i = 0; i < D; ++i) out[i] = c.pos[i];
    } else {
      for (int i = 0; i < D; ++i) {
        double s = 0.0;
        for (int v = 0; v < NV; ++v) s = s + c.pos[v * D + i];
        out[i] = s / (double)NV;
      }
    }
  }

  // sort_cells_in_voxels_step_1 (update_mechanics.rs:418-477).
  void sort1(int s) {
    Box &b = boxes[s];
    std::vector<std::pair<uint64_t, Entry>> movers;
    for (Voxel &v : b.voxels) {
      std::vector<Entry> stay;
      stay.reserve(v.cells.size());
      for (Entry &e : v.cells) {
        double kp[D];
        key_point(e.c, kp);
        uint64_t p;
        int r = dom.index_of(kp, p);
        if (r == 0 && p != v.plain)
          movers.emplace_back(v.plain, e);
        else
          stay.push_back(e);  // errors are collected and dropped; the cell stays
      }
      v.cells.swap(stay);
    }
    for (auto &mv : movers) {
      double kp[D];
      key_point(mv.second.c, kp);
      uint64_t p;
      if (dom.index_of(kp, p) != 0) {
        set_error(b, OR_EBOUNDARY, (int64_t)mv.second.c.id);
        return;
      }
      Voxel *tv = voxel_local(b, p);
      if (tv)
        tv->cells.push_back(mv.second);
      else
        mb_cell[s][sub_of[p]].push_back(SendCell{mv.first, mv.second});
    }
  }

  // sort_cells_in_voxels_step_2 (update_mechanics.rs:485-513), determinism = true.
  void sort2(int s) {
    Box &b = boxes[s];
    std::vector<SendCell> rec;
    for (int t = 0; t < S; ++t) {
      auto &q = mb_cell[t][s];
      rec.insert(rec.end(), q.begin(), q.end());
      q.clear();
    }
    std::stable_sort(rec.begin(), rec.end(), [](const SendCell &x, const SendCell &y) {
      return x.source < y.source;
    });
    for (SendCell &sc : rec) {
      double kp[D];
      key_point(sc.e.c, kp);
      uint64_t p;
      if (dom.index_of(kp, p) != 0) {
        set_error(b, OR_EBOUNDARY, (int64_t)sc.e.c.id);
        return;
      }
      Voxel *tv = voxel_local(b, p);
      if (!tv) {
        set_error(b, OR_EINDEX, (int64_t)sc.e.c.id);
        return;
      }
      tv->cells.push_back(sc.e);
    }
  }

  // Neighbour statistics of the visit in step 1 (debug only; single-threaded).
  void neighbor_stats(uint32_t *n_cand, uint32_t *n_inter, uint64_t *hash) {
    std::vector<Voxel *> all(dom.n_total, nullptr);
    for (Box &b : boxes)
      for (Voxel &v : b.voxels) all[v.plain] = &v;
    for (Box &b : boxes)
      for (Voxel &v : b.voxels)
        for (Entry &e : v.cells) {
          uint32_t nc = 0, ni = 0;
          uint64_t h = 0;
          auto visit = [&](Voxel &w) {
            for (Entry &o : w.cells) {
              if (&o == &e) continue;
              ++nc;
              h += mix64(o.c.id);
              if constexpr (NV == 1) {
                double f1[NC], f2[NC];
                if (morse<D>(e.c.pos, o.c.pos, prm.radius, prm.radius, prm.cutoff, prm.strength,
                             prm.stiffness, f1, f2))
                  ++ni;
              } else {
                // in-range vertex/segment evaluations of e.calc(e, o) (own perspective)
                for (int i = 0; i < NV; ++i)
                  for (int j = 0; j + 1 < NV; ++j) {
                    double q[D], t, f1[D], f2[D];
                    nearest_point<D>(e.c.pos + i * D, o.c.pos + j * D, o.c.pos + (j + 1) * D, q,
                                     t);
                    if (morse<D>(e.c.pos + i * D, q, prm.radius, prm.radius, prm.cutoff,
                                 prm.strength, prm.stiffness, f1, f2))
                      ++ni;
                  }
              }
            }
          };
          visit(v);
          for (uint64_t nb : v.nbrs) visit(*all[nb]);
          n_cand[e.c.id] = nc;
          n_inter[e.c.id] = ni;
          hash[e.c.id] = h;
        }
  }

  int setup(const or_config &cfg, int64_t n, const double *pos, const double *vel) {
    n_agents = n;
    S = cfg.n_subdomains;
    int r = subdomain_map(dom, (uint64_t)S, sub_of);
    if (r) return r;
    // Domain::decompose (concepts-derive/src/domain.rs:292-400): cells go to their
    // subdomain in input order; CartesianCuboid SortCells uses get_voxel_index_of_raw.
    std::vector<std::vector<Cell>> per_sub(S);
    for (int64_t i = 0; i < n; ++i) {
      Cell c;
      c.id = (uint64_t)i;
      std::memcpy(c.pos, pos + i * NC, sizeof(c.pos));
      std::memcpy(c.vel, vel + i * NC, sizeof(c.vel));
      c.slen = slen_in ? slen_in[i] : prm.spring_length;
      c.grate = cyc.growth;
      double kp[D];
      key_point(c, kp);
      uint64_t p;
      int rr = dom.index_of_raw(kp, p);
      if (rr == 1) return OR_EBOUNDARY;
      if (rr == 2) return OR_EINDEX;
      per_sub[sub_of[p]].push_back(c);
    }
    // construct_simulation_runner (chili/datastructures.rs:51-217) and
    // insert_initial_cells (datastructures.rs:278-299).
    boxes.resize(S);
    uint64_t p0 = 0;
    for (int s = 0; s < S; ++s) {
      Box &b = boxes[s];
      b.lo = p0;
      while (p0 < dom.n_total && sub_of[p0] == (uint32_t)s) ++p0;
      b.hi = p0;
      b.voxels.resize(b.hi - b.lo);
      for (uint64_t q = b.lo; q < b.hi; ++q) {
        Voxel &v = b.voxels[q - b.lo];
        v.plain = q;
        neighbors_of(dom, q, v.nbrs);
      }
      for (Cell &c : per_sub[s]) {
        double kp[D];
        key_point(c, kp);
        uint64_t p;
        if (dom.index_of(kp, p) != 0) return OR_EBOUNDARY;
        Voxel *v = voxel_local(b, p);
        if (!v) return OR_EBOUNDARY;
        Entry e;
        e.c = c;
        zero(e.a.force);
        v->cells.push_back(e);
        v->id_counter += 1;  // insert_initial_cells (datastructures.rs:296)
      }
    }
    mb_pos.assign(S, std::vector<std::vector<PosInfo>>(S));
    mb_force.assign(S, std::vector<std::vector<ForceInfo>>(S));
    mb_cell.assign(S, std::vector<std::vector<SendCell>>(S));
    return OR_OK;
  }

  // The macro-generated per-thread loop (core-proc-macro/src/run_sim.rs:363-403).
  void worker(int s, int64_t n_steps, std::barrier<> *bar, int64_t *err_step) {
    for (int64_t step = 1; step <= n_steps; ++step) {
      Box &b = boxes[s];
      bool last = (step == n_steps);
      if (b.error == OR_OK) step1(s);
      if (bar) bar->arrive_and_wait();
      if (b.error == OR_OK) step2(s);
      if (bar) bar->arrive_and_wait();
      if (b.error == OR_OK) step3(s);
      if (b.error == OR_OK) update_local(s, last, step_base + step - 1);
      if (b.error == OR_OK && cyc.on) cycle4(s);
      if (b.error == OR_OK) boundary(s);
      if (b.error == OR_OK) sort1(s);
      if (bar) bar->arrive_and_wait();
      if (b.error == OR_OK) sort2(s);
      if (bar) bar->arrive_and_wait();  // BarrierSync::store_error
      if (got_error.load()) {
        if (b.error != OR_OK && *err_step < 0) *err_step = step;
        break;
      }
    }
  }

  int run(int64_t n_steps, or_debug *dbg) {
    std::vector<int64_t> err_steps(S, -1);
    want_debug = dbg && dbg->force_last;
    if (want_debug) dbg_force.assign((size_t)n_agents * NC, 0.0);
    auto go = [&](int64_t steps) {
      if (steps <= 0) return;
      struct Advance {  // the random stream's step index continues across calls
        int64_t &base, n;
        ~Advance() { base += n; }
      } adv{step_base, steps};
      if (S == 1) {
        worker(0, steps, nullptr, &err_steps[0]);
      } else {
        std::barrier<> bar(S);
        std::vector<std::thread> th;
        for (int s = 0; s < S; ++s)
          th.emplace_back([&, s] { worker(s, steps, &bar, &err_steps[s]); });
        for (auto &t : th) t.join();
      }
    };
    bool stats = dbg && (dbg->n_cand || dbg->n_inter || dbg->cand_hash);
    if (stats && n_steps >= 1) {
      go(n_steps - 1);
      if (!got_error.load()) {
        std::vector<uint32_t> nc(n_agents), ni(n_agents);
        std::vector<uint64_t> h(n_agents);
        neighbor_stats(nc.data(), ni.data(), h.data());
        if (dbg->n_cand) std::memcpy(dbg->n_cand, nc.data(), sizeof(uint32_t) * n_agents);
        if (dbg->n_inter) std::memcpy(dbg->n_inter, ni.data(), sizeof(uint32_t) * n_agents);
        if (dbg->cand_hash) std::memcpy(dbg->cand_hash, h.data(), sizeof(uint64_t) * n_agents);
        go(1);
      }
    } else {
      go(n_steps);
    }
    int code = OR_OK;
    if (dbg) {
      dbg->error_agent = -1;
      dbg->error_step = -1;
    }
    for (int s = 0; s < S; ++s)
      if (boxes[s].error != OR_OK) {
        code = boxes[s].error;
        if (dbg) {
          dbg->error_agent = boxes[s].err_agent;
          dbg->error_step = err_steps[s];
        }
        break;
      }
    return code;
  }

  void export_state(double *pos, double *vel, or_debug *dbg) {
    size_t k = 0;
    for (Box &b : boxes)
      for (Voxel &v : b.voxels)
        for (Entry &e : v.cells) {
          if (dbg && dbg->order_out) dbg->order_out[k++] = e.c.id;
          std::memcpy(pos + e.c.id * NC, e.c.pos, sizeof(e.c.pos));
          std::memcpy(vel + e.c.id * NC, e.c.vel, sizeof(e.c.vel));
          if (dbg && dbg->voxel_out) dbg->voxel_out[e.c.id] = (uint32_t)v.plain;
        }
    if (dbg && dbg->force_last)
      std::memcpy(dbg->force_last, dbg_force.data(), sizeof(double) * dbg_force.size());
  }

  // Storage-order export of a cell-cycle run; false when the output arrays are too short.
  bool export_cycle(or_cycle &o) {
    int64_t n = 0;
    for (Box &b : boxes)
      for (Voxel &v : b.voxels) n += (int64_t)v.cells.size();
    o.n_out = n;
    if (n > o.cap_out) return false;
    int64_t k = 0;
    for (Box &b : boxes)
      for (Voxel &v : b.voxels)
        for (Entry &e : v.cells) {
          if (o.ids_out) o.ids_out[k] = e.c.id;
          if (o.parent_out) o.parent_out[k] = e.c.parent;
          if (o.pos_out) std::memcpy(o.pos_out + k * NC, e.c.pos, sizeof(e.c.pos));
          if (o.vel_out) std::memcpy(o.vel_out + k * NC, e.c.vel, sizeof(e.c.vel));
          if (o.spring_length_out) o.spring_length_out[k] = e.c.slen;
          if (o.growth_rate_out) o.growth_rate_out[k] = e.c.grate;
          if (o.voxel_out) o.voxel_out[k] = (uint32_t)v.plain;
          ++k;
        }
    return true;
  }
};

template <int D, int NV>
int32_t run_t(const or_config &cfg, const Domain &dom, int64_t n, double *pos, double *vel,
              int64_t n_steps, or_debug *dbg, double *elapsed) {
  auto sim = std::make_unique<Sim<D, NV>>();
  sim->dom = dom;
  sim->prm = Params{cfg.mass,      cfg.damping,   cfg.spring_tension, cfg.rigidity,
                    cfg.spring_length, cfg.radius, cfg.stiffness, cfg.cutoff,
                    cfg.strength,  cfg.dt,        cfg.solver_order, cfg.kind,
                    cfg.diffusion, cfg.kb_temperature, cfg.rng_seed};
  sim->cap = cfg.solver_order - 1;
  int r = sim->setup(cfg, n, pos, vel);
  if (r) return r;
  auto t0 = std::chrono::steady_clock::now();
  r = sim->run(n_steps, dbg);
  auto t1 = std::chrono::steady_clock::now();
  if (elapsed) *elapsed = std::chrono::duration<double>(t1 - t0).count();
  sim->export_state(pos, vel, dbg);
  return r;
}

template <int D, int NV>
int32_t run_cycle_t(const or_config &cfg, const Domain &dom, or_cycle &cy, int64_t n,
                    const double *pos, const double *vel, int64_t n_steps) {
  auto sim = std::make_unique<Sim<D, NV>>();
  sim->dom = dom;
  sim->prm = Params{cfg.mass,      cfg.damping,   cfg.spring_tension, cfg.rigidity,
                    cfg.spring_length, cfg.radius, cfg.stiffness, cfg.cutoff,
                    cfg.strength,  cfg.dt,        cfg.solver_order, cfg.kind,
                    cfg.diffusion, cfg.kb_temperature, cfg.rng_seed};
  sim->cap = cfg.solver_order - 1;
  sim->cyc.on = true;
  sim->cyc.growth = cy.growth_rate;
  sim->cyc.div_len = cy.division_length;
  sim->cyc.sense = cy.sense_range;
  sim->cyc.sat = cy.sense_saturation;
  sim->slen_in = cy.spring_length_in;
  int r = sim->setup(cfg, n, pos, vel);
  if (r) return r;
  or_debug dbg;
  std::memset(&dbg, 0, sizeof(dbg));
  r = sim->run(n_steps, &dbg);
  cy.error_agent = dbg.error_agent;
  cy.error_step = dbg.error_step;
  if (!sim->export_cycle(cy) && r == OR_OK) r = OR_EINVAL;
  return r;
}

}  // namespace oracle_impl

using namespace oracle_impl;

int32_t oracle_cycle_rods2(const or_config &cfg, const Domain &dom, or_cycle &cy, int64_t n,
                           const double *pos, const double *vel, int64_t n_steps);
int32_t oracle_cycle_rods3(const or_config &cfg, const Domain &dom, or_cycle &cy, int64_t n,
                           const double *pos, const double *vel, int64_t n_steps);

#define ORACLE_CYCLE_DEF(NAME, D)                                                         \
  int32_t NAME(const or_config &cfg, const Domain &dom, or_cycle &cy, int64_t n,           \
               const double *pos, const double *vel, int64_t n_steps) {                   \
    switch (cfg.n_vertices) {                                                             \
      case 2: return run_cycle_t<D, 2>(cfg, dom, cy, n, pos, vel, n_steps);               \
      case 3: return run_cycle_t<D, 3>(cfg, dom, cy, n, pos, vel, n_steps);               \
      case 4: return run_cycle_t<D, 4>(cfg, dom, cy, n, pos, vel, n_steps);               \
      case 5: return run_cycle_t<D, 5>(cfg, dom, cy, n, pos, vel, n_steps);               \
      case 6: return run_cycle_t<D, 6>(cfg, dom, cy, n, pos, vel, n_steps);               \
      case 7: return run_cycle_t<D, 7>(cfg, dom, cy, n, pos, vel, n_steps);               \
      case 8: return run_cycle_t<D, 8>(cfg, dom, cy, n, pos, vel, n_steps);               \
      default: return OR_EINVAL;                                                          \
    }                                                                                     \
  }

// The rod instantiations are compiled in separate units (ORACLE_PART 2 and 3) so the
// oracle builds in parallel.
int32_t oracle_run_rods2(const or_config &cfg, const Domain &dom, int64_t n, double *pos,
                         double *vel, int64_t n_steps, or_debug *dbg, double *elapsed);
int32_t oracle_run_rods3(const or_config &cfg, const Domain &dom, int64_t n, double *pos,
                         double *vel, int64_t n_steps, or_debug *dbg, double *elapsed);

#define ORACLE_RODS_DEF(NAME, D)                                                          \
  int32_t NAME(const or_config &cfg, const Domain &dom, int64_t n, double *pos,           \
               double *vel, int64_t n_steps, or_debug *dbg, double *elapsed) {            \
    switch (cfg.n_vertices) {                                                             \
      case 2: return run_t<D, 2>(cfg, dom, n, pos, vel, n_steps, dbg, elapsed);           \
      case 3: return run_t<D, 3>(cfg, dom, n, pos, vel, n_steps, dbg, elapsed);           \
      case 4: return run_t<D, 4>(cfg, dom, n, pos, vel, n_steps, dbg, elapsed);           \
      case 5: return run_t<D, 5>(cfg, dom, n, pos, vel, n_steps, dbg, elapsed);           \
      case 6: return run_t<D, 6>(cfg, dom, n, pos, vel, n_steps, dbg, elapsed);           \
      case 7: return run_t<D, 7>(cfg, dom, n, pos, vel, n_steps, dbg, elapsed);           \
      case 8: return run_t<D, 8>(cfg, dom, n, pos, vel, n_steps, dbg, elapsed);           \
      default: return OR_EINVAL;                                                          \
    }                                                                                     \
  }

#if ORACLE_PART == 2 || ORACLE_PART == -1
ORACLE_RODS_DEF(oracle_run_rods2, 2)
ORACLE_CYCLE_DEF(oracle_cycle_rods2, 2)
#endif
#if ORACLE_PART == 3 || ORACLE_PART == -1
ORACLE_RODS_DEF(oracle_run_rods3, 3)
ORACLE_CYCLE_DEF(oracle_cycle_rods3, 3)
#endif

#if ORACLE_PART == 0 || ORACLE_PART == -1

extern "C" {

int32_t or_run(const or_config *cfg, int64_t n_agents, double *pos, double *vel,
               int64_t n_steps, or_debug *dbg, double *elapsed_s) {
  if (!cfg || n_agents < 0 || n_steps < 0) return OR_EINVAL;
  if (cfg->solver_order < 1 || cfg->solver_order > 3) return OR_EINVAL;
  if (cfg->n_subdomains < 1) return OR_EINVAL;
  if ((cfg->kind == OR_KIND_BROWNIAN && !(cfg->kb_temperature != 0.0)) ||
      (cfg->kind == OR_KIND_SPHERE && cfg->diffusion != 0.0))
    return OR_EINVAL;
  Domain dom;
  int r = make_domain(*cfg, dom);
  if (r) return r;
  if (cfg->kind == OR_KIND_SPHERE || cfg->kind == OR_KIND_BROWNIAN ||
      cfg->kind == OR_KIND_LANGEVIN) {
    if (cfg->dim == 2) return run_t<2, 1>(*cfg, dom, n_agents, pos, vel, n_steps, dbg, elapsed_s);
    return run_t<3, 1>(*cfg, dom, n_agents, pos, vel, n_steps, dbg, elapsed_s);
  }
  if (cfg->kind == OR_KIND_ROD) {
    if (cfg->dim == 2) return oracle_run_rods2(*cfg, dom, n_agents, pos, vel, n_steps, dbg, elapsed_s);
    return oracle_run_rods3(*cfg, dom, n_agents, pos, vel, n_steps, dbg, elapsed_s);
  }
  return OR_EINVAL;
}

int32_t or_run_cycle(const or_config *cfg, or_cycle *cyc, int64_t n_agents,
                     const double *pos, const double *vel, int64_t n_steps) {
  if (!cfg || !cyc || n_agents < 0 || n_steps < 0 || (n_agents > 0 && (!pos || !vel)))
    return OR_EINVAL;
  if (cfg->kind != OR_KIND_ROD || cfg->solver_order < 1 || cfg->solver_order > 3 ||
      cfg->n_subdomains < 1 || !(cyc->sense_saturation != 0.0))
    return OR_EINVAL;
  cyc->n_out = 0;
  cyc->error_agent = cyc->error_step = -1;
  Domain dom;
  int r = make_domain(*cfg, dom);
  if (r) return r;
  if (cfg->dim == 2) return oracle_cycle_rods2(*cfg, dom, *cyc, n_agents, pos, vel, n_steps);
  return oracle_cycle_rods3(*cfg, dom, *cyc, n_agents, pos, vel, n_steps);
}

void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  philox4x32_10(ctr, key, out);
}

void or_normals(uint64_t seed, uint64_t step, uint64_t id, int32_t n, double *out) {
  normals(seed, step, id, n, out);
}

int32_t or_domain_voxels(const or_config *cfg, int64_t *n_voxels_out, double *dx_out) {
  Domain dom;
  int r = make_domain(*cfg, dom);
  if (r) return r;
  for (int i = 0; i < cfg->dim; ++i) {
    n_voxels_out[i] = (int64_t)dom.nvox[i];
    dx_out[i] = dom.dx[i];
  }
  return OR_OK;
}

int32_t or_get_decomp_res(uint64_t n_voxel, uint64_t n_regions, uint64_t *n, uint64_t *m,
                          uint64_t *average_len) {
  return get_decomp_res(n_voxel, n_regions, *n, *m, *average_len) ? OR_OK : OR_EDECOMPOSE;
}

int32_t or_subdomain_map(const or_config *cfg, uint32_t *out) {
  Domain dom;
  int r = make_domain(*cfg, dom);
  if (r) return r;
  std::vector<uint32_t> map;
  r = subdomain_map(dom, (uint64_t)cfg->n_subdomains, map);
  if (r) return r;
  std::memcpy(out, map.data(), sizeof(uint32_t) * map.size());
  return OR_OK;
}

int32_t or_voxel_neighbors(const or_config *cfg, uint64_t plain, uint64_t *out) {
  Domain dom;
  int r = make_domain(*cfg, dom);
  if (r) return -r;
  if (plain >= dom.n_total) return -OR_EINDEX;
  std::vector<uint64_t> nb;
  neighbors_of(dom, plain, nb);
  std::memcpy(out, nb.data(), sizeof(uint64_t) * nb.size());
  return (int32_t)nb.size();
}

int32_t or_initial_voxels(const or_config *cfg, int64_t n_agents, const double *pos,
                          uint32_t *out) {
  Domain dom;
  int r = make_domain(*cfg, dom);
  if (r) return r;
  int nv = cfg->kind == OR_KIND_ROD ? cfg->n_vertices : 1;
  int D = cfg->dim;
  for (int64_t i = 0; i < n_agents; ++i) {
    double kp[3];
    for (int c = 0; c < D; ++c) {
      double s = 0.0;
      if (nv == 1) {
        s = pos[i * D + c];
      } else {
        for (int v = 0; v < nv; ++v) s = s + pos[(i * nv + v) * D + c];
        s = s / (double)nv;
      }
      kp[c] = s;
    }
    uint64_t p;
    int rr = dom.index_of_raw(kp, p);
    if (rr == 1) return OR_EBOUNDARY;
    if (rr == 2) return OR_EINDEX;
    out[i] = (uint32_t)p;
  }
  return OR_OK;
}

void or_nearest_point_from_point_to_line(int32_t dim, const double *point, const double *a,
                                         const double *b, double *dist, double *nearest,
                                         double *rel_length) {
  if (dim == 2)
    *dist = nearest_point<2>(point, a, b, nearest, *rel_length);
  else
    *dist = nearest_point<3>(point, a, b, nearest, *rel_length);
}

int32_t or_morse(int32_t dim, const double *own, const double *ext, double own_radius,
                 double ext_radius, double cutoff, double strength, double stiffness,
                 double *f_own, double *f_ext) {
  if (dim == 2)
    return morse<2>(own, ext, own_radius, ext_radius, cutoff, strength, stiffness, f_own, f_ext);
  return morse<3>(own, ext, own_radius, ext_radius, cutoff, strength, stiffness, f_own, f_ext);
}

// solvers.rs:303-310
double or_euler(double x, double dx, double dt, double dx_rand) {
  return (dx * dt + x) * 1.0 + dx_rand * dt;
}
// solvers.rs:332-347
double or_adams_bashforth_2(double x, double dx0, double dx1, double dt, double dx_rand) {
  const double f0 = 3.0 / 2.0, f1 = -1.0 / 2.0;
  return ((dx0 * f0 + dx1 * f1) * dt + x) * 1.0 + dx_rand * dt;
}
// solvers.rs:313-329
double or_adams_bashforth_3(double x, double dx0, double dx1, double dx2, double dt,
                            double dx_rand) {
  const double f0 = 23.0 / 12.0, f1 = -16.0 / 12.0, f2 = 5.0 / 12.0;
  return ((dx0 * f0 + (dx1 * f1 + dx2 * f2)) * dt + x) * 1.0 + dx_rand * dt;
}

}  // extern "C"
#endif  // ORACLE_PART == 0
