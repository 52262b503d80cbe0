// crg_sort.cu -- device cell list: voxel keys, counting sort and state gather.
//
// Replaces chili's per-voxel Vec storage and its re-sort
// (cellular_raza-core/src/backend/chili/update_mechanics.rs:418-513) with one global
// counting sort per step.  The order inside a voxel reproduces chili's exactly:
//   class 0: agents that stayed (drain+partition keeps their order, :431-455),
//   class 1: movers from a voxel of the same subdomain, pushed in source order (:459-466),
//   class 2: movers from another subdomain, received and sorted by source voxel (:496-498),
// and inside each class by the previous cell-list position, which is the previous
// (voxel, position-in-voxel) order.  Slots are taken with atomics and then each voxel's
// segment is sorted by (class, previous position), so the result is deterministic.
#include "crg_internal.cuh"
#include "crg_kernels.h"

namespace crg {

namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t x) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  return x;
}

// Block-wide exclusive scan of one value per thread; returns the exclusive prefix and
// writes the block total to *total.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t x, uint32_t *total) {
  __shared__ uint32_t warp_tot[32];
  __shared__ uint32_t block_tot;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = (blockDim.x + 31) >> 5;
  uint32_t incl = warp_incl_scan(x);
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t t = (lane < nwarps) ? warp_tot[lane] : 0u;
    uint32_t ti = warp_incl_scan(t);
    if (lane < nwarps) warp_tot[lane] = ti - t;  // exclusive prefix of each warp
    if (lane == 31) block_tot = ti;              // total (nwarps <= 32)
  }
  __syncthreads();
  uint32_t res = warp_tot[warp] + incl - x;
  *total = block_tot;
  __syncthreads();
  return res;
}

// Voxel range [lo, hi) of the simulation whose current step failed (failed_sim), empty if
// none or if `status` is null (scans that are not a cell-list re-sort).  Its agents keep
// their voxels, so its histogram entries are the voxel sizes of the current cell list.
struct FailedRange {
  uint32_t lo = 0, hi = 0;
  __device__ FailedRange(const int32_t *status, const SimDev *sims) {
    const int32_t f = status ? failed_sim(status) : -1;
    if (f >= 0) {
      lo = sims[f].voxel_off;
      hi = lo + sims[f].n_vox;
    }
  }
  __device__ bool has(uint32_t v) const { return v - lo < hi - lo; }
};

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(uint32_t *__restrict__ count,
                                                              uint32_t n, uint32_t *bsum,
                                                              const int32_t *status,
                                                              const SimDev *sims,
                                                              const uint32_t *old_start) {
  const FailedRange fr(status, sims);
  const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k)
    if (base + k < n) {
      uint32_t c = count[base + k];
      if (fr.has(base + k)) {  // k_scan_final reads the corrected entry
        c = old_start[base + k + 1] - old_start[base + k];
        count[base + k] = c;
      }
      s += c;
    }
  uint32_t tot;
  block_excl_scan(s, &tot);
  if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

// Single block: exclusive scan of the block sums in place; grand total -> start[n].
__global__ void __launch_bounds__(kScanThreads) k_scan_blocks(uint32_t *bsum, uint32_t nb,
                                                              uint32_t *start, uint32_t n) {
  uint32_t carry = 0;
  for (uint32_t b0 = 0; b0 < nb; b0 += kScanThreads) {
    uint32_t j = b0 + threadIdx.x;
    uint32_t x = (j < nb) ? bsum[j] : 0u;
    uint32_t tot;
    uint32_t ex = block_excl_scan(x, &tot);
    if (j < nb) bsum[j] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0) start[n] = carry;
}

// Final pass: start[j] = exclusive prefix; count[j] = 0 (reused as the scatter cursor).
__global__ void __launch_bounds__(kScanThreads) k_scan_final(uint32_t *__restrict__ count,
                                                             uint32_t n,
                                                             const uint32_t *__restrict__ bsum,
                                                             uint32_t *__restrict__ start) {
  const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = (base + k < n) ? count[base + k] : 0u;
    s += v[k];
  }
  uint32_t tot;
  uint32_t ex = block_excl_scan(s, &tot) + bsum[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) {
      start[base + k] = ex;
      count[base + k] = 0u;
    }
    ex += v[k];
  }
}

// Whole scan in one block when the voxels fit one tile (small packs): start[j] = exclusive
// prefix, count[j] = 0, start[n] = total.
// The voxel sizes of a failed simulation are read from `start` before the first barrier of
// the scan, and start is written after it.
__global__ void __launch_bounds__(kScanThreads) k_scan_single(uint32_t *__restrict__ count,
                                                              uint32_t n, uint32_t *start,
                                                              const int32_t *status,
                                                              const SimDev *sims) {
  const FailedRange fr(status, sims);
  const uint32_t base = threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = (base + k < n) ? count[base + k] : 0u;
    if (base + k < n && fr.has(base + k)) v[k] = start[base + k + 1] - start[base + k];
    s += v[k];
  }
  uint32_t tot;
  uint32_t ex = block_excl_scan(s, &tot);
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) {
      start[base + k] = ex;
      count[base + k] = 0u;
    }
    ex += v[k];
  }
  if (threadIdx.x == 0) start[n] = tot;
}

// Slot assignment.  Sort key = class << 62 | rank << 31 | index, where the rank is the
// agent's previous position (with divisions: its position in chili's pre-sort order, the
// daughters of a voxel following its other agents) and the index locates its state.
// The agents of a simulation whose step failed keep their voxel and their place (class 0,
// rank = current position), so their slots are their current positions.
__global__ void k_scatter(const SortArgs A) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.n_agents) return;
  const int32_t f = A.initial ? -1 : failed_sim(A.status);
  const bool keep = f >= 0 && i - A.sims[f].agent_off < A.sims[f].n_agents;
  uint32_t k = A.nkey[i];
  if (keep) {
    k = A.key[i];
    A.nkey[i] = k;
  }
  uint32_t cls = 0;
  if (!A.initial && !keep) {
    const uint32_t old = A.key[i];
    if (k != old) {
      const uint32_t s = (A.n_sims == 1) ? 0u : A.sim_of_voxel ? A.sim_of_voxel[k] : 0u;
      const SimDev &S = A.sims[s];
      cls = (subdomain_of(S, k - S.voxel_off) == subdomain_of(S, old - S.voxel_off)) ? 1u : 2u;
    }
  }
  if (k >= A.n_vox) {
    invariant_failed(A.status, kSiteScatterKey, i);
    return;
  }
  const uint32_t slot = A.start[k] + atomicAdd(&A.count[k], 1u);
  if (slot >= A.n_agents) {
    invariant_failed(A.status, kSiteScatterSlot, i);
    return;
  }
  const uint32_t rank = (A.srank && !keep) ? A.srank[i] : i;
  A.tmp[slot] = ((uint64_t)cls << 62) | ((uint64_t)rank << 31) | (uint64_t)i;
}

constexpr int kSegThreads = 256;  // voxels per block of k_segsort
constexpr uint32_t kSegShort = 32;    // segments up to this length: one thread, insertion sort
constexpr uint32_t kSegSmem = 2048;   // longer ones up to this length: in shared memory

// Sorts t[0..m) ascending in place with all threads of the block (every thread calls it).
// A bitonic network over the next power of two p >= m in the form whose compare-exchanges
// all put the smaller key first: per merge size k, each element of the first half of a run
// of k against its mirror in the second half, then half-cleaners at distances k/4 .. 1.
// Positions m..p-1 stand for +infinity: a real key only ever moves to a lower position by a
// swap with a larger one, so it never reaches them, and pairs that touch them never swap.
// O(m log^2 m) work, (log2 p)(log2 p + 1)/2 barriers.  Keys are distinct (they hold the
// agent index).
__device__ void block_bitonic(uint64_t *t, uint32_t m) {
  uint32_t p = 1;
  while (p < m) p <<= 1;
  for (uint32_t k = 2; k <= p; k <<= 1) {
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t x = threadIdx.x; x < (p >> 1); x += blockDim.x) {
        const uint32_t blk = x / j, off = x - blk * j;
        uint32_t a, b;
        if (j == (k >> 1)) {  // mirror stage of a merge of two runs of k / 2
          a = blk * k + off;
          b = blk * k + k - 1 - off;
        } else {  // half-cleaner over blocks of 2 j
          a = blk * 2 * j + off;
          b = a + j;
        }
        if (b < m) {
          const uint64_t ta = t[a], tb = t[b];
          if (tb < ta) {
            t[a] = tb;
            t[b] = ta;
          }
        }
      }
      __syncthreads();
    }
  }
}

// One thread per voxel: order the voxel's segment of slot keys and reset its histogram
// counter.  Segments hold ~2 agents in the configured workloads and are insertion-sorted by
// their thread; a longer one (a coarse grid, a dense cluster) goes to a list in shared
// memory and is sorted by the whole block afterwards, in shared memory up to kSegSmem
// entries and in place in global memory beyond, so a voxel with 2^20 agents costs
// O(m log^2 m) rather than O(m^2).
__global__ void __launch_bounds__(kSegThreads) k_segsort(const SortArgs A) {
  __shared__ uint32_t sLong[kSegThreads];
  __shared__ uint32_t nLong;
  __shared__ uint64_t sBuf[kSegSmem];
  if (threadIdx.x == 0) nLong = 0;
  __syncthreads();
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < A.n_vox) {
    const uint32_t s0 = A.start[v], s1 = A.start[v + 1];
    A.count[v] = 0u;
    if (s0 > s1 || s1 > A.n_agents) {
      invariant_failed(A.status, kSiteSegRange, v);
    } else if (s1 - s0 > kSegShort) {
      sLong[atomicAdd(&nLong, 1u)] = v;
    } else if (s1 - s0 >= 2) {
      uint64_t *t = A.tmp;
      for (uint32_t a = s0 + 1; a < s1; ++a) {
        uint64_t x = t[a];
        uint32_t b = a;
        while (b > s0 && t[b - 1] > x) {
          t[b] = t[b - 1];
          --b;
        }
        t[b] = x;
      }
    }
  }
  __syncthreads();
  const uint32_t n_long = nLong;
  for (uint32_t q = 0; q < n_long; ++q) {
    const uint32_t w = sLong[q];
    const uint32_t s0 = A.start[w], m = A.start[w + 1] - s0;  // checked above
    if (m <= kSegSmem) {
      for (uint32_t x = threadIdx.x; x < m; x += blockDim.x) sBuf[x] = A.tmp[s0 + x];
      __syncthreads();
      block_bitonic(sBuf, m);
      for (uint32_t x = threadIdx.x; x < m; x += blockDim.x) A.tmp[s0 + x] = sBuf[x];
      __syncthreads();
    } else {
      block_bitonic(A.tmp + s0, m);
    }
  }
}

// One thread per slot: move the updated state into cell-list order and refresh the FP32
// offsets from the voxel corner.
__global__ void k_gather(const SortArgs A) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s == 0 && A.step_ctr) {
    *A.step_ctr += 1;
    // the failed simulation as the next step's force kernels see it (sim_frozen)
    const int32_t code = A.status[0];
    A.status[6] = code == 0 ? 0 : code == CRG_EINTERNAL ? -1 : A.status[4] + 1;
  }
  if (s >= A.n_agents) return;
  // a simulation whose step failed keeps its current state (its slots are its positions)
  const int32_t f = A.initial ? -1 : failed_sim(A.status);
  if (f >= 0 && s - A.sims[f].agent_off < A.sims[f].n_agents) return;
  uint32_t src = (uint32_t)(A.tmp[s] & 0x7fffffffull);
  if (src >= A.n_agents) {
    invariant_failed(A.status, kSiteGatherSrc, s);
    src = s;
  }
  // Loads before stores: the state arrays never overlap, but nothing tells the compiler,
  // so a load written after a store waits for the store's order.  The key, id and the first
  // four components are read together (one memory round trip for a sphere, not one per
  // component), the rest four at a time below.
  const int nc = A.nc;
  const int64_t cap = A.cap;
  uint32_t k = A.nkey[src];
  const uint64_t idv = A.nid[src];
  double gp[4], gv[4];
#pragma unroll
  for (int q = 0; q < 4; ++q)
    if (q < nc) {
      gp[q] = A.npos[q * cap + src];
      gv[q] = A.nvel[q * cap + src];
    }
  if (k >= A.n_vox) {
    invariant_failed(A.status, kSiteGatherKey, s);
    k = 0;
  }
  A.key[s] = k;
  A.id[s] = idv;
  const uint32_t sim = (A.n_sims == 1) ? 0u : A.sim_of_voxel[k];
  const SimDev &S = A.sims[sim];
  int idx[3] = {0, 0, 0};
  {
    uint32_t v = k - S.voxel_off;
    for (int i = S.dim - 1; i >= 0; --i) {
      idx[i] = (int)(v % (uint32_t)S.nvox[i]);
      v /= (uint32_t)S.nvox[i];
    }
  }
  const int dim = S.dim;
  // voxel_centre of the agent's voxel per axis, tabled (named, not an array: the axis of a
  // component is only known at run time)
  const double cen0 = A.vcen[S.cen_off[0] + idx[0]];
  const double cen1 = A.vcen[S.cen_off[1] + idx[1]];
  const double cen2 = dim == 3 ? A.vcen[S.cen_off[2] + idx[2]] : 0.0;
  float ov[3] = {0.f, 0.f, 0.f};  // spheres: written together, interleaved
  for (int c0 = 0; c0 < nc; c0 += 4) {
    if (c0 > 0) {
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (c0 + q < nc) {
          gp[q] = A.npos[(c0 + q) * cap + src];
          gv[q] = A.nvel[(c0 + q) * cap + src];
        }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int c = c0 + q;
      if (c >= nc) break;
      A.pos[c * cap + s] = gp[q];
      A.vel[c * cap + s] = gv[q];
      const int axis = c % dim;
      float o = (float)(gp[q] - (axis == 0 ? cen0 : axis == 1 ? cen1 : cen2));
      // Offsets far outside the voxel (an agent kept in its old voxel because its new
      // index fell outside the grid) would weaken the prefilter's error bound: mark them
      // NaN so every comparison involving them falls through to the exact FP64 path.
      if (!(fabsf(o) <= S.off_lim)) o = __int_as_float(0x7fc00000);
      if (A.off_aos) {
        if (c == 0) ov[0] = o;
        else if (c == 1) ov[1] = o;
        else ov[2] = o;
      } else {
        A.off[c * cap + s] = o;
      }
    }
  }
  if (A.off_aos == 4)
    reinterpret_cast<float4 *>(A.off)[s] = make_float4(ov[0], ov[1], ov[2], 0.f);
  else if (A.off_aos == 2)
    reinterpret_cast<float2 *>(A.off)[s] = make_float2(ov[0], ov[1]);
  if (A.hist) {
    for (int c = 0; c < 2 * nc; ++c) A.hist[c * cap + s] = A.nhist[c * cap + src];
    A.hmeta[s] = A.nhmeta[src];
  }
  if (A.slen) {
    A.slen[s] = A.nslen[src];
    A.grate[s] = A.ngrate[src];
    A.parent[s] = A.nparent[src];
  }
}

// Initial voxel keys from the caller's agents (input order), as Domain::decompose does it
// with CartesianCuboid::get_voxel_index_of_raw (cartesian_cuboid_n.rs:320-337): a key
// point with pos[i] <= min[i] is a BoundaryError; an index outside the grid is an
// IndexError ("could not find voxel index", concepts-derive/src/domain.rs:367-373).
// Rods use the centroid row_sum / nrows (bacterial_rods.rs:368-372).
__global__ void k_init_keys(const SortArgs A, int nv) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.n_agents) return;
  uint32_t sim = 0;
  if (A.n_sims > 1) {
    int lo = 0, hi = A.n_sims;
    while (hi - lo > 1) {
      int mid = (lo + hi) >> 1;
      if (A.sim_agent_off[mid] <= i) lo = mid; else hi = mid;
    }
    sim = (uint32_t)lo;
  }
  const SimDev &S = A.sims[sim];
  const int dim = S.dim;
  const int64_t cap = A.cap;
  double kp[3];
  for (int a = 0; a < dim; ++a) {
    double s = 0.0;
    if (nv == 1) {
      s = A.npos[a * cap + i];
    } else {
      for (int v = 0; v < nv; ++v) s = dadd(s, A.npos[(v * dim + a) * cap + i]);
      s = ddiv(s, (double)nv);
    }
    kp[a] = s;
  }
  int bad = 0;
  for (int a = 0; a < dim; ++a)
    if (S.min[a] >= kp[a]) bad = 1;
  uint32_t plain = 0;
  if (!bad) {
    int r = (dim == 3) ? voxel_of<3>(S, kp, plain) : voxel_of<2>(S, kp, plain);
    if (r == 1) bad = 1;
    if (r == 2) bad = 2;
  }
  if (bad) {
    set_status(A.status, bad == 1 ? CRG_EBOUNDARY : CRG_EINDEX, A.nid[i], 0);
    plain = 0;
  }
  const uint32_t k = S.voxel_off + plain;
  A.nkey[i] = k;
  atomicAdd(&A.count[k], 1u);
}

// Kept simulations of a repack: state copied in cell-list order, keys shifted to the new
// voxel offsets, histogram counted (the insertion sort that follows keeps this order).
__global__ void k_repack(const RepackArgs A) {
  const uint32_t j = A.first + blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= A.last) return;
  int lo = 0, hi = A.n_keep;  // dst_off[lo] <= j < dst_off[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (A.dst_off[mid] <= j) lo = mid; else hi = mid;
  }
  const uint32_t s = A.src_off[lo] + (j - A.dst_off[lo]);
  for (int c = 0; c < A.nc; ++c) {
    A.dpos[c * A.dcap + j] = A.spos[c * A.scap + s];
    A.dvel[c * A.dcap + j] = A.svel[c * A.scap + s];
  }
  if (A.has_hist) {
    for (int c = 0; c < 2 * A.nc; ++c) A.dhist[c * A.dcap + j] = A.shist[c * A.scap + s];
    A.dhmeta[j] = A.shmeta[s];
  }
  A.did[j] = A.sid[s];
  const uint32_t k = (uint32_t)((int64_t)A.skey[s] + A.key_shift[lo]);
  A.dkey[j] = k;
  atomicAdd(&A.dcount[k], 1u);
}

// Agent-major host layout [n][nc] -> component-major device layout [nc][cap].
__global__ void k_transpose_in(const double *__restrict__ src, double *__restrict__ dst,
                               uint32_t n, int nc, int64_t cap) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int c = 0; c < nc; ++c) dst[c * cap + i] = src[(int64_t)i * nc + c];
}

__global__ void k_transpose_out(const double *__restrict__ src, double *__restrict__ dst,
                                uint32_t n, int nc, int64_t cap) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int c = 0; c < nc; ++c) dst[(int64_t)i * nc + c] = src[c * cap + i];
}

// Per-agent values of the cell list ([nc][cap], slot s) back to the agent-major layout and
// the order of the arrays the cell list was built from: row = the index field of the slot key
// the insertion sort left in tmp.
__global__ void k_unsort_out(const double *__restrict__ src, const uint64_t *__restrict__ tmp,
                             double *__restrict__ dst, uint32_t n, int nc, int64_t cap,
                             int32_t *status) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const uint32_t row = (uint32_t)(tmp[s] & 0x7fffffffull);
  if (row >= n) {
    invariant_failed(status, kSiteGatherSrc, s);
    return;
  }
  for (int c = 0; c < nc; ++c) dst[(int64_t)row * nc + c] = src[c * cap + s];
}

}  // namespace

static inline unsigned grid_for(uint64_t n, unsigned block) {
  return (unsigned)((n + block - 1) / block);
}

// status / sims non-null: a cell-list re-sort, which takes the voxel sizes of a simulation
// whose step failed from the current cell list (k_scan_reduce, k_scan_single).
static void scan_impl(uint32_t *count, uint32_t n, uint32_t *start, uint32_t *bsum,
                      const int32_t *status, const SimDev *sims, cudaStream_t st) {
  const uint32_t nb = (n + kScanTile - 1) / kScanTile;
  if (nb <= 1) {
    k_scan_single<<<1, kScanThreads, 0, st>>>(count, n, start, status, sims);
  } else {
    k_scan_reduce<<<nb, kScanThreads, 0, st>>>(count, n, bsum, status, sims, start);
    k_scan_blocks<<<1, kScanThreads, 0, st>>>(bsum, nb, start, n);
    k_scan_final<<<nb, kScanThreads, 0, st>>>(count, n, bsum, start);
  }
}

void launch_scan(uint32_t *count, uint32_t n, uint32_t *start, uint32_t *bsum,
                 cudaStream_t st) {
  scan_impl(count, n, start, bsum, nullptr, nullptr, st);
}

void launch_sort(const SortArgs &A, uint32_t *bsum, cudaStream_t st) {
  scan_impl(A.count, A.n_vox, A.start, bsum, A.initial ? nullptr : A.status, A.sims, st);
  if (A.n_agents) k_scatter<<<grid_for(A.n_agents, 256), 256, 0, st>>>(A);
  k_segsort<<<grid_for(A.n_vox, kSegThreads), kSegThreads, 0, st>>>(A);
  if (A.n_agents) k_gather<<<grid_for(A.n_agents, 256), 256, 0, st>>>(A);
}

int sort_kernel_count(uint32_t n_vox) { return n_vox <= (uint32_t)kScanTile ? 4 : 6; }

void launch_repack(const RepackArgs &A, cudaStream_t st) {
  if (A.last > A.first) k_repack<<<grid_for(A.last - A.first, 256), 256, 0, st>>>(A);
}

void launch_init_keys(const SortArgs &A, int nv, cudaStream_t st) {
  if (A.n_agents) k_init_keys<<<grid_for(A.n_agents, 256), 256, 0, st>>>(A, nv);
}

void launch_transpose_in(const double *src, double *dst, uint32_t n, int nc, int64_t cap,
                         cudaStream_t st) {
  if (n) k_transpose_in<<<grid_for(n, 256), 256, 0, st>>>(src, dst, n, nc, cap);
}

void launch_transpose_out(const double *src, double *dst, uint32_t n, int nc, int64_t cap,
                          cudaStream_t st) {
  if (n) k_transpose_out<<<grid_for(n, 256), 256, 0, st>>>(src, dst, n, nc, cap);
}

void launch_unsort_out(const double *src, const uint64_t *tmp, double *dst, uint32_t n, int nc,
                       int64_t cap, int32_t *status, cudaStream_t st) {
  if (n) k_unsort_out<<<grid_for(n, 256), 256, 0, st>>>(src, tmp, dst, n, nc, cap, status);
}

}  // namespace crg

// ---------------------------------------------------------------------------------------
// crg_cell_list_noalloc: the cell list of caller-owned device points without allocating.
//
// The scratch the counting sort needs (voxel histogram, scan block sums, slot keys, status
// word) lives in one fixed device array compiled into the library.  Host code cannot use
// the array's name as a device address (in host code the name refers to a host-side
// shadow), so the device address is looked up once per device with cudaGetSymbolAddress
// and handed to the kernels.
// ---------------------------------------------------------------------------------------
#include <mutex>

namespace {

constexpr uint32_t kNaMaxPoints = CRG_NOALLOC_MAX_POINTS;
constexpr uint32_t kNaMaxVoxels = CRG_NOALLOC_MAX_VOXELS;
constexpr size_t kNaAlign = 256;
constexpr size_t na_round(size_t b) { return (b + kNaAlign - 1) / kNaAlign * kNaAlign; }
constexpr size_t kNaCountOff = 0;
constexpr size_t kNaCountBytes = na_round(sizeof(uint32_t) * ((size_t)kNaMaxVoxels + 1));
constexpr size_t kNaBsumOff = kNaCountOff + kNaCountBytes;
constexpr size_t kNaBsumBytes = na_round(sizeof(uint32_t) * ((size_t)kNaMaxVoxels / 4096 + 2));
constexpr size_t kNaTmpOff = kNaBsumOff + kNaBsumBytes;
constexpr size_t kNaTmpBytes = na_round(sizeof(uint64_t) * (size_t)kNaMaxPoints);
constexpr size_t kNaStatusOff = kNaTmpOff + kNaTmpBytes;
constexpr size_t kNaBytes = kNaStatusOff + na_round(sizeof(int32_t) * 4);  // 12,584,704 B

// Shared by every call on a device; keeps the previous call's contents.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

constexpr int kNaMaxDevices = 64;
std::mutex g_noalloc_mutex;
void *g_noalloc_ptr[kNaMaxDevices] = {};

// Voxel index of every point with crg_upload's insertion rules; histogram into count.
template <int D>
__global__ void k_noalloc_keys(const crg::SimDev S, uint32_t n, const double *__restrict__ pos,
                               uint32_t *__restrict__ voxel, uint32_t *count, int32_t *status) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double p[D];
  int bad = 0;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    p[a] = pos[(size_t)a * n + i];
    if (S.min[a] >= p[a]) bad = 1;
  }
  uint32_t plain = 0;
  if (!bad) {
    const int r = crg::voxel_of<D>(S, p, plain);
    if (r == 1) bad = 1;
    if (r == 2) bad = 2;
  }
  if (bad) {
    atomicCAS(&status[0], 0, bad == 1 ? CRG_EBOUNDARY : CRG_EINDEX);  // first error wins
    plain = 0;
  }
  voxel[i] = plain;
  atomicAdd(&count[plain], 1u);
}

__global__ void k_noalloc_order(const uint64_t *__restrict__ tmp, uint32_t n,
                                uint32_t *__restrict__ order) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) order[s] = (uint32_t)(tmp[s] & 0x7fffffffull);  // the index field of the sort key
}

}  // namespace

extern "C" int32_t crg_cell_list_noalloc(const crg_domain *d, int64_t n, const double *pos_dev,
                                         uint32_t *voxel_out, uint32_t *order_out,
                                         uint32_t *start_out, void *stream) {
  if (!d || n < 0 || n > (int64_t)kNaMaxPoints || !start_out) return CRG_EINVAL;
  if (n > 0 && (!pos_dev || !voxel_out || !order_out)) return CRG_EINVAL;
  if (d->dim != 2 && d->dim != 3) return CRG_EINVAL;
  // Grid of CartesianCuboid::from_boundaries_and_interaction_range / _and_n_voxels
  // (cellular_raza-building-blocks/src/domains/cartesian_cuboid_n.rs:183-256).
  crg::SimDev S;
  memset(&S, 0, sizeof(S));
  S.dim = d->dim;
  S.nvox[0] = S.nvox[1] = S.nvox[2] = 1;
  uint64_t total = 1;
  for (int a = 0; a < d->dim; ++a) {
    if (!(d->min[a] < d->max[a])) return CRG_EBOUNDARY;
    S.min[a] = d->min[a];
    S.max[a] = d->max[a];
    uint64_t nv;
    if (d->voxel_mode == 0) {
      if (!(d->interaction_range > 0.0)) return CRG_EINVAL;
      const double f = floor((d->max[a] - d->min[a]) / d->interaction_range);
      if (!(f > -1.0 && f < 18446744073709551616.0)) return CRG_EBOUNDARY;
      nv = (uint64_t)f < 1 ? 1 : (uint64_t)f;
      S.dx[a] = (d->max[a] - d->min[a]) / f;
    } else {
      if (d->n_voxels[a] <= 0) return CRG_EINVAL;
      nv = (uint64_t)d->n_voxels[a];
      S.dx[a] = (d->max[a] - d->min[a]) / (double)nv;
    }
    S.inv_dxf[a] = (float)(1.0 / S.dx[a]);
    if (nv > kNaMaxVoxels) return CRG_EINVAL;
    total *= nv;
    if (total > kNaMaxVoxels) return CRG_EINVAL;
    S.nvox[a] = (int32_t)nv;
  }
  S.n_vox = (uint32_t)total;

  // One-time set-up per device: the device address of the scratch array.
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNaMaxDevices) return CRG_ECUDA;
  void *base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
      void *p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return CRG_ECUDA;
      g_noalloc_ptr[dev] = p;
    }
    base = g_noalloc_ptr[dev];
  }
  unsigned char *b = static_cast<unsigned char *>(base);
  uint32_t *count = reinterpret_cast<uint32_t *>(b + kNaCountOff);
  uint32_t *bsum = reinterpret_cast<uint32_t *>(b + kNaBsumOff);
  uint64_t *tmp = reinterpret_cast<uint64_t *>(b + kNaTmpOff);
  int32_t *status = reinterpret_cast<int32_t *>(b + kNaStatusOff);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const uint32_t un = (uint32_t)n, nvox = S.n_vox;

  // The histogram and the status word must start at zero; the slot keys are fully
  // rewritten by the scatter.
  if (cudaMemsetAsync(count, 0, sizeof(uint32_t) * ((size_t)nvox + 1), st) != cudaSuccess ||
      cudaMemsetAsync(status, 0, sizeof(int32_t) * 4, st) != cudaSuccess)
    return CRG_ECUDA;
  if (un) {
    const unsigned grid = (un + 255) / 256;
    if (S.dim == 3)
      k_noalloc_keys<3><<<grid, 256, 0, st>>>(S, un, pos_dev, voxel_out, count, status);
    else
      k_noalloc_keys<2><<<grid, 256, 0, st>>>(S, un, pos_dev, voxel_out, count, status);
  }
  crg::SortArgs A;
  memset(&A, 0, sizeof(A));
  A.n_sims = 1;
  A.nc = S.dim;
  A.initial = 1;
  A.cap = (int64_t)n;
  A.n_agents = un;
  A.n_vox = nvox;
  A.nkey = voxel_out;
  A.count = count;
  A.start = start_out;
  A.tmp = tmp;
  A.status = status;
  const uint32_t nb = (nvox + crg::kScanTile - 1) / crg::kScanTile;
  crg::k_scan_reduce<<<nb, crg::kScanThreads, 0, st>>>(count, nvox, bsum, nullptr, nullptr,
                                                       nullptr);
  crg::k_scan_blocks<<<1, crg::kScanThreads, 0, st>>>(bsum, nb, start_out, nvox);
  crg::k_scan_final<<<nb, crg::kScanThreads, 0, st>>>(count, nvox, bsum, start_out);
  if (un) crg::k_scatter<<<(un + 255) / 256, 256, 0, st>>>(A);
  crg::k_segsort<<<(nvox + crg::kSegThreads - 1) / crg::kSegThreads, crg::kSegThreads, 0, st>>>(A);
  if (un) k_noalloc_order<<<(un + 255) / 256, 256, 0, st>>>(tmp, un, order_out);
  if (cudaGetLastError() != cudaSuccess) return CRG_ECUDA;
  int32_t h_status[4] = {0, 0, 0, 0};
  if (cudaMemcpyAsync(h_status, status, sizeof(h_status), cudaMemcpyDeviceToHost, st) !=
          cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return CRG_ECUDA;
  return h_status[0];
}
