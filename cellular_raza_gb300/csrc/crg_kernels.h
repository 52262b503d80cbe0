// crg_kernels.h -- host-side launch wrappers shared between the crg translation units.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace crg {

struct SimDev;
struct PackArgs;

// Arguments of the cell-list kernels (crg_sort.cu).
struct SortArgs {
  const SimDev *sims;
  const uint32_t *sim_agent_off;  // [n_sims + 1]
  const uint32_t *sim_of_voxel;   // [n_vox] (batch handles only)
  int32_t n_sims;
  int32_t nc;      // components per agent (n_vertices * dim)
  int32_t initial; // 1 for the insertion sort after crg_upload (every agent class 0)
  int64_t cap;
  uint32_t n_agents;
  uint32_t n_vox;
  // sorted state (written by the gather)
  double *pos, *vel;
  uint64_t *id;
  uint32_t *key;
  float *off;
  int32_t off_aos;     // spheres: floats per agent of the interleaved offsets (4 in 3D, 2 in
                       // 2D); 0: component-major [nc][cap] (rods)
  const double *vcen;  // voxel centres per simulation and axis (SimDev::cen_off)
  double *hist;
  uint8_t *hmeta;
  // updated state in the previous order (read by the gather)
  const double *npos, *nvel;
  const uint64_t *nid;
  uint32_t *nkey;
  const double *nhist;
  const uint8_t *nhmeta;
  // scratch
  uint32_t *count;  // [n_vox]
  uint32_t *start;  // [n_vox + 1]
  uint64_t *tmp;    // [cap]
  int32_t *status;
  int64_t *step_ctr;
  // cell cycle (null when off): per-agent state moved with the agents, and the rank of
  // each agent in chili's pre-sort order when divisions inserted daughters (else the
  // agent's index is its rank)
  double *slen, *grate;
  uint64_t *parent;
  const double *nslen, *ngrate;
  const uint64_t *nparent;
  const uint32_t *srank;
};

// Copy of kept simulations from one pack into the "next" arrays of another (crg_repack).
struct RepackArgs {
  const double *spos, *svel, *shist;
  const uint64_t *sid;
  const uint32_t *skey;
  const uint8_t *shmeta;
  int64_t scap;
  double *dpos, *dvel, *dhist;
  uint64_t *did;
  uint32_t *dkey;
  uint8_t *dhmeta;
  uint32_t *dcount;
  int64_t dcap;
  int32_t nc, has_hist, n_keep;
  const uint32_t *dst_off;   // [n_keep + 1] destination agent offsets
  const uint32_t *src_off;   // [n_keep]     source agent offsets
  const int64_t *key_shift;  // [n_keep]     destination minus source voxel offset
  uint32_t first, last;      // destination index range of the kept agents
};
void launch_repack(const RepackArgs &A, cudaStream_t st);

void launch_sort(const SortArgs &A, uint32_t *bsum, cudaStream_t st);
// Exclusive prefix sum of count[0..n) into start[0..n] (start[n] = total); zeroes count.
// bsum: n / 4096 + 2 entries.
void launch_scan(uint32_t *count, uint32_t n, uint32_t *start, uint32_t *bsum,
                 cudaStream_t st);
int sort_kernel_count(uint32_t n_vox);  // kernels one launch_sort issues
void launch_init_keys(const SortArgs &A, int nv, cudaStream_t st);
void launch_transpose_in(const double *src, double *dst, uint32_t n, int nc, int64_t cap,
                         cudaStream_t st);
void launch_transpose_out(const double *src, double *dst, uint32_t n, int nc, int64_t cap,
                          cudaStream_t st);
// Cell-list values [nc][cap] -> agent-major rows in the order of the upload that built the
// cell list (through the insertion sort's slot table tmp).
void launch_unsort_out(const double *src, const uint64_t *tmp, double *dst, uint32_t n, int nc,
                       int64_t cap, int32_t *status, cudaStream_t st);

// Force + integrator + boundary + next voxel key (+ histogram) for one step.
void launch_spheres_step(int dim, int precision, const PackArgs &P, int block, cudaStream_t st);
// k0 / k1 (optional) are recorded on st right before and after the dominant force kernel,
// k2 / k3 around the update kernel of the pass-list path.
void launch_rods_step(int dim, int nv, int precision, const PackArgs &P, int block,
                      cudaStream_t st, cudaEvent_t k0 = nullptr, cudaEvent_t k1 = nullptr,
                      cudaEvent_t k2 = nullptr, cudaEvent_t k3 = nullptr);
int prepare_rods(int dim, int nv);  // 0 on success
int prepare_spheres(int dim, int precision);  // 0 on success
// Cell cycle of rods: neighbour counts of this step (before the update kernel), and after
// the update and the scan of its division flags, the divisions (n_div > 0), then the voxel
// counters (launched once the divisions are known to have succeeded).
void launch_rods_sense(int dim, int nv, const PackArgs &P, cudaStream_t st);
void launch_rods_divide(int dim, int nv, const PackArgs &P, uint32_t n_div, cudaStream_t st);
void launch_cycle_counters(const PackArgs &P, cudaStream_t st);
// Voxel counters from the first cell list; per-agent values from upload order to the cell
// list through the upload sort's slot table (tmp).
void launch_cycle_init(const PackArgs &P, cudaStream_t st);
void launch_cycle_permute(double *dst, const double *src, const uint64_t *tmp, uint32_t n,
                          cudaStream_t st);
// Diagnostics over the current cell list.
void launch_neighbor_stats(int dim, int nv, const PackArgs &P, uint32_t *n_cand,
                           uint32_t *n_inter, uint64_t *hash, cudaStream_t st);

int measure_fma_peaks(double *fp64_tflops, double *fp32_tflops);
int check_division(int64_t n, uint64_t seed, int64_t *mismatches, int64_t *fast);

}  // namespace crg
