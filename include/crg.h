/*
 * crg.h -- C ABI of the GB300 mechanics/interaction backend for cellular_raza's chili loop.
 *
 * One handle runs one or more independent simulations ("a pack") on the current CUDA
 * device.  A step is the chili Mechanics+Interaction step:
 *   update_mechanics_interaction_step_1/2/3   (cellular_raza-core/src/backend/chili/
 *                                              update_mechanics.rs:153-382)
 *   local_mechanics_update                    (update_mechanics.rs:530-559)
 *   apply_boundary                            (update_mechanics.rs:387-406)
 *   sort_cells_in_voxels_step_1/2             (update_mechanics.rs:418-513)
 * with NewtonDamped{2,3}D + MorsePotential spheres or RodMechanics + RodInteraction<Morse>
 * rods on a CartesianCuboid with reflecting walls.
 *
 * Conventions: every call returns a status (CRG_OK = 0, else one of CRG_E*); the caller
 * owns every host array and no pointer is retained past a call; the library owns device
 * memory for the lifetime of the handle.  A handle is single-threaded; different handles
 * may be used from different threads.  Nothing here aborts or traps.
 *
 * Host arrays of positions/velocities are agent-major: [n][n_vertices][dim] doubles
 * (n_vertices = 1 for spheres), matching RodMechanics::pos rows
 * (cellular_raza-building-blocks/src/cell_building_blocks/bacterial_rods.rs:82-107) and
 * NewtonDamped::pos (mechanics.rs:14-80).
 */
#ifndef CRG_H
#define CRG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The first five mirror chili's SimulationError variants
 * (cellular_raza-core/src/backend/chili/errors.rs:73-122). */
#define CRG_OK 0
#define CRG_ECALC 1       /* CalcError */
#define CRG_EBOUNDARY 2   /* BoundaryError (agent left the domain after reflection) */
#define CRG_EINDEX 3      /* IndexError (agent outside every voxel at insertion) */
#define CRG_EDECOMPOSE 4  /* DecomposeError (n_subdomains cannot split the voxels) */
#define CRG_EINVAL 5      /* invalid argument */
#define CRG_ENOMEM 6      /* device allocation failed / admission budget exceeded */
#define CRG_ECUDA 7       /* CUDA runtime error */
#define CRG_ETIMEDOUT 8   /* bounded device-side wait expired */
#define CRG_ENOTSUP 9     /* feature outside what this library supports */
#define CRG_EINTERNAL 10  /* a device-side invariant check failed; the access was skipped
                             (crg_last_error: agent = index, step = check site) */

#define CRG_KIND_SPHERE 0   /* NewtonDamped{2,3}D + MorsePotential */
#define CRG_KIND_ROD 1      /* RodMechanics<f64,D> + RodInteraction<MorsePotential> */
#define CRG_KIND_BROWNIAN 2 /* Brownian{2,3}D + MorsePotential (mechanics.rs:228-374) */
#define CRG_KIND_LANGEVIN 3 /* Langevin{2,3}D + MorsePotential (mechanics.rs:376-475) */
/* Stochastic mechanics (Brownian, Langevin, RodMechanics with diffusion != 0) draw their
 * Wiener increments from a counter-based stream: Philox4x32-10 keyed by rng_seed, counter
 * (draw, pack step, agent id), Box-Muller normals.  The reference's per-voxel ChaCha8
 * streams (chili/datastructures.rs:180-182) are replaced, so results match the reference
 * in distribution, and a simulation's random stream does not depend on its voxel, its
 * subdomain or its batch neighbours. */

#define CRG_PREC_F64 0    /* every operation in FP64, in the reference's order */
#define CRG_PREC_MIXED 1  /* FP32 pair forces with Kahan sums; FP64 state and update
                           * (spheres, Brownian, Langevin and rods; not with the cell cycle,
                           * CRG_ENOTSUP) */

#define CRG_WEIGHTS_CHILI 0    /* chili's subdomain-dependent pair weights (default) */
#define CRG_WEIGHTS_PHYSICAL 1 /* every pair with weight 1 (not reference behaviour) */

/* CartesianCuboid (cellular_raza-building-blocks/src/domains/cartesian_cuboid_n.rs:65-72)
 * plus chili's Settings::n_threads (cellular_raza-core/src/backend/chili/setup.rs:17-27),
 * which sets the number of subdomains and with it chili's pair weights. */
typedef struct crg_domain {
  int32_t dim;        /* 2 or 3 */
  int32_t voxel_mode; /* 0: from_boundaries_and_interaction_range (:183-222)
                         1: from_boundaries_and_n_voxels (:226-256) */
  double min[3];
  double max[3];
  double interaction_range; /* voxel_mode 0 */
  int64_t n_voxels[3];      /* voxel_mode 1 */
  int32_t n_subdomains;     /* chili n_threads (>= 1) */
  int32_t weight_mode;      /* CRG_WEIGHTS_* */
} crg_domain;

/* Agent model: Mechanics + Interaction parameters shared by every agent of a simulation.
 *   spheres: NewtonDamped (mass, damping) + MorsePotential (radius, stiffness = potential_
 *            stiffness, cutoff, strength)  (mechanics.rs:14-204, interaction.rs:184-299)
 *   rods:    RodMechanics (spring_tension, rigidity, spring_length, damping, diffusion)
 *            + RodInteraction(MorsePotential)  (bacterial_rods.rs:82-337)
 * solver_order is run_simulation!'s mechanics_solver_order (1 Euler, 2 AB2, 3 AB3;
 * cellular_raza-core-proc-macro/src/kwargs.rs:219-230). */
typedef struct crg_model {
  int32_t kind;         /* CRG_KIND_* */
  int32_t n_vertices;   /* rods: vertices per rod (2..8); spheres: 1 */
  int32_t solver_order; /* 1, 2 or 3 */
  int32_t precision;    /* CRG_PREC_* */
  double mass, damping;
  double spring_tension, rigidity, spring_length, diffusion;
  double radius, stiffness, cutoff, strength;
  double dt;
  double kb_temperature; /* Brownian / Langevin k_B T */
  uint64_t rng_seed;     /* seed of the stochastic mechanics' random stream */
  /* Cell cycle (rods, single-simulation handles; 0 = off): the bacterial-rods agent's
   * Cycle + NeighborSensing (cellular_raza-examples/bacterial_rods/src/main.rs:48-112).
   * Each step every rod counts the vertex pairs it shares with the agents it meets that
   * are closer than sense_range (n); its growth rate becomes growth_rate * (sense_saturation
   * - n) / sense_saturation, at least 0, when n > 0, else growth_rate; its spring length
   * grows by rate * dt, and past division_length it divides (RodMechanics::divide with the
   * Morse radius, bacterial_rods.rs:586-663).  Agent counts then change from step to step. */
  int32_t cycle;
  double growth_rate, division_length, sense_range, sense_saturation;
} crg_model;

/* Identifiers of agents made or renamed by a division: chili's CellIdentifier::Division(
 * voxel plain index, voxel counter) (cellular_raza-concepts/src/cell.rs:18-25, chili/
 * update_cycle.rs:30-64), encoded as CRG_ID_DIVISION | voxel << 32 | counter.  Initial
 * agents keep the ids given to crg_upload and have parent CRG_NO_PARENT. */
#define CRG_ID_DIVISION (1ull << 63)
#define CRG_NO_PARENT (~0ull)

typedef struct crg_ctx crg_ctx;

/* Creates a handle for one simulation with room for `capacity` agents.
 * Replaces construct_simulation_runner (chili/datastructures.rs:51-217). */
int32_t crg_create(const crg_domain *domain, const crg_model *model, int64_t capacity,
                   crg_ctx **out);

/* Creates a handle for `n_sims` independent simulations stepped by the same launches
 * (batched form).  All models share kind, n_vertices, dim, precision and solver_order;
 * parameters, domains and agent counts may differ.  capacities[s] bounds sim s. */
int32_t crg_create_batch(int32_t n_sims, const crg_domain *domains, const crg_model *models,
                         const int64_t *capacities, crg_ctx **out);

/* Copies agents in from host memory and sorts them into voxels.  `ids` may be NULL
 * (then agent k gets id k, like CellIdentifier::Initial(k)).  For a batch handle,
 * counts[s] agents of sim s follow each other in the arrays (pass n = sum(counts));
 * for a single handle pass counts = NULL.  Replaces Domain::decompose +
 * insert_initial_cells (concepts-derive/src/domain.rs:292-400,
 * chili/datastructures.rs:278-299): an agent with pos <= min on some axis is
 * CRG_EBOUNDARY, one outside every voxel CRG_EINDEX. */
int32_t crg_upload(crg_ctx *ctx, int64_t n, const int64_t *counts, const double *pos,
                   const double *vel, const uint64_t *ids);

/* Advances every simulation of the handle by n_steps chili steps (the macro-generated
 * loop body, cellular_raza-core-proc-macro/src/run_sim.rs:380-403).  Stops at the first
 * device-reported error and returns it; crg_last_error gives the agent and the step.
 * The step that fails is not committed for the simulation that raised the error, and later
 * steps leave that simulation unchanged (chili stops a run at its first error,
 * chili/errors.rs:73-122): a single-simulation handle then holds the state after its last
 * successful step, which crg_step_count reports.  crg_clear_error lets it continue. */
int32_t crg_step(crg_ctx *ctx, int64_t n_steps);

/* Interaction forces without a step: the per-agent force that chili's
 * update_mechanics_interaction_step_1/2/3 accumulate into AuxStorageMechanics::current_force
 * (cellular_raza-core/src/backend/chili/update_mechanics.rs:153-382, add_force in
 * chili/aux_storage.rs:120-129), with chili's pair weights for the handle's n_subdomains.
 * pos: [n][n_vertices][dim] doubles (n_vertices = 1 for point agents) listing the agents of
 * every voxel in the order that voxel's Vec holds them (voxels in any order); force receives
 * [n][n_vertices][dim] in the same order.  This is the body of a step-1 hook
 * (run_simulation!'s update_mechanics_interaction_step_1 kwarg, cellular_raza-core-proc-macro/
 * src/run_sim.rs:150-157,251-256) for a chili run with one subdomain: the hook adds the
 * forces to each cell's aux storage and chili's own local_mechanics_update, apply_boundary
 * and re-sort run unchanged.  The handle's agents are replaced by these (as crg_upload with
 * zero velocities).  Single-simulation handles without a cell cycle; otherwise CRG_ENOTSUP. */
int32_t crg_forces(crg_ctx *ctx, int64_t n, const double *pos, double *force);

/* Copies the current agents out in cell-list order (sorted by voxel).  Any pointer may be
 * NULL.  voxel receives the voxel plain index (per simulation). */
int32_t crg_download(crg_ctx *ctx, double *pos, double *vel, uint64_t *ids, uint32_t *voxel);

/* ---- continuous batching --------------------------------------------------------------
 * chili runs one simulation per run_simulation! call; serving many requests needs three more
 * primitives (no counterpart in the reference beyond the per-simulation semantics above). */

/* A simulation whose pack step counter reaches stop_step is frozen: later steps leave its
 * state untouched, so one launch can carry simulations that need different step counts. */
int32_t crg_set_sim_stop(crg_ctx *ctx, int32_t sim, int64_t stop_step);

/* Steps the handle has run since its creation or last upload (its step counter). */
int32_t crg_step_count(crg_ctx *ctx, int64_t *steps);

/* Agents of one simulation of the handle (cell-list order), like crg_download. */
int32_t crg_sim_download(crg_ctx *ctx, int32_t sim, int64_t *n, double *pos, double *vel,
                         uint64_t *ids);

/* Returns the handle's error code, stores the index of the simulation that raised it in
 * *sim and clears it so the other simulations can continue. */
int32_t crg_clear_error(crg_ctx *ctx, int32_t *sim);

/* New handle = simulations `keep[0..n_keep)` of `src` with their device-resident state
 * (cell-list order, solver history; copied device to device) + n_new simulations from
 * host memory (agents of all new simulations back to back, like crg_upload).  In the new
 * handle the new simulations come first (indices 0..n_new-1), then the kept ones in the
 * order given; the step counter starts at 0 and every stop step is unset.  `src` is left
 * unchanged (destroy it when done). */
int32_t crg_repack(crg_ctx *src, int32_t n_keep, const int32_t *keep, int32_t n_new,
                   const crg_domain *new_domains, const crg_model *new_models,
                   const int64_t *new_caps, const int64_t *new_counts, const double *new_pos,
                   const double *new_vel, crg_ctx **out);

/* ---- serving ----------------------------------------------------------------------------
 * A request server keeps many simulations resident on the device and advances them together
 * (continuous batching): requests are admitted first-come first-served while their
 * estimated device footprint fits `hbm_budget_bytes`, counting the transient copy of a
 * class's unfinished simulations that a pack rebuild holds (so the device never holds more
 * than the budget); admitted simulations join the running pack of their class (kind, dim,
 * vertices, precision, solver order) without moving the running ones off the device
 * (crg_repack); every simulation stops exactly after its own number of steps
 * (crg_set_sim_stop); the packs advance `steps_per_tick` steps between admissions, each on
 * its own stream, all of them enqueued before the server waits for any, so different classes
 * overlap on the device.  A result is bit-identical to running the same simulation alone.
 * A request whose footprint exceeds half the budget is refused at submit (CRG_ENOMEM).
 * One background thread drives the device; submit/wait are thread-safe. */
typedef struct crg_server crg_server;
int32_t crg_server_create(int64_t hbm_budget_bytes, int32_t steps_per_tick, crg_server **out);
/* Queues one simulation (inputs copied; n agents [n][nv][dim]); returns a ticket. */
int32_t crg_server_submit(crg_server *srv, const crg_domain *domain, const crg_model *model,
                          int64_t n, const double *pos, const double *vel, int64_t n_steps,
                          uint64_t *ticket);
/* Waits up to timeout_s (< 0: forever) for a ticket; on completion copies its final state
 * (cell-list order, ids give the input index) and the submit-to-completion latency, and
 * forgets the ticket.  Returns the request's status, or CRG_ETIMEDOUT. */
int32_t crg_server_wait(crg_server *srv, uint64_t ticket, double timeout_s, int64_t *n,
                        double *pos, double *vel, uint64_t *ids, double *latency_s);
int32_t crg_server_stats(crg_server *srv, int64_t *queued, int64_t *active, int64_t *completed,
                         int64_t *bytes_in_use, int64_t *agent_steps);
int32_t crg_server_destroy(crg_server *srv);

/* Number of agents currently held (total over simulations of a batch). */
int32_t crg_agent_count(crg_ctx *ctx, int64_t *n);

/* Cell cycle: per-rod spring lengths in the order of the arrays given to the last
 * crg_upload (call after it and before stepping; default: the model's spring_length). */
int32_t crg_set_spring_lengths(crg_ctx *ctx, const double *spring_length);

/* Cell cycle: per-agent spring length, growth rate and parent identifier, in the order
 * of crg_download.  Any pointer may be NULL.  A step whose divisions would take the agent
 * count past the handle's capacity first grows the handle (at least twice the capacity,
 * state moved through a checkpoint, the same stream) and then takes the step, as chili's
 * growable Vecs do; CRG_ENOMEM only when that allocation fails.  A DivisionError is
 * CRG_ECALC. */
int32_t crg_download_cycle(crg_ctx *ctx, double *spring_length, double *growth_rate,
                           uint64_t *parent);

/* First error seen on the device: code, agent id and 1-based step (or -1). */
int32_t crg_last_error(crg_ctx *ctx, int64_t *agent, int64_t *step);

/* Device-side checkpoint of the whole handle state (cell list, velocities, solver history,
 * step counter): CRG_SNAPSHOT_SAVE copies it into a second device buffer (allocated on the
 * first save), CRG_SNAPSHOT_RESTORE copies it back.  chili has no checkpoint (planned,
 * cellular_raza-core/src/lib.rs:14-22); its save points (chili/datastructures.rs:349-396)
 * persist the same state. */
#define CRG_SNAPSHOT_SAVE 0
#define CRG_SNAPSHOT_RESTORE 1
int32_t crg_snapshot(crg_ctx *ctx, int32_t op);

/* Host checkpoint of the handle's simulation state: positions, velocities, ids, the cell
 * list in its storage order, FP32 offsets, solver history, the step counter, and per
 * simulation its agent range, stop step and own step count; with the cell cycle also every
 * rod's spring length, growth rate and parent and every voxel's division counter.  crg_checkpoint_size gives the bytes needed;
 * crg_checkpoint_save writes them to host memory; crg_checkpoint_load, on a handle created
 * with the same domains, models and capacities (a fresh one, or the same one later),
 * restores the state so that stepping continues bit for bit as if it had not stopped.
 * The blob starts with a header that load checks (magic, version, kind, dimension,
 * vertices, solver order, simulation and voxel counts, and a hash of every field of the
 * domains, models and capacities); load also checks the cell starts (monotone, from 0 to
 * the agent count, each simulation's first voxel at its first agent) before any copy.  Replaces nothing in the
 * reference: chili's save points store cells through serde for analysis, and resuming a
 * run from them is not implemented there (cellular_raza-core/src/lib.rs:14-22). */
int32_t crg_checkpoint_size(crg_ctx *ctx, int64_t *bytes);
int32_t crg_checkpoint_save(crg_ctx *ctx, void *buf, int64_t bytes);
int32_t crg_checkpoint_load(crg_ctx *ctx, const void *buf, int64_t bytes);

/* The CUDA stream (cudaStream_t) every launch of the handle is issued on, for callers that
 * order their own work or events against it. */
int32_t crg_get_stream(crg_ctx *ctx, void **stream);

/* Autotuner: times `steps` steps of every force-kernel shape this handle can use (kernel
 * variant x block size x tile, the tile for the persistent sphere kernel) on the handle's
 * current state, restoring that state after each trial (crg_snapshot), and keeps the
 * fastest: *variant and *block receive the chosen CRG_OPT_KERNEL_VARIANT / CRG_OPT_BLOCK
 * values, *ms_per_step its time; the chosen CRG_OPT_TILE is read with crg_get_option.  The
 * simulation state is unchanged on return.  Cell-cycle handles: the rod walk and kernel
 * shapes, each trial started from a host checkpoint and timed on the host clock. */
int32_t crg_autotune(crg_ctx *ctx, int64_t steps, int64_t *variant, int64_t *block,
                     double *ms_per_step);

/* Destroys the handle and frees its device memory. */
int32_t crg_destroy(crg_ctx *ctx);

/* Human-readable name of a status code (static string). */
const char *crg_strerror(int32_t code);

/* ---- options and diagnostics ------------------------------------------------------- */
#define CRG_OPT_PREFILTER 1  /* 1 (default): FP32 candidate prefilter on; 0: off */
#define CRG_OPT_GRAPH_CHUNK 2 /* steps per captured CUDA graph (0 disables graphs) */
#define CRG_OPT_BLOCK 3       /* threads per block of the force kernel (autotuner); rods'
                              * pass list: 32 walks with a warp per rod, 128 with a thread
                              * per rod, 0 by size (a warp per rod up to 16,384 rods) */
int32_t crg_set_option(crg_ctx *ctx, int32_t option, int64_t value);
/* The current value of an option (CRG_OPT_PASS_LIST: the pass list's capacity in passes;
 * CRG_OPT_DEBUG_FORCES: 1 while forces are captured).  CRG_EINVAL for an unknown option. */
int32_t crg_get_option(crg_ctx *ctx, int32_t option, int64_t *value);

/* Interaction force accumulated during the most recent step, [n][nv][dim] in the order
 * of the ids array (same layout as crg_download's ids).  Capture must have been enabled
 * with crg_set_option(ctx, CRG_OPT_DEBUG_FORCES, 1) before that step. */
#define CRG_OPT_DEBUG_FORCES 5
/* Force kernel: 0 (default) automatic; 1 one thread per agent (the simple reference
 * formulation).  FP64 rods: 0 = pass list (walk, pass kernel, bend, update), 1 thread per
 * rod (also the pass list's overflow fallback); mixed rods always run the pass list.  FP64
 * spheres: 0 = agent groups up to 38,912
 * agents, lane per agent above; 2 agent groups (CRG_OPT_BLOCK 16 or 32: lanes per agent,
 * else 8); 3 lane per agent (warp-packed survivors;
 * CRG_OPT_BLOCK 64 scans 64 candidates per lane and round instead of 32).  Mixed spheres:
 * 3 lane per agent (warp-packed survivors), else one thread per agent.  All variants of one
 * precision produce identical results. */
#define CRG_OPT_KERNEL_VARIANT 6
/* Rods, default kernel: capacity of the pass list in passes (one pass = one candidate pair
 * half, about 11 per rod in a dense 2D colony).  A step whose list does not fit computes its
 * forces with the rod-level kernel instead (same results) and the list is grown to fit at
 * the end of crg_step.  Created with 12 passes per rod of capacity. */
#define CRG_OPT_PASS_LIST 7
/* Spheres, thread-per-agent kernel (CRG_OPT_KERNEL_VARIANT 1, or the mixed default): 0
 * (default) one thread per agent in a grid over all agents; k in 1..16 the persistent form,
 * as many blocks as the SMs hold at once (CRG_OPT_BLOCK threads, a multiple of 64; 128 when
 * 0), each claiming tiles of CRG_OPT_BLOCK x k consecutive agents of the cell list until
 * none is left.  The results do not depend on it. */
#define CRG_OPT_TILE 8
int32_t crg_debug_forces(crg_ctx *ctx, double *force, uint64_t *ids);

/* Neighbour statistics of the CURRENT cell list (what the next step will visit): per agent
 * the number of candidate partners in its 3^D voxel neighbourhood, the number with
 * 0 < d <= cutoff (spheres), and a sum of splitmix64(id) over the candidates; in the order
 * of ids. */
int32_t crg_debug_neighbor_stats(crg_ctx *ctx, uint32_t *n_cand, uint32_t *n_inter,
                                 uint64_t *cand_hash, uint64_t *ids);

/* Device time of the kernels of the last crg_step call, split by phase (ms):
 * [0] force+update, [1] sort; [2] number of kernels launched; [3] the dominant force
 * kernel alone (rods: the pass kernel; spheres: the force kernel); [4] the rod update
 * kernel alone (pass-list rod path; else 0).  Requires CRG_OPT_PROFILE = 1: the steps still
 * run from captured CUDA graphs, which then carry event nodes between the phases, and the
 * host reads the times after every chunk of 32 steps. */
#define CRG_OPT_PROFILE 4
int32_t crg_profile(crg_ctx *ctx, double *out5);

/* Measures the FP64 and FP32 fused-multiply-add throughput of the current device with a
 * dependent-chain microbenchmark (TFLOP/s, 2 flops per FMA). */
int32_t crg_measure_fma_peaks(double *fp64_tflops, double *fp32_tflops);

/* Checks the FP64 rod pass kernel's division (a quotient from b's correctly rounded
 * reciprocal, with FMA residual corrections) against the IEEE division on n generated
 * operand pairs: rod-like values, random exponents across the fast path's range, quotients
 * next to rounding midpoints, all-ones and power-of-two divisors.  *mismatches receives
 * the pairs whose bits differ (0 expected), *fast the pairs that took the fast path. */
int32_t crg_check_division(int64_t n, uint64_t seed, int64_t *mismatches, int64_t *fast);

/* ---- cell list without device allocation -------------------------------------------
 * No counterpart in the reference: chili keeps its cells in per-voxel Vecs and never
 * builds a device cell list.
 *
 * Builds the voxel index and the cell list of n points that already live in device
 * memory, using only the caller's buffers and a scratch area compiled into this library
 * (a fixed device array of about 12.6 MB, present on every GPU that loads the library
 * until the process exits).  It calls no cudaMalloc/cudaFree and no allocating library
 * routine.  It is meant for callers that cannot allocate device memory at this point:
 * a host whose device memory is owned by its own arena or pool (a Rust caller managing
 * memory through its own allocator), a serving loop whose HBM budget is fully committed to
 * admitted jobs, or a latency-critical loop that must not pay for cudaMalloc/cudaFree,
 * which can synchronise the whole device.
 *
 *   pos_dev    device, component-major [dim][n] doubles (point i, axis a at a * n + i)
 *   voxel_out  device [n]: voxel plain index of point i, with the insertion rules of
 *              crg_upload (pos <= min on some axis: CRG_EBOUNDARY; outside every voxel:
 *              CRG_EINDEX; the first offending point index is not reported)
 *   order_out  device [n]: the point index held by each slot of the cell list (voxels
 *              ascending, input order inside a voxel) -- the order crg_upload produces
 *   start_out  device [n_voxels + 1]: first slot of every voxel, start_out[n_voxels] = n
 *   stream     cudaStream_t to run on (NULL: the default stream); the call synchronizes
 *              it before returning (it reads the status word back), so it cannot be
 *              called while that stream is being captured
 *
 * Limits: n <= CRG_NOALLOC_MAX_POINTS and n_voxels <= CRG_NOALLOC_MAX_VOXELS, otherwise
 * CRG_EINVAL before anything runs.  All calls share the scratch array: calls that overlap
 * on the GPU (different streams or threads at the same time) race and must be serialised
 * by the caller.  The first call on a device looks up the scratch address on that device
 * (cudaGetSymbolAddress). */
#define CRG_NOALLOC_MAX_POINTS (1 << 20)
#define CRG_NOALLOC_MAX_VOXELS (1 << 20)
int32_t crg_cell_list_noalloc(const crg_domain *domain, int64_t n, const double *pos_dev,
                              uint32_t *voxel_out, uint32_t *order_out, uint32_t *start_out,
                              void *stream);

#ifdef __cplusplus
}
#endif
#endif /* CRG_H */
