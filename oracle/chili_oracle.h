/*
 * chili_oracle.h -- C ABI of the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain C++ restatement of cellular_raza's
 * chili mechanics/interaction step (cellular_raza-core/src/backend/chili) with the
 * building blocks it calls (NewtonDamped, MorsePotential, RodMechanics,
 * RodInteraction, CartesianCuboid).  It exists to check the CUDA path and to
 * provide the timed CPU baseline.  Nothing in the product links or calls it.
 *
 * The reference is Rust and cannot be compiled in this environment (no cargo,
 * no vendored crates), so parity is anchored on this restatement plus the
 * known-answer tests the reference ships (doc tests and unit tests, see
 * tests/test_oracle.py).
 */
#ifndef CHILI_ORACLE_H
#define CHILI_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Agent kinds. */
#define OR_KIND_SPHERE 0   /* NewtonDamped{2,3}D + MorsePotential            */
#define OR_KIND_ROD 1      /* RodMechanics<f64,D> + RodInteraction<Morse>      */
#define OR_KIND_BROWNIAN 2 /* Brownian{2,3}D + MorsePotential (mechanics.rs:228-374) */
#define OR_KIND_LANGEVIN 3 /* Langevin{2,3}D + MorsePotential (mechanics.rs:376-475) */

/* Status codes (mirror chili's SimulationError variants). */
#define OR_OK 0
#define OR_ECALC 1
#define OR_EBOUNDARY 2
#define OR_EINDEX 3
#define OR_EDECOMPOSE 4
#define OR_EINVAL 5

typedef struct or_config {
  int32_t dim;          /* 2 or 3 */
  int32_t kind;         /* OR_KIND_* */
  int32_t n_vertices;   /* rods: vertices per rod; spheres: 1 */
  int32_t solver_order; /* run_simulation! mechanics_solver_order: 1 Euler, 2 AB2, 3 AB3 */
  int32_t n_subdomains; /* chili Settings::n_threads (one worker thread each) */
  int32_t voxel_mode;   /* 0: from_boundaries_and_interaction_range, 1: from_boundaries_and_n_voxels */
  double min[3];
  double max[3];
  double interaction_range;
  int64_t n_voxels[3];
  /* mechanics */
  double mass;    /* NewtonDamped mass */
  double damping; /* NewtonDamped damping_constant / RodMechanics damping */
  double spring_tension, rigidity, spring_length, diffusion; /* RodMechanics */
  /* MorsePotential */
  double radius, stiffness, cutoff, strength;
  double dt;
  /* stochastic mechanics: Brownian / Langevin k_B T, and the seed of the random stream */
  double kb_temperature;
  uint64_t rng_seed;
} or_config;

/* Optional outputs describing the LAST step that was run. */
typedef struct or_debug {
  double *force_last;    /* [n][nv][dim]: interaction force accumulated in the last step */
  uint32_t *voxel_out;   /* [n]: voxel plain index after the last re-sort */
  uint32_t *n_cand;      /* [n]: candidate partners scanned in the last step */
  uint32_t *n_inter;     /* [n]: partners with 0 < d <= cutoff (spheres) */
  uint64_t *cand_hash;   /* [n]: sum of mix(id) over candidate partners */
  uint64_t *order_out;   /* [n]: agent ids in chili's storage order (voxels ascending,
                            each voxel's Vec order) after the last step */
  int64_t error_agent;   /* filled on error: agent id, else -1 */
  int64_t error_step;    /* filled on error: 1-based step, else -1 */
} or_debug;

/* Runs n_steps chili steps.  pos/vel are [n][nv][dim] in agent-id order (the agent id
 * is the input index, chili's CellIdentifier::Initial(n)); they are overwritten with
 * the final state.  Returns OR_OK or an error code. */
int32_t or_run(const or_config *cfg, int64_t n_agents, double *pos, double *vel,
               int64_t n_steps, or_debug *dbg, double *elapsed_s);

/* Cell cycle of the bacterial-rods agent (cellular_raza-examples/bacterial_rods/src/
 * main.rs:48-112): NeighborSensing counts vertex pairs of an agent and every partner it
 * meets that are closer than sense_range; react_to_neighbors sets the growth rate to
 * growth_rate * (sense_saturation - n) / sense_saturation (at least 0) when n > 0, else
 * growth_rate; Cycle::update_cycle grows the spring length by rate * dt and divides past
 * division_length with RodMechanics::divide (bacterial_rods.rs:586-663).  Daughters and
 * dividing parents get CellIdentifier::Division(voxel, counter), encoded as
 * OR_ID_DIVISION | voxel << 32 | counter; the parent of an initial agent is OR_NO_PARENT. */
#define OR_ID_DIVISION (1ull << 63)
#define OR_NO_PARENT (~0ull)

typedef struct or_cycle {
  double growth_rate, division_length, sense_range, sense_saturation;
  const double *spring_length_in; /* [n] initial spring lengths (NULL: cfg->spring_length) */
  int64_t cap_out;                /* room in the output arrays (agents) */
  int64_t n_out;                  /* agents after the run (also set when cap_out is short) */
  uint64_t *ids_out, *parent_out; /* [cap_out], chili's storage order */
  double *pos_out, *vel_out;      /* [cap_out][nv][dim] */
  double *spring_length_out, *growth_rate_out; /* [cap_out] */
  uint32_t *voxel_out;            /* [cap_out] */
  int64_t error_agent, error_step;
} or_cycle;

/* Runs n_steps chili steps of rods with the cell cycle (aspects Mechanics, Interaction,
 * Cycle, NeighborSensing).  Outputs in storage order; OR_EINVAL when cap_out is short. */
int32_t or_run_cycle(const or_config *cfg, or_cycle *cyc, int64_t n_agents,
                     const double *pos, const double *vel, int64_t n_steps);

/* The random stream of the stochastic mechanics (shared definition with the GPU path):
 * Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) and the standard normals drawn from it
 * for agent `id` at pack step `step`: n values, two per Philox block (Box-Muller). */
void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
void or_normals(uint64_t seed, uint64_t step, uint64_t id, int32_t n, double *out);

/* Domain helpers (known-answer tests). */
int32_t or_domain_voxels(const or_config *cfg, int64_t *n_voxels_out, double *dx_out);
int32_t or_get_decomp_res(uint64_t n_voxel, uint64_t n_regions, uint64_t *n, uint64_t *m,
                          uint64_t *average_len);
/* subdomain id per voxel plain index; out has prod(n_voxels) entries. */
int32_t or_subdomain_map(const or_config *cfg, uint32_t *out);
/* neighbours of one voxel (ascending plain index); returns the count (<= 26). */
int32_t or_voxel_neighbors(const or_config *cfg, uint64_t plain, uint64_t *out);
/* Initial voxel plain index of each agent (decompose + insert_initial_cells), or error. */
int32_t or_initial_voxels(const or_config *cfg, int64_t n_agents, const double *pos,
                          uint32_t *out);

/* Building blocks (known-answer tests). */
void or_nearest_point_from_point_to_line(int32_t dim, const double *point, const double *a,
                                         const double *b, double *dist, double *nearest,
                                         double *rel_length);
int32_t or_morse(int32_t dim, const double *own, const double *ext, double own_radius,
                 double ext_radius, double cutoff, double strength, double stiffness,
                 double *f_own, double *f_ext);
/* solvers.rs euler / adams_bashforth_2 / adams_bashforth_3 on scalars. */
double or_euler(double x, double dx, double dt, double dx_rand);
double or_adams_bashforth_2(double x, double dx0, double dx1, double dt, double dx_rand);
double or_adams_bashforth_3(double x, double dx0, double dx1, double dx2, double dt,
                            double dx_rand);

#ifdef __cplusplus
}
#endif
#endif
